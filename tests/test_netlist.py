"""The netlist reader (kronspice_gb300/netlist.py): SPICE text to the engine's
Circuit and analyses, as circuit.FromDeck builds them (circuit/builder.go:307),
without a GPU.  The reference's own netlists go through the same reader when the
golden fixtures are made (tests/golden/make_reference_fixtures.py)."""
import numpy as np
import pytest

from kronspice_gb300 import netlist
from kronspice_gb300 import circuit as kc

RC = """RC low-pass with a parameter and a subcircuit
.param rval = {2*500}
.subckt stage in out r=1k
R1 in out {r}
C1 out 0 10n
.ends
V1 in 0 DC 1 AC 1 PULSE(0 1 0 1u 1u 50u 100u)
X1 in mid stage r={rval}
RL mid 0 10k
.tran 1u 200u
.ac dec 10 10 1meg
.end
"""


def test_read_builds_the_circuit_and_analyses():
    ckt, an = netlist.read(RC)
    b = kc.Builder("ref")
    b.voltage_source("V1", "in", "0", 1.0, wave="pulse", args=[0, 1, 0, 1e-6, 1e-6, 50e-6, 100e-6], ac=(1.0, 0.0))
    b.resistor("R1", "in", "mid", 1e3).capacitor("C1", "mid", "0", 10e-9).resistor("RL", "mid", "0", 1e4)
    want = b.build()
    el, v, _ = ckt.pack()
    el2, v2, _ = want.pack()
    assert np.array_equal(el["kind"], el2["kind"]) and np.allclose(v, v2, rtol=1e-15)
    assert [a["kind"] for a in an] == ["tran", "ac"]
    assert an[0]["step"] == pytest.approx(1e-6) and an[0]["stop"] == pytest.approx(200e-6)
    assert an[1]["variation"] == "dec" and an[1]["fstop"] == pytest.approx(1e6)


def test_switch_and_nonlinear_reactive_lines():
    ckt, _ = netlist.read("""t
V1 c 0 DC 1
R1 c a 1k
S1 a 0 c 0 sw1 ON
CN a 0 Q=pwl(-1 -1u 0 0 1 1u) SCALE=SIN(1 0.2 1k)
.model sw1 SW(VT=0.5 VH=0.1)
.op
.end
""")
    kinds = [e.kind for e in ckt.elements]
    assert kinds == ["V", "R", "S", "CN"]
    s = ckt.elements[2]
    assert s.has_ic and s.ic == 1.0
    cn = ckt.elements[3]
    assert cn.curve == [-1, -1e-6, 0, 0, 1, 1e-6] and cn.wave == "sin" and cn.args == [1, 0.2, 1e3]


@pytest.mark.parametrize("text,why", [
    ("t\nV1 a 0 1\nZ1 a 0 1k\n.end\n", "unsupported element"),
    ("t\n.param a = {b+1}\n.param b = {a}\nR1 x 0 {a}\nV1 x 0 1\n.end\n", "depends on itself"),
    ("t\nV1 a 0 1\nR1 a 0 1k\n.noise v(a) V1 dec 10 1 1k\n.end\n", "unsupported control line"),
])
def test_read_refuses_what_it_cannot_read(text, why):
    with pytest.raises(netlist.NetlistError) as e:
        netlist.read(text)
    assert why in str(e.value)
