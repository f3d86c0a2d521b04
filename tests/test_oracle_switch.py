"""Switches (device/switch.go) in the oracle and on the host, without a GPU.

The oracle's restatement against the reference's own switch tests
(device/switch_test.go) at the circuit level: the hysteresis sequence of
TestSwitchHysteresis as a chained DC sweep (each point's state referred to the
previous accepted one), the smooth switch's linearization (TestSmoothSwitchJacobian)
through the operating point and the small-signal response, and the relaxation
oscillator's period.  The golden netlists switch_dc, switch_rc_tran and
switch_relax_tran are pinned in test_oracle_golden.  Then the host's
validateSwitch and the torn engine's refusals.
"""
import numpy as np
import pytest

from kronspice_gb300 import analysis
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc


def hysteresis_circuit(vh=0.2, ron=1.0, roff=1e6):
    b = kc.Builder("hysteresis")
    b.voltage_source("V1", "ctl", "0", 0.0)
    b.voltage_source("V2", "dd", "0", 5.0)
    b.resistor("R1", "dd", "out", 1e3)
    b.model("sw", "sw", {"vt": 1.0, "vh": vh, "ron": ron, "roff": roff})
    b.vswitch("S1", "out", "0", "ctl", "0", "sw")
    return b.build()


def test_hysteresis_sequence_as_a_chained_sweep():
    """TestSwitchHysteresis (device/switch_test.go:35-57): on above VT + VH, off
    below VT - VH, the accepted state held in between."""
    ckt = hysteresis_circuit()
    pk = orc.Packed.of(ckt)
    ctl = [0, 1.1, 1.3, 1, 0.85, 0.7, 1.15]
    want = [False, False, True, True, True, False, False]
    st, x, cur, msg = orc.dc(pk, ckt.element_index("V1"), ctl)
    assert st == 0, msg
    out = x[:, ckt.node_index("out") - 1]
    on = 5 * 1 / (1 + 1e3)
    off = 5 * 1e6 / (1e6 + 1e3)
    for k, w in enumerate(want):
        assert abs(out[k] - (on if w else off)) <= 1e-9 * off, (ctl[k], out[k], w)
    # a sweep down from above the band keeps the switch on inside it
    st, x, _, _ = orc.dc(pk, ckt.element_index("V1"), [2.0, 1.0, 0.85])
    assert st == 0 and np.all(np.abs(x[:, ckt.node_index("out") - 1] - on) <= 1e-12)


def smooth_g(c, vt, vh, ron, roff):
    """ngspice's smooth switch (device/switch.go:151-162): ln R a cubic in
    x = (c - VT)/|VH| with zero slope at RON and ROFF."""
    x = (c - vt) / abs(vh)
    if x >= 1:
        return 1 / ron
    if x <= -1:
        return 1 / roff
    lr = np.log(ron / roff)
    return np.exp(-(np.log(np.sqrt(ron * roff)) + lr * (3 * x - x ** 3) / 4))


@pytest.mark.parametrize("vin", [0.6, 0.9, 1.0, 1.2, 1.45, 2.0])
def test_smooth_switch_operating_point_and_small_signal(vin):
    """The smooth switch is a nonlinear resistor in its control: the operating
    point carries i = g(c) v, and the AC response at a low frequency is the
    derivative of the DC transfer (the linearization's transconductance k = v dg/dc)."""
    vt, vh, ron, roff = 1.0, -0.5, 10.0, 1e5

    def build(v):
        b = kc.Builder("smooth")
        b.voltage_source("V1", "ctl", "0", v, ac=(1.0, 0.0))
        b.resistor("RC", "ctl", "0", 1e3)
        b.voltage_source("V2", "dd", "0", 5.0)
        b.resistor("R1", "dd", "out", 1e3)
        b.model("sm", "sw", {"vt": vt, "vh": vh, "ron": ron, "roff": roff})
        b.vswitch("S1", "out", "0", "ctl", "0", "sm")
        return b.build()
    ckt = build(vin)
    st, x, cur, _, msg = orc.op(orc.Packed.of(ckt))
    assert st == 0, msg
    vout = x[ckt.node_index("out") - 1]
    g = smooth_g(vin, vt, vh, ron, roff)
    assert abs((5 - vout) / 1e3 - g * vout) <= 1e-9 * (5 - vout) / 1e3 + 1e-15
    assert abs(cur[ckt.element_index("S1")] - g * vout) <= 1e-9 * abs(g * vout) + 1e-15
    # d vout / d vin by central differences of the DC solution against the AC gain
    d = 1e-6
    vp = orc.op(orc.Packed.of(build(vin + d)))[1][ckt.node_index("out") - 1]
    vm = orc.op(orc.Packed.of(build(vin - d)))[1][ckt.node_index("out") - 1]
    st, xa, msg = orc.ac(orc.Packed.of(ckt), [1e-3])
    assert st == 0, msg
    gain = xa[0, ckt.node_index("out") - 1]
    fd = (vp - vm) / (2 * d)
    assert abs(gain.imag) <= 1e-9 * (abs(gain.real) + 1e-12)
    assert abs(gain.real - fd) <= 1e-5 * (abs(fd) + 1e-9), (gain, fd)


def test_relaxation_period():
    """The relaxation oscillator of switch_relax_tran: the capacitor charges
    through 10k towards 5 V until the switch turns on at 3 V, discharges through
    RON = 1k in parallel towards 5/11 V until it turns off at 2 V; period
    tau1 ln((5-2)/(5-3)) + tau2 ln((3-5/11)/(2-5/11)), located to the step
    limiter's 1 % of a step."""
    b = kc.Builder("relax")
    b.voltage_source("V1", "vcc", "0", 5.0)
    b.resistor("R1", "vcc", "c", 1e4)
    b.capacitor("C1", "c", "0", 1e-6, ic=0.0)
    b.model("swh", "sw", {"vt": 2.5, "vh": 0.5, "ron": 1e3, "roff": 1e12})
    b.vswitch("S1", "c", "0", "c", "0", "swh")
    ckt = b.build()
    spec = orc.TranSpec(10e-6, 30e-3, 0.0, 0.0, 1, 0, 0, 0, 0, 0, 0)
    st, t, x, cur, steps, iters, msg = orc.tran(orc.Packed.of(ckt), spec)
    assert st == 0, msg
    v = x[:, ckt.node_index("c") - 1]
    rise = [t[k] for k in range(1, len(t)) if v[k - 1] < 2.5 <= v[k]]
    tau1, rp = 1e4 * 1e-6, 1e4 * 1e3 / 1.1e4
    period = tau1 * np.log(3 / 2) + rp * 1e-6 * np.log((3 - 5 / 11) / (2 - 5 / 11))
    got = np.diff(rise[1:])
    assert len(got) >= 4
    assert np.all(np.abs(got - period) <= 2e-3 * period), (got, period)


def test_switch_validation_on_the_host():
    """validateSwitch (circuit/switch.go:52-72) and validateControl."""
    def one(**kw):
        b = kc.Builder("v")
        b.voltage_source("V1", "a", "0", 1.0).resistor("R1", "a", "0", 1e3)
        b.voltage_source("V2", "d", "0", 1.0).resistor("R2", "d", "o", 1e3)
        b.model("sw", "sw", kw.get("model", {"vt": 1, "vh": 0.1}))
        b.model("csw", "csw", {"it": 1e-3, "ih": 1e-4})
        if kw.get("current"):
            b.iswitch("W1", "o", "0", kw.get("src", "V1"), "csw")
        else:
            b.vswitch("S1", "o", "0", "a", kw.get("cn", "0"), "sw", on=kw.get("on"))
        return b.build()
    assert analysis.validate(one()) is None
    assert analysis.validate(one(current=True)) is None
    assert "RON != ROFF" in str(analysis.validate(one(model={"vt": 1, "vh": -0.1, "ron": 5, "roff": 5})))
    assert "always 0" in str(analysis.validate(one(cn="a")))
    assert "not a voltage source" in str(analysis.validate(one(current=True, src="R1")))
    assert "RON and ROFF" in str(analysis.validate(one(model={"vt": 1, "ron": 0})))
    c = one()
    el, vals, _ = c.pack()
    vals[int(el[c.element_index("S1")]["param"]) + 4] = 0.5  # an initial state that is neither ON nor OFF
    assert "ON (1) or OFF (0)" in str(analysis.validate_packed(el, c.n_nodes, vals))


def test_tearing_a_switch():
    """tearTerminals (kron/jacobian.go:136-170): an S switch tears with its
    control nodes, a W switch is refused; the torn engine refuses a smooth
    switch (its transconductance entries are not in the values-free plan)."""
    b = kc.Builder("tear")
    b.voltage_source("V1", "a", "0", 1.0)
    b.resistor("R1", "a", "b", 1e3).resistor("R2", "b", "0", 1e3)
    b.resistor("R3", "a", "c", 1e3).resistor("R4", "c", "0", 1e3)
    b.voltage_source("VS", "c", "d", 0.0).resistor("R5", "d", "0", 1e3)
    b.model("sw", "sw", {"vt": 0.3, "vh": 0.1}).model("csw", "csw", {"it": 1e-4})
    b.vswitch("S1", "b", "c", "a", "b", "sw")
    b.iswitch("W1", "b", "d", "VS", "csw")
    c = b.build()
    pk = orc.Packed.of(c)
    st, pairs, msg = orc.torn_cuts(pk, [c.element_index("S1")])
    assert st == 0, msg
    # b, c and the control nodes a, b: the pairs of {b, c, a}
    assert len(pairs) == 3
    st, pairs, msg = orc.torn_cuts(pk, [c.element_index("W1")])
    assert st != 0 and "branch-current unknown" in msg
    el, vals, _ = c.pack()
    vals[int(el[c.element_index("S1")]["param"]) + 1] = -0.1  # VH < 0: the smooth switch
    with pytest.raises(RuntimeError) as e:
        analysis.TornBatch(el, c.n_nodes, vals[None, :], [c.element_index("R1")])
    assert "smooth switches" in str(e.value)
