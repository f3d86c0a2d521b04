"""Pin the oracle's element results and energy ledger against the reference's own tests.

Known answers of analysis/op_test.go (TestDivider :24-52, TestCurrentSourceDirection
:54-67, TestAbsorbingSourceIsOutflow :69-85), analysis/negres_test.go
(TestNegativeResistorDivider :19-45), analysis/tran_test.go (TestRCStep :47-74,
TestLCOscillatorConservesEnergy :119-160) and the coverage test
analysis/ledger_golden_test.go (TestGoldenLedgers: every golden operating point
balances to 1e-12, every golden transient to 1e-9, Tellegen's sum vanishes on the
two-terminal circuits).
"""
import json
import math
import os

import numpy as np
import pytest

from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_cases.json")) as f:
    CASES = json.load(f)["cases"]

R, L, T = orc.RES, orc.LEDGER, orc.TPOINT


def near(a, b, tol):
    return abs(a - b) <= tol


def relative_residual(led):
    """output.Ledger.RelativeResidual (output/result.go:100-109)."""
    res = abs(led[L["residual"]])
    if led[L["scale"]] == 0 or res <= max(1e-21, led[L["roundoff"]]):
        return 0.0
    return res / led[L["scale"]]


def op(ckt, **kw):
    st, x, elem, led, _, msg = orc.op_results(orc.Packed.of(ckt), orc.options(**kw))
    assert st == 0, msg
    return x, elem, led


def test_divider():
    ckt = (kc.Builder("div").voltage_source("V1", "in", "0", 10).resistor("R1", "in", "out", 1e3)
           .resistor("R2", "out", "0", 1e3).build())
    x, elem, led = op(ckt)
    assert near(x[ckt.node_index("out") - 1], 5, 1e-12)
    assert near(elem[0, R["current"]], -5e-3, 1e-15)  # current into the + terminal
    assert near(led[L["inflow"]], 0.05, 1e-15) and near(led[L["dissipation"]], 0.05, 1e-15)
    assert relative_residual(led) <= 1e-12


def test_current_source_direction():
    ckt = kc.Builder("i").current_source("I1", "0", "a", 2e-3).resistor("R1", "a", "0", 1e3).build()
    x, elem, led = op(ckt)
    assert near(x[0], 2, 1e-12)
    assert near(led[L["inflow"]], 4e-3, 1e-15)


def test_absorbing_source_is_outflow():
    ckt = (kc.Builder("charge").voltage_source("V1", "a", "0", 9).voltage_source("V2", "b", "0", 5)
           .resistor("R1", "a", "b", 100).build())
    _, _, led = op(ckt)
    i = 4.0 / 100
    assert near(led[L["inflow"]], 9 * i, 1e-12)
    assert near(led[L["outflow"]], 5 * i, 1e-12)
    assert near(led[L["dissipation"]], 4 * i, 1e-12)


def test_negative_resistor_divider():
    ckt = (kc.Builder("neg").voltage_source("V1", "in", "0", 10).resistor("R1", "in", "out", 1e3)
           .resistor("R2", "out", "0", -500).build())
    x, elem, led = op(ckt)
    assert near(x[ckt.node_index("out") - 1], -10, 1e-12)
    assert near(led[L["model_supplied"]], 0.2, 1e-15)
    assert near(led[L["inflow"]], 0.2, 1e-15)
    assert near(led[L["dissipation"]], 0.4, 1e-15)
    assert relative_residual(led) <= 1e-12
    # the negative resistance takes nothing in through its thermal port
    assert elem[2, R["exterior_power"]] == 0 and elem[2, R["model_supplied"]] != 0


def tran(ckt, step, stop, uic=False, start=0.0, max_step=0.0):
    spec = orc.TranSpec(step, stop, start, max_step, int(uic), 0, 0, 0, 0, 0, 0)
    out = orc.tran_results(orc.Packed.of(ckt), spec, orc.options())
    assert out[0] == 0, out[-1]
    return out


def test_rc_step():
    b = kc.Builder("rc").voltage_wave("V1", "in", "0", "pulse", [0, 1, 0, 1e-9, 1e-9, 1, 2])
    ckt = b.resistor("R1", "in", "out", 1e3).capacitor("C1", "out", "0", 1e-6).build()
    st, t, x, elem, led, summ, steps, _, _ = tran(ckt, 10e-6, 5e-3)
    vf = 1 - math.exp(-5)
    want = 0.5 * 1e-6 * vf * vf
    assert abs(summ[orc.TSUM["stored_end"]] - want) <= 1e-3 * want
    assert abs(summ[orc.TSUM["energy_dissipated"]] / summ[orc.TSUM["stored_end"]] - 1) <= 0.02
    assert summ[orc.TSUM["max_relative_residual"]] <= 1e-9
    assert steps <= 2000
    # the recorded currents and powers are the element rows of each point
    assert np.allclose(elem[:, 1, 1], (x[:, 0] - x[:, 1]) * elem[:, 1, 0], rtol=1e-12, atol=1e-18)


def test_lc_oscillator_conserves_energy():
    Lh, C = 1e-3, 1e-6
    ckt = kc.Builder("lc").capacitor("C1", "a", "0", C, ic=1.0).inductor("L1", "a", "0", Lh).build()
    period = 2 * math.pi * math.sqrt(Lh * C)
    st, t, x, elem, led, summ, *_ = tran(ckt, period / 200, 10 * period, uic=True)
    e0 = 0.5 * C
    assert np.all(np.abs(led[:, T["stored_energy"]] - e0) <= 1e-3 * e0)
    assert summ[orc.TSUM["energy_in"]] == 0 and summ[orc.TSUM["energy_dissipated"]] == 0


def _runnable(c):
    return c["skip"] is None


def _uic(c):
    return any(a["kind"] == "tran" and a["uic"] for a in c["circuit"]["analyses"])


OP_CASES = [c for c in CASES if _runnable(c) and not _uic(c)]
TRAN_CASES = [c for c in CASES if _runnable(c) and any(a["kind"] == "tran" for a in c["circuit"]["analyses"])]


@pytest.mark.parametrize("case", OP_CASES, ids=[c["name"] for c in OP_CASES])
def test_golden_operating_point_ledger(case):
    ckt = kc.from_dict(case["circuit"])
    x, elem, led = op(ckt)
    assert relative_residual(led) <= 1e-12, led
    # Tellegen on circuits of two-terminal elements (em/efficiency.go:106-120)
    if all(e.kind in "RCLVID" for e in ckt.elements):
        v = np.concatenate([[0.0], x[:ckt.n_nodes - 1]])
        p = np.array([(v[ckt.node_index(e.nodes[0])] - v[ckt.node_index(e.nodes[1])]) * elem[k, R["current"]]
                      for k, e in enumerate(ckt.elements)])
        assert abs(p.sum()) <= max(1e-12 * np.abs(p).sum(), 1e-21)


@pytest.mark.parametrize("case", TRAN_CASES, ids=[c["name"] for c in TRAN_CASES])
def test_golden_transient_ledger(case):
    ckt = kc.from_dict(case["circuit"])
    tr = [a for a in case["circuit"]["analyses"] if a["kind"] == "tran"][-1]
    out = tran(ckt, tr["step"], tr["stop"], uic=tr["uic"], start=tr["start"], max_step=tr["max_step"])
    summ = out[5]
    assert summ[orc.TSUM["max_relative_residual"]] <= 1e-9


def test_ledger_coverage():
    assert len(OP_CASES) >= 25 and len(TRAN_CASES) >= 8
