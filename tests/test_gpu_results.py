"""GPU parity of the element results and the energy ledger against the oracle.

ks_op_results / ks_tran_results compute each element's operating point (voltage,
current, absorbed and storage power, stored energy, exterior and model-supplied
power) and the ledger on the device at the accepted solution, from the
linearization of each device's last load, as (*Sim).result (analysis/op.go:361-403)
and the transient recorder (analysis/tran.go:291-386) do.  Both sides solve to a
tight Newton tolerance, so the results agree to the solution's own agreement; the
ledger must balance as the reference requires (relative residual <= 1e-12 at an
operating point, <= 1e-9 over a transient: analysis/ledger_golden_test.go).
"""
import json
import math
import os

import numpy as np
import pytest

from kronspice_gb300 import analysis, build, workloads
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
R, L, TP, TS = analysis.RES, analysis.LEDGER, analysis.TPOINT, analysis.TSUM
TIGHT = dict(reltol=1e-9, vntol=1e-12, abstol=1e-15)


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def relative_residual(led):
    """output.Ledger.RelativeResidual (output/result.go:100-109)."""
    res = abs(led[L["residual"]])
    if led[L["scale"]] == 0 or res <= max(1e-21, led[L["roundoff"]]):
        return 0.0
    return res / led[L["scale"]]


def gpu_op(ckt, **kw):
    el, vals, _ = ckt.pack()
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, len(vals)), vals[None, :])
    x, st, it, elem, led = b.op_results(analysis.Options(kernel="generic", **kw))
    return st[0], x[0], elem[0], led[0]


# Newton stops a device current within reltol * |i| + abstol (1e-15 A here), so
# currents near the gmin floor agree to about that absolute level
IABS = 1e-14


def close(a, b, scale, rtol=1e-6, atol=1e-18):
    return np.abs(a - b) <= rtol * np.abs(b) + 1e-9 * scale + atol


with open(os.path.join(ROOT, "tests", "golden", "reference_cases.json")) as f:
    CASES = [c for c in json.load(f)["cases"] if not c["skip"]]
OP_CASES = [c for c in CASES if not any(a["kind"] == "tran" and a["uic"] for a in c["circuit"]["analyses"])]
TRAN_CASES = [c for c in CASES if any(a["kind"] == "tran" for a in c["circuit"]["analyses"])]


@pytest.mark.parametrize("case", OP_CASES, ids=[c["name"] for c in OP_CASES])
def test_golden_operating_point_results(case):
    ckt = kc.from_dict(case["circuit"])
    st, x, elem, led = gpu_op(ckt, **TIGHT)
    ost, ox, oelem, oled, _, msg = orc.op_results(orc.Packed.of(ckt), orc.options(**TIGHT))
    assert st == 0 and ost == 0, msg
    scale = max(oled[L["scale"]], 1e-30)
    iscale = np.abs(oelem[:, R["current"]]).max() + 1e-30
    pabs = IABS * (np.abs(ox).max() + 1)  # the current floor times the largest voltage
    assert np.all(close(elem[:, R["voltage"]], oelem[:, R["voltage"]], 1.0))
    assert np.all(close(elem[:, R["current"]], oelem[:, R["current"]], iscale, atol=IABS))
    for col in ("power", "storage_power", "exterior_power", "model_supplied"):
        assert np.all(close(elem[:, R[col]], oelem[:, R[col]], scale, atol=pabs)), col
    assert np.all(close(elem[:, R["stored_energy"]], oelem[:, R["stored_energy"]],
                        np.abs(oelem[:, R["stored_energy"]]).max() + 1e-30))
    for col in ("inflow", "outflow", "dissipation", "storage_rate", "model_supplied", "scale"):
        assert close(led[L[col]], oled[L[col]], scale, atol=len(ckt.elements) * pabs), col
    # the round-off estimate of the last linear system, and the balance itself
    assert abs(led[L["roundoff"]] - oled[L["roundoff"]]) <= 1e-6 * oled[L["roundoff"]] + 1e-30
    assert relative_residual(led) <= 1e-12, led


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bjt_ce_batch_results(precision):
    """Every circuit of a BJT batch: currents and powers against the oracle, the
    ledger balanced (mixed precision to em.DefaultTolerance)."""
    el, nn, vals = workloads.bjt_ce_batch(512, seed=21)
    b = analysis.Batch(analysis.Plan(el, nn, vals.shape[1]), vals)
    x, st, it, elem, led = b.op_results(analysis.Options(precision=precision, **TIGHT))
    assert b.last_kernel == "generic"
    pk = orc.Packed(el, nn, vals[0])
    bound = 1e-12 if precision == "fp64" else 1e-9
    for c in range(0, 512, 7):
        pk.values[:] = vals[c]
        ost, ox, oelem, oled, _, msg = orc.op_results(pk, orc.options(**TIGHT))
        assert st[c] == ost
        if ost:
            assert not elem[c].any() and not led[c].any()
            continue
        scale = oled[L["scale"]]
        pabs = IABS * (np.abs(ox).max() + 1)
        assert np.all(close(elem[c, :, R["current"]], oelem[:, R["current"]], np.abs(oelem[:, R["current"]]).max(),
                            atol=IABS))
        assert np.all(close(elem[c, :, R["power"]], oelem[:, R["power"]], scale, atol=pabs))
        assert close(led[c, L["dissipation"]], oled[L["dissipation"]], scale, atol=len(el) * pabs)
        assert relative_residual(led[c]) <= bound
    ok = st == 0
    assert ok.mean() > 0.99
    assert max(relative_residual(led[c]) for c in np.nonzero(ok)[0]) <= bound


def test_known_answers_on_gpu():
    """TestDivider, TestAbsorbingSourceIsOutflow, TestNegativeResistorDivider
    (analysis/op_test.go:24-85, analysis/negres_test.go:19-45) on the device."""
    ckt = (kc.Builder("div").voltage_source("V1", "in", "0", 10).resistor("R1", "in", "out", 1e3)
           .resistor("R2", "out", "0", 1e3).build())
    st, x, elem, led = gpu_op(ckt)
    assert st == 0 and abs(elem[0, R["current"]] + 5e-3) <= 1e-15
    assert abs(led[L["inflow"]] - 0.05) <= 1e-15 and abs(led[L["dissipation"]] - 0.05) <= 1e-15
    ckt = (kc.Builder("charge").voltage_source("V1", "a", "0", 9).voltage_source("V2", "b", "0", 5)
           .resistor("R1", "a", "b", 100).build())
    st, x, elem, led = gpu_op(ckt)
    i = 4.0 / 100
    assert abs(led[L["inflow"]] - 9 * i) <= 1e-12 and abs(led[L["outflow"]] - 5 * i) <= 1e-12
    assert abs(led[L["dissipation"]] - 4 * i) <= 1e-12
    ckt = (kc.Builder("neg").voltage_source("V1", "in", "0", 10).resistor("R1", "in", "out", 1e3)
           .resistor("R2", "out", "0", -500).build())
    st, x, elem, led = gpu_op(ckt)
    assert st == 0
    assert abs(led[L["model_supplied"]] - 0.2) <= 1e-15 and abs(led[L["inflow"]] - 0.2) <= 1e-15
    assert abs(led[L["dissipation"]] - 0.4) <= 1e-15
    assert elem[2, R["exterior_power"]] == 0 and relative_residual(led) <= 1e-12


def ospec(sp):
    return orc.TranSpec(sp.step, sp.stop, sp.start, sp.max_step, int(sp.uic), 1 if sp.method == "be" else 2,
                        int(sp.fixed_step), sp.max_steps, sp.chgtol, sp.trtol, sp.min_step)


@pytest.mark.parametrize("case", TRAN_CASES, ids=[c["name"] for c in TRAN_CASES])
def test_golden_transient_ledger_fixed_step(case):
    """The golden transients on the fixed-step grid of their print step: every
    point's currents, powers and ledger row against the oracle's."""
    ckt = kc.from_dict(case["circuit"])
    tr = [a for a in case["circuit"]["analyses"] if a["kind"] == "tran"][-1]
    sp = analysis.TranSpec(step=tr["step"], stop=tr["stop"], uic=tr["uic"], fixed_step=True)
    el, vals, _ = ckt.pack()
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, len(vals)), vals[None, :])
    wave, _, elem, led, summ, npts, st, steps, it = b.tran_results(sp, analysis.Options(**TIGHT))
    out = orc.tran_results(orc.Packed.of(ckt), ospec(sp), orc.options(**TIGHT))
    ost, ot, ox, oelem, oled, osumm, osteps = out[:7]
    assert st[0] == ost, out[-1]
    if ost:
        return
    k = len(ot)
    assert int(npts[0]) == k
    g_elem, g_led = elem[:k, 0], led[:k, 0]
    peak = np.abs(oled[:, :TP["residual"]]).sum(axis=1).max() + 1e-30
    ipk = np.abs(oelem[..., 0]).max() + 1e-30
    pabs = IABS * (np.abs(ox).max() + 1)
    assert np.all(np.abs(g_elem[..., 0] - oelem[..., 0]) <= 1e-5 * np.abs(oelem[..., 0]) + 1e-6 * ipk + IABS)
    assert np.all(np.abs(g_elem[..., 1] - oelem[..., 1]) <= 1e-5 * np.abs(oelem[..., 1]) + 1e-6 * peak + pabs)
    for col in ("inflow", "outflow", "dissipation", "storage_rate", "stored_energy"):
        ref = oled[:, TP[col]]
        pk = np.abs(ref).max() + 1e-30
        atol = 0 if col == "stored_energy" else len(ckt.elements) * pabs
        assert np.all(np.abs(g_led[:, TP[col]] - ref) <= 1e-5 * np.abs(ref) + 1e-6 * pk + atol), col
    assert summ[0, TS["max_relative_residual"]] <= 1e-9
    for col in ("energy_in", "energy_dissipated", "stored_end"):
        assert abs(summ[0, TS[col]] - osumm[TS[col]]) <= 1e-5 * abs(osumm[TS[col]]) + 1e-6 * (
            abs(osumm[TS["energy_in"]]) + abs(osumm[TS["stored_end"]]) + 1e-30), col


@pytest.mark.parametrize("case", TRAN_CASES, ids=[c["name"] for c in TRAN_CASES])
def test_golden_transient_ledger_adaptive(case):
    """The golden transients as the reference runs them (LTE control, breakpoints):
    the ledger balances to em.DefaultTolerance and the energies match the oracle's."""
    ckt = kc.from_dict(case["circuit"])
    tr = [a for a in case["circuit"]["analyses"] if a["kind"] == "tran"][-1]
    sp = analysis.TranSpec(step=tr["step"], stop=tr["stop"], start=tr["start"], max_step=tr["max_step"], uic=tr["uic"])
    el, vals, _ = ckt.pack()
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, len(vals)), vals[None, :])
    cap = 100000
    wave, tim, elem, led, summ, npts, st, steps, it = b.tran_results(sp, analysis.Options(), capacity=cap)
    out = orc.tran_results(orc.Packed.of(ckt), ospec(sp), capacity=cap)
    assert st[0] == 0 and out[0] == 0, out[-1]
    osumm = out[5]
    assert summ[0, TS["max_relative_residual"]] <= 1e-9
    ref = abs(osumm[TS["energy_in"]]) + abs(osumm[TS["stored_end"]]) + abs(osumm[TS["energy_dissipated"]]) + 1e-30
    for col in ("energy_in", "energy_out", "energy_dissipated", "stored_start", "stored_end"):
        assert abs(summ[0, TS[col]] - osumm[TS[col]]) <= 1e-3 * ref, col


def test_lc_oscillator_conserves_energy_on_gpu():
    """TestLCOscillatorConservesEnergy (analysis/tran_test.go:119-160) on the device."""
    Lh, C = 1e-3, 1e-6
    ckt = kc.Builder("lc").capacitor("C1", "a", "0", C, ic=1.0).inductor("L1", "a", "0", Lh).build()
    period = 2 * math.pi * math.sqrt(Lh * C)
    sp = analysis.TranSpec(step=period / 200, stop=10 * period, uic=True)
    el, vals, _ = ckt.pack()
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, len(vals)), vals[None, :])
    wave, tim, elem, led, summ, npts, st, steps, it = b.tran_results(sp, capacity=20000)
    assert st[0] == 0
    k = int(npts[0])
    e0 = 0.5 * C
    assert np.all(np.abs(led[0, :k, TP["stored_energy"]] - e0) <= 1e-3 * e0)
    assert summ[0, TS["energy_in"]] == 0 and summ[0, TS["energy_dissipated"]] == 0


def test_rc_ladder_batch_ledger():
    """A fixed-step batch (the RC-ladder workload): every circuit's ledger balances
    and its energies match the oracle's."""
    el, nn, vals = workloads.rc_ladder_batch(64, seed=5)
    sp = analysis.TranSpec(step=10e-9, stop=1e-6, fixed_step=True)
    b = analysis.Batch(analysis.Plan(el, nn, vals.shape[1]), vals)
    wave, _, elem, led, summ, npts, st, steps, it = b.tran_results(sp, analysis.Options(reltol=1e-6))
    assert np.all(st == 0)
    assert np.all(summ[:, TS["max_relative_residual"]] <= 1e-9)
    pk = orc.Packed(el, nn, vals[0])
    for c in range(0, 64, 9):
        pk.values[:] = vals[c]
        out = orc.tran_results(pk, ospec(sp), orc.options(reltol=1e-6), capacity=200)
        assert out[0] == 0
        osumm = out[5]
        for col in ("energy_in", "energy_dissipated", "stored_end", "integration_mismatch"):
            ref = abs(osumm[TS["energy_in"]]) + 1e-30
            assert abs(summ[c, TS[col]] - osumm[TS[col]]) <= 1e-6 * ref, col
