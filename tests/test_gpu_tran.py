"""GPU parity of the batched transient against the CPU FP64 oracle and the golden waveforms.

Fixed-step batches (the RC-ladder workload, a diode rectifier) must match the
oracle point by point; adaptive transients of the reference's golden netlists
(LTE control, breakpoints, BE/trapezoidal switching) must take the oracle's
time grid and match the golden tables with CompareTable's tolerance
(internal/golden/golden.go:184-214).
"""
import json
import os

import numpy as np
import pytest

from kronspice_gb300 import analysis, build, workloads
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

import golden_compare as gc

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def ospec(sp):
    return orc.TranSpec(sp.step, sp.stop, sp.start, sp.max_step, int(sp.uic), 1 if sp.method == "be" else 2,
                        int(sp.fixed_step), sp.max_steps, sp.chgtol, sp.trtol, sp.min_step)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rc_ladder_fixed_step_batch(precision):
    el, nn, vals = workloads.rc_ladder_batch(256, seed=3)
    sp = analysis.TranSpec(step=10e-9, stop=2e-6, fixed_step=True)
    plan = analysis.Plan(el, nn, vals.shape[1])
    wave, _, npts, st, steps, it = analysis.Batch(plan, vals).tran(sp, analysis.Options(reltol=1e-6, precision=precision))
    assert np.all(st == 0) and np.all(npts == 201) and np.all(steps == 200)
    so, xo, so_steps, io = orc.batch_tran(orc.Packed(el, nn, vals), 256, ospec(sp), orc.options(reltol=1e-6))
    assert np.all(so == 0)
    rel = 1e-9 if precision == "fp64" else 1e-6
    assert np.all(np.abs(wave - xo) <= rel * np.abs(xo) + 1e-9), np.abs(wave - xo).max()


def rectifier_batch(n, seed):
    b = kc.Builder("rectifier")
    b.voltage_wave("V1", "in", "0", "sin", [0, 10, 1e3])
    b.model("dr", "d", {"is": 1e-14, "n": 1, "cjo": 5e-12, "tt": 5e-9})
    b.diode("D1", "in", "out", "dr")
    b.resistor("R1", "out", "0", 1e3)
    b.capacitor("C1", "out", "0", 10e-6)
    c = b.build()
    el, v0, _ = c.pack()
    g = np.random.default_rng(seed)
    vals = np.tile(v0, (n, 1))
    vals[:, int(el[2]["param"])] *= np.exp(g.uniform(-1, 1, n))  # R1
    vals[:, int(el[3]["param"])] *= np.exp(g.uniform(-1, 1, n))  # C1
    return el, c.n_nodes, vals


def test_diode_rectifier_fixed_step_batch():
    el, nn, vals = rectifier_batch(128, 9)
    sp = analysis.TranSpec(step=5e-6, stop=2e-3, fixed_step=True)
    plan = analysis.Plan(el, nn, vals.shape[1])
    wave, _, npts, st, steps, it = analysis.Batch(plan, vals).tran(sp, analysis.Options(reltol=1e-6))
    so, xo, so_steps, io = orc.batch_tran(orc.Packed(el, nn, vals), 128, ospec(sp), orc.options(reltol=1e-6))
    assert np.array_equal(st, so) and np.all(so == 0)
    assert np.array_equal(steps, so_steps)
    volt = np.abs(xo) + 0
    assert np.all(np.abs(wave[..., :2] - xo[..., :2]) <= 1e-6 * volt[..., :2] + 1e-6)


@pytest.mark.parametrize("kernel", ["generic", "specialized"])
def test_step_predictor_rectifier_batch(kernel):
    """Newton from the extrapolated history (ks_options.step_predictor) on the
    diode rectifier at a tight tolerance: a fifth fewer iterations, the same
    waveforms within the tolerance."""
    el, nn, vals = rectifier_batch(128, 9)
    sp = analysis.TranSpec(step=5e-6, stop=2e-3, fixed_step=True)
    b = analysis.Batch(analysis.Plan(el, nn, vals.shape[1]), vals)
    w0, _, n0, st0, steps0, it0 = b.tran(sp, analysis.Options(reltol=1e-6, kernel=kernel))
    w1, _, n1, st1, steps1, it1 = b.tran(sp, analysis.Options(reltol=1e-6, kernel=kernel, step_predictor=True))
    assert np.all(st0 == 0) and np.all(st1 == 0) and np.array_equal(steps0, steps1)
    assert it1.sum() < 0.9 * it0.sum(), (it1.sum(), it0.sum())
    so, xo, so_steps, io = orc.batch_tran(orc.Packed(el, nn, vals), 128, ospec(sp), orc.options(reltol=1e-6))
    assert np.all(so == 0)
    assert np.all(np.abs(w1[..., :2] - xo[..., :2]) <= 1e-5 * np.abs(xo[..., :2]) + 1e-5)


def test_step_predictor_adaptive_golden():
    """Adaptive golden transients with the predictor: the same accepted grid to
    within a few steps and the golden tables still met."""
    for case in TRAN_CASES:
        ckt = kc.from_dict(case["circuit"])
        tr = [a for a in case["circuit"]["analyses"] if a["kind"] == "tran"][-1]
        sp = analysis.TranSpec(step=tr["step"], stop=tr["stop"], start=tr["start"], max_step=tr["max_step"],
                               uic=tr["uic"])
        el, vals, _ = ckt.pack()
        b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, len(vals)), vals[None, :])
        wave, tim, npts, st, steps, it = b.tran(sp, analysis.Options(step_predictor=True), capacity=200000)
        assert st[0] == 0, case["name"]
        k = int(npts[0])
        t = list(tim[0, :k])
        x = wave[0, :k]

        def get(name):
            if not name.startswith("v("):
                return None
            i = ckt.node_index(name[2:-1])
            return None if i < 0 else (np.zeros(k) if i == 0 else list(x[:, i - 1]))
        want = case["golden"]["independent"]
        want = dict(want, names=[nm for nm in want["names"] if nm.startswith("v(")])
        if want["names"]:
            assert not gc.compare_table(t, get, want), case["name"]


with open(os.path.join(ROOT, "tests", "golden", "reference_cases.json")) as f:
    CASES = [c for c in json.load(f)["cases"] if not c["skip"]]
TRAN_CASES = [c for c in CASES if any(a["kind"] == "tran" for a in c["circuit"]["analyses"])]


@pytest.mark.parametrize("case", TRAN_CASES, ids=[c["name"] for c in TRAN_CASES])
def test_golden_adaptive_transient_on_gpu(case):
    ckt = kc.from_dict(case["circuit"])
    tr = [a for a in case["circuit"]["analyses"] if a["kind"] == "tran"][-1]
    sp = analysis.TranSpec(step=tr["step"], stop=tr["stop"], start=tr["start"], max_step=tr["max_step"], uic=tr["uic"])
    el, vals, _ = ckt.pack()
    plan = analysis.Plan(el, ckt.n_nodes, len(vals))
    cap = 200000
    wave, tim, npts, st, steps, it = analysis.Batch(plan, vals[None, :]).tran(sp, analysis.Options(), capacity=cap)
    assert st[0] == 0
    k = int(npts[0])
    t = list(tim[0, :k])
    x = wave[0, :k]
    # same algorithm as the oracle: same accepted steps
    ost, ot, ox, ocur, osteps, oiters, msg = orc.tran(orc.Packed.of(ckt), ospec(sp), capacity=cap)
    assert ost == 0
    assert abs(steps[0] - osteps) <= max(2, 0.01 * osteps)

    def get(name):
        if not name.startswith("v("):
            return None
        i = ckt.node_index(name[2:-1])
        return None if i < 0 else (np.zeros(k) if i == 0 else list(x[:, i - 1]))
    want = case["golden"]["independent"]
    want = dict(want, names=[nm for nm in want["names"] if nm.startswith("v(")])
    if not want["names"]:
        # current-only goldens (rl_step: i(l1)): compare the inductor branch current
        li = ckt.element_index("l1")
        _, isv = orc.unknowns(orc.Packed.of(ckt))
        br = [i for i in range(len(isv)) if not isv[i]]
        y = list(x[:, br[-1]])
        want2 = case["golden"]["independent"]
        assert not gc.compare_table(t, lambda nm: y, want2)
        return
    assert not gc.compare_table(t, get, want)


def test_uic_transient_matches_oracle():
    b = kc.Builder("lc")
    b.inductor("L1", "a", "0", 1e-3, ic=1e-3)
    b.capacitor("C1", "a", "0", 1e-6, ic=0.5)
    b.resistor("R1", "a", "0", 1e3)
    c = b.build()
    sp = analysis.TranSpec(step=1e-6, stop=2e-4, uic=True)
    el, vals, _ = c.pack()
    plan = analysis.Plan(el, c.n_nodes, len(vals))
    wave, tim, npts, st, steps, it = analysis.Batch(plan, vals[None, :]).tran(sp, capacity=100000)
    ost, ot, ox, _, osteps, _, msg = orc.tran(orc.Packed.of(c), ospec(sp), capacity=100000)
    assert st[0] == 0 and ost == 0
    k = int(npts[0])
    assert k == len(ot)
    assert np.allclose(tim[0, :k], ot, rtol=1e-9, atol=1e-15)
    assert np.allclose(wave[0, :k], ox, rtol=1e-6, atol=1e-9)


def test_bad_tran_spec_is_rejected():
    el, nn, vals = workloads.rc_ladder_batch(2)
    plan = analysis.Plan(el, nn, vals.shape[1])
    with pytest.raises(RuntimeError, match="invalid transient"):
        analysis.Batch(plan, vals).tran(analysis.TranSpec(step=-1, stop=1e-6, fixed_step=True))
