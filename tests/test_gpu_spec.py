"""Per-topology kernels (the plan's element program compiled by NVRTC) on the GPU.

They instantiate the same device templates as the generic kernels with every
element a compile-time constant, so they must reproduce the oracle exactly as
the generic kernels do (same statuses, node voltages within the SPICE
tolerances, FP64 within 1e-9 relative with the same Newton iteration counts),
and agree with the generic kernels circuit by circuit.
"""
import dataclasses
import time

import numpy as np
import pytest

from kronspice_gb300 import analysis, build, workloads
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
RELTOL, VNTOL, ABSTOL = 1e-6, 1e-6, 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def tol(x_ref, isv, rel=RELTOL):
    return np.where(isv, VNTOL, ABSTOL) + rel * np.abs(x_ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bjt_ce_specialized_matches_oracle_and_generic(precision):
    el, nn, vals = workloads.bjt_ce_batch(4096, seed=11)
    plan = analysis.Plan(el, nn, vals.shape[1])
    b = analysis.Batch(plan, vals)
    og = analysis.Options(reltol=RELTOL, precision=precision, kernel="generic")
    xg, sg, ig = b.op(og)
    assert b.last_kernel == "generic"
    xs, ss, is_ = b.op(dataclasses.replace(og, kernel="specialized"))
    assert b.last_kernel == "specialized-registers"
    so, xo, io = orc.batch_op(orc.Packed(el, nn, vals), vals.shape[0], orc.options(reltol=RELTOL))
    _, isv = orc.unknowns(orc.Packed(el, nn, vals[0]))
    assert np.array_equal(ss, so), np.nonzero(ss != so)
    ok = so == 0
    assert ok.mean() > 0.99
    err = np.abs(xs[ok] - xo[ok])
    assert np.all(err <= tol(xo[ok], isv)), err.max()
    assert np.array_equal(ss, sg)
    if precision == "fp64":
        assert np.all(err <= 1e-9 * np.abs(xo[ok]) + np.where(isv, 1e-12, 1e-18))
        assert (is_ == io).mean() > 0.99
        assert (is_ == ig).mean() > 0.99
    assert np.all(np.abs(xs[ok] - xg[ok]) <= tol(xg[ok], isv))


def test_auto_choice():
    el, nn, vals = workloads.bjt_ce_batch(4096, seed=2)
    plan = analysis.Plan(el, nn, vals.shape[1])
    b = analysis.Batch(plan, vals)
    b.op(analysis.Options(reltol=RELTOL))
    assert b.last_kernel == "specialized-registers"
    small = analysis.Batch(plan, vals[:64])
    small.op(analysis.Options(reltol=RELTOL))
    assert small.last_kernel == "generic"
    t0 = time.perf_counter()
    kname, _ = plan.specialize("op")  # compiled once per plan and process
    assert kname == "specialized-registers" and time.perf_counter() - t0 < 0.5


def ospec(sp):
    return orc.TranSpec(sp.step, sp.stop, sp.start, sp.max_step, int(sp.uic), 1 if sp.method == "be" else 2,
                        int(sp.fixed_step), sp.max_steps, sp.chgtol, sp.trtol, sp.min_step)


@pytest.mark.parametrize("sections,kind", [(3, "specialized-registers"), (5, "specialized-shared")])
def test_rc_ladder_specialized_transient(sections, kind):
    """Fixed-step RC ladders: 5 unknowns (registers) and 7 (shared memory)."""
    el, nn, vals = workloads.rc_ladder_batch(256, seed=3, sections=sections)
    sp = analysis.TranSpec(step=10e-9, stop=1e-6, fixed_step=True)
    plan = analysis.Plan(el, nn, vals.shape[1])
    b = analysis.Batch(plan, vals)
    wave, _, npts, st, steps, it = b.tran(sp, analysis.Options(reltol=1e-6, kernel="specialized"))
    assert b.last_kernel == kind
    assert np.all(st == 0) and np.all(npts == 101) and np.all(steps == 100)
    so, xo, so_steps, io = orc.batch_tran(orc.Packed(el, nn, vals), 256, ospec(sp), orc.options(reltol=1e-6))
    assert np.all(so == 0)
    assert np.all(np.abs(wave - xo) <= 1e-9 * np.abs(xo) + 1e-9), np.abs(wave - xo).max()


def test_diode_rectifier_specialized_adaptive_transient():
    """LTE-controlled steps with breakpoints through the per-topology kernel:
    the oracle's time grid and waveforms."""
    b = kc.Builder("rectifier")
    b.voltage_wave("V1", "in", "0", "pulse", [0, 5, 1e-6, 1e-7, 1e-7, 2e-6, 5e-6])
    b.model("dr", "d", {"is": 1e-14, "n": 1, "cjo": 5e-12, "tt": 5e-9})
    b.diode("D1", "in", "out", "dr")
    b.resistor("R1", "out", "0", 1e3)
    b.capacitor("C1", "out", "0", 1e-9)
    c = b.build()
    el, v0, _ = c.pack()
    g = np.random.default_rng(4)
    vals = np.tile(v0, (64, 1))
    vals[:, int(el[2]["param"])] *= np.exp(g.uniform(-1, 1, 64))
    plan = analysis.Plan(el, c.n_nodes, len(v0))
    bt = analysis.Batch(plan, vals)
    sp = analysis.TranSpec(step=1e-7, stop=1e-5)
    cap = 4096
    wave, tim, npts, st, steps, it = bt.tran(sp, analysis.Options(reltol=1e-6, kernel="specialized"), capacity=cap)
    assert bt.last_kernel == "specialized-registers"
    gw, gt, gnp, gst, gsteps, git = bt.tran(sp, analysis.Options(reltol=1e-6, kernel="generic"), capacity=cap)
    assert np.all(st == 0) and np.array_equal(st, gst)
    assert np.all(np.abs(steps - gsteps) <= 2)
    for i in range(0, 64, 8):
        ost, ot, ox, _, osteps, _, _ = orc.tran(orc.Packed(el, c.n_nodes, vals[i]), ospec(sp), orc.options(reltol=1e-6),
                                             capacity=cap)
        assert ost == 0
        assert abs(steps[i] - osteps) <= max(2, 0.01 * osteps)
        k = int(npts[i])
        # the waveform at the oracle's accepted times, by interpolation of ours
        for j in range(ox.shape[1]):
            y = np.interp(ot, tim[i, :k], wave[i, :k, j])
            assert np.all(np.abs(y - ox[:, j]) <= 1e-3 * np.abs(ox[:, j]) + 2e-3), (i, j)
