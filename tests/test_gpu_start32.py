"""GPU parity of the FP32 start stage and of the learned start's basin check.

The FP32 stage (ks_options.fp32_start_iters) runs Newton in FP32 from the
start before the FP64 solve; the FP64 Newton, its convergence test and its
fallback chain stay the reference's, so every circuit must still return the
oracle's status and node voltages within the SPICE tolerance the analyses run
at, while the FP64 iterations drop.  The basin check (ks_options.start_check)
solves a circuit again from InitJct when its solution ends far from the given
start; with it, a start that lands far away returns exactly the standard
start's result.
"""
import json
import os

import numpy as np
import pytest

from kronspice_gb300 import analysis, build, workloads
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RELTOL, VNTOL, ABSTOL = 1e-6, 1e-6, 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def tol(x_ref, isv, rel=RELTOL):
    return np.where(isv, VNTOL, ABSTOL) + rel * np.abs(x_ref)


def oracle_op(el, nn, vals, x0=None):
    so, xo, io = orc.batch_op(orc.Packed(el, nn, vals), vals.shape[0], orc.options(reltol=RELTOL), x0=x0)
    _, isv = orc.unknowns(orc.Packed(el, nn, vals[0]))
    return so, xo, io, isv


@pytest.mark.parametrize("kernel", ["specialized", "generic"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bjt_ce_fp32_stage_matches_oracle(kernel, precision):
    el, nn, vals = workloads.bjt_ce_batch(4096, seed=11)
    so, xo, io, isv = oracle_op(el, nn, vals)
    b = analysis.Batch(analysis.Plan(el, nn, vals.shape[1]), vals)
    x1, s1, i1 = b.op(analysis.Options(reltol=RELTOL, precision=precision, kernel=kernel))
    xg, sg, ig = b.op(analysis.Options(reltol=RELTOL, precision=precision, kernel=kernel, fp32_start_iters=60))
    assert np.array_equal(sg, so), np.nonzero(sg != so)
    ok = so == 0
    assert ok.mean() > 0.99
    assert np.all(np.abs(xg[ok] - xo[ok]) <= tol(xo[ok], isv)), np.abs(xg[ok] - xo[ok]).max()
    # the FP64 Newton starts next to the solution: far fewer FP64 iterations
    assert ig[ok].mean() < 0.5 * i1[ok].mean(), (ig[ok].mean(), i1[ok].mean())
    assert ig[ok].max() <= i1[ok].max()


def test_cmos_opamp_fp32_stage_matches_oracle():
    """Level-1 op-amps on the generic kernel (9 unknowns, eight MOSFETs)."""
    el, nn, vals = workloads.cmos_opamp_batch(2048, seed=13)
    so, xo, io, isv = oracle_op(el, nn, vals)
    b = analysis.Batch(analysis.Plan(el, nn, vals.shape[1]), vals)
    x1, s1, i1 = b.op(analysis.Options(reltol=RELTOL, precision="mixed"))
    xg, sg, ig = b.op(analysis.Options(reltol=RELTOL, precision="mixed", fp32_start_iters=200))
    assert np.array_equal(sg, so), np.nonzero(sg != so)
    ok = so == 0
    assert ok.mean() > 0.98
    assert np.all(np.abs(xg[ok] - xo[ok]) <= tol(xo[ok], isv, 1e-5)), np.abs(xg[ok] - xo[ok]).max()
    # most circuits finish in a couple of FP64 iterations; the few whose FP32
    # chain fails run the FP64 chain as before
    assert np.median(ig[ok]) <= 3 and np.median(i1[ok]) > 10, (np.median(ig[ok]), np.median(i1[ok]))


def test_fp32_stage_from_a_given_start():
    """x0 near the solution (NodeSet): the stage refines it, the FP64 solve finishes."""
    el, nn, vals = workloads.bjt_ce_batch(2048, seed=5)
    so, xo, io, isv = oracle_op(el, nn, vals)
    x0 = xo * (1 + 2e-2)
    b = analysis.Batch(analysis.Plan(el, nn, vals.shape[1]), vals)
    xg, sg, ig = b.op(analysis.Options(reltol=RELTOL, precision="mixed", fp32_start_iters=60), x0)
    assert np.array_equal(sg, so)
    ok = so == 0
    assert np.all(np.abs(xg[ok] - xo[ok]) <= tol(xo[ok], isv))
    assert ig[ok].mean() <= 3.0, ig[ok].mean()


with open(os.path.join(ROOT, "tests", "golden", "reference_cases.json")) as f:
    OP_CASES = [c for c in json.load(f)["cases"] if not c["skip"] and c["circuit"]["analyses"][0]["kind"] == "op"]


@pytest.mark.parametrize("case", OP_CASES, ids=[c["name"] for c in OP_CASES])
def test_golden_op_with_fp32_stage(case):
    """Every golden operating point (levels 2 and 3 skip the stage) still meets the
    oracle.  The stage changes the Newton path, so both solve at reltol 1e-6 and
    may differ by up to each one's own tolerance."""
    ckt = kc.from_dict(case["circuit"])
    res, errs = analysis.op_batch([ckt], analysis.Options(reltol=RELTOL, precision="mixed", fp32_start_iters=100))
    assert errs[0] is None, errs[0]
    st, xo, _, _, _ = orc.op(orc.Packed.of(ckt), orc.options(reltol=RELTOL))
    assert st == 0
    _, isv = orc.unknowns(orc.Packed.of(ckt))
    assert np.all(np.abs(res[0].x - xo) <= 2 * tol(xo, isv, RELTOL))


def test_start_check_resolves_from_initjct():
    """A start 1 V off at every node converges to the same operating point but
    ends farther than start_check from it: every circuit is solved again from
    InitJct, and the FP64 result is the standard start's, bit for bit."""
    el, nn, vals = workloads.bjt_ce_batch(1024, seed=3)
    so, xo, io, isv = oracle_op(el, nn, vals)
    b = analysis.Batch(analysis.Plan(el, nn, vals.shape[1]), vals)
    opt = dict(reltol=RELTOL, precision="fp64", kernel="generic")
    xs, ss, is_ = b.op(analysis.Options(**opt))
    x0 = xo.copy()
    x0[:, :nn - 1] += 1.0
    xn, sn, in_ = b.op(analysis.Options(**opt), x0)
    xc, sc, ic = b.op(analysis.Options(start_check=0.5, **opt), x0)
    ok = so == 0
    assert np.array_equal(sc, ss) and np.array_equal(sc, so)
    assert np.array_equal(xc[ok], xs[ok])
    # the check ran both solves: its iterations are the given start's plus InitJct's
    both = (sn == 0) & ok
    assert np.array_equal(ic[both], in_[both] + is_[both])
    # a tight start passes the check untouched
    xt, st_, it_ = b.op(analysis.Options(start_check=0.5, **opt), xo)
    xu, su, iu = b.op(analysis.Options(**opt), xo)
    assert np.array_equal(xt, xu) and np.array_equal(it_, iu)
