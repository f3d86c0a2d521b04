"""GPU parity of the batched operating point against the CPU FP64 oracle.

The engine (FP64 plain and FP32-LU/FP64-residual mixed precision) must return
the oracle's status for every circuit and node voltages within the SPICE
tolerance the analyses run at (reltol 1e-6, vntol 1e-6 V, abstol 1e-12 A);
plain FP64 takes the same Newton path as the oracle, so it must also agree to
1e-9 relative with the same iteration counts for nearly every circuit.
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
RELTOL, VNTOL, ABSTOL = 1e-6, 1e-6, 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def tol(x_ref, isv, rel=RELTOL):
    return np.where(isv, VNTOL, ABSTOL) + rel * np.abs(x_ref)


def run_both(el, nn, vals, opt_gpu, opt_cpu, x0=None):
    plan = analysis.Plan(el, nn, vals.shape[1])
    b = analysis.Batch(plan, vals)
    xg, sg, ig = b.op(opt_gpu, x0)
    pk = orc.Packed(el, nn, vals)
    so, xo, io = orc.batch_op(pk, vals.shape[0], opt_cpu, x0=x0)
    _, isv = orc.unknowns(orc.Packed(el, nn, vals[0]))
    return (xg, sg, ig), (xo, so, io), isv


@pytest.mark.parametrize("precision,passes", [("fp64", 0), ("mixed", 0), ("mixed", 1)])
def test_bjt_ce_batch_matches_oracle(precision, passes):
    """mixed: every linear solve refined from the FP64 residual (default), or one
    unchecked pass per Newton step (passes=1, well-conditioned systems)."""
    el, nn, vals = workloads.bjt_ce_batch(4096, seed=11)
    og = analysis.Options(reltol=RELTOL, precision=precision, mixed_passes=passes)
    oc = orc.options(reltol=RELTOL)
    (xg, sg, ig), (xo, so, io), isv = run_both(el, nn, vals, og, oc)
    assert np.array_equal(sg, so), np.nonzero(sg != so)
    ok = so == 0
    assert ok.mean() > 0.99
    err = np.abs(xg[ok] - xo[ok])
    assert np.all(err <= tol(xo[ok], isv)), err.max()
    if precision == "fp64":
        assert np.all(err <= 1e-9 * np.abs(xo[ok]) + np.where(isv, 1e-12, 1e-18))
        assert (ig == io).mean() > 0.99


def test_bjt_ce_nodeset_start():
    # a start near the solution (Options.NodeSet, analysis/newton.go:221-243) converges in fewer iterations
    el, nn, vals = workloads.bjt_ce_batch(1024, seed=5)
    oc = orc.options(reltol=RELTOL)
    so, xo, io = orc.batch_op(orc.Packed(el, nn, vals), 1024, oc)
    x0 = xo * (1 + 1e-4)
    og = analysis.Options(reltol=RELTOL, precision="mixed")
    (xg, sg, ig), (xo2, so2, io2), isv = run_both(el, nn, vals, og, oc, x0=x0)
    assert np.array_equal(sg, so2)
    ok = so2 == 0
    assert np.all(np.abs(xg[ok] - xo2[ok]) <= tol(xo2[ok], isv))
    assert ig[ok].mean() < 0.6 * io[ok].mean()


with open(os.path.join(ROOT, "tests", "golden", "reference_cases.json")) as f:
    CASES = [c for c in json.load(f)["cases"] if not c["skip"]]
OP_CASES = [c for c in CASES if c["circuit"]["analyses"][0]["kind"] == "op"]
DC_CASES = [c for c in CASES if c["circuit"]["analyses"][0]["kind"] == "dc"]


@pytest.mark.parametrize("case", OP_CASES, ids=[c["name"] for c in OP_CASES])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_golden_op_on_gpu(case, precision):
    ckt = kc.from_dict(case["circuit"])
    res, errs = analysis.op_batch([ckt], analysis.Options(precision=precision))
    assert errs[0] is None, errs[0]
    x = res[0].x
    st, xo, cur, _, _ = orc.op(orc.Packed.of(ckt))
    assert st == 0
    _, isv = orc.unknowns(orc.Packed.of(ckt))
    assert np.all(np.abs(x - xo) <= tol(xo, isv, 1e-6))
    want = case["golden"]["independent"]["values"]
    got = {}
    for k in want:
        if k.startswith("v("):
            i = ckt.node_index(k[2:-1])
            got[k] = 0.0 if i == 0 else x[i - 1]
    assert not gc.compare_values(got, {k: v for k, v in want.items() if k in got})


@pytest.mark.parametrize("case", DC_CASES, ids=[c["name"] for c in DC_CASES])
def test_golden_dc_sweep_points_on_gpu(case):
    """Every sweep point as one circuit of a batch (cold start each), against the
    golden sweep with CompareSweep's tolerances (internal/golden/golden.go:341-372)."""
    ckt = kc.from_dict(case["circuit"])
    a = case["circuit"]["analyses"][0]
    pts = gc.sweep_values(a["start"], a["stop"], a["step"])
    el, v0, _ = ckt.pack()
    k = ckt.element_index(a["source"])
    vals = np.tile(v0, (len(pts), 1))
    vals[:, int(el[k]["param"])] = pts
    plan = analysis.Plan(el, ckt.n_nodes, len(v0))
    x, st, it = analysis.Batch(plan, vals).op(analysis.Options())
    assert np.all(st == 0), st
    want = case["golden"]["independent"]
    names = [nm for nm in want["names"] if nm.startswith("v(")]
    if not names:
        pytest.skip("golden sweep holds only currents")

    def get(nm):
        i = ckt.node_index(nm[2:-1])
        return np.zeros(len(pts)) if i == 0 else x[:, i - 1]
    sub = dict(want, names=names)
    assert not gc.compare_sweep(pts, get, sub)


@pytest.mark.parametrize("case", DC_CASES, ids=[c["name"] for c in DC_CASES])
def test_golden_dc_sweep_chained_on_gpu(case):
    """ks_dc_sweep: the sweep's points in order, each warm-started from the
    previous one (analysis/dc.go:104-128), against the oracle's chained sweep
    and the golden table."""
    ckt = kc.from_dict(case["circuit"])
    a = case["circuit"]["analyses"][0]
    pts = gc.sweep_values(a["start"], a["stop"], a["step"])
    el, v0, _ = ckt.pack()
    k = ckt.element_index(a["source"])
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, len(v0)), v0[None, :])
    x, st, npts, it = b.dc_sweep(k, pts, analysis.Options(precision="fp64"))
    assert st[0] == 0 and npts[0] == len(pts), st
    ost, ox, _, msg = orc.dc(orc.Packed.of(ckt), k, pts)
    assert ost == 0, msg
    _, isv = orc.unknowns(orc.Packed.of(ckt))
    assert np.all(np.abs(x[0] - ox) <= tol(ox, isv, 1e-6)), np.abs(x[0] - ox).max()
    want = case["golden"]["independent"]
    names = [nm for nm in want["names"] if nm.startswith("v(")]
    if names:
        def get(nm):
            i = ckt.node_index(nm[2:-1])
            return np.zeros(len(pts)) if i == 0 else x[0, :, i - 1]
        assert not gc.compare_sweep(pts, get, dict(want, names=names))


@pytest.mark.parametrize("name,inner,outer,vals2", [
    ("bjt_output_dc", "VCE", "IB", [5e-6, 10e-6, 20e-6, 40e-6]),
    ("mos1_idvd_dc", "VDS", "VGS", [1.0, 1.5, 2.5, 4.0]),
])
def test_nested_dc_sweep_on_gpu(name, inner, outer, vals2):
    """A second, outer swept source (analysis/dc.go:100-111): the family of
    output characteristics in one chained sweep, against the oracle's."""
    case = [c for c in DC_CASES if c["name"] == name][0]
    ckt = kc.from_dict(case["circuit"])
    a = case["circuit"]["analyses"][0]
    pts = gc.sweep_values(a["start"], a["stop"], a["step"])
    el, v0, _ = ckt.pack()
    k, k2 = ckt.element_index(inner), ckt.element_index(outer)
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, len(v0)), v0[None, :])
    x, st, npts, it = b.dc_sweep(k, pts, analysis.Options(precision="fp64"), src2=k2, values2=vals2)
    assert st[0] == 0 and npts[0] == len(pts) * len(vals2), st
    ost, ox, _, msg = orc.dc2(orc.Packed.of(ckt), k, pts, k2, vals2)
    assert ost == 0, msg
    _, isv = orc.unknowns(orc.Packed.of(ckt))
    assert np.all(np.abs(x[0] - ox) <= tol(ox, isv, 1e-6)), np.abs(x[0] - ox).max()
    # the last outer value's inner sweep is the single sweep at that value (to
    # the Newton tolerance: the two start each point from different iterates)
    v1 = v0.copy()
    v1[int(el[k2]["param"])] = vals2[-1]
    ost1, ox1, _, _ = orc.dc(orc.Packed(el, ckt.n_nodes, v1), k, pts)
    assert ost1 == 0
    assert np.all(np.abs(x[0, -len(pts):] - ox1) <= tol(ox1, isv, 1e-3))


def test_dc_sweep_refusals():
    ckt = kc.from_dict(DC_CASES[0]["circuit"])
    el, v0, _ = ckt.pack()
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, len(v0)), v0[None, :])
    r = [i for i, e in enumerate(ckt.elements) if e.kind not in ("V", "I")][0]
    with pytest.raises(Exception) as e:
        b.dc_sweep(r, [0.0, 1.0])
    assert "swept source not found" in str(e.value)


def test_typed_errors():
    # TestSingularVoltageLoop, analysis/op_test.go:87: two sources in parallel
    b = kc.Builder("loop")
    b.voltage_source("V1", "a", "0", 1.0)
    b.voltage_source("V2", "a", "0", 2.0)
    b.resistor("R1", "a", "0", 1e3)
    # TestNoConvergenceIsTyped, analysis/newton_test.go:64: ITL1 = 2 without fallbacks
    d = kc.Builder("diode")
    d.voltage_source("V1", "a", "0", 5.0)
    d.resistor("R1", "a", "b", 1e3)
    d.model("dm", "d", {"is": 1e-14})
    d.diode("D1", "b", "0", "dm")
    opt = analysis.Options(itl1=2, no_gmin_stepping=True, no_source_stepping=True, no_pseudo_transient=True)
    res, errs = analysis.op_batch([b.build(), d.build()], opt)
    assert isinstance(errs[0], analysis.ErrSingularMatrix)
    assert isinstance(errs[1], analysis.ErrNoConvergence)
    # the same diode converges with the defaults
    res, errs = analysis.op_batch([d.build()])
    assert errs[0] is None and 0.5 < res[0].node_voltages[2] < 0.8


def test_fallback_chain_matches_oracle():
    # TestSteppingAgrees-style: force each fallback by ITL1 small; results match the oracle path
    el, nn, vals = workloads.bjt_ce_batch(512, seed=7)
    for kw in ({"no_source": True, "no_pt": True}, {"no_gmin": True, "no_pt": True}, {"no_gmin": True, "no_source": True}):
        og = analysis.Options(itl1=4, no_gmin_stepping=kw.get("no_gmin", False),
                              no_source_stepping=kw.get("no_source", False), no_pseudo_transient=kw.get("no_pt", False))
        oc = orc.options(itl1=4, **kw)
        (xg, sg, ig), (xo, so, io), isv = run_both(el, nn, vals, og, oc)
        assert np.array_equal(sg, so)
        ok = so == 0
        assert np.all(np.abs(xg[ok] - xo[ok]) <= tol(xo[ok], isv, 1e-3))


@pytest.mark.parametrize("precision,passes", [("fp64", 0), ("mixed", 0)])
def test_cmos_opamp_batch_matches_oracle(precision, passes):
    """Level-1 two-stage op-amp variants (the 24-D parameter workload)."""
    el, nn, vals = workloads.cmos_opamp_batch(2048, seed=13)
    og = analysis.Options(reltol=RELTOL, precision=precision, mixed_passes=passes)
    oc = orc.options(reltol=RELTOL)
    (xg, sg, ig), (xo, so, io), isv = run_both(el, nn, vals, og, oc)
    assert np.array_equal(sg, so), np.nonzero(sg != so)
    ok = so == 0
    assert ok.mean() > 0.98
    assert np.all(np.abs(xg[ok] - xo[ok]) <= tol(xo[ok], isv, 1e-5))
