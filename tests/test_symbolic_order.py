"""Pin the host's sparse symbolic analysis against the reference's ordering.

The reference's sparse backend keeps every entry the loads stamp as a slot for
the rest of the run (solver/sparse.go:114-143) and orders the columns by
minimumDegree of that pattern (:154-187, :412-452).  The engine's symbolic
analysis (ks_sparse_analyze / ks_sparse_pattern, one fixed pivot sequence per
circuit and analysis) restates the same pattern from the devices' stamp
sequences and the same minimum degree.  The orders must be identical, column for
column, wherever the reference's run stamped every entry a device can stamp.
The one difference by contract: a fixed pivot sequence holds every entry any
Newton iteration may stamp, while the reference's pattern only has the entries
its own iterations stamped; a MOSFET that stays in cutoff through a whole
operating point (level 1: gm = gds = gmbs = 0) never stamps its channel, and
there the engine's order is still minimumDegree of its own pattern, bit for bit.
"""
import json
import os

import numpy as np
import pytest

from kronspice_gb300 import analysis, workloads
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_cases.json")) as f:
    CASES = [c for c in json.load(f)["cases"] if not c["skip"]]
TRAN_CASES = [c for c in CASES if any(a["kind"] == "tran" for a in c["circuit"]["analyses"])]


def offdiag(p):
    q = p.copy()
    np.fill_diagonal(q, False)
    return q


def both(ckt, tr=None):
    el, vals, _ = ckt.pack()
    spec = None
    if tr is not None:
        spec = orc.TranSpec(tr["step"], tr["stop"], tr["start"], tr["max_step"], int(tr["uic"]), 0, 0, 0, 0, 0, 0)
    st, oorder, opat = orc.sparse_order(orc.Packed(el, ckt.n_nodes, vals), spec)
    q, prow, epat = analysis.sparse_analysis(el, ckt.n_nodes, vals, step=0.0 if tr is None else tr["step"])
    return st, oorder, opat, q, prow, epat


def cutoff_mosfets(ckt):
    """The MOSFETs whose drain current at the oracle's operating point is only
    their junctions' gmin leakage (below 0.1 nA): no channel current."""
    el, vals, _ = ckt.pack()
    st, x, elem, led, _, _ = orc.op_results(orc.Packed(el, ckt.n_nodes, vals))
    assert st == 0
    return [e.name for k, e in enumerate(ckt.elements) if e.kind == "M" and abs(elem[k, orc.RES["current"]]) <= 1e-10]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_operating_point_order_matches_reference(case):
    ckt = kc.from_dict(case["circuit"])
    st, oorder, opat, q, prow, epat = both(ckt)
    if case["name"] == "switch_relax_tran":
        # a relaxation oscillator has no consistent switch state at DC: its
        # operating point does not converge (device/switch.go:39-42); the golden
        # transient starts from UIC
        assert st == 3  # KS_STATUS_NO_CONVERGENCE
        return
    assert st == 0
    # the minimum degree restatement itself, bit for bit, on the engine's pattern
    assert np.array_equal(orc.min_degree(epat), q)
    # every entry the reference's run stamped is in the engine's pattern
    assert np.all(~offdiag(opat) | offdiag(epat))
    extra = offdiag(epat) & ~offdiag(opat)
    if not extra.any():
        assert np.array_equal(q, oorder)
        return
    # only the channels of MOSFETs the operating point left in cutoff: at most
    # (d', g), (s', g), (d', s'), (s', d') each
    off = cutoff_mosfets(ckt)
    assert off, "extra entries without a cutoff transistor"
    assert extra.sum() <= 4 * len(off)


@pytest.mark.parametrize("case", TRAN_CASES, ids=[c["name"] for c in TRAN_CASES])
def test_transient_order_matches_reference(case):
    ckt = kc.from_dict(case["circuit"])
    tr = [a for a in case["circuit"]["analyses"] if a["kind"] == "tran"][-1]
    st, oorder, opat, q, prow, epat = both(ckt, tr)
    assert st == 0
    assert np.array_equal(offdiag(opat), offdiag(epat))
    assert np.array_equal(q, oorder)


def test_operating_point_orders_of_random_netlists():
    """200 seeded random netlists (10 to 400 nodes; R, C, L, diodes, a source):
    the engine's column order is the reference's, column for column."""
    for ckt in workloads.random_netlists(200, seed=7):
        st, oorder, opat, q, prow, epat = both(ckt)
        assert st == 0
        assert np.array_equal(offdiag(opat), offdiag(epat))
        assert np.array_equal(q, oorder)
        # the pivot rows are a permutation (every step pivots a distinct row)
        assert np.array_equal(np.sort(prow), np.arange(len(q)))


def test_transient_orders_of_random_netlists():
    """The transient pattern (companion stamps added) of 40 of them."""
    for ckt in workloads.random_netlists(40, seed=8, nodes=(10, 120)):
        tr = dict(step=1e-7, stop=2e-6, start=0.0, max_step=0.0, uic=False)
        st, oorder, opat, q, prow, epat = both(ckt, tr)
        assert st == 0
        assert np.array_equal(offdiag(opat), offdiag(epat))
        assert np.array_equal(q, oorder)


def test_only_cutoff_inverters_differ():
    """The golden operating points whose order differs from the reference's are
    exactly the level-1 CMOS inverters at input 0 (NMOS in cutoff)."""
    differ = []
    for case in CASES:
        ckt = kc.from_dict(case["circuit"])
        st, oorder, opat, q, prow, epat = both(ckt)
        if not np.array_equal(q, oorder):
            differ.append(case["name"])
    assert sorted(differ) == ["mos1_cmos_vtc", "mos1_inv_tran"], differ


def lu_and_reach(ckt, step=0.0):
    el, vals, _ = ckt.pack()
    q, prow, epat = analysis.sparse_analysis(el, ckt.n_nodes, vals, step=step)
    lu = analysis.sparse_lu_pattern(el, ckt.n_nodes, vals, step=step)
    reach, bad = orc.reach_pattern(epat, q, prow)
    return lu, reach, bad


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_lu_pattern_is_the_reach_of_the_pivot_sequence(case):
    """The engine's L + U slots (row-wise symbolic elimination on its fixed pivot
    sequence) are the reference's Gilbert-Peierls reach sets (solver/sparse.go:
    301-352) for the same pattern, column order and pivot rows, entry for entry,
    at the operating point and, for the transient netlists, at their step."""
    ckt = kc.from_dict(case["circuit"])
    lu, reach, bad = lu_and_reach(ckt)
    assert bad == -1 and np.array_equal(lu, reach)
    for a in case["circuit"]["analyses"]:
        if a["kind"] == "tran":
            lu, reach, bad = lu_and_reach(ckt, a["step"])
            assert bad == -1 and np.array_equal(lu, reach)


def test_lu_patterns_of_random_netlists_are_their_reach():
    fill = 0
    for ckt in workloads.random_netlists(120, seed=9, nodes=(10, 200)):
        lu, reach, bad = lu_and_reach(ckt)
        assert bad == -1 and np.array_equal(lu, reach)
        el, vals, _ = ckt.pack()
        q, prow, epat = analysis.sparse_analysis(el, ckt.n_nodes, vals)
        fill += int(lu.sum()) - int(epat[np.ix_(prow, q)].sum())
    assert fill > 1000  # the factors' fill is part of what is compared


def test_pivot_rows_of_the_golden_operating_points():
    """The engine's pivot rows (chosen once, on a representative matrix) are the
    ones the reference's last factorization of the operating point pivoted on
    (threshold partial pivoting with the diagonal preferred, solver/sparse.go:
    256-281) on every golden netlist whose column order is the reference's.  On
    circuits whose junctions or companions change which entry dominates a column,
    they may differ: a fixed pivot failing its run-time threshold hands the solve
    to partial pivoting, so results do not depend on it."""
    compared = 0
    for case in CASES:
        ckt = kc.from_dict(case["circuit"])
        el, vals, _ = ckt.pack()
        st, order, _, piv = orc.sparse_order(orc.Packed(el, ckt.n_nodes, vals), None, None, pivots=True)
        q, prow, _ = analysis.sparse_analysis(el, ckt.n_nodes, vals)
        if st != 0 or not np.array_equal(order, q):
            continue
        assert np.array_equal(piv, prow), case["name"]
        compared += 1
    assert compared >= 40
