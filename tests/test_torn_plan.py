"""The torn engine's symbolic plan (ks_torn_plan, host only) is the reference's.

buildPlan (kron/jacobian.go:296-389) is integer work: the pieces are the
connected components of the Jacobian's pattern without the torn node pairs,
numbered in order of their first unknown, and the coupling rows are the rows of
entries that join two pieces.  The engine must reproduce it exactly; the oracle
restates it (oracle/oracle_torn.hpp) on the pattern of a backward-Euler step.
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


def same_plan(el, nn, vals, cut):
    pk = orc.Packed(el, nn, vals)
    st, pairs, msg = orc.torn_cuts(pk, cut)
    assert st == 0, msg
    opiece, orows, onp = orc.torn_plan(pk, pairs, 1e-9)
    piece, rows, _, _ = analysis.torn_plan(el, nn, len(vals), cut)
    assert np.array_equal(piece, opiece)
    assert sorted(rows.tolist()) == sorted(orows.tolist())
    return onp


def test_golden_netlists_tear_as_the_reference():
    compared = split = 0
    for case in CASES:
        ckt = kc.from_dict(case["circuit"])
        el, vals, _ = ckt.pack()
        pk = orc.Packed(el, ckt.n_nodes, vals)
        single = [i for i in range(len(ckt.elements))
                  if orc.torn_cuts(pk, [i])[0] == 0 and len(orc.torn_cuts(pk, [i])[1])]
        cuts = [[i] for i in single] + ([single] if len(single) > 1 else [])
        for cut in cuts:
            try:
                npieces = same_plan(el, ckt.n_nodes, vals, cut)
            except ValueError:
                continue  # the oracle's one-step transient does not run for this netlist
            compared += 1
            split += npieces > 1
    assert compared >= 70 and split >= 35, (compared, split)


@pytest.mark.parametrize("N,P,loads", [(16, 2, 16), (64, 4, 64)])
def test_power_grid_pieces(N, P, loads):
    el, nn, vals, torn, c = workloads.power_grid_batch(1, N=N, P=P, loads=loads)
    assert same_plan(el, nn, vals[0], torn) == P * P


def test_full_power_grid_plan():
    """256 x 256 grid: 16 pieces of 4,096 grid nodes plus their pad and source
    branch, 3,036 coupling rows (both ends of the 1,536 torn resistors, corners
    counted once), a band of 65 + 65 after the pseudo-peripheral order."""
    el, nn, vals, torn, c = workloads.power_grid_batch(1)
    piece, rows, max_piece, max_band = analysis.torn_plan(el, nn, vals.shape[1], torn)
    assert piece.max() + 1 == 16
    assert np.bincount(piece).tolist() == [4098] * 16
    assert len(rows) == 3036 and max_piece == 4098 and max_band == 130
