"""The oracle's DC sweeps (analysis/dc.go:51-133) without a GPU: a nested sweep
with one outer value is the single sweep at that value (bit for bit: the
override and the DC value are the same number), and its later outer values chain
warm from the previous inner sweep's end while landing on the same points to the
Newton tolerance.  The golden sweeps are pinned in test_oracle_golden."""
import json
import os

import numpy as np

from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

import golden_compare as gc

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_cases.json")) as f:
    CASES = {c["name"]: c for c in json.load(f)["cases"]}


def test_nested_sweep_of_the_bjt_output_family():
    case = CASES["bjt_output_dc"]
    ckt = kc.from_dict(case["circuit"])
    a = case["circuit"]["analyses"][0]
    pts = gc.sweep_values(a["start"], a["stop"], a["step"])
    el, v0, _ = ckt.pack()
    k, k2 = ckt.element_index("VCE"), ckt.element_index("IB")
    ib = [5e-6, 10e-6, 20e-6, 40e-6]
    st, x, cur, msg = orc.dc2(orc.Packed.of(ckt), k, pts, k2, ib)
    assert st == 0, msg
    assert x.shape[0] == len(pts) * len(ib)
    _, isv = orc.unknowns(orc.Packed.of(ckt))
    for j, v in enumerate(ib):
        vals = v0.copy()
        vals[int(el[k2]["param"])] = v
        s1, x1, _, _ = orc.dc(orc.Packed(el, ckt.n_nodes, vals), k, pts)
        assert s1 == 0
        got = x[j * len(pts):(j + 1) * len(pts)]
        if j == 0:
            assert np.array_equal(got, x1)  # the same chain from the same cold start
        else:
            assert np.all(np.abs(got - x1) <= np.where(isv, 1e-6, 1e-12) + 1e-3 * np.abs(x1))
    # the collector current rises with the base current at every VCE past saturation
    br = int(np.flatnonzero(~np.asarray(isv, bool))[0])  # the VCE branch current (the only branch)
    ic = -x[:, br].reshape(len(ib), len(pts))  # positive into the collector
    assert np.all(np.diff(ic[:, np.asarray(pts) > 1.0], axis=0) > 0)
