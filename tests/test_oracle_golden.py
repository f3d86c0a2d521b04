"""Pin the CPU oracle against the reference's golden vectors.

Mirrors TestGolden and TestNgspiceTwin (analysis/op_test.go:116-158, checkGolden
:161-284; AC at :214-236): every in-scope golden netlist runs on the dense and on the sparse
backend and must match the independent reference (testdata/golden) and the
ngspice-39 twin (testdata/golden/ngspice) with internal/golden/golden.go's
tolerances.  The fixtures come from tests/golden/make_reference_fixtures.py.
"""
import json
import os

import numpy as np
import pytest

import golden_compare as gc
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_cases.json")) as f:
    CASES = json.load(f)["cases"]

PARAMS = []
for c in CASES:
    for src in ("independent", "ngspice"):
        if src in c["golden"]:
            for be in ((1, 2) if src == "independent" else (0,)):
                PARAMS.append(pytest.param(c, src, be, id="%s/%s/%s" % (c["name"], src, ["auto", "dense", "sparse"][be])))


def _getter_op(ckt, x, cur):
    def get(name):
        if name.startswith("v("):
            node = name[2:-1]
            i = ckt.node_index(node)
            if i == 0:
                return 0.0
            return None if i < 0 else x[i - 1]
        k = ckt.element_index(name[2:-1])
        return None if k < 0 else cur[k]
    return get


def run_case(case, src, backend):
    if case["skip"]:
        pytest.skip(case["skip"])
    ckt = kc.from_dict(case["circuit"])
    pk = orc.Packed.of(ckt)
    want = case["golden"][src]
    opt = orc.options(backend=backend)
    an = case["circuit"]["analyses"]
    if want["kind"] == "values":
        st, x, cur, _, msg = orc.op(pk, opt)
        assert st == 0, msg
        get = _getter_op(ckt, x, cur)
        got = {k: get(k) for k in want["values"] if get(k) is not None}
        return gc.compare_values(got, want["values"])
    dcs = [a for a in an if a["kind"] == "dc"]
    if dcs:
        a = dcs[0]
        vals = gc.sweep_values(a["start"], a["stop"], a["step"])
        k = ckt.element_index(a["source"])
        st, x, cur, msg = orc.dc(pk, k, vals, opt)
        assert st == 0, msg

        def get(name):
            if name.startswith("v("):
                i = ckt.node_index(name[2:-1])
                return None if i < 0 else (np.zeros(len(vals)) if i == 0 else x[:, i - 1])
            e = ckt.element_index(name[2:-1])
            return None if e < 0 else cur[:, e]
        return gc.compare_sweep(vals, get, want)
    acs = [a for a in an if a["kind"] == "ac"]
    if acs:
        a = acs[0]
        freqs = gc.ac_frequencies(a["variation"], a["points"], a["fstart"], a["fstop"])
        st, x, msg = orc.ac(pk, freqs, opt)
        assert st == 0, msg

        def get(node):
            i = ckt.node_index(node)
            return None if i < 0 else (np.zeros(len(freqs), complex) if i == 0 else x[:, i - 1])
        return gc.compare_ac(freqs, get, want)
    tr = [a for a in an if a["kind"] == "tran"][-1]
    spec = orc.TranSpec(tr["step"], tr["stop"], tr["start"], tr["max_step"], int(tr["uic"]), 0, 0, 0, 0, 0, 0)
    st, t, x, cur, steps, iters, msg = orc.tran(pk, spec, opt)
    assert st == 0, msg
    t = list(t)

    def get(name):
        if name.startswith("v("):
            i = ckt.node_index(name[2:-1])
            return None if i < 0 else (np.zeros(len(t)) if i == 0 else list(x[:, i - 1]))
        e = ckt.element_index(name[2:-1])
        return None if e < 0 else list(cur[:, e])
    if src == "ngspice":
        return gc.compare_table_at_sim(t, get, want)
    return gc.compare_table(t, get, want)


@pytest.mark.parametrize("case,src,backend", PARAMS)
def test_oracle_matches_golden(case, src, backend):
    msgs = run_case(case, src, backend)
    assert not msgs, "\n".join(msgs)


def test_in_scope_cases_are_many():
    # every one of the reference's 45 golden netlists uses only the engine's
    # element kinds and analyses (OP, DC sweep, transient, AC)
    assert sum(1 for c in CASES if not c["skip"]) == 45
