"""GPU parity of the torn solves (ks_torn_*) against the oracle.

The engine tears each variant's Jacobian as kron.JacobianTearing does and
refines every solve against the exact Jacobian to a componentwise backward
error of 1e-14 (kron/jacobian.go:551-589), so its Newton iterates are those of
an untorn solve up to round-off: operating points and backward-Euler
transients of seeded power grids must match the oracle's untorn runs (and its
restatement of the torn solver) to 1e-9 of the largest node voltage, with and
without factor reuse.  The reference's own tearing cases (TestJacobianErrors,
kron/jacobian_test.go:284-308) are refused with its messages.
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
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def grid(V, N, P, loads, seed=0):
    el, nn, vals, torn, c = workloads.power_grid_batch(V, seed=seed, N=N, P=P, loads=loads)
    return el, nn, vals, torn, c


@pytest.mark.parametrize("reuse", [True, False])
def test_power_grid_op_matches_oracle(reuse):
    el, nn, vals, torn, c = grid(4, 16, 2, 16)
    tb = analysis.TornBatch(el, nn, vals, torn)
    assert tb.pieces == 4 and tb.coupling_rows > 0
    x, st, it, stats = tb.op(analysis.Options(reltol=1e-6), reuse=reuse)
    assert np.all(st == 0), st
    for v in range(len(vals)):
        s0, x0, _, it0, msg = orc.op(orc.Packed(el, nn, vals[v]), orc.options(reltol=1e-6))
        assert s0 == 0, msg
        assert np.abs(x[v] - x0).max() <= 1e-9 * np.abs(x0).max(), np.abs(x[v] - x0).max()
        assert it[v] == it0
    if not reuse:
        assert stats["refactors"] == stats["solves"]


@pytest.mark.parametrize("reuse", [True, False])
def test_power_grid_transient_matches_oracle(reuse):
    el, nn, vals, torn, c = grid(3, 16, 2, 16, seed=1)
    tb = analysis.TornBatch(el, nn, vals, torn)
    spec = analysis.TranSpec(step=0.1e-9, stop=40 * 0.1e-9, fixed_step=True, method="be")
    probes = np.arange(0, tb.n, 7)
    wave, x, st, steps, it, stats = tb.tran(spec, analysis.Options(reltol=1e-6), reuse=reuse, probes=probes)
    assert np.all(st == 0) and np.all(steps == 40), (st, steps)
    ospec = orc.TranSpec(0.1e-9, 40 * 0.1e-9, 0.0, 0.0, 0, 1, 1, 0, 0.0, 0.0, 0.0)
    for v in range(len(vals)):
        r = orc.tran(orc.Packed(el, nn, vals[v]), ospec, orc.options(reltol=1e-6))
        assert r[0] == 0, r[-1]
        xo = r[2]
        assert xo.shape[0] == wave.shape[0]
        scale = np.abs(xo).max()
        assert np.abs(wave[:, v, :] - xo[:, probes]).max() <= 1e-9 * scale
        assert np.abs(x[v] - xo[-1]).max() <= 1e-9 * scale
        assert it[v] == r[5]
    if reuse:
        assert stats["refactors"] < stats["solves"] // 4, stats


def test_medium_grid_transient_matches_oracle_restatement():
    """64 x 64 grid in 16 pieces of 256 nodes: the torn oracle (the reference's
    algorithm restated) and the engine agree step by step."""
    el, nn, vals, torn, c = grid(2, 64, 4, 64, seed=2)
    tb = analysis.TornBatch(el, nn, vals, torn)
    assert tb.pieces == 16
    spec = analysis.TranSpec(step=0.1e-9, stop=10 * 0.1e-9, fixed_step=True, method="be")
    probes = np.arange(0, tb.n, 13)
    wave, x, st, steps, it, stats = tb.tran(spec, analysis.Options(reltol=1e-6), probes=probes)
    assert np.all(st == 0)
    ospec = orc.TranSpec(0.1e-9, 10 * 0.1e-9, 0.0, 0.0, 0, 1, 1, 0, 0.0, 0.0, 0.0)
    for v in range(len(vals)):
        pk = orc.Packed(el, nn, vals[v])
        s, pairs, msg = orc.torn_cuts(pk, torn)
        assert s == 0, msg
        s, t, xo, nsteps, its, ostats, msg = orc.tran_torn(pk, ospec, pairs, orc.options(reltol=1e-6))
        assert s == 0 and ostats["max_pieces"] == 16, msg
        assert np.abs(wave[:, v, :] - xo[:, probes]).max() <= 1e-9 * np.abs(xo).max()


with open(os.path.join(HERE, "golden", "reference_cases.json")) as f:
    OP_CASES = [c for c in json.load(f)["cases"] if not c["skip"] and c["circuit"]["analyses"][0]["kind"] == "op"]


@pytest.mark.parametrize("case", OP_CASES, ids=[c["name"] for c in OP_CASES])
def test_golden_operating_points_torn(case):
    """Each golden operating-point netlist torn along all its tearable elements
    (jacobianCuts, kron/jacobian_test.go:25-42) still meets its golden values."""
    ckt = kc.from_dict(case["circuit"])
    el, vals, _ = ckt.pack()
    pk = orc.Packed(el, ckt.n_nodes, vals)
    cut = []
    for i in range(len(ckt.elements)):
        st, pairs, _ = orc.torn_cuts(pk, [i])
        if st == 0 and len(pairs):
            cut.append(i)
    tb = analysis.TornBatch(el, ckt.n_nodes, vals, cut)
    x, st, it, stats = tb.op(analysis.Options())
    assert st[0] == 0, st
    want = case["golden"]["independent"]
    got = {}
    for k in want["values"]:
        if k.startswith("v("):
            i = ckt.node_index(k[2:-1])
            if i >= 0:
                got[k] = 0.0 if i == 0 else x[0, i - 1]
    msgs = gc.compare_values(got, {k: v for k, v in want["values"].items() if k.startswith("v(")})
    assert not msgs, msgs


def test_untorn_mode_matches_oracle():
    """reuse="untorn": every system solved untorn (one band LU per connected
    component of the whole Jacobian, the solver of the untorn fallback): the
    power-grid transient matches the oracle's untorn run, and no solve is torn."""
    el, nn, vals, torn, c = grid(2, 16, 2, 16, seed=4)
    tb = analysis.TornBatch(el, nn, vals, torn)
    spec = analysis.TranSpec(step=0.1e-9, stop=20 * 0.1e-9, fixed_step=True, method="be")
    probes = np.arange(0, tb.n, 5)
    wave, x, st, steps, it, stats = tb.tran(spec, analysis.Options(reltol=1e-6), reuse="untorn", probes=probes)
    assert np.all(st == 0) and np.all(steps == 20), (st, steps)
    assert stats["refactors"] == stats["solves"] and 0 < stats["untorn"] <= len(vals) * stats["solves"], stats
    ospec = orc.TranSpec(0.1e-9, 20 * 0.1e-9, 0.0, 0.0, 0, 1, 1, 0, 0.0, 0.0, 0.0)
    for v in range(len(vals)):
        r = orc.tran(orc.Packed(el, nn, vals[v]), ospec, orc.options(reltol=1e-6))
        assert r[0] == 0, r[-1]
        scale = np.abs(r[2]).max()
        assert np.abs(wave[:, v, :] - r[2][:, probes]).max() <= 1e-9 * scale
        assert it[v] == r[5]


def test_singular_circuit_falls_back_untorn():
    """TestJacobianErrors' fallback case (kron/jacobian_test.go:298-305): two
    voltage sources in parallel, torn along R1.  The torn solve fails, the
    variant is solved untorn, and the untorn LU reports what plain MNA reports:
    a singular matrix, for both variants of the batch."""
    b = kc.Builder("loop")
    b.voltage_source("V1", "1", "0", 1.0)
    b.voltage_source("V2", "1", "0", 2.0)
    b.resistor("R1", "1", "2", 1e3)
    b.resistor("R2", "2", "0", 1e3)
    ckt = b.build()
    el, v0, _ = ckt.pack()
    names = [e.name for e in ckt.elements]
    vals = np.tile(v0, (2, 1))
    vals[1, int(el[names.index("V2")]["param"])] = 0.0  # still two sources in parallel: singular as well
    opt = analysis.Options(no_gmin_stepping=True, no_source_stepping=True, no_pseudo_transient=True)
    tb = analysis.TornBatch(el, ckt.n_nodes, vals, [names.index("R1")])
    x, st, it, stats = tb.op(opt)
    so, xo, _, _, msg = orc.op(orc.Packed(el, ckt.n_nodes, vals[0]),
                               orc.options(no_gmin=True, no_source=True, no_pt=True))
    assert so == 1 and "singular" in msg, msg
    assert np.all(st == 1), st  # KS_STATUS_SINGULAR from the untorn LU
    assert stats["untorn"] >= 2, stats


@pytest.mark.parametrize("N,P,loads", [(16, 2, 16), (64, 4, 64)])
def test_fp32_factors_transient_matches_oracle(N, P, loads):
    """precision="mixed": the applications stream FP32 copies of the band and
    interconnection factors while the refinement's residual stays FP64 against
    the exact Jacobian, so each solve still reaches a backward error of 1e-14
    and the transient matches the oracle's untorn run as closely as with FP64
    factors (more refinement passes per solve)."""
    el, nn, vals, torn, c = grid(2, N, P, loads, seed=5)
    tb = analysis.TornBatch(el, nn, vals, torn)
    spec = analysis.TranSpec(step=0.1e-9, stop=15 * 0.1e-9, fixed_step=True, method="be")
    probes = np.arange(0, tb.n, 11)
    wave, x, st, steps, it, stats = tb.tran(spec, analysis.Options(reltol=1e-6, precision="mixed"), probes=probes)
    w64, x64, st64, steps64, it64, stats64 = tb.tran(spec, analysis.Options(reltol=1e-6), probes=probes)
    assert np.all(st == 0) and np.all(steps == 15), (st, steps)
    assert stats["not_accepted"] == 0 and stats["untorn"] == 0, stats
    assert stats["refines"] >= stats64["refines"]
    ospec = orc.TranSpec(0.1e-9, 15 * 0.1e-9, 0.0, 0.0, 0, 1, 1, 0, 0.0, 0.0, 0.0)
    for v in range(len(vals)):
        r = orc.tran(orc.Packed(el, nn, vals[v]), ospec, orc.options(reltol=1e-6))
        assert r[0] == 0, r[-1]
        scale = np.abs(r[2]).max()
        assert np.abs(wave[:, v, :] - r[2][:, probes]).max() <= 1e-9 * scale
        assert np.array_equal(it[v], it64[v])


def test_step_predictor_on_the_power_grid():
    """Each time step's Newton starting from the extrapolated history
    (ks_options.step_predictor) converges to the oracle's points within the
    Newton tolerance.  On the grid it saves no iterations: the pads' branch
    currents relax exponentially over a few steps after every load edge, and the
    extrapolation misses them by far more than the 1e-3 relative current
    tolerance, so a step still takes the two solves it takes from the last point."""
    el, nn, vals, torn, c = grid(3, 16, 2, 16, seed=4)
    tb = analysis.TornBatch(el, nn, vals, torn)
    spec = analysis.TranSpec(step=0.1e-9, stop=60 * 0.1e-9, fixed_step=True, method="be")
    probes = np.arange(0, tb.n, 5)
    _, _, st0, steps0, it0, _ = tb.tran(spec, analysis.Options(), probes=probes)
    wave, x, st, steps, it, stats = tb.tran(spec, analysis.Options(step_predictor=True), probes=probes)
    assert np.all(st == 0) and np.all(st0 == 0) and np.all(steps == 60)
    assert it.sum() <= it0.sum(), (it, it0)
    w6, x6, st6, _, it6, _ = tb.tran(spec, analysis.Options(reltol=1e-6, step_predictor=True), probes=probes)
    assert np.all(st6 == 0)
    ospec = orc.TranSpec(0.1e-9, 60 * 0.1e-9, 0.0, 0.0, 0, 1, 1, 0, 0.0, 0.0, 0.0)
    for v in range(len(vals)):
        r = orc.tran(orc.Packed(el, nn, vals[v]), ospec, orc.options(reltol=1e-6))
        assert r[0] == 0, r[-1]
        xo = r[2]
        assert np.all(np.abs(w6[:, v, :] - xo[:, probes]) <= 1e-6 * np.abs(xo[:, probes]) + 2e-6)


@pytest.mark.parametrize("name,cut", [("switch_rc_tran", "R1"), ("nlcap_tran", "R1"), ("varind_tran", "R1"),
                                      ("nlind_tran", "R1")])
def test_switches_and_nonlinear_reactive_torn(name, cut):
    """Switches (abrupt) and the nonlinear / time-varying C and L in the torn
    engine's fixed-step transient: four seeded variants of a golden netlist torn
    along a resistor match the oracle's untorn runs."""
    case = [c for c in json.load(open(os.path.join(HERE, "golden", "reference_cases.json")))["cases"]
            if c["name"] == name][0]
    ckt = kc.from_dict(case["circuit"])
    el, v0, _ = ckt.pack()
    g = np.random.default_rng(12)
    vals = np.tile(v0, (4, 1))
    for k, e in enumerate(ckt.elements):
        if e.kind == "R":
            vals[:, int(el[k]["param"])] *= g.uniform(0.8, 1.25, 4)
    tb = analysis.TornBatch(el, ckt.n_nodes, vals, [ckt.element_index(cut)])
    nsteps = 400
    spec = analysis.TranSpec(step=5e-6, stop=nsteps * 5e-6, fixed_step=True, method="be")
    probes = np.arange(tb.n)
    wave, x, st, steps, it, stats = tb.tran(spec, analysis.Options(reltol=1e-6), probes=probes)
    assert np.all(st == 0) and np.all(steps == nsteps), (st, steps)
    ospec = orc.TranSpec(5e-6, nsteps * 5e-6, 0.0, 0.0, 0, 1, 1, 0, 0.0, 0.0, 0.0)
    for v in range(len(vals)):
        r = orc.tran(orc.Packed(el, ckt.n_nodes, vals[v]), ospec, orc.options(reltol=1e-6))
        assert r[0] == 0, r[-1]
        scale = np.abs(r[2]).max(axis=0) + 1e-12
        assert np.all(np.abs(wave[:, v, :] - r[2]) <= 1e-6 * scale), (v, np.abs(wave[:, v, :] - r[2]).max())

