"""GPU parity of the controlled sources (E, F, G, H) and mutual inductances (K).

device/controlled.go and device/mutual.go on every kernel family: batches of the
reference's golden circuits with seeded gains, coupling coefficients and
inductances on the per-topology kernels (operating point and fixed-step
transient) and on the generic ones, and circuits of different topologies in one
multi-topology batch, all against the oracle.  The golden cases themselves
(controlled_op, mutual_ac, mutual_tran) run in the golden parametrizations of
test_gpu_op, test_gpu_tran, test_gpu_ac and test_gpu_results.
"""
import json
import os

import numpy as np
import pytest

from kronspice_gb300 import analysis, build
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_cases.json")) as f:
    CASES = {c["name"]: c for c in json.load(f)["cases"]}
RELTOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def variants(name, n, seed, kinds):
    """n copies of a golden circuit with the values of the given element kinds
    scaled by log-uniform factors in [1/1.3, 1.3] (coupling coefficients kept in (0, 1))."""
    ckt = kc.from_dict(CASES[name]["circuit"])
    el, v0, _ = ckt.pack()
    g = np.random.default_rng(seed)
    vals = np.tile(v0, (n, 1))
    for k, e in enumerate(ckt.elements):
        if e.kind in kinds:
            col = int(el[k]["param"])
            f = np.exp(g.uniform(np.log(1 / 1.3), np.log(1.3), n))
            vals[:, col] = np.minimum(vals[:, col] * f, 0.99) if e.kind == "K" else vals[:, col] * f
    return ckt, el, vals


@pytest.mark.parametrize("kernel", ["specialized", "generic"])
def test_controlled_sources_batch(kernel):
    ckt, el, vals = variants("controlled_op", 2048, 1, "EFGHR")
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, vals.shape[1]), vals)
    x, st, it = b.op(analysis.Options(reltol=RELTOL, kernel=kernel))
    assert b.last_kernel.startswith(kernel[:4])
    assert np.all(st == 0)
    pk = orc.Packed(el, ckt.n_nodes, vals[0])
    for c in range(0, 2048, 37):
        pk.values[:] = vals[c]
        ost, ox, _, _, msg = orc.op(pk, orc.options(reltol=RELTOL))
        assert ost == 0, msg
        assert np.allclose(x[c], ox, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("kernel", ["specialized", "generic"])
def test_mutual_inductance_transient_batch(kernel):
    ckt, el, vals = variants("mutual_tran", 2048, 2, "LKR")
    sp = analysis.TranSpec(step=2e-6, stop=2e-4, fixed_step=True)
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, vals.shape[1]), vals)
    wave, _, npts, st, steps, it = b.tran(sp, analysis.Options(reltol=RELTOL, kernel=kernel))
    assert np.all(st == 0) and np.all(npts == 101)
    ospec = orc.TranSpec(2e-6, 2e-4, 0.0, 0.0, 0, 2, 1, 0, 0.0, 0.0, 0.0)
    sample = np.arange(0, 2048, 97)
    so, xo, so_steps, io = orc.batch_tran(orc.Packed(el, ckt.n_nodes, vals[sample]), len(sample), ospec,
                                          orc.options(reltol=RELTOL))
    assert np.all(so == 0)
    assert np.allclose(wave[:, sample, :], xo, rtol=1e-7, atol=1e-10)


def test_mutual_inductance_ac_batch():
    ckt, el, vals = variants("mutual_ac", 256, 3, "LKC")
    freqs = np.logspace(4, 8, 41)
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, vals.shape[1]), vals)
    x, st, it = b.ac(freqs, analysis.Options())
    assert np.all(st == 0)
    pk = orc.Packed(el, ckt.n_nodes, vals[0])
    for c in range(0, 256, 17):
        pk.values[:] = vals[c]
        ost, ox, msg = orc.ac(pk, freqs)
        assert ost == 0, msg
        g = x[c][..., 0] + 1j * x[c][..., 1] if x.ndim == 4 else x[c]
        assert np.allclose(g, ox, rtol=1e-9, atol=1e-15)


def test_multi_topology_batch_with_controlled_and_mutual():
    """controlled_op, mutual_tran and a BJT stage of different sizes in one batch."""
    circuits = [kc.from_dict(CASES[n]["circuit"]) for n in ("controlled_op", "mutual_tran", "bjt_ce_op")] * 16
    mb = analysis.MultiBatch(circuits)
    xs, st, it = mb.op(analysis.Options(reltol=RELTOL))
    assert np.all(st == 0)
    for c, x in zip(circuits[:3], xs[:3]):
        ost, ox, _, _, msg = orc.op(orc.Packed.of(c), orc.options(reltol=RELTOL))
        assert ost == 0, msg
        _, isv = orc.unknowns(orc.Packed.of(c))
        tol = np.where(isv, 1e-6, 1e-12) + 2e-6 * np.abs(ox)
        assert np.all(np.abs(x - ox) <= tol)
    sp = analysis.TranSpec(step=2e-6, stop=1e-4, fixed_step=True)
    waves, st, steps, it = mb.tran(sp, analysis.Options(reltol=RELTOL))
    assert np.all(st == 0)
    ospec = orc.TranSpec(2e-6, 1e-4, 0.0, 0.0, 0, 2, 1, 0, 0.0, 0.0, 0.0)
    r = orc.tran(orc.Packed.of(circuits[1]), ospec, orc.options(reltol=RELTOL))
    assert r[0] == 0
    assert np.allclose(waves[1], r[2], rtol=1e-6, atol=1e-9)
