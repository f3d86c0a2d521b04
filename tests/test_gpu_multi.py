"""Batches of circuits of different topologies and sizes (one warp per circuit,
sparse LU on the host's fixed pivot sequence) against the CPU FP64 oracle,
which solves each circuit on its own with the reference's solver choice (dense
below 30 unknowns, sparse above)."""
import numpy as np
import pytest

from kronspice_gb300 import analysis, build, workloads
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
RELTOL, VNTOL, ABSTOL = 1e-6, 1e-6, 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


@pytest.fixture(scope="module")
def circuits():
    return workloads.random_netlists(96, seed=7, nodes=(10, 80))


def tol(x_ref, isv, rel):
    return np.where(isv, VNTOL, ABSTOL) + rel * np.abs(x_ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multi_op_matches_oracle(circuits, precision):
    mb = analysis.MultiBatch(circuits)
    xs, st, it = mb.op(analysis.Options(reltol=RELTOL, precision=precision))
    bad = []
    for k, c in enumerate(circuits):
        pk = orc.Packed.of(c)
        so, xo, _, _, _ = orc.op(pk, orc.options(reltol=RELTOL))
        if st[k] != so:
            bad.append((k, int(st[k]), so))
            continue
        if so == 0:
            _, isv = orc.unknowns(pk)
            if not np.all(np.abs(xs[k] - xo) <= tol(xo, isv, 1e-5)):
                bad.append((k, float(np.abs(xs[k] - xo).max())))
    assert not bad, bad[:10]
    assert (st == 0).mean() > 0.95


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multi_fixed_step_transient_matches_oracle(circuits, precision):
    sub = circuits[:48]
    mb = analysis.MultiBatch(sub)
    sp = analysis.TranSpec(step=5e-9, stop=1e-6, fixed_step=True)
    waves, st, steps, it = mb.tran(sp, analysis.Options(reltol=RELTOL, precision=precision))
    ospec = orc.TranSpec(sp.step, sp.stop, 0.0, 0.0, 0, 2, 1, 0, 0.0, 0.0, 0.0)
    bad = []
    for k, c in enumerate(sub):
        el, vals, _ = c.pack()
        pk = orc.Packed(el, c.n_nodes, vals[None, :])
        so, xo, so_steps, _ = orc.batch_tran(pk, 1, ospec, orc.options(reltol=RELTOL))
        if st[k] != so[0]:
            bad.append((k, int(st[k]), int(so[0])))
            continue
        if so[0] != 0:
            continue
        assert steps[k] == so_steps[0]
        ref = xo[:, 0, :]
        nn = c.n_nodes - 1
        err = np.abs(waves[k][:, :nn] - ref[:, :nn])
        if not np.all(err <= 1e-5 * np.abs(ref[:, :nn]) + 1e-5):
            bad.append((k, float(err.max())))
    assert not bad, bad[:10]
    assert (st == 0).mean() > 0.9
