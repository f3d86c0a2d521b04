"""The operating-point autotuner (ks_options.autotune): the first call for a plan
and batch-size bucket times the kernels the batch can run (per-topology and
generic, 1, 2 or 4 circuits per thread), keeps the fastest in the plan, and the
results are those of the untuned call (the same algorithm) and the oracle's."""
import numpy as np
import pytest

from kronspice_gb300 import analysis, build, workloads
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def test_autotune_picks_keeps_and_matches():
    el, nn, vals = workloads.bjt_ce_batch(16384, seed=0)
    plan = analysis.Plan(el, nn, vals.shape[1])
    b = analysis.Batch(plan, vals)
    x0, st0, it0 = b.op(analysis.Options(reltol=1e-6, precision="fp64"))
    assert plan.tuned(16384) is None
    x1, st1, it1 = b.op(analysis.Options(reltol=1e-6, precision="fp64", autotune=True))
    t = plan.tuned(16384)
    assert t is not None and t[0] in ("generic", "specialized-reg", "specialized-smem") and t[1] in (1, 2, 4)
    assert t[2] > 0
    assert np.array_equal(st0, st1) and np.all(st1 == 0)
    assert np.allclose(x1, x0, rtol=1e-7, atol=1e-10)
    # later calls of the bucket reuse the choice; another bucket is tuned on its own
    b.op(analysis.Options(reltol=1e-6, precision="fp64", autotune=True))
    assert plan.tuned(16384) == t and plan.tuned(20000) == t  # 16,384 and 20,000 share the 2^14 bucket
    assert plan.tuned(10000) is None
    pk = orc.Packed(el, nn, vals[0])
    _, isv = orc.unknowns(pk)
    for c in range(0, 16384, 1021):
        pk.values[:] = vals[c]
        ost, ox, _, _, msg = orc.op(pk, orc.options(reltol=1e-6))
        assert ost == 0, msg
        assert np.all(np.abs(x1[c] - ox) <= np.where(isv, 1e-6, 1e-12) + 1e-6 * np.abs(ox))
