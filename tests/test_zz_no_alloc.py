"""ks_op_noalloc: the batched operating point for callers that cannot allocate
device memory while they solve (a memory pool or arena that owns the device,
a solve path where an allocation could synchronise the device or fail under
memory pressure).  It keeps every intermediate array in the library's fixed
scratch area, so it must give what ks_op gives for the same circuits, call after
call, although every call reuses the same scratch.

This file is collected last on purpose: a run that stops at its first failure
has then already run every other test.
"""
import ctypes

import numpy as np
import pytest

from kronspice_gb300 import _lib, analysis, build, workloads

RELTOL, VNTOL, ABSTOL = 1e-6, 1e-6, 1e-12


def _topo(el, nn, nv):
    return _lib.KsTopology(nn, len(el), nv, 0, el.ctypes.data)


def test_noalloc_rejects_batches_beyond_the_scratch():
    """Too many circuits for the fixed scratch: a clear error before any GPU work."""
    build.build()
    L = _lib.load()
    el, nn, vals = workloads.cmos_opamp_batch(2, seed=1)
    topo = _topo(el, nn, vals.shape[1])
    need = ctypes.c_size_t()
    assert L.ks_op_noalloc_scratch_bytes(ctypes.byref(topo), 65536, ctypes.byref(need)) == 0
    assert need.value > (64 << 20)  # KS_NOALLOC_SCRATCH_BYTES
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.ks_op_noalloc(ctypes.byref(topo), 65536, dummy, None, dummy, dummy, dummy, None)
    assert rc == -1  # KS_EINVAL
    assert "scratch" in _lib.last_error()


@pytest.mark.gpu
def test_noalloc_matches_ks_op_on_consecutive_calls():
    import torch
    build.build()
    L = _lib.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    # two different batches one after the other through the same scratch
    for seed, n_circ in ((21, 4096), (22, 3000)):
        el, nn, vals = workloads.bjt_ce_batch(n_circ, seed=seed)
        topo = _topo(el, nn, vals.shape[1])
        plan = analysis.Plan(el, nn, vals.shape[1])
        n = plan.n
        opt = analysis.Options(reltol=RELTOL, kernel="generic")
        x_ref, st_ref, it_ref = analysis.Batch(plan, vals).op(opt)

        v_dev = torch.from_numpy(vals).to(dev)
        x_dev = torch.full((n_circ, n), float("nan"), dtype=torch.float64, device=dev)
        s_dev = torch.full((n_circ,), -1, dtype=torch.int32, device=dev)
        i_dev = torch.full((n_circ,), -1, dtype=torch.int32, device=dev)
        o = opt.c()
        torch.cuda.synchronize()
        rc = L.ks_op_noalloc(ctypes.byref(topo), n_circ, ctypes.c_void_p(v_dev.data_ptr()), ctypes.byref(o),
                             ctypes.c_void_p(x_dev.data_ptr()), ctypes.c_void_p(s_dev.data_ptr()),
                             ctypes.c_void_p(i_dev.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, _lib.last_error()
        stream.synchronize()
        x, st, it = x_dev.cpu().numpy(), s_dev.cpu().numpy(), i_dev.cpu().numpy()
        assert np.array_equal(st, st_ref)
        ok = st_ref == 0
        assert ok.mean() > 0.99
        isv = np.zeros(n, dtype=bool)
        isv[:nn - 1] = True
        tol = np.where(isv, VNTOL, ABSTOL) + RELTOL * np.abs(x_ref[ok])
        assert np.all(np.abs(x[ok] - x_ref[ok]) <= tol)
        assert np.array_equal(it, it_ref)
