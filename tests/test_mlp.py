"""The learned Newton start: the CPU FP64 network is pinned by finite differences
(CPU), the engine's tensor-core forward/backward kernels match it (GPU), training
on plain-solver solutions reduces the loss, and the learned start cuts the Newton
iterations of the BJT batch while the results stay within the SPICE tolerance of
the oracle (GPU)."""
import ctypes

import numpy as np
import pytest

import mlp_oracle as mo

SHAPES = [(64, 7), (64, 64), (64, 64), (4, 64)]


def test_cpu_network_gradient_matches_finite_differences():
    g = np.random.default_rng(0)
    p = mo.init(SHAPES, 1)
    X = g.normal(size=(5, 7))
    T = g.normal(size=(5, 4))
    grad, loss = mo.grad(p, SHAPES, X, T)
    for k in g.choice(len(p), 40, replace=False):
        e = np.zeros_like(p); e[k] = 1e-6
        fd = (mo.grad(p + e, SHAPES, X, T)[1] - mo.grad(p - e, SHAPES, X, T)[1]) / 2e-6
        assert abs(fd - grad[k]) <= 1e-6 * max(1, abs(fd)), (k, fd, grad[k])


@pytest.mark.gpu
def test_gpu_gradients_match_cpu_network():
    from kronspice_gb300 import build, learned_start as ls
    build.build()
    m = ls.MLP(7, 4, hidden=256, seed=3)
    shapes = m.layer_shapes()
    g = np.random.default_rng(1)
    p = mo.init(shapes, 2).astype(np.float32)
    m.set_params(p)
    assert np.allclose(m.get_params(), p)
    X = g.normal(size=(300, 7)).astype(np.float32)
    T = g.normal(size=(300, 4)).astype(np.float32)
    gg, loss = m.grad(X, T)
    gc, lc = mo.grad(p.astype(np.float64), shapes, X.astype(np.float64), T.astype(np.float64), round_bf16=True)
    assert abs(loss * 4 - lc) <= 2e-2 * lc  # engine reports the per-element mean
    k = 0
    for (o, i) in shapes:
        for size in (o * i, o):
            a, b = gg[k:k + size], gc[k:k + size]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30))
            assert rel < 5e-2 and cos > 0.998, (o, i, size, rel, cos)
            k += size


@pytest.mark.gpu
def test_learned_start_cuts_newton_iterations():
    import torch
    from kronspice_gb300 import analysis, build, learned_start as ls, workloads
    from oracle import oracle as orc
    build.build()
    dev = torch.device("cuda", 0)
    el, nn, vals = workloads.bjt_ce_batch(8192, seed=0)
    plan = analysis.Plan(el, nn, vals.shape[1])
    batch = analysis.Batch(plan, vals)
    start = ls.train_for("bjt_ce", el, nn, vals, batch, dev, n_train=262144, epochs=40)
    assert start.info["final_loss"] < 1e-3
    stream = torch.cuda.current_stream(dev)
    x0 = start.predict(stream)
    torch.cuda.synchronize()
    x0h = x0.cpu().numpy()
    opt_m = analysis.Options(reltol=1e-6, precision="mixed")
    xl, sl, il = batch.op(opt_m, x0h)
    xp, sp_, ip = batch.op(analysis.Options(reltol=1e-6, precision="fp64"))
    so, xo, io = orc.batch_op(orc.Packed(el, nn, vals), 8192, orc.options(reltol=1e-6))
    assert np.array_equal(sl == 0, so == 0)
    ok = so == 0
    _, isv = orc.unknowns(orc.Packed(el, nn, vals[0]))
    tol = np.where(isv, 1e-6, 1e-12) + 1e-6 * np.abs(xo[ok])
    assert np.all(np.abs(xl[ok] - xo[ok]) <= tol)
    # the prediction is close and the Newton work drops
    err = np.abs(x0h[ok, :nn - 1] - xo[ok, :nn - 1]).mean()
    assert err < 0.1, err
    assert il.mean() < 0.7 * ip.mean(), (il.mean(), ip.mean())
