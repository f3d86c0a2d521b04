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
            assert rel < 1e-2 and cos > 0.9999, (o, i, size, rel, cos)
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


@pytest.mark.gpu
def test_fused_inference_matches_cpu_network():
    """ks_mlp_predict (features, three hidden layers, output and decode in one
    kernel) against the CPU network on the same BF16-rounded weights and
    activations, for a batch that is not a multiple of the kernel's 64-row tile."""
    import torch
    from kronspice_gb300 import analysis, build, workloads, learned_start as ls
    build.build()
    el, nn, vals = workloads.bjt_ce_batch(1000, seed=4)
    plan = analysis.Plan(el, nn, vals.shape[1])
    batch = analysis.Batch(plan, vals)
    cols, logmask, scale_col = ls.feature_spec("bjt_ce", el)
    m = ls.MLP(len(cols), nn - 1, hidden=256, seed=3)
    shapes = m.layer_shapes()
    p = mo.init(shapes, 5).astype(np.float32)
    m.set_params(p)
    F = ls.features_host(vals, cols, logmask)
    fmean, fstd = F.mean(0), F.std(0) + 1e-12
    tmean = np.linspace(0.1, 0.9, nn - 1)
    tstd = np.full(nn - 1, 0.2)
    m.set_io(cols, logmask, fmean, fstd, tmean, tstd, scale_col)
    x0 = torch.zeros((1000, plan.n), dtype=torch.float64, device="cuda")
    m.predict(batch, x0.data_ptr())
    torch.cuda.synchronize()
    got = x0.cpu().numpy()
    # CPU: FP32 features, BF16 inputs, weights and hidden activations
    f32 = vals[:, cols].astype(np.float32)
    for j in range(len(cols)):
        if (logmask >> j) & 1:
            f32[:, j] = np.log(f32[:, j])
    Xs = ((f32 - fmean.astype(np.float32)) / fstd.astype(np.float32)).astype(np.float64)
    params = [(mo.to_bf16(W), b) for W, b in mo.unpack(p.astype(np.float64), shapes)]
    Y, _ = mo.forward(params, mo.to_bf16(Xs), round_bf16=True)
    sc = vals[:, scale_col]
    y_gpu = (got[:, :nn - 1] / sc[:, None] - tmean) / tstd
    assert np.all(np.abs(y_gpu - Y) <= 0.03 + 0.02 * np.abs(Y)), np.abs(y_gpu - Y).max()
    assert np.all(got[:, nn - 1:] == 0.0)


@pytest.mark.gpu
def test_opamp_learned_start_matches_oracle_on_bench_seed():
    """The op-amp workload's chosen path: the network trained on the GPU on
    plain-solver operating points, its prediction refined by the FP32 Newton
    stage, FP32 LU with FP64 residual, the learned start's basin check, on the
    first 8,192 circuits of the bench's batch (65,536 variants, seed 0).  Every
    status must equal the oracle's and every node voltage must lie within
    reltol 1e-6 / vntol 1e-6 V of it; the learned start must cut the FP64 Newton
    iterations against the standard start."""
    import torch
    from kronspice_gb300 import analysis, build, learned_start as ls, workloads
    from oracle import oracle as orc
    build.build()
    dev = torch.device("cuda", 0)
    el, nn, vals = workloads.cmos_opamp_batch(65536, seed=0)
    vals = np.ascontiguousarray(vals[:8192])
    batch = analysis.Batch(analysis.Plan(el, nn, vals.shape[1]), vals)
    start = ls.train_for("cmos_opamp", el, nn, vals, batch, dev, n_train=262144, epochs=40)
    assert start.start_check > 0
    stream = torch.cuda.current_stream(dev)
    x0 = start.predict(stream)
    torch.cuda.synchronize()
    x0h = x0.cpu().numpy()
    so, xo, io = orc.batch_op(orc.Packed(el, nn, vals), len(vals), orc.options(reltol=1e-6))
    ok = so == 0
    assert ok.mean() > 0.99
    chosen = analysis.Options(reltol=1e-6, precision="mixed", fp32_start_iters=6000, start_check=start.start_check)
    learned_only = analysis.Options(reltol=1e-6, precision="mixed")
    xp, sp_, ip = batch.op(analysis.Options(reltol=1e-6, precision="fp64"))
    for opt in (chosen, learned_only):
        xl, sl, il = batch.op(opt, x0h)
        assert np.array_equal(sl, so), np.nonzero(sl != so)
        dv = np.abs(xl[ok, :nn - 1] - xo[ok, :nn - 1])
        assert np.all(dv <= 1e-6 + 1e-6 * np.abs(xo[ok, :nn - 1])), dv.max()
        assert np.median(il[ok]) <= 0.25 * np.median(ip[ok]), (np.median(il[ok]), np.median(ip[ok]))
