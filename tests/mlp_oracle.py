"""CPU FP64 restatement of the learned-start network (test infrastructure).

Same layout and loss as the engine's MLP (kronspice_gb300/csrc/ks_mlp.cu):
layers in -> H -> H -> H -> out, ReLU on the hidden layers, parameters per layer
W [out][in] row-major then b [out]; loss L = sum over rows and outputs of
(y - t)^2 divided by the number of rows (reported as the per-element mean).
"""
import numpy as np


def unpack(p, shapes):
    out, k = [], 0
    for (o, i) in shapes:
        W = p[k:k + o * i].reshape(o, i); k += o * i
        b = p[k:k + o]; k += o
        out.append((W, b))
    return out


def forward(params, X, round_bf16=False):
    acts = [X]
    h = X
    for l, (W, b) in enumerate(params):
        z = h @ W.T + b
        if l < len(params) - 1:
            h = np.maximum(z, 0)
            if round_bf16:
                h = to_bf16(h)
            acts.append(h)
        else:
            h = z
    return h, acts


def grad(p, shapes, X, T, round_bf16=False):
    """Gradients of the loss.  round_bf16: the engine's storage precision, BF16
    weights, inputs, activations and backward deltas (the loss gradient and each
    ReLU-masked delta rounded to BF16 as the GEMM epilogues store them), every
    product accumulated wide."""
    params = unpack(np.asarray(p, dtype=np.float64), shapes)
    if round_bf16:
        params = [(to_bf16(W), b) for W, b in params]
        X = to_bf16(X)
    Y, acts = forward(params, X, round_bf16)
    rows = X.shape[0]
    loss = np.sum((Y - T) ** 2) / rows
    d = 2 * (Y - T) / rows
    if round_bf16:
        d = to_bf16(d)
    grads = [None] * len(params)
    for l in range(len(params) - 1, -1, -1):
        W, b = params[l]
        grads[l] = (d.T @ acts[l], d.sum(0))
        if l > 0:
            d = (d @ W) * (acts[l] > 0)
            if round_bf16:
                d = to_bf16(d)
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return flat, loss


def to_bf16(a):
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16  # round to nearest even
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def init(shapes, seed=0):
    g = np.random.default_rng(seed)
    parts = []
    for (o, i) in shapes:
        parts.append(g.uniform(-1, 1, o * i) * np.sqrt(6.0 / i))
        parts.append(g.uniform(-0.1, 0.1, o))
    return np.concatenate(parts)
