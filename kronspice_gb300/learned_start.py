"""Learned Newton start: an MLP on the GPU's tensor cores predicts each circuit's
operating point from its parameter vector (the role of Options.NodeSet,
analysis/op.go:39-43, applied by analysis/newton.go:221-243).

The network is trained on operating points the plain FP64 GPU solver computes
for a training batch of the same topology, by the engine's own BF16 forward and
backward kernels (kronspice_gb300/csrc/ks_mlp.cu).  At solve time Newton starts
from the prediction, corrects it, and the usual gmin / source-stepping chain
takes over for any circuit whose Newton from the prediction fails.
"""
import ctypes
import json
import os
import time

import numpy as np

from . import _lib, analysis, workloads


def _setup_ctypes(L):
    if getattr(L, "_mlp_ready", False):
        return
    P = ctypes.c_void_p
    L.ks_mlp_create.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, ctypes.POINTER(P)]
    L.ks_mlp_destroy.argtypes = [P]
    L.ks_mlp_destroy.restype = None
    L.ks_mlp_num_params.argtypes = [P, P]
    L.ks_mlp_get_params.argtypes = [P, P]
    L.ks_mlp_set_params.argtypes = [P, P]
    L.ks_mlp_set_io.argtypes = [P, P, ctypes.c_uint64, P, P, P, P, ctypes.c_int32]
    L.ks_mlp_grad.argtypes = [P, P, P, ctypes.c_int32, P, P]
    L.ks_mlp_train.argtypes = [P, P, P, P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_float, P, P]
    L.ks_mlp_predict.argtypes = [P, P, P, P]
    L._mlp_ready = True


class MLP:
    """Handle of a ks_mlp (BF16 MLP in -> H -> H -> H -> out)."""

    def __init__(self, in_dim, out_dim, hidden=256, seed=0):
        self.L = _lib.load()
        _setup_ctypes(self.L)
        self.in_dim, self.out_dim, self.hidden = in_dim, out_dim, hidden
        h = ctypes.c_void_p()
        analysis._check(self.L.ks_mlp_create(in_dim, hidden, out_dim, seed, ctypes.byref(h)), "ks_mlp_create")
        self.handle = h
        n = ctypes.c_int64()
        self.L.ks_mlp_num_params(h, ctypes.byref(n))
        self.n_params = n.value

    def layer_shapes(self):
        ins = [self.in_dim, self.hidden, self.hidden, self.hidden]
        outs = [self.hidden, self.hidden, self.hidden, self.out_dim]
        return list(zip(outs, ins))

    def get_params(self):
        p = np.zeros(self.n_params, dtype=np.float32)
        analysis._check(self.L.ks_mlp_get_params(self.handle, p.ctypes.data), "ks_mlp_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        analysis._check(self.L.ks_mlp_set_params(self.handle, p.ctypes.data), "ks_mlp_set_params")

    def grad(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = ctypes.c_float()
        analysis._check(self.L.ks_mlp_grad(self.handle, X.ctypes.data, T.ctypes.data, X.shape[0], g.ctypes.data,
                                           ctypes.byref(loss)), "ks_mlp_grad")
        return g, loss.value

    def set_io(self, cols, logmask, fmean, fstd, tmean, tstd, scale_col=-1):
        self._io = [np.ascontiguousarray(a, dtype=d) for a, d in
                    ((cols, np.int32), (fmean, np.float32), (fstd, np.float32), (tmean, np.float32), (tstd, np.float32))]
        c, fm, fs, tm, ts = self._io
        self._logmask, self._scale_col = int(logmask), int(scale_col)
        analysis._check(self.L.ks_mlp_set_io(self.handle, c.ctypes.data, int(logmask), fm.ctypes.data, fs.ctypes.data,
                                             tm.ctypes.data, ts.ctypes.data, int(scale_col)), "ks_mlp_set_io")

    def train(self, batch, x_dev, idx_dev, n_train, epochs, mb, lr, stream=None):
        loss = ctypes.c_float()
        analysis._check(self.L.ks_mlp_train(self.handle, batch.handle, x_dev, idx_dev, n_train, epochs, mb,
                                            ctypes.c_float(lr), ctypes.byref(loss), stream), "ks_mlp_train")
        return loss.value

    def predict(self, batch, x0_dev, stream=None):
        analysis._check(self.L.ks_mlp_predict(self.handle, batch.handle, x0_dev, stream), "ks_mlp_predict")

    def __del__(self):
        if getattr(self, "handle", None) and _lib._lib is not None:
            self.L.ks_mlp_destroy(self.handle)
            self.handle = None


def feature_spec(name, el):
    """(value columns, log mask, output scale column) of a workload's parameter
    vector: the node voltages are predicted as fractions of the supply."""
    if name == "bjt_ce":
        q = int(el[5]["param"])
        from .circuit import Q_KEYS
        cols = [q + Q_KEYS.index("is"), q + Q_KEYS.index("bf")] + [int(el[k]["param"]) for k in range(1, 5)] + \
               [int(el[0]["param"])]
        logmask = 0b0111101
        return cols, logmask, int(el[0]["param"])
    if name == "cmos_opamp":
        cols, logs, scale = workloads.cmos_opamp_feature_columns(el)
        return cols, sum(1 << j for j, lg in enumerate(logs) if lg), scale
    raise KeyError(name)


def features_host(vals, cols, logmask):
    f = vals[:, cols].astype(np.float64).copy()
    for j in range(len(cols)):
        if (logmask >> j) & 1:
            f[:, j] = np.log(f[:, j])
    return f


class LearnedStart:
    """A trained MLP bound to one batch: predict() fills x0 for ks_op_async.

    start_check (volts) is the network's own error bound: a circuit whose
    solution ends farther than this from its prediction at any node is solved
    again from the standard start (ks_options.start_check), which catches a
    prediction that led Newton to another operating point."""
    launches_per_step = 1  # the fused inference kernel

    def __init__(self, mlp, batch, x0, info):
        self.mlp, self.batch, self.x0, self.info = mlp, batch, x0, info
        self.start_check = float(info.get("start_check_v", 0.0))

    def predict(self, stream):
        self.mlp.predict(self.batch, self.x0.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        return self.x0

    def save(self, path):
        """The trained network and its input/output normalisation (.npz)."""
        c, fm, fs, tm, ts = self.mlp._io
        np.savez(path, params=self.mlp.get_params(), dims=np.array([self.mlp.in_dim, self.mlp.hidden,
                                                                   self.mlp.out_dim]),
                 cols=c, fmean=fm, fstd=fs, tmean=tm, tstd=ts,
                 io=np.array([self.mlp._logmask, self.mlp._scale_col]), info=json.dumps(self.info))

    @classmethod
    def load(cls, path, batch, device):
        import torch
        z = np.load(path)
        i, h, o = (int(v) for v in z["dims"])
        mlp = MLP(i, o, h, seed=7)
        logmask, scale_col = (int(v) for v in z["io"])
        mlp.set_io(z["cols"], logmask, z["fmean"], z["fstd"], z["tmean"], z["tstd"], scale_col)
        mlp.set_params(z["params"])
        x0 = torch.zeros((batch.n_circ, batch.plan.n), dtype=torch.float64, device=device)
        info = dict(json.loads(str(z["info"])), loaded_from=os.path.basename(path))
        return cls(mlp, batch, x0, info)


def train_for(name, el, nn, vals, batch, device, n_train=131072, epochs=40, mb=2048, lr=2e-3, seed=1000,
              reltol=1e-6, hidden=256):
    """Train a learned start for a workload on `n_train` fresh circuits of the same
    topology solved by the plain FP64 GPU solver, then bind it to `batch`."""
    import torch
    t0 = time.perf_counter()
    gen = {"bjt_ce": workloads.bjt_ce_batch, "cmos_opamp": workloads.cmos_opamp_batch}[name]
    _, _, tv = gen(n_train, seed)
    plan = analysis.Plan(el, nn, tv.shape[1])
    tb = analysis.Batch(plan, tv)
    n = plan.n
    x = torch.zeros((n_train, n), dtype=torch.float64, device=device)
    st = torch.zeros(n_train, dtype=torch.int32, device=device)
    it = torch.zeros(n_train, dtype=torch.int32, device=device)
    stream = torch.cuda.current_stream(device)
    sh = ctypes.c_void_p(stream.cuda_stream) if stream.cuda_stream else None
    tb.op_async(analysis.Options(reltol=reltol, precision="fp64"), None, x.data_ptr(), st.data_ptr(), it.data_ptr(), sh)
    torch.cuda.synchronize()
    t_solve = time.perf_counter() - t0
    ok = (st.cpu().numpy() == 0)
    xs = x.cpu().numpy()
    cols, logmask, scale_col = feature_spec(name, el)
    F = features_host(tv, cols, logmask)
    dout = nn - 1
    Y = xs[:, :dout] / (tv[:, scale_col:scale_col + 1] if scale_col >= 0 else 1.0)
    fmean, fstd = F[ok].mean(0), F[ok].std(0) + 1e-12
    tmean, tstd = Y[ok].mean(0), Y[ok].std(0) + 1e-6
    mlp = MLP(len(cols), dout, hidden, seed=7)
    mlp.set_io(cols, logmask, fmean, fstd, tmean, tstd, scale_col)
    g = np.random.default_rng(seed)
    idx_ok = np.nonzero(ok)[0].astype(np.int32)
    n_use = (len(idx_ok) // mb) * mb
    losses = []
    t1 = time.perf_counter()
    idx_dev = torch.empty(n_use, dtype=torch.int32, device=device)
    per_round = 4
    for r in range(0, epochs, per_round):
        perm = g.permutation(idx_ok)[:n_use].astype(np.int32)
        idx_dev.copy_(torch.from_numpy(perm))
        frac = r / max(1, epochs)
        lr_r = lr * (0.5 * (1 + np.cos(np.pi * frac)))  # cosine decay per round
        losses.append(mlp.train(tb, x.data_ptr(), idx_dev.data_ptr(), n_use, min(per_round, epochs - r), mb,
                                float(lr_r), sh))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    # the network's error on its training circuits sets its basin check: at least
    # four times the 99.9th percentile and 1.5 times the largest node-voltage error
    # (a solution that far from its prediction is not the network's usual miss)
    # and 0.1 V
    xp = torch.zeros((n_train, n), dtype=torch.float64, device=device)
    mlp.predict(tb, xp.data_ptr(), sh)
    torch.cuda.synchronize()
    pe = np.abs(xp.cpu().numpy()[ok, :dout] - xs[ok, :dout]).max(axis=1)
    check = max(0.1, 4.0 * float(np.percentile(pe, 99.9)), 1.5 * float(pe.max()))
    del xp
    x0 = torch.zeros((batch.n_circ, n), dtype=torch.float64, device=device)
    info = {"n_train": int(n_use), "epochs": epochs, "minibatch": mb, "final_loss": losses[-1],
            "train_solve_s": t_solve, "train_s": t_train, "hidden": hidden, "layers": "in-%d-%d-%d-out" % (hidden, hidden, hidden),
            "pred_err_v": {"p50": float(np.percentile(pe, 50)), "p99": float(np.percentile(pe, 99)),
                           "p99.9": float(np.percentile(pe, 99.9)), "max": float(pe.max())},
            "start_check_v": check}
    del tb
    return LearnedStart(mlp, batch, x0, info)


def for_workload(name, el, nn, vals, batch, device, cache=None):
    """The bench's learned start: 1,048,576 plain-solver operating points (or the
    network saved at `cache` by an earlier run, which it saves otherwise)."""
    if cache and os.path.exists(cache):
        return LearnedStart.load(cache, batch, device)
    ls = train_for(name, el, nn, vals, batch, device, n_train=1 << 20, epochs=60 if name == "bjt_ce" else 40,
                   mb=4096, lr=2e-3)
    if cache:
        ls.save(cache)
    return ls
