"""ctypes binding of the CPU FP64 oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the engine (kronspice_gb300) never does.  build() compiles the
oracle from oracle/*.cpp with g++ into oracle/_build/.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libks_oracle.so")
SOURCES = ["ks_oracle.cpp"]
HEADERS = ["ks_oracle.h", "oracle_solver.hpp", "oracle_devices.hpp", "oracle_bjt.hpp", "oracle_mos.hpp",
           "oracle_torn.hpp"]


def build(force=False):
    srcs = [os.path.join(HERE, s) for s in SOURCES + HEADERS] + [os.path.join(HERE, "..", "include", "kronspice_gpu.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in srcs):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", tmp,
                           os.path.join(HERE, "ks_oracle.cpp"), "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


class Topology(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int32), ("n_elem", ctypes.c_int32), ("n_values", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("elem", ctypes.c_void_p)]


class Options(ctypes.Structure):
    _fields_ = [("reltol", ctypes.c_double), ("abstol", ctypes.c_double), ("vntol", ctypes.c_double),
                ("gmin", ctypes.c_double), ("itl1", ctypes.c_int32), ("itl4", ctypes.c_int32),
                ("no_gmin_stepping", ctypes.c_int32), ("no_source_stepping", ctypes.c_int32),
                ("no_pseudo_transient", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("backend", ctypes.c_int32), ("max_iter_total", ctypes.c_int32),
                ("deadline_s", ctypes.c_double), ("mixed_passes", ctypes.c_int32),
                ("fp32_start_iters", ctypes.c_int32), ("start_check", ctypes.c_double),
                ("ledger_tol", ctypes.c_double), ("skip_energy_check", ctypes.c_int32),
                ("step_predictor", ctypes.c_int32), ("autotune", ctypes.c_int32)]


class TranSpec(ctypes.Structure):
    _fields_ = [("step", ctypes.c_double), ("stop", ctypes.c_double), ("start", ctypes.c_double),
                ("max_step", ctypes.c_double), ("uic", ctypes.c_int32), ("method", ctypes.c_int32),
                ("fixed_step", ctypes.c_int32), ("max_steps", ctypes.c_int32), ("chgtol", ctypes.c_double),
                ("trtol", ctypes.c_double), ("min_step", ctypes.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        L.kso_op.argtypes = [P, P, P, P, P, P, P, ctypes.c_char_p, ctypes.c_int]
        L.kso_dc.argtypes = [P, P, P, ctypes.c_int, P, ctypes.c_int, P, P, ctypes.c_char_p, ctypes.c_int]
        L.kso_reach_pattern.argtypes = [ctypes.c_int, P, P, P, P]
        L.kso_dc2.argtypes = [P, P, P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int, P, ctypes.c_int, P, P,
                              ctypes.c_char_p, ctypes.c_int]
        L.kso_tran.argtypes = [P, P, P, P, ctypes.c_int, P, P, P, P, P, P, ctypes.c_char_p, ctypes.c_int]
        L.kso_op_results.argtypes = [P, P, P, P, P, P, P, P, ctypes.c_char_p, ctypes.c_int]
        L.kso_sparse_order.argtypes = [P, P, P, P, P, P, P, P]
        L.kso_min_degree.argtypes = [ctypes.c_int, P, P]
        L.kso_min_degree.restype = None
        L.kso_tran_results.argtypes = [P, P, P, P, ctypes.c_int, P, P, P, P, P, P, P, P, ctypes.c_char_p,
                                       ctypes.c_int]
        L.kso_batch_op.argtypes = [P, P, ctypes.c_int, P, P, ctypes.c_int, P, P, P]
        L.kso_batch_tran.argtypes = [P, P, ctypes.c_int, P, P, ctypes.c_int, P, P, P, P]
        L.kso_unknowns.argtypes = [P, P, P, P]
        L.kso_ac.argtypes = [P, P, P, P, ctypes.c_int, P, ctypes.c_char_p, ctypes.c_int]
        L.kso_torn_plan.argtypes = [P, P, P, ctypes.c_int, ctypes.c_double, P, P, P, ctypes.c_int, P]
        L.kso_torn_cuts.argtypes = [P, P, ctypes.c_int, P, ctypes.c_int, P, ctypes.c_char_p, ctypes.c_int]
        L.kso_op_torn.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_double, P, P, P, ctypes.c_char_p, ctypes.c_int]
        L.kso_tran_torn.argtypes = [P, P, P, P, P, ctypes.c_int, ctypes.c_double, ctypes.c_int, P, P, P, P, P, P,
                                    ctypes.c_char_p, ctypes.c_int]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


class Packed:
    """A topology plus value vectors, kept alive for the C calls."""

    def __init__(self, elements, n_nodes, values):
        self.elements = np.ascontiguousarray(elements)
        self.values = np.ascontiguousarray(values, dtype=np.float64)
        nv = self.values.shape[-1]
        self.topo = Topology(n_nodes, len(self.elements), nv, 0, self.elements.ctypes.data)

    @classmethod
    def of(cls, circuit):
        el, vals, _ = circuit.pack()
        return cls(el, circuit.n_nodes, vals)

    def tref(self):
        return ctypes.byref(self.topo)


def options(reltol=0.0, abstol=0.0, vntol=0.0, gmin=0.0, itl1=0, itl4=0, backend=0,
            no_gmin=False, no_source=False, no_pt=False, deadline_s=0.0, ledger_tol=0.0, skip_energy_check=False):
    return Options(reltol, abstol, vntol, gmin, itl1, itl4, int(no_gmin), int(no_source), int(no_pt),
                   0, backend, 0, deadline_s, 0, 0, 0.0, ledger_tol, int(skip_energy_check), 0)


def unknowns(pk):
    n = ctypes.c_int32()
    rc = lib().kso_unknowns(pk.tref(), _ptr(pk.values), ctypes.byref(n), None)
    if rc:
        raise ValueError("kso_unknowns failed")
    isv = np.zeros(n.value, dtype=np.int32)
    lib().kso_unknowns(pk.tref(), _ptr(pk.values), ctypes.byref(n), _ptr(isv))
    return n.value, isv.astype(bool)


def op(pk, opt=None, x0=None):
    """(status, x, element currents, iterations, message)."""
    n, _ = unknowns(pk)
    x = np.zeros(n)
    cur = np.zeros(max(1, len(pk.elements)))
    it = ctypes.c_int32()
    err = ctypes.create_string_buffer(512)
    o = opt or options()
    x0a = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
    st = lib().kso_op(pk.tref(), _ptr(pk.values), ctypes.byref(o), _ptr(x0a), _ptr(x), _ptr(cur),
                      ctypes.byref(it), err, 512)
    return st, x, cur[:len(pk.elements)], it.value, err.value.decode()


RES_COLS, LEDGER_COLS, TPOINT_COLS, TSUM_COLS = 7, 8, 7, 8
RES = dict(voltage=0, current=1, power=2, storage_power=3, stored_energy=4, exterior_power=5, model_supplied=6)
LEDGER = dict(inflow=0, outflow=1, dissipation=2, storage_rate=3, model_supplied=4, residual=5, scale=6, roundoff=7)
TPOINT = dict(inflow=0, outflow=1, dissipation=2, storage_rate=3, model_supplied=4, residual=5, stored_energy=6)
TSUM = dict(max_relative_residual=0, energy_in=1, energy_out=2, energy_dissipated=3, energy_model_supplied=4,
            stored_start=5, stored_end=6, integration_mismatch=7)


def op_results(pk, opt=None, x0=None):
    """analysis.OP with its result: (status, x, elem [ne][RES_COLS], ledger [LEDGER_COLS], iters, message)."""
    n, _ = unknowns(pk)
    x = np.zeros(n)
    elem = np.zeros((max(1, len(pk.elements)), RES_COLS))
    led = np.zeros(LEDGER_COLS)
    it = ctypes.c_int32()
    err = ctypes.create_string_buffer(512)
    o = opt or options()
    x0a = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
    st = lib().kso_op_results(pk.tref(), _ptr(pk.values), ctypes.byref(o), _ptr(x0a), _ptr(x), _ptr(elem), _ptr(led),
                              ctypes.byref(it), err, 512)
    return st, x, elem[:len(pk.elements)], led, it.value, err.value.decode()


def tran_results(pk, spec, opt=None, capacity=200000):
    """analysis.Tran with the Waveform's element series and ledger:
    (status, t, x, elem [k][ne][2], ledger [k][TPOINT_COLS], summary [TSUM_COLS], steps, iters, message)."""
    n, _ = unknowns(pk)
    ne = max(1, len(pk.elements))
    t = np.zeros(capacity)
    x = np.zeros((capacity, n))
    elem = np.zeros((capacity, ne, 2))
    led = np.zeros((capacity, TPOINT_COLS))
    summ = np.zeros(TSUM_COLS)
    npts, steps, it = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    err = ctypes.create_string_buffer(512)
    o = opt or options()
    st = lib().kso_tran_results(pk.tref(), _ptr(pk.values), ctypes.byref(spec), ctypes.byref(o), capacity, _ptr(t),
                                _ptr(x), _ptr(elem), _ptr(led), _ptr(summ), ctypes.byref(npts), ctypes.byref(steps),
                                ctypes.byref(it), err, 512)
    k = npts.value
    return (st, t[:k], x[:k], elem[:k, :len(pk.elements)], led[:k], summ, steps.value, it.value,
            err.value.decode())


def sparse_order(pk, spec=None, opt=None, pivots=False):
    """The sparse backend's column order after an operating point (or a transient
    when spec is given) and the pattern it ordered: (status, order [n], pattern [n][n] bool)
    and, with pivots, the A rows its last factorization pivoted on per step."""
    n, _ = unknowns(pk)
    order = np.zeros(n, dtype=np.int32)
    pat = np.zeros((n, n), dtype=np.uint8)
    piv = np.zeros(n, dtype=np.int32)
    o = opt or options()
    st = lib().kso_sparse_order(pk.tref(), _ptr(pk.values), None if spec is None else ctypes.byref(spec),
                                ctypes.byref(o), None, _ptr(order), _ptr(pat), _ptr(piv) if pivots else None)
    if pivots:
        return st, order, pat.astype(bool), piv
    return st, order, pat.astype(bool)


def min_degree(pattern):
    """minimumDegree (solver/sparse.go:412-452) of an n x n pattern."""
    p = np.ascontiguousarray(pattern, dtype=np.uint8)
    order = np.zeros(p.shape[0], dtype=np.int32)
    lib().kso_min_degree(p.shape[0], _ptr(p), _ptr(order))
    return order


def dc(pk, src, vals, opt=None):
    n, _ = unknowns(pk)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    x = np.zeros((len(vals), n))
    cur = np.zeros((len(vals), len(pk.elements)))
    err = ctypes.create_string_buffer(512)
    o = opt or options()
    st = lib().kso_dc(pk.tref(), _ptr(pk.values), ctypes.byref(o), src, _ptr(vals), len(vals), _ptr(x),
                      _ptr(cur), err, 512)
    return st, x, cur, err.value.decode()


def reach_pattern(A, q, prow):
    """The reference's Gilbert-Peierls reach sets for a fixed pivot sequence:
    (pattern [n][n] bool in step coordinates, first step whose pivot row is
    outside its reach or -1)."""
    A = np.ascontiguousarray(A, dtype=np.uint8)
    n = A.shape[0]
    q = np.ascontiguousarray(q, dtype=np.int32)
    prow = np.ascontiguousarray(prow, dtype=np.int32)
    out = np.zeros((n, n), dtype=np.uint8)
    bad = lib().kso_reach_pattern(n, _ptr(A), _ptr(q), _ptr(prow), _ptr(out))
    return out.astype(bool), bad


def dc2(pk, src, vals, src2, vals2, opt=None):
    """analysis.DC with a second, outer source (the inner one stepping fastest)."""
    n, _ = unknowns(pk)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    vals2 = np.ascontiguousarray(vals2, dtype=np.float64)
    total = len(vals) * len(vals2)
    x = np.zeros((total, n))
    cur = np.zeros((total, len(pk.elements)))
    err = ctypes.create_string_buffer(512)
    o = opt or options()
    st = lib().kso_dc2(pk.tref(), _ptr(pk.values), ctypes.byref(o), src, _ptr(vals), len(vals), src2, _ptr(vals2),
                       len(vals2), _ptr(x), _ptr(cur), err, 512)
    return st, x, cur, err.value.decode()


def tran(pk, spec, opt=None, capacity=200000, currents=True):
    n, _ = unknowns(pk)
    t = np.zeros(capacity)
    x = np.zeros((capacity, n))
    cur = np.zeros((capacity, len(pk.elements))) if currents else None
    npts, steps, it = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    err = ctypes.create_string_buffer(512)
    o = opt or options()
    st = lib().kso_tran(pk.tref(), _ptr(pk.values), ctypes.byref(spec), ctypes.byref(o), capacity, _ptr(t),
                        _ptr(x), _ptr(cur), ctypes.byref(npts), ctypes.byref(steps), ctypes.byref(it), err, 512)
    k = npts.value
    return (st, t[:k], x[:k], None if cur is None else cur[:k], steps.value, it.value, err.value.decode())


def ac(pk, freqs, opt=None):
    """AC sweep (analysis/ac.go): (status, x [nf][n] complex, message)."""
    n, _ = unknowns(pk)
    f = np.ascontiguousarray(freqs, dtype=np.float64)
    x = np.zeros((len(f), n, 2))
    err = ctypes.create_string_buffer(512)
    o = opt or options()
    st = lib().kso_ac(pk.tref(), _ptr(pk.values), ctypes.byref(o), _ptr(f), len(f), _ptr(x), err, 512)
    return st, x[..., 0] + 1j * x[..., 1], err.value.decode()


TORN_STATS = ("solves", "factors", "reuses", "stale", "fallbacks", "refines", "max_pieces")


def torn_cuts(pk, elems):
    """NewJacobianTearing's cut (kron/jacobian.go:92-232): (status, pairs [k][2], message)."""
    e = np.ascontiguousarray(elems, dtype=np.int32)
    cap = 64 * max(1, len(e))
    pairs = np.zeros((cap, 2), dtype=np.int32)
    npairs = ctypes.c_int32()
    err = ctypes.create_string_buffer(512)
    st = lib().kso_torn_cuts(pk.tref(), _ptr(e), len(e), _ptr(pairs), cap, ctypes.byref(npairs), err, 512)
    return st, pairs[:npairs.value].copy(), err.value.decode()


def torn_plan(pk, pairs, h):
    """buildPlan's (piece of each unknown, coupling rows) for one backward-Euler step of length h."""
    n, _ = unknowns(pk)
    p = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
    piece = np.zeros(n, dtype=np.int32)
    rows = np.zeros(n, dtype=np.int32)
    npc, nr = ctypes.c_int32(), ctypes.c_int32()
    st = lib().kso_torn_plan(pk.tref(), _ptr(pk.values), _ptr(p), len(p), float(h), _ptr(piece), ctypes.byref(npc),
                             _ptr(rows), n, ctypes.byref(nr))
    if st:
        raise ValueError("kso_torn_plan failed")
    return piece, rows[:nr.value].copy(), npc.value


def op_torn(pk, pairs, opt=None, reuse_tol=0.0):
    """analysis.OP with Options.Solver = kron.JacobianTearing: (status, x, iters, stats, message)."""
    n, _ = unknowns(pk)
    p = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
    x = np.zeros(n)
    it = ctypes.c_int32()
    stats = np.zeros(7, dtype=np.int64)
    err = ctypes.create_string_buffer(512)
    st = lib().kso_op_torn(pk.tref(), _ptr(pk.values), ctypes.byref(opt or options()), _ptr(p), len(p),
                           float(reuse_tol), _ptr(x), ctypes.byref(it), _ptr(stats), err, 512)
    return st, x, it.value, dict(zip(TORN_STATS, stats.tolist())), err.value.decode()


def tran_torn(pk, spec, pairs, opt=None, reuse_tol=0.0, capacity=200000):
    """analysis.Tran with every linear system solved torn: (status, t, x [npts][n], steps, iters, stats, message)."""
    n, _ = unknowns(pk)
    p = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
    t = np.zeros(capacity)
    x = np.zeros((capacity, n))
    npts, steps, it = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    stats = np.zeros(7, dtype=np.int64)
    err = ctypes.create_string_buffer(512)
    st = lib().kso_tran_torn(pk.tref(), _ptr(pk.values), ctypes.byref(spec), ctypes.byref(opt or options()), _ptr(p),
                             len(p), float(reuse_tol), capacity, _ptr(t), _ptr(x), ctypes.byref(npts),
                             ctypes.byref(steps), ctypes.byref(it), _ptr(stats), err, 512)
    k = npts.value
    return st, t[:k].copy(), x[:k].copy(), steps.value, it.value, dict(zip(TORN_STATS, stats.tolist())), err.value.decode()


def batch_op(pk, nc, opt=None, x0=None, nthreads=0):
    n, _ = unknowns(Packed(pk.elements, pk.topo.n_nodes, pk.values[0]))
    x = np.zeros((nc, n))
    st = np.zeros(nc, dtype=np.int32)
    it = np.zeros(nc, dtype=np.int32)
    o = opt or options()
    x0a = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
    lib().kso_batch_op(pk.tref(), _ptr(pk.values), nc, ctypes.byref(o), _ptr(x0a), nthreads, _ptr(x),
                       _ptr(st), _ptr(it))
    return st, x, it


def batch_tran(pk, nc, spec, opt=None, nthreads=0, record=True):
    n, _ = unknowns(Packed(pk.elements, pk.topo.n_nodes, pk.values[0]))
    npts = int(round(spec.stop / spec.step)) + 1
    x = np.zeros((npts, nc, n)) if record else None
    st = np.zeros(nc, dtype=np.int32)
    steps = np.zeros(nc, dtype=np.int32)
    it = np.zeros(nc, dtype=np.int32)
    o = opt or options()
    lib().kso_batch_tran(pk.tref(), _ptr(pk.values), nc, ctypes.byref(spec), ctypes.byref(o), nthreads,
                         _ptr(x), _ptr(st), _ptr(steps), _ptr(it))
    return st, x, steps, it
