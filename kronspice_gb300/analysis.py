"""Batched analyses on the GB300 engine: the host-side mirror of kronspice's analysis package.

``op_batch(circuits, opt)`` is analysis.OP (analysis/op.go:331) for many
circuits in one call; ``tran_batch`` is analysis.Tran (analysis/tran.go:70).
Circuits are grouped by topology, each group is one plan and one batch on the
GPU.  Each circuit gets back its solution or its typed error, with the same
sentinels as the reference (solver/matrix.go:15-20, analysis/newton.go:20,
analysis/tran.go:18-22, circuit/circuit.go:21-31), so callers such as a GA
fitness function can classify failures unchanged.
"""
import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .circuit import ELEMENT_DTYPE


class KronspiceError(Exception):
    """Base of the engine's typed errors."""


class ErrSingularMatrix(KronspiceError):
    """solver.ErrSingularMatrix (solver/matrix.go:17)."""


class ErrNonFinite(KronspiceError):
    """solver.ErrNonFinite (solver/matrix.go:19)."""


class ErrNoConvergence(KronspiceError):
    """analysis.ErrNoConvergence (analysis/newton.go:20)."""


class ErrTimestepTooSmall(KronspiceError):
    """analysis.ErrTimestepTooSmall (analysis/tran.go:19)."""


class ErrTooManySteps(KronspiceError):
    """analysis.ErrTooManySteps (analysis/tran.go:20)."""


class ErrInterrupted(KronspiceError):
    """context deadline or cancel (analysis/op.go:81-89)."""


class ErrLedgerResidual(KronspiceError):
    """em.ErrLedgerResidual (em/energy.go:18): the energy ledger does not balance."""


class ErrValidation(KronspiceError):
    """circuit.Validate failures (ErrFloatingNode, ErrBadValue, ... circuit/circuit.go:21-31)."""


class ErrFloatingNode(ErrValidation):
    """circuit.ErrFloatingNode (circuit/circuit.go:23)."""


STATUS_ERRORS = {1: (ErrSingularMatrix, "solver: singular matrix"),
                 2: (ErrNonFinite, "solver: non-finite value in system"),
                 3: (ErrNoConvergence, "analysis: no convergence"),
                 4: (ErrTimestepTooSmall, "analysis: timestep too small"),
                 5: (ErrTooManySteps, "analysis: too many time steps"),
                 6: (ErrInterrupted, "analysis interrupted: context deadline exceeded"),
                 7: (KronspiceError, "not run"),
                 8: (ErrLedgerResidual, "em: energy ledger does not balance")}

# Columns of the element results and the ledgers (include/kronspice_gpu.h)
RES_COLS, LEDGER_COLS, TPOINT_COLS, TSUM_COLS = 7, 8, 7, 8
RES = dict(voltage=0, current=1, power=2, storage_power=3, stored_energy=4, exterior_power=5, model_supplied=6)
LEDGER = dict(inflow=0, outflow=1, dissipation=2, storage_rate=3, model_supplied=4, residual=5, scale=6, roundoff=7)
TPOINT = dict(inflow=0, outflow=1, dissipation=2, storage_rate=3, model_supplied=4, residual=5, stored_energy=6)
TSUM = dict(max_relative_residual=0, energy_in=1, energy_out=2, energy_dissipated=3, energy_model_supplied=4,
            stored_start=5, stored_end=6, integration_mismatch=7)

PREC = {"fp64": 0, "mixed": 1}
# GPU kernel choice: "auto" (per-topology kernels for large batches), "generic", "specialized"
KERNEL = {"auto": 0, "generic": 3, "specialized": 4}
ANALYSIS = {"op": 0, "tran": 1}
KERNEL_NAMES = {-1: None, 0: "generic", 1: "specialized-registers", 2: "specialized-shared"}


@dataclass
class Options:
    """analysis.Options (analysis/op.go:22-62) plus the engine's precision mode."""
    reltol: float = 0.0
    abstol: float = 0.0
    vntol: float = 0.0
    gmin: float = 0.0
    itl1: int = 0
    itl4: int = 0
    no_gmin_stepping: bool = False
    no_source_stepping: bool = False
    no_pseudo_transient: bool = False
    precision: str = "fp64"
    max_iter_total: int = 0
    deadline_s: float = 0.0
    kernel: str = "auto"
    mixed_passes: int = 0
    fp32_start_iters: int = 0   # FP32 Newton stage before the FP64 solve (operating points; 0: off)
    start_check: float = 0.0    # re-solve from InitJct when the solution ends this far (V) from x0 (0: off)
    ledger_tol: float = 0.0     # Options.LedgerTolerance (0: 1e-9)
    skip_energy_check: bool = False  # Options.SkipEnergyCheck
    step_predictor: bool = False     # transients: each step's Newton starts from the extrapolated history
    autotune: bool = False           # operating points: time the kernels on the first call, keep the fastest

    def c(self):
        return _lib.KsOptions(self.reltol, self.abstol, self.vntol, self.gmin, self.itl1, self.itl4,
                              int(self.no_gmin_stepping), int(self.no_source_stepping),
                              int(self.no_pseudo_transient), PREC[self.precision], KERNEL[self.kernel],
                              self.max_iter_total, self.deadline_s, self.mixed_passes, int(self.fp32_start_iters),
                              float(self.start_check), float(self.ledger_tol), int(self.skip_energy_check),
                              int(self.step_predictor), int(self.autotune))


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed (%d): %s" % (what, rc, _lib.last_error()))


def status_error(status):
    if status == 0:
        return None
    cls, msg = STATUS_ERRORS.get(int(status), (KronspiceError, "status %d" % status))
    return cls(msg)


class Plan:
    """One topology after the host symbolic pass (ks_plan_create)."""

    def __init__(self, elements, n_nodes, n_values):
        L = _lib.load()
        self.elements = np.ascontiguousarray(elements, dtype=ELEMENT_DTYPE)
        self.n_nodes = int(n_nodes)
        self.topo = _lib.KsTopology(self.n_nodes, len(self.elements), int(n_values), 0, self.elements.ctypes.data)
        h = ctypes.c_void_p()
        _check(L.ks_plan_create(ctypes.byref(self.topo), ctypes.byref(h)), "ks_plan_create")
        self.handle = h
        n = ctypes.c_int32()
        _check(L.ks_plan_info(h, ctypes.byref(n), None, None), "ks_plan_info")
        self.n = n.value

    def specialize(self, analysis="op"):
        """Compile (or load from the cache) the per-topology kernel of one
        analysis ("op" or "tran") now: (kernel name, NVRTC seconds)."""
        k, t = ctypes.c_int32(), ctypes.c_double()
        _check(_lib.load().ks_plan_specialize(self.handle, ANALYSIS[analysis], ctypes.byref(k), ctypes.byref(t)),
               "ks_plan_specialize")
        return KERNEL_NAMES[k.value], t.value

    def tuned(self, n_circ, analysis="op"):
        """The autotuner's choice for n_circ circuits (ks_plan_tuned): (kernel name,
        circuits per thread, winning trial's ms), or None when not tuned."""
        k, c, ms = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double()
        rc = _lib.load().ks_plan_tuned(self.handle, ANALYSIS[analysis], int(n_circ), ctypes.byref(k), ctypes.byref(c),
                                       ctypes.byref(ms))
        if rc != 0:
            return None
        return {0: "generic", 1: "specialized-reg", 2: "specialized-smem"}[k.value], c.value, ms.value

    def kernel_source(self, analysis="op"):
        L = _lib.load()
        n = ctypes.c_size_t()
        _check(L.ks_plan_kernel_source(self.handle, ANALYSIS[analysis], None, 0, ctypes.byref(n)),
               "ks_plan_kernel_source")
        buf = ctypes.create_string_buffer(n.value + 1)
        _check(L.ks_plan_kernel_source(self.handle, ANALYSIS[analysis], buf, n.value + 1, None),
               "ks_plan_kernel_source")
        return buf.value.decode()

    def __del__(self):
        if getattr(self, "handle", None) and _lib._lib is not None:
            _lib._lib.ks_plan_destroy(self.handle)
            self.handle = None


class Batch:
    """n circuits of one plan with their values resident on the GPU (ks_batch_create)."""

    def __init__(self, plan, values):
        L = _lib.load()
        self.plan = plan
        self.values = np.ascontiguousarray(values, dtype=np.float64)
        self.n_circ = self.values.shape[0]
        h = ctypes.c_void_p()
        _check(L.ks_batch_create(plan.handle, self.n_circ, self.values.ctypes.data, ctypes.byref(h)),
               "ks_batch_create")
        self.handle = h

    @property
    def last_kernel(self):
        """Kernel that ran the last analysis: "generic", "specialized-registers",
        "specialized-shared" (None before the first)."""
        return KERNEL_NAMES[_lib.load().ks_batch_last_kernel(self.handle)]

    def set_values(self, values):
        self.values = np.ascontiguousarray(values, dtype=np.float64)
        _check(_lib.load().ks_batch_set_values(self.handle, self.values.ctypes.data, 0, None), "ks_batch_set_values")

    def op(self, opt=None, x0=None, stream=None):
        """(x [n_circ][n], status [n_circ], iterations [n_circ]) through ks_op (host buffers)."""
        o = (opt or Options()).c()
        x = np.zeros((self.n_circ, self.plan.n))
        st = np.zeros(self.n_circ, dtype=np.int32)
        it = np.zeros(self.n_circ, dtype=np.int32)
        x0a = None
        if x0 is not None:
            x0a = np.ascontiguousarray(x0, dtype=np.float64)
            assert x0a.shape == (self.n_circ, self.plan.n)
        _check(_lib.load().ks_op(self.handle, ctypes.byref(o), None if x0a is None else x0a.ctypes.data,
                                 x.ctypes.data, st.ctypes.data, it.ctypes.data, stream), "ks_op")
        return x, st, it

    def op_results(self, opt=None, x0=None, stream=None):
        """analysis.OP with its results for every circuit (ks_op_results): (x, status,
        iterations, elem [n_circ][n_elem][RES_COLS], ledger [n_circ][LEDGER_COLS])."""
        o = (opt or Options()).c()
        B, ne = self.n_circ, len(self.plan.elements)
        x = np.zeros((B, self.plan.n))
        st = np.zeros(B, dtype=np.int32)
        it = np.zeros(B, dtype=np.int32)
        elem = np.zeros((B, ne, RES_COLS))
        led = np.zeros((B, LEDGER_COLS))
        x0a = None
        if x0 is not None:
            x0a = np.ascontiguousarray(x0, dtype=np.float64)
            assert x0a.shape == (B, self.plan.n)
        _check(_lib.load().ks_op_results(self.handle, ctypes.byref(o), None if x0a is None else x0a.ctypes.data,
                                         x.ctypes.data, st.ctypes.data, it.ctypes.data, elem.ctypes.data,
                                         led.ctypes.data, stream), "ks_op_results")
        return x, st, it, elem, led

    def tran_results(self, spec, opt=None, capacity=0, stream=None):
        """analysis.Tran with the Waveform's element series and ledger (ks_tran_results):
        (wave, time, elem [..][n_elem][2], ledger [..][TPOINT_COLS], summary [n_circ][TSUM_COLS],
        npts, status, steps, iters), laid out as tran() lays out the waveforms."""
        L = _lib.load()
        o = (opt or Options()).c()
        sp = spec.c() if hasattr(spec, "c") else spec
        B, n, ne = self.n_circ, self.plan.n, len(self.plan.elements)
        if sp.fixed_step:
            lead = (int(round(sp.stop / sp.step)) + 1, B)
            tim = None
        else:
            lead = (B, capacity)
            tim = np.zeros(lead)
        wave = np.zeros(lead + (n,))
        elem = np.zeros(lead + (ne, 2))
        led = np.zeros(lead + (TPOINT_COLS,))
        summ = np.zeros((B, TSUM_COLS))
        np_, st, steps, it = (np.zeros(B, dtype=np.int32) for _ in range(4))
        rc = L.ks_tran_results(self.handle, ctypes.byref(sp), ctypes.byref(o), int(capacity),
                               None if tim is None else tim.ctypes.data, wave.ctypes.data, elem.ctypes.data,
                               led.ctypes.data, summ.ctypes.data, np_.ctypes.data, st.ctypes.data, steps.ctypes.data,
                               it.ctypes.data, stream)
        _check(rc, "ks_tran_results")
        return wave, tim, elem, led, summ, np_, st, steps, it

    def tran(self, spec, opt=None, capacity=0, record=True, stream=None):
        """analysis.Tran for every circuit (ks_tran).  Fixed-step specs return
        (wave [n_points][n_circ][n], None, npts, status, steps, iters); adaptive specs
        return (wave [n_circ][capacity][n], time [n_circ][capacity], npts, ...)."""
        L = _lib.load()
        o = (opt or Options()).c()
        sp = spec.c() if hasattr(spec, "c") else spec
        B, n = self.n_circ, self.plan.n
        if sp.fixed_step:
            npts = int(round(sp.stop / sp.step)) + 1
            wave = np.zeros((npts, B, n)) if record else None
            tim = None
        else:
            wave = np.zeros((B, capacity, n)) if record else None
            tim = np.zeros((B, capacity)) if record else None
        np_ = np.zeros(B, dtype=np.int32)
        st = np.zeros(B, dtype=np.int32)
        steps = np.zeros(B, dtype=np.int32)
        it = np.zeros(B, dtype=np.int32)
        rc = L.ks_tran(self.handle, ctypes.byref(sp), ctypes.byref(o), int(capacity),
                       None if tim is None else tim.ctypes.data, None if wave is None else wave.ctypes.data,
                       np_.ctypes.data, st.ctypes.data, steps.ctypes.data, it.ctypes.data, stream)
        _check(rc, "ks_tran")
        return wave, tim, np_, st, steps, it

    def tran_async(self, spec, opt, capacity, time_dev, wave_dev, npts_dev, status_dev, steps_dev, iters_dev,
                   stream):
        """ks_tran_async on device pointers (ints; 0 or None where not wanted) on a CUDA stream handle."""
        o = (opt or Options()).c()
        sp = spec.c() if hasattr(spec, "c") else spec
        _check(_lib.load().ks_tran_async(self.handle, ctypes.byref(sp), ctypes.byref(o), int(capacity), time_dev,
                                         wave_dev, npts_dev, status_dev, steps_dev, iters_dev, stream),
               "ks_tran_async")

    def ac(self, freqs, opt=None, x0=None, stream=None):
        """analysis.AC for every circuit (ks_ac): (x [n_circ][n_freq][n] complex,
        status [n_circ], operating-point iterations [n_circ])."""
        o = (opt or Options()).c()
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        if f.ndim != 1 or len(f) == 0:
            raise ValueError("ac: freqs must be a non-empty 1-D array")
        x = np.zeros((self.n_circ, len(f), self.plan.n, 2))
        st = np.zeros(self.n_circ, dtype=np.int32)
        it = np.zeros(self.n_circ, dtype=np.int32)
        x0a = None
        if x0 is not None:
            x0a = np.ascontiguousarray(x0, dtype=np.float64)
            assert x0a.shape == (self.n_circ, self.plan.n)
        _check(_lib.load().ks_ac(self.handle, ctypes.byref(o), None if x0a is None else x0a.ctypes.data,
                                 f.ctypes.data, len(f), x.ctypes.data, st.ctypes.data, it.ctypes.data, stream),
               "ks_ac")
        return x[..., 0] + 1j * x[..., 1], st, it

    def dc_sweep(self, src, values, opt=None, src2=None, values2=None, stream=None):
        """analysis.DC for every circuit (ks_dc_sweep): element `src` takes `values`
        in order (for each of `values2` of an outer source `src2` in turn), each
        point warm-started from the previous one.  (x [n_circ][n_points][n], with
        the inner source stepping fastest, status [n_circ], points solved
        [n_circ], Newton iterations [n_circ])."""
        o = (opt or Options()).c()
        v = np.ascontiguousarray(values, dtype=np.float64)
        if v.ndim != 1 or len(v) == 0:
            raise ValueError("dc_sweep: values must be a non-empty 1-D array")
        if src2 is not None and (values2 is None or len(values2) == 0):
            raise ValueError("dc_sweep: an outer source needs a non-empty values2")
        v2 = None if src2 is None else np.ascontiguousarray(values2, dtype=np.float64)
        total = len(v) * (1 if v2 is None else len(v2))
        x = np.zeros((self.n_circ, total, self.plan.n))
        st = np.zeros(self.n_circ, dtype=np.int32)
        pts = np.zeros(self.n_circ, dtype=np.int32)
        it = np.zeros(self.n_circ, dtype=np.int32)
        _check(_lib.load().ks_dc_sweep(self.handle, ctypes.byref(o), int(src), v.ctypes.data, len(v),
                                       -1 if v2 is None else int(src2), None if v2 is None else v2.ctypes.data,
                                       0 if v2 is None else len(v2), x.ctypes.data, st.ctypes.data, pts.ctypes.data,
                                       it.ctypes.data, stream), "ks_dc_sweep")
        return x, st, pts, it

    def ac_async(self, opt, x0_dev, freqs_dev, n_freq, x_dev, status_dev, iters_dev, stream):
        """ks_ac_async on device pointers (ints) on a CUDA stream handle."""
        o = (opt or Options()).c()
        _check(_lib.load().ks_ac_async(self.handle, ctypes.byref(o), x0_dev, freqs_dev, n_freq, x_dev, status_dev,
                                       iters_dev, stream), "ks_ac_async")

    def ac_at_async(self, opt, x_op_dev, status_dev, freqs_dev, n_freq, x_dev, out_status_dev, stream):
        """ks_ac_at: the sweep alone about given operating points (device pointers)."""
        o = (opt or Options()).c()
        _check(_lib.load().ks_ac_at(self.handle, ctypes.byref(o), x_op_dev, status_dev, freqs_dev, n_freq, x_dev,
                                    out_status_dev, stream), "ks_ac_at")

    def cancel_word(self):
        """The batch's cancel word (ks_batch_cancel_word) as a ctypes int32 in
        mapped page-locked memory: set .value = 1 to interrupt the batch's
        running analysis, 0 before the next one."""
        p = ctypes.POINTER(ctypes.c_int32)()
        _check(_lib.load().ks_batch_cancel_word(self.handle, ctypes.byref(p)), "ks_batch_cancel_word")
        return p.contents

    def op_async(self, opt, x0_dev, x_dev, status_dev, iters_dev, stream):
        """ks_op_async on device pointers (ints) on a CUDA stream handle."""
        o = (opt or Options()).c()
        _check(_lib.load().ks_op_async(self.handle, ctypes.byref(o), x0_dev, x_dev, status_dev, iters_dev, stream),
               "ks_op_async")

    def __del__(self):
        if getattr(self, "handle", None) and _lib._lib is not None:
            _lib._lib.ks_batch_destroy(self.handle)
            self.handle = None


class MultiBatch:
    """Circuits of different topologies and sizes in one batch (ks_multi_create):
    the GPU gives each circuit a warp and a sparse system with a fixed pivot
    sequence from the host's symbolic analysis."""

    def __init__(self, circuits):
        L = _lib.load()
        self._els, topos, vals, offs = [], [], [], []
        nv = 0
        for c in circuits:
            if isinstance(c, tuple):
                el, nn, v = c
            else:
                el, v, _ = c.pack()
                nn = c.n_nodes
            el = np.ascontiguousarray(el, dtype=ELEMENT_DTYPE)
            self._els.append(el)
            topos.append(_lib.KsTopology(int(nn), len(el), len(v), 0, el.ctypes.data))
            vals.append(np.asarray(v, dtype=np.float64))
            offs.append(nv)
            nv += len(v)
        self.n_circ = len(topos)
        self._topos = (_lib.KsTopology * self.n_circ)(*topos)
        self._vals = np.ascontiguousarray(np.concatenate(vals))
        self._offs = np.asarray(offs, dtype=np.int64)
        h = ctypes.c_void_p()
        _check(L.ks_multi_create(self.n_circ, self._topos, self._vals.ctypes.data, self._offs.ctypes.data,
                                 ctypes.byref(h)), "ks_multi_create")
        self.handle = h
        N, F, fl = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self.n = np.zeros(self.n_circ, dtype=np.int32)
        _check(L.ks_multi_info(h, ctypes.byref(N), ctypes.byref(F), ctypes.byref(fl), self.n.ctypes.data),
               "ks_multi_info")
        self.total_unknowns, self.factor_slots, self.lu_flops = N.value, F.value, fl.value
        self.x_off = np.concatenate([[0], np.cumsum(self.n)[:-1]]).astype(np.int64)

    def op(self, opt=None):
        """([x_c], status, iters) for every circuit."""
        o = (opt or Options()).c()
        x = np.zeros(self.total_unknowns)
        st = np.zeros(self.n_circ, dtype=np.int32)
        it = np.zeros(self.n_circ, dtype=np.int32)
        _check(_lib.load().ks_multi_op(self.handle, ctypes.byref(o), x.ctypes.data, st.ctypes.data, it.ctypes.data),
               "ks_multi_op")
        return [x[a:a + n] for a, n in zip(self.x_off, self.n)], st, it

    def tran(self, spec, opt=None):
        """Fixed-step transient: ([wave_c [n_points][n_c]], status, steps, iters)."""
        o = (opt or Options()).c()
        sp = spec.c() if hasattr(spec, "c") else spec
        npts = int(round(sp.stop / sp.step)) + 1
        w = np.zeros(npts * self.total_unknowns)
        st = np.zeros(self.n_circ, dtype=np.int32)
        steps = np.zeros(self.n_circ, dtype=np.int32)
        it = np.zeros(self.n_circ, dtype=np.int32)
        _check(_lib.load().ks_multi_tran(self.handle, ctypes.byref(sp), ctypes.byref(o), w.ctypes.data,
                                         st.ctypes.data, steps.ctypes.data, it.ctypes.data), "ks_multi_tran")
        waves = [w[npts * a:npts * (a + n)].reshape(npts, n) for a, n in zip(self.x_off, self.n)]
        return waves, st, steps, it

    def tran_async(self, spec, opt, wave_dev, npts_dev, status_dev, steps_dev, iters_dev, stream):
        o = (opt or Options()).c()
        sp = spec.c() if hasattr(spec, "c") else spec
        _check(_lib.load().ks_multi_tran_async(self.handle, ctypes.byref(sp), ctypes.byref(o), wave_dev, npts_dev,
                                               status_dev, steps_dev, iters_dev, stream), "ks_multi_tran_async")

    def __del__(self):
        if getattr(self, "handle", None) and _lib._lib is not None:
            _lib._lib.ks_multi_destroy(self.handle)
            self.handle = None


TORN_STATS = ("solves", "refactors", "refines", "max_passes", "not_accepted", "pieces", "coupling_rows", "max_band",
              "band_doubles", "launches", "refactor_us", "apply_us", "load_us", "residual_us", "untorn")


def torn_plan(elements, n_nodes, n_values, torn):
    """The tearing of a topology on the host (ks_torn_plan): (piece of each
    unknown, coupling rows, largest piece, largest band)."""
    L = _lib.load()
    el = np.ascontiguousarray(elements, dtype=ELEMENT_DTYPE)
    tr = np.ascontiguousarray(torn, dtype=np.int32)
    topo = _lib.KsTopology(int(n_nodes), len(el), int(n_values), 0, el.ctypes.data)
    n = ctypes.c_int32()
    _check(L.ks_unknowns(ctypes.byref(topo), ctypes.byref(n), None), "ks_unknowns")
    piece = np.zeros(n.value, dtype=np.int32)
    rows = np.zeros(n.value, dtype=np.int32)
    npc, nr, mp, mb = (ctypes.c_int32() for _ in range(4))
    _check(L.ks_torn_plan(ctypes.byref(topo), tr.ctypes.data if len(tr) else None, len(tr), piece.ctypes.data,
                          ctypes.byref(npc), rows.ctypes.data, n.value, ctypes.byref(nr), ctypes.byref(mp),
                          ctypes.byref(mb)), "ks_torn_plan")
    return piece, rows[:nr.value].copy(), mp.value, mb.value


def sparse_lu_pattern(elements, n_nodes, values, step=0.0):
    """The L + U slots of the host's fixed pivot sequence (ks_sparse_analyze): an
    [n][n] bool matrix in step coordinates (row i: the row pivoting at step i,
    column k: the column eliminated at step k), fill included."""
    L = _lib.load()
    el = np.ascontiguousarray(elements, dtype=ELEMENT_DTYPE)
    v = np.ascontiguousarray(values, dtype=np.float64)
    topo = _lib.KsTopology(int(n_nodes), len(el), len(v), 0, el.ctypes.data)
    n, slots = ctypes.c_int32(), ctypes.c_int64()
    _check(L.ks_sparse_analyze(ctypes.byref(topo), v.ctypes.data, float(step), ctypes.byref(n), ctypes.byref(slots),
                               None, None, None, None, None), "ks_sparse_analyze")
    rowptr = np.zeros(n.value + 1, dtype=np.int32)
    cols = np.zeros(slots.value, dtype=np.int32)
    _check(L.ks_sparse_analyze(ctypes.byref(topo), v.ctypes.data, float(step), None, None, None, None, None,
                               rowptr.ctypes.data, cols.ctypes.data), "ks_sparse_analyze")
    out = np.zeros((n.value, n.value), dtype=bool)
    for i in range(n.value):
        out[i, cols[rowptr[i]:rowptr[i + 1]]] = True
    return out


def sparse_analysis(elements, n_nodes, values, step=0.0):
    """The host's sparse analysis of one circuit (ks_sparse_analyze, ks_sparse_pattern):
    (column order [n], pivot rows [n], pattern [n][n] bool); step > 0: the
    transient's pattern and pivots."""
    L = _lib.load()
    el = np.ascontiguousarray(elements, dtype=ELEMENT_DTYPE)
    v = np.ascontiguousarray(values, dtype=np.float64)
    topo = _lib.KsTopology(int(n_nodes), len(el), len(v), 0, el.ctypes.data)
    n = ctypes.c_int32()
    _check(L.ks_unknowns(ctypes.byref(topo), ctypes.byref(n), None), "ks_unknowns")
    pcol = np.zeros(n.value, dtype=np.int32)
    prow = np.zeros(n.value, dtype=np.int32)
    pat = np.zeros((n.value, n.value), dtype=np.uint8)
    _check(L.ks_sparse_analyze(ctypes.byref(topo), v.ctypes.data, float(step), None, None, None, prow.ctypes.data,
                               pcol.ctypes.data, None, None), "ks_sparse_analyze")
    _check(L.ks_sparse_pattern(ctypes.byref(topo), v.ctypes.data, int(step > 0), None, pat.ctypes.data),
           "ks_sparse_pattern")
    return pcol, prow, pat.astype(bool)


class TornBatch:
    """Variants of one large topology solved torn into pieces (ks_torn_create):
    kron.JacobianTearing as analysis.Options.Solver, batched over the variants."""

    def __init__(self, elements, n_nodes, values, torn):
        L = _lib.load()
        self._el = np.ascontiguousarray(elements, dtype=ELEMENT_DTYPE)
        self.values = np.ascontiguousarray(values, dtype=np.float64)
        if self.values.ndim == 1:
            self.values = self.values[None, :]
        self.n_var = self.values.shape[0]
        self._torn = np.ascontiguousarray(torn, dtype=np.int32)
        topo = _lib.KsTopology(int(n_nodes), len(self._el), self.values.shape[1], 0, self._el.ctypes.data)
        h = ctypes.c_void_p()
        _check(L.ks_torn_create(ctypes.byref(topo), self.n_var, self.values.ctypes.data,
                                self._torn.ctypes.data if len(self._torn) else None, len(self._torn), ctypes.byref(h)),
               "ks_torn_create")
        self.handle = h
        info = [ctypes.c_int32() for _ in range(5)]
        L.ks_torn_info(self.handle, *[ctypes.byref(i) for i in info])
        self.n, self.pieces, self.coupling_rows, self.max_piece, self.max_band = (i.value for i in info)

    def set_stream(self, stream):
        """Run the later analyses on a CUDA stream handle (None: the batch's own)."""
        _check(_lib.load().ks_torn_set_stream(self.handle, stream), "ks_torn_set_stream")

    @staticmethod
    def _mode(reuse):
        """ks_torn's reuse argument: True (keep factors while they refine), False
        (refactor at every solve) or "untorn" (every system untorn)."""
        return 2 if reuse == "untorn" else int(bool(reuse))

    def op(self, opt=None, reuse=True):
        """(x [n_var][n], status, iterations, stats) of analysis.OP for every variant."""
        o = (opt or Options()).c()
        x = np.zeros((self.n_var, self.n))
        st = np.zeros(self.n_var, dtype=np.int32)
        it = np.zeros(self.n_var, dtype=np.int32)
        stats = np.zeros(15, dtype=np.int64)
        _check(_lib.load().ks_torn_op(self.handle, ctypes.byref(o), self._mode(reuse), x.ctypes.data, st.ctypes.data,
                                      it.ctypes.data, stats.ctypes.data), "ks_torn_op")
        return x, st, it, dict(zip(TORN_STATS, stats.tolist()))

    def tran(self, spec, opt=None, reuse=True, probes=()):
        """Fixed-step analysis.Tran of every variant: (wave [n_points][n_var][n_probes],
        last x [n_var][n], status, steps, iterations, stats)."""
        o = (opt or Options()).c()
        sp = spec.c() if hasattr(spec, "c") else spec
        npts = int(round(sp.stop / sp.step)) + 1
        pr = np.ascontiguousarray(probes, dtype=np.int32)
        wave = np.zeros((npts, self.n_var, len(pr)))
        x = np.zeros((self.n_var, self.n))
        st = np.zeros(self.n_var, dtype=np.int32)
        steps = np.zeros(self.n_var, dtype=np.int32)
        it = np.zeros(self.n_var, dtype=np.int32)
        stats = np.zeros(15, dtype=np.int64)
        _check(_lib.load().ks_torn_tran(self.handle, ctypes.byref(sp), ctypes.byref(o), self._mode(reuse),
                                        pr.ctypes.data if len(pr) else None, len(pr),
                                        wave.ctypes.data if len(pr) else None, x.ctypes.data, st.ctypes.data,
                                        steps.ctypes.data, it.ctypes.data, stats.ctypes.data), "ks_torn_tran")
        return wave, x, st, steps, it, dict(zip(TORN_STATS, stats.tolist()))

    def __del__(self):
        if getattr(self, "handle", None) and _lib._lib is not None:
            _lib._lib.ks_torn_destroy(self.handle)
            self.handle = None


def validate(circuit, transient=False):
    """circuit.Validate: None or the typed validation error."""
    el, vals, _ = circuit.pack()
    return validate_packed(el, circuit.n_nodes, vals, transient)


def validate_packed(el, n_nodes, vals, transient=False):
    """circuit.Validate of a packed topology and value vector."""
    el = np.ascontiguousarray(el)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    topo = _lib.KsTopology(n_nodes, len(el), len(vals), 0, el.ctypes.data)
    rc = _lib.load().ks_validate(ctypes.byref(topo), vals.ctypes.data, int(transient))
    if rc == 0:
        return None
    msg = _lib.last_error()
    if "no path to ground" in msg:
        return ErrFloatingNode(msg)
    return ErrValidation(msg)


@dataclass
class TranSpec:
    """analysis.TranSpec + TranOptions (analysis/tran.go:26-40) plus the fixed-step batch mode."""
    step: float
    stop: float
    start: float = 0.0
    max_step: float = 0.0
    uic: bool = False
    method: str = "trap"
    fixed_step: bool = False
    max_steps: int = 0
    chgtol: float = 0.0
    trtol: float = 0.0
    min_step: float = 0.0

    def c(self):
        return _lib.KsTranSpec(self.step, self.stop, self.start, self.max_step, int(self.uic),
                               1 if self.method == "be" else 2, int(self.fixed_step), self.max_steps, self.chgtol,
                               self.trtol, self.min_step)


@dataclass
class Result:
    """The parts of output.Result (output/result.go:112-119) the engine computes."""
    node_names: list
    node_voltages: np.ndarray          # [n_nodes], ground first
    x: np.ndarray                      # all MNA unknowns
    iterations: int = 0
    extra: dict = field(default_factory=dict)


def op_batch(circuits, opt=None, nodeset=None):
    """analysis.OP for every circuit: (results, errors), one entry per circuit."""
    opt = opt or Options()
    results, errors = [None] * len(circuits), [None] * len(circuits)
    groups = {}
    packed = []
    for i, c in enumerate(circuits):
        err = validate(c)
        if err is not None:
            errors[i] = err
            packed.append(None)
            continue
        el, vals, key = c.pack()
        packed.append((el, vals))
        groups.setdefault(key, []).append(i)
    for key, idx in groups.items():
        el = packed[idx[0]][0]
        nv = len(packed[idx[0]][1])
        plan = Plan(el, circuits[idx[0]].n_nodes, nv)
        vals = np.stack([packed[i][1] for i in idx])
        b = Batch(plan, vals)
        x0 = None
        if nodeset is not None:
            x0 = np.zeros((len(idx), plan.n))
            for r, i in enumerate(idx):
                ns = nodeset[i]
                if ns is not None:
                    x0[r, :len(ns)] = ns
        x, st, it = b.op(opt, x0)
        for r, i in enumerate(idx):
            if st[r] != 0:
                errors[i] = status_error(st[r])
                continue
            c = circuits[i]
            nv_ = np.zeros(c.n_nodes)
            nv_[1:] = x[r, :c.n_nodes - 1]
            results[i] = Result(list(c.node_names), nv_, x[r].copy(), int(it[r]))
    return results, errors


class ErrBadACSpec(KronspiceError):
    """analysis.ErrBadACSpec (analysis/ac.go:16)."""


MAX_AC_POINTS = 1_000_000  # analysis/ac.go:29


@dataclass
class ACSpec:
    """analysis.ACSpec (analysis/ac.go:19-24)."""
    variation: str   # "dec", "oct" or "lin"
    points: int      # per decade / per octave, or total for lin
    fstart: float
    fstop: float

    def frequencies(self):
        """ACSpec.Frequencies (analysis/ac.go:33-72): the sweep's frequencies in Hz."""
        import math
        p, f0, f1 = self.points, self.fstart, self.fstop
        if p < 1 or f1 < f0 or f0 < 0 or math.isnan(f0 + f1) or math.isinf(f1):
            raise ErrBadACSpec("analysis: invalid AC specification: %r" % (self,))
        if self.variation == "lin":
            if p == 1:
                return np.array([f0])
            step = (f1 - f0) / (p - 1)
            out = [f0 + k * step for k in range(p)]
        elif self.variation in ("dec", "oct"):
            if f0 <= 0:
                raise ErrBadACSpec("analysis: invalid AC specification: logarithmic sweep needs fstart > 0")
            ratio = math.pow(10.0 if self.variation == "dec" else 2.0, 1.0 / p)
            n = int(math.floor(math.log(f1 / f0) / math.log(ratio) + 1e-9)) + 1
            if n > MAX_AC_POINTS:
                raise ErrBadACSpec("analysis: invalid AC specification: %d points" % n)
            out = [f0 * math.pow(ratio, k) for k in range(n)]
        else:
            raise ErrBadACSpec("analysis: invalid AC specification: sweep type %r" % self.variation)
        if len(out) > MAX_AC_POINTS:
            raise ErrBadACSpec("analysis: invalid AC specification: %d points" % len(out))
        return np.array(out)


@dataclass
class ACResult:
    """The phasor part of output.ACResult (output/result.go): V[node][freq], ground first."""
    node_names: list
    freq: np.ndarray
    node_voltages: np.ndarray          # [n_nodes][n_freq] complex, row 0 (ground) zero
    x: np.ndarray                      # [n_freq][n] complex, all MNA unknowns
    iterations: int = 0


def ac_batch(circuits, spec, opt=None):
    """analysis.AC for every circuit: (results, errors), one entry per circuit."""
    opt = opt or Options()
    freqs = spec.frequencies() if hasattr(spec, "frequencies") else np.asarray(spec, dtype=np.float64)
    results, errors = [None] * len(circuits), [None] * len(circuits)
    groups, packed = {}, []
    for i, c in enumerate(circuits):
        err = validate(c)
        if err is not None:
            errors[i] = err
            packed.append(None)
            continue
        el, vals, key = c.pack()
        packed.append((el, vals))
        groups.setdefault(key, []).append(i)
    for key, idx in groups.items():
        el = packed[idx[0]][0]
        plan = Plan(el, circuits[idx[0]].n_nodes, len(packed[idx[0]][1]))
        b = Batch(plan, np.stack([packed[i][1] for i in idx]))
        x, st, it = b.ac(freqs, opt)
        for r, i in enumerate(idx):
            if st[r] != 0:
                errors[i] = status_error(st[r])
                continue
            c = circuits[i]
            v = np.zeros((c.n_nodes, len(freqs)), dtype=complex)
            v[1:] = x[r, :, :c.n_nodes - 1].T
            results[i] = ACResult(list(c.node_names), freqs, v, x[r].copy(), int(it[r]))
    return results, errors
