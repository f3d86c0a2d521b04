"""ctypes binding of libkronspice_gpu.so (include/kronspice_gpu.h).

The library is built in-tree by kronspice_gb300.build (nvcc, sm_103a).  Loading
fails loudly when it is missing: the engine has no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libkronspice_gpu.so")


class KsTopology(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int32), ("n_elem", ctypes.c_int32), ("n_values", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("elem", ctypes.c_void_p)]


class KsOptions(ctypes.Structure):
    _fields_ = [("reltol", ctypes.c_double), ("abstol", ctypes.c_double), ("vntol", ctypes.c_double),
                ("gmin", ctypes.c_double), ("itl1", ctypes.c_int32), ("itl4", ctypes.c_int32),
                ("no_gmin_stepping", ctypes.c_int32), ("no_source_stepping", ctypes.c_int32),
                ("no_pseudo_transient", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("backend", ctypes.c_int32), ("max_iter_total", ctypes.c_int32),
                ("deadline_s", ctypes.c_double), ("mixed_passes", ctypes.c_int32),
                ("fp32_start_iters", ctypes.c_int32), ("start_check", ctypes.c_double),
                ("ledger_tol", ctypes.c_double), ("skip_energy_check", ctypes.c_int32),
                ("step_predictor", ctypes.c_int32), ("autotune", ctypes.c_int32)]


class KsTranSpec(ctypes.Structure):
    _fields_ = [("step", ctypes.c_double), ("stop", ctypes.c_double), ("start", ctypes.c_double),
                ("max_step", ctypes.c_double), ("uic", ctypes.c_int32), ("method", ctypes.c_int32),
                ("fixed_step", ctypes.c_int32), ("max_steps", ctypes.c_int32), ("chgtol", ctypes.c_double),
                ("trtol", ctypes.c_double), ("min_step", ctypes.c_double)]


# every symbol include/kronspice_gpu.h declares
EXPORTS = ["ks_version", "ks_last_error", "ks_validate", "ks_unknowns", "ks_plan_create", "ks_plan_destroy",
           "ks_plan_info", "ks_batch_create", "ks_batch_set_values", "ks_batch_destroy", "ks_op", "ks_op_async",
           "ks_tran", "ks_tran_async", "ks_tran_points", "ks_plan_specialize", "ks_plan_kernel_source",
           "ks_batch_last_kernel", "ks_op_noalloc", "ks_op_noalloc_scratch_bytes", "ks_multi_create",
           "ks_multi_destroy", "ks_multi_info", "ks_multi_op", "ks_multi_op_async", "ks_multi_tran",
           "ks_multi_tran_async", "ks_sparse_analyze", "ks_ac", "ks_ac_async", "ks_ac_at", "ks_dc_sweep", "ks_plan_tuned", "ks_torn_create",
           "ks_torn_destroy", "ks_torn_plan", "ks_torn_set_stream", "ks_torn_info", "ks_torn_op", "ks_torn_tran",
           "ks_fp64_peak", "ks_batch_cancel_word", "ks_op_results", "ks_op_results_async", "ks_tran_results",
           "ks_tran_results_async", "ks_sparse_pattern"]

_lib = None


class EngineMissing(RuntimeError):
    pass


def load(build_if_missing=False):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build
            build.build()
        else:
            raise EngineMissing("kronspice_gb300: %s is not built (run kronspice_gb300/build.py); "
                                "the engine has no CPU fallback" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    L.ks_version.restype = ctypes.c_char_p
    L.ks_last_error.restype = ctypes.c_char_p
    L.ks_validate.argtypes = [P, P, ctypes.c_int]
    L.ks_unknowns.argtypes = [P, P, P]
    L.ks_plan_create.argtypes = [P, ctypes.POINTER(ctypes.c_void_p)]
    L.ks_plan_destroy.argtypes = [P]
    L.ks_plan_destroy.restype = None
    L.ks_plan_info.argtypes = [P, P, P, P]
    L.ks_batch_create.argtypes = [P, ctypes.c_int32, P, ctypes.POINTER(ctypes.c_void_p)]
    L.ks_batch_set_values.argtypes = [P, P, ctypes.c_int, P]
    L.ks_batch_destroy.argtypes = [P]
    L.ks_batch_destroy.restype = None
    L.ks_op.argtypes = [P, P, P, P, P, P, P]
    L.ks_op_async.argtypes = [P, P, P, P, P, P, P]
    L.ks_tran.argtypes = [P, P, P, ctypes.c_int32, P, P, P, P, P, P, P]
    L.ks_tran_async.argtypes = [P, P, P, ctypes.c_int32, P, P, P, P, P, P, P]
    L.ks_op_results.argtypes = [P, P, P, P, P, P, P, P, P]
    L.ks_op_results_async.argtypes = [P, P, P, P, P, P, P, P, P]
    L.ks_tran_results.argtypes = [P, P, P, ctypes.c_int32, P, P, P, P, P, P, P, P, P, P]
    L.ks_tran_results_async.argtypes = [P, P, P, ctypes.c_int32, P, P, P, P, P, P, P, P, P, P]
    L.ks_tran_points.argtypes = [P, P]
    L.ks_plan_specialize.argtypes = [P, ctypes.c_int32, P, P]
    L.ks_plan_kernel_source.argtypes = [P, ctypes.c_int32, ctypes.c_char_p, ctypes.c_size_t, P]
    L.ks_batch_last_kernel.argtypes = [P]
    L.ks_op_noalloc.argtypes = [P, ctypes.c_int32, P, P, P, P, P, P]
    L.ks_op_noalloc_scratch_bytes.argtypes = [P, ctypes.c_int32, P]
    L.ks_multi_create.argtypes = [ctypes.c_int32, P, P, P, ctypes.POINTER(ctypes.c_void_p)]
    L.ks_sparse_analyze.argtypes = [P, P, ctypes.c_double, P, P, P, P, P, P, P]
    L.ks_sparse_pattern.argtypes = [P, P, ctypes.c_int32, P, P]
    L.ks_multi_destroy.argtypes = [P]
    L.ks_multi_destroy.restype = None
    L.ks_multi_info.argtypes = [P, P, P, P, P]
    L.ks_multi_op.argtypes = [P, P, P, P, P]
    L.ks_multi_op_async.argtypes = [P, P, P, P, P, P]
    L.ks_multi_tran.argtypes = [P, P, P, P, P, P, P]
    L.ks_multi_tran_async.argtypes = [P, P, P, P, P, P, P, P, P]
    L.ks_ac.argtypes = [P, P, P, P, ctypes.c_int32, P, P, P, P]
    L.ks_ac_async.argtypes = [P, P, P, P, ctypes.c_int32, P, P, P, P]
    L.ks_ac_at.argtypes = [P, P, P, P, P, ctypes.c_int32, P, P, P]
    L.ks_plan_tuned.argtypes = [P, ctypes.c_int32, ctypes.c_int64, P, P, P]
    L.ks_dc_sweep.argtypes = [P, P, ctypes.c_int32, P, ctypes.c_int32, ctypes.c_int32, P, ctypes.c_int32, P, P, P,
                              P, P]
    L.ks_torn_create.argtypes = [P, ctypes.c_int32, P, P, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]
    L.ks_torn_destroy.argtypes = [P]
    L.ks_torn_destroy.restype = None
    L.ks_torn_set_stream.argtypes = [P, P]
    L.ks_torn_plan.argtypes = [P, P, ctypes.c_int32, P, P, P, ctypes.c_int32, P, P, P]
    L.ks_torn_info.argtypes = [P, P, P, P, P, P]
    L.ks_torn_op.argtypes = [P, P, ctypes.c_int32, P, P, P, P]
    L.ks_torn_tran.argtypes = [P, P, P, ctypes.c_int32, P, ctypes.c_int32, P, P, P, P, P, P]
    L.ks_fp64_peak.argtypes = [P, P]
    L.ks_batch_cancel_word.argtypes = [P, P]
    _lib = L
    return L


def last_error():
    return load().ks_last_error().decode()
