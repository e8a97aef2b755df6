"""ctypes binding of include/fastem_gpu.h (libfastem_gpu.so, built in-tree).

There is no fallback: if the native library is missing or cannot be loaded
every entry point raises, so a test that passes has run the CUDA path.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfastem_gpu.so")

FEM_OK = 0
FEM_ERR_BAD_ARG = 1
FEM_ERR_CUDA = 2
FEM_ERR_CHOLESKY = 3
FEM_ERR_COND_ABORT = 4
FEM_ERR_TIMEOUT = 5
FEM_ERR_NO_DEVICE = 6
FEM_ERR_STATE = 7
FEM_ERR_UNSUPPORTED = 8

PREC = {"fp64": 0, "fp32": 1, "mixed": 2}

# every symbol include/fastem_gpu.h declares
EXPORTS = [
    "fem_api_version", "fem_last_error",
    "fem_em_config_default", "fem_em_create", "fem_em_destroy", "fem_em_set_parameters",
    "fem_em_upload", "fem_em_upload_device", "fem_em_set_params", "fem_em_get_params",
    "fem_em_train", "fem_em_init_densities", "fem_em_precompute", "fem_em_mstep",
    "fem_em_max_condition", "fem_em_selftest_wait_expiry", "fem_em_get_posteriors", "fem_em_retrieve_classes",
    "fem_em_posterior_correlation",
    "fem_em_get_factors", "fem_em_timing_reset", "fem_em_timing_get", "fem_em_timing_total",
    "fem_em_timing_covariance",
    "fem_em_batch_create", "fem_em_batch_destroy", "fem_em_batch_set_parameters",
    "fem_em_batch_upload", "fem_em_batch_upload_packed", "fem_em_batch_set_params",
    "fem_em_batch_get_params", "fem_em_batch_train", "fem_em_batch_trace",
    "fem_em_batch_fail_component", "fem_em_batch_timing_enable", "fem_em_batch_timing",
    "fem_em_batch_timing_classes", "fem_em_batch_tuning_default", "fem_em_batch_create_tuned",
    "fem_em_batch_get_tuning",
    "fem_km_config_default", "fem_km_create", "fem_km_destroy", "fem_km_upload",
    "fem_km_upload_device", "fem_km_init_data_structures", "fem_km_compute_mse_and_correct",
    "fem_km_correct_without_mse",
    "fem_km_run", "fem_km_get_assignment", "fem_km_seed", "fem_km_set_rng_state", "fem_km_get_rng_state",
    "fem_km_stats",
    "fem_km_classify_noalloc",
]


class FemError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("fastem status %d: %s" % (status, msg))
        self.status = status


class CholeskyError(FemError):
    """EMException("Cholesky decomposition failed") of the reference."""


class ConditionAbort(FemError):
    """EMException("Condition number of a covariance matrix is too high")."""


class EmConfig(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("device", ctypes.c_int), ("max_sweeps", ctypes.c_int),
                ("eps", ctypes.c_double), ("abort_thr", ctypes.c_double),
                ("reg_coef", ctypes.c_double), ("svd", ctypes.c_int)]


class BatchTuning(ctypes.Structure):
    """fem_em_batch_tuning: points per means / covariance item per dimension class."""
    _fields_ = [("means_chunk", ctypes.c_int * 4), ("cov_chunk", ctypes.c_int * 4)]


class KmConfig(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("device", ctypes.c_int), ("seed", ctypes.c_uint64),
                ("repair", ctypes.c_int)]


_LIB = None


def lib():
    """Load libfastem_gpu.so (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise ImportError("libfastem_gpu.so not built: run `python -c \"import __graft_entry__ as g; "
                          "g.build()\"` (the CUDA path has no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    P, i32, i64, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
    pP = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "fem_api_version": ([], i32),
        "fem_last_error": ([], ctypes.c_char_p),
        "fem_em_config_default": ([ctypes.POINTER(EmConfig)], None),
        "fem_em_create": ([i32, i64, i32, ctypes.POINTER(EmConfig), pP], i32),
        "fem_em_destroy": ([P], None),
        "fem_em_set_parameters": ([P, i32, f64, f64, f64], i32),
        "fem_em_upload": ([P, P, i64], i32),
        "fem_em_upload_device": ([P, P, i64], i32),
        "fem_em_set_params": ([P, P, P, P], i32),
        "fem_em_get_params": ([P, P, P, P], i32),
        "fem_em_train": ([P, i32, P, P, i32, P, P], i32),
        "fem_em_init_densities": ([P, P], i32),
        "fem_em_precompute": ([P, P], i32),
        "fem_em_mstep": ([P], i32),
        "fem_em_max_condition": ([P, P], i32),
        "fem_em_selftest_wait_expiry": ([P, i64, P], i32),
        "fem_em_get_posteriors": ([P, P], i32),
        "fem_em_retrieve_classes": ([P, P], i32),
        "fem_em_posterior_correlation": ([P, P], i32),
        "fem_em_get_factors": ([P, P, P], i32),
        "fem_em_timing_reset": ([P, i32], i32),
        "fem_em_timing_get": ([P, P, P, P, P], i32),
        "fem_em_timing_total": ([P, P, P], i32),
        "fem_em_timing_covariance": ([P, P], i32),
        "fem_em_batch_create": ([i32, P, P, P, ctypes.POINTER(EmConfig), pP], i32),
        "fem_em_batch_destroy": ([P], None),
        "fem_em_batch_set_parameters": ([P, i32, f64, f64, f64], i32),
        "fem_em_batch_upload": ([P, i32, P, i64], i32),
        "fem_em_batch_upload_packed": ([P, P], i32),
        "fem_em_batch_set_params": ([P, i32, P, P, P], i32),
        "fem_em_batch_get_params": ([P, i32, P, P, P], i32),
        "fem_em_batch_train": ([P, i32, P, P, P], i32),
        "fem_em_batch_trace": ([P, i32, P, P, i32], i32),
        "fem_em_batch_fail_component": ([P, i32, P], i32),
        "fem_em_batch_timing_enable": ([P, i32], i32),
        "fem_em_batch_timing": ([P, P, P, P], i32),
        "fem_em_batch_timing_classes": ([P, P], i32),
        "fem_em_batch_tuning_default": ([ctypes.POINTER(BatchTuning)], None),
        "fem_em_batch_create_tuned": ([i32, P, P, P, ctypes.POINTER(EmConfig), ctypes.POINTER(BatchTuning), pP],
                                      i32),
        "fem_em_batch_get_tuning": ([P, ctypes.POINTER(BatchTuning)], i32),
        "fem_km_config_default": ([ctypes.POINTER(KmConfig)], None),
        "fem_km_create": ([i32, i64, i32, ctypes.POINTER(KmConfig), pP], i32),
        "fem_km_destroy": ([P], None),
        "fem_km_upload": ([P, P, i64], i32),
        "fem_km_upload_device": ([P, P, i64], i32),
        "fem_km_init_data_structures": ([P], i32),
        "fem_km_compute_mse_and_correct": ([P, P, P, P], i32),
        "fem_km_correct_without_mse": ([P, P, P], i32),
        "fem_km_run": ([P, P, f64, i32, P, P], i32),
        "fem_km_get_assignment": ([P, P], i32),
        "fem_km_seed": ([P, ctypes.c_uint64], i32),
        "fem_km_set_rng_state": ([P, ctypes.c_char_p], i32),
        "fem_km_get_rng_state": ([P, ctypes.c_char_p, ctypes.c_size_t], i32),
        "fem_km_stats": ([P, P, P, P], i32),
        "fem_km_classify_noalloc": ([i32, i64, i32, P, P, P, P, i32, P], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _LIB = L
    return L


def last_error():
    return lib().fem_last_error().decode(errors="replace")


def check(status):
    if status == FEM_OK:
        return
    msg = last_error()
    if status == FEM_ERR_CHOLESKY:
        raise CholeskyError(status, msg)
    if status == FEM_ERR_COND_ABORT:
        raise ConditionAbort(status, msg)
    raise FemError(status, msg)


def ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def f32rows(X):
    X = np.asarray(X)
    if X.dtype != np.float32 or not X.flags.c_contiguous:
        X = np.ascontiguousarray(X, dtype=np.float32)
    return X
