"""ctypes binding of libsmartcore_gb300.so (the C ABI in include/smartcore_gb300.h).

The library is required: importing a compute entry point without it raises,
and every compute call needs a CUDA device.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from .error import Failed, FailedError

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsmartcore_gb300.so")

SC_OK, SC_ERR_INVALID, SC_ERR_CUDA, SC_ERR_OOM, SC_ERR_TIMEOUT, SC_ERR_INTERNAL = range(6)
F32, F64 = 0, 1
ROW_MAJOR, COL_MAJOR = 0, 1
MEM_HOST, MEM_DEVICE = 0, 1
FORM_FP64, FORM_SPLIT_BF16 = 0, 1
RNG_SMALL, RNG_STD = 0, 1
KNN_UNIFORM, KNN_DISTANCE = 0, 1

# Every symbol include/smartcore_gb300.h declares, with its ctypes signature.
_P, _I32, _I64, _U64, _D = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_double
SIGNATURES = {
    "sc_last_error": ([], C.c_char_p),
    "sc_abi_version": ([], _I32),
    "sc_device_ok": ([], _I32),
    "sc_kmeanspp_draws": ([_I32, _U64, _I64, _I64, _P, _P], _I32),
    "sc_kmeans_fit": ([_P, _I32, _I32, _I64, _I64, _I64, _I64, _I64, _I64, _P, _I32, _P, _P, _P, _P, _P], _I32),
    "sc_kmeans_predict": ([_P, _I32, _I32, _I64, _I64, _I64, _P, _I64, _I32, _P], _I32),
    "sc_kmeans_create": ([_P, _I32, _I32, _I32, _I64, _I64, _I64, _I32, _P], _I32),
    "sc_kmeans_seed": ([_P, _I64, _I64, _P], _I32),
    "sc_kmeans_set_centroids": ([_P, _I64, _P], _I32),
    "sc_kmeans_iterate": ([_P, _I64, _I32, _P], _I32),
    "sc_kmeans_get": ([_P, _P, _P, _P, _P, _P], _I32),
    "sc_kmeans_stream": ([_P], _P),
    "sc_kmeans_stats": ([_P, _P, _P], _I32),
    "sc_kmeans_sum_stats": ([_P, _P], _I32),
    "sc_kmeans_profile": ([_P, _I32], _I32),
    "sc_kmeans_profile_read": ([_P, _P, _P], _I32),
    "sc_kernel_launches": ([], _I64),
    "sc_kmeans_sync": ([_P], _I32),
    "sc_kmeans_step_noalloc": ([_P, _I32, _I64, _I64, _P, _I64, _P, _P, _P, _P], _I32),
    "sc_kmeans_destroy": ([_P], None),
    "sc_kmeans_fit_batched": ([_P, _I64, _I32, _I32], _I32),
    "sc_batch_tune": ([C.c_char_p], _I32),
    "sc_batch_tune_load": ([C.c_char_p], _I32),
    "sc_batch_tune_get": ([_I32, _I32, _P, _P], _I32),
    "sc_kmeans_set_wait_limit": ([_P, _I64], _I32),
    "sc_debug_fail_alloc_after": ([_I64], _I32),
    "sc_debug_live_allocations": ([], _I64),
    "sc_debug_knn_candidate_cap": ([_I64], _I32),
    "sc_debug_knn_chunk_queries": ([_I64], _I32),
    "sc_debug_batch_variant": ([_I32], _I32),
    "sc_knn_create": ([_P, _I32, _I32, _I32, _I64, _I64, _I64, _P], _I32),
    "sc_knn_find": ([_P, _P, _I32, _I32, _I64, _I64, _I64, _I32, _I32, _P, _P], _I32),
    "sc_knn_find_radius": ([_P, _P, _I32, _I32, _I64, _I64, _D, _I32, _P, _I64, _P, _P, _P], _I32),
    "sc_fastpair": ([_P, _P, _P, _P, _P], _I32),
    "sc_dbscan_fit": ([_P, _D, _I64, _I32, _P, _P], _I32),
    "sc_dbscan_predict": ([_P, _P, _I32, _I32, _I64, _I64, _D, _I32, _P, _I64, _P], _I32),
    "sc_knn_classify": ([_P, _P, _I32, _I32, _I64, _I64, _I64, _I32, _I32, _P, _I64, _P], _I32),
    "sc_knn_regress": ([_P, _P, _I32, _I32, _I64, _I64, _I64, _I32, _I32, _P, _P], _I32),
    "sc_knn_stream": ([_P], _P),
    "sc_knn_stats": ([_P, _P], _I32),
    "sc_knn_destroy": ([_P], None),
}



class KMeansProblem(C.Structure):
    """sc_kmeans_problem of include/smartcore_gb300.h."""
    _fields_ = [("x", _P), ("layout", _I32), ("status", _I32), ("n", _I64), ("d", _I64), ("ld", _I64),
                ("k", _I64), ("max_iter", _I64), ("first_index", _I64), ("uniforms", _P),
                ("centroids_out", _P), ("sizes_out", _P), ("labels_out", _P), ("distortion_out", _P),
                ("iters_out", _P), ("rescored", _I64), ("pp_replays", _I64)]


_lib = None
_lock = threading.Lock()


def load():
    """Load the library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"{LIB_PATH} is missing: build it with `python -m smartcore_gb300.build` "
                    "(the GPU path has no CPU fallback)")
            L = C.CDLL(LIB_PATH)
            for name, (args, res) in SIGNATURES.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = res
            _lib = L
    return _lib


def last_error() -> str:
    return load().sc_last_error().decode(errors="replace")


def check(status: int, kind: FailedError = FailedError.FitFailed):
    """Raise Failed for a non-zero sc_status, with the library's message."""
    if status == SC_OK:
        return
    msg = last_error()
    if status == SC_ERR_INVALID:
        raise Failed(kind, msg)
    raise Failed(FailedError.InvalidStateError, f"[status {status}] {msg}")


def ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)
