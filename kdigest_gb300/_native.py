"""ctypes binding of libkdigest_gb300.so (the C-ABI in include/kdigest_gb300.h).

The library is the only compute path: there is no CPU fallback.  Importing
this module on a machine without the built library raises immediately.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libkdigest_gb300.so")

KD_OK, KD_EINVAL, KD_EEMPTY, KD_ERANGE, KD_ECONVERGE, KD_ENOMEM, KD_ECUDA, KD_ETIMEOUT = range(8)
KD_K0, KD_K1, KD_K2, KD_K3 = 0, 1, 2, 3
KD_CLOCK_COUNT, KD_CLOCK_TIME = 0, 1
KD_PTR_DEVICE = 1
KD_OPT_FORCE_EXACT_K, KD_OPT_MAX_LEVELS, KD_OPT_STAGE_TIMING, KD_OPT_GRAPHS = 1, 2, 3, 4
KD_OPT_SMALL_TILE_CAP, KD_OPT_LARGE_BLOCKS_PER_SM, KD_OPT_SMALL_BLOCKS_PER_SM = 5, 6, 7
KD_OPT_CONCURRENT_TILES = 8
KD_OPT_FRONT_STREAMS = 9
KD_OPT_TEST_WAIT = 10
STAGES = ("prep", "sort", "plan", "level0", "levels", "commit")

EXPORTED = (
    "kd_version", "kd_status_string", "kd_session_create", "kd_session_destroy",
    "kd_last_error", "kd_session_sync", "kd_session_set_option", "kd_session_stream",
    "kd_session_stats", "kd_session_reset_stats",
    "kd_compress", "kd_store_create", "kd_store_destroy", "kd_store_ingest",
    "kd_store_quantile", "kd_store_cdf", "kd_store_merge", "kd_store_get_digest",
    "kd_store_set_digest", "kd_store_to_bytes", "kd_store_from_bytes", "kd_store_stats",
    "kd_store_counts", "kd_compress_noalloc",
    "kd_server_create", "kd_server_submit", "kd_server_advance", "kd_server_wait",
    "kd_server_flush", "kd_server_stats", "kd_server_destroy",
    "kd_store_export", "kd_store_import",
    "kd_keymap_create", "kd_keymap_map", "kd_keymap_lookup", "kd_keymap_size", "kd_keymap_destroy",
    "kd_store_add", "kd_store_flush", "kd_store_merge_into", "kd_store_ingest_many",
    "kd_store_query_batch", "kd_grouped_compress", "kd_quantile", "kd_cdf", "kd_merge",
    "kd_server_latency", "kd_server_memory", "kd_server_groups", "kd_selftest_fp64",
    "kd_session_alloc_stats",
)
KD_REQ_INGEST, KD_REQ_QUANTILE, KD_REQ_CDF = 0, 1, 2

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double


class KdError(RuntimeError):
    """A non-zero status from the engine (message from kd_last_error)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code
        self.message = message


_lib = None


def load(path: str = LIB_PATH):
    """Load the engine library; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"kdigest_gb300 native library not found at {path}; build it with "
            "`python -m kdigest_gb300.build` (requires nvcc)")
    L = ctypes.CDLL(path)
    L.kd_version.restype = ctypes.c_int
    L.kd_status_string.restype = ctypes.c_char_p
    L.kd_status_string.argtypes = [ctypes.c_int]
    L.kd_session_create.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(_P)]
    L.kd_session_destroy.argtypes = [_P]
    L.kd_last_error.restype = ctypes.c_char_p
    L.kd_last_error.argtypes = [_P]
    L.kd_session_sync.argtypes = [_P]
    L.kd_session_set_option.argtypes = [_P, ctypes.c_int, ctypes.c_int]
    L.kd_session_stream.restype = _P
    L.kd_session_stream.argtypes = [_P]
    L.kd_session_stats.argtypes = [_P, _P, ctypes.c_int, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]
    L.kd_session_reset_stats.argtypes = [_P]
    L.kd_compress.argtypes = [_P, ctypes.c_int, _D, _P, _P, _I64, ctypes.c_int, _P, _P, _I64,
                              ctypes.POINTER(_I64)]
    L.kd_store_create.argtypes = [_P, _I64, ctypes.c_int, _D, _D, ctypes.POINTER(_P)]
    L.kd_store_destroy.argtypes = [_P]
    L.kd_store_ingest.argtypes = [_P, _P, _P, _I64, ctypes.c_int, _D, ctypes.c_int]
    L.kd_store_ingest_many.argtypes = [_P, _I64, _P, _P, _P, ctypes.c_int, _P, ctypes.c_int,
                                       ctypes.POINTER(_I64)]
    L.kd_store_quantile.argtypes = [_P, _P, _P, _I64, _P, ctypes.c_int]
    L.kd_store_cdf.argtypes = [_P, _P, _P, _I64, _P, ctypes.c_int]
    L.kd_store_query_batch.argtypes = [_P, _P, _P, _I64, _P, _P, _P, _I64, _P, ctypes.c_int]
    L.kd_grouped_compress.argtypes = [_P, ctypes.c_int, _D, _I64, _P, _P, _I64, _P, _P, _P, _P,
                                      _P, _P, _P, _I64, ctypes.POINTER(_I64), _P, _P]
    L.kd_quantile.argtypes = [_P, _P, _I64, _P, _P, _P, _P, _P, _P, _I64, _P, ctypes.c_int]
    L.kd_cdf.argtypes = [_P, _P, _I64, _P, _P, _P, _P, _P, _P, _I64, _P, ctypes.c_int]
    L.kd_merge.argtypes = [_P, ctypes.c_int, _D, _P, _I64, _P, _P, _P, _I64, _P, _P, _P, _P, _I64,
                           ctypes.POINTER(_I64)]
    L.kd_store_merge.argtypes = [_P, _P, _P, _P, _I64]
    L.kd_store_get_digest.argtypes = [_P, ctypes.c_uint32, _P, _P, _P, _I64, ctypes.POINTER(_I64)]
    L.kd_store_set_digest.argtypes = [_P, ctypes.c_uint32, _P, _P, _P, _I64]
    L.kd_store_to_bytes.argtypes = [_P, ctypes.c_uint32, _P, _I64, ctypes.POINTER(_I64)]
    L.kd_store_from_bytes.argtypes = [_P, ctypes.c_uint32, _P, _I64]
    L.kd_store_counts.argtypes = [_P, _P, ctypes.c_int]
    L.kd_store_export.argtypes = [_P, _P, _I64, _P, _I64, _P, ctypes.c_int]
    L.kd_store_import.argtypes = [_P, _P, _I64, _P, _P, ctypes.c_int]
    L.kd_server_create.argtypes = [_P, _D, ctypes.c_size_t, ctypes.POINTER(_P)]
    L.kd_server_submit.argtypes = [_P, ctypes.c_int, _D, _P, _P, _I64, _P, ctypes.POINTER(_I64)]
    L.kd_server_advance.argtypes = [_P, _D]
    L.kd_server_wait.argtypes = [_P, _I64, _D, ctypes.POINTER(ctypes.c_int)]
    L.kd_server_flush.argtypes = [_P]
    L.kd_server_stats.argtypes = [_P, _P, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                                  ctypes.POINTER(_D)]
    L.kd_server_destroy.argtypes = [_P]
    L.kd_server_latency.argtypes = [_P, _I64, ctypes.POINTER(_D)]
    L.kd_server_memory.argtypes = [_P, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t),
                                   ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
    L.kd_server_groups.argtypes = [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                                   ctypes.POINTER(_D), ctypes.POINTER(_I64), ctypes.POINTER(_D)]
    L.kd_selftest_fp64.argtypes = [ctypes.c_int, _P, _P, _I64, _P]
    L.kd_session_alloc_stats.argtypes = [_P, ctypes.POINTER(_I64), ctypes.POINTER(_D)]
    L.kd_compress_noalloc.argtypes = [ctypes.c_int, _D, _P, _P, _I64, ctypes.c_int, _P, _P, _I64,
                                      ctypes.POINTER(_I64), _P, ctypes.c_char_p, ctypes.c_int]
    L.kd_store_stats.argtypes = [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                                 ctypes.POINTER(ctypes.c_size_t)]
    L.kd_store_add.argtypes = [_P, _P, _P, _P, _I64, ctypes.c_int]
    L.kd_store_flush.argtypes = [_P]
    L.kd_store_merge_into.argtypes = [_P, _P]
    L.kd_keymap_create.argtypes = [_P, _I64, ctypes.POINTER(_P)]
    L.kd_keymap_map.argtypes = [_P, _P, _I64, _P, ctypes.c_int]
    L.kd_keymap_lookup.argtypes = [_P, _P, _I64, _P, ctypes.c_int]
    L.kd_keymap_size.restype = _I64
    L.kd_keymap_size.argtypes = [_P]
    L.kd_keymap_destroy.argtypes = [_P]
    _lib = L
    return L


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)
