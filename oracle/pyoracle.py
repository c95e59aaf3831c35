"""ctypes binding of the C oracle (test infrastructure only).

The oracle restates the reference kdigest algorithms on the CPU in FP64.  It is
imported only by the tests, by ``__graft_entry__.smoke`` and by the CPU-baseline
leg of ``bench.py`` -- as the checker or the timed reference, never as the
product path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libkd_oracle.so")

OK, EINVAL, EEMPTY, ERANGE, ECONVERGE = 0, 1, 2, 3, 4
K0, K1, K2, K3 = 0, 1, 2, 3

_D = ctypes.c_double
_I64 = ctypes.c_int64
_P = ctypes.c_void_p


def build(force: bool = False) -> str:
    """Compile the oracle with make (cc -ffp-contract=off)."""
    if force and os.path.exists(_LIB_PATH):
        os.remove(_LIB_PATH)
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.kdo_tile_compress.restype = ctypes.c_int
        L.kdo_tile_compress.argtypes = [ctypes.c_int, _D, _P, _P, ctypes.c_int, _P, _P, _P]
        L.kdo_tile_compress_literal.restype = ctypes.c_int
        L.kdo_tile_compress_literal.argtypes = [ctypes.c_int, _D, _P, _P, ctypes.c_int, _P, _P, _P]
        L.kdo_set_math.argtypes = [ctypes.c_int]
        L.kdo_get_math.restype = ctypes.c_int
        L.kdo_set_sums.argtypes = [ctypes.c_int]
        L.kdo_get_sums.restype = ctypes.c_int
        L.kdo_ppath_compress.restype = _I64
        L.kdo_ppath_compress.argtypes = [ctypes.c_int, _D, _P, _P, _I64, _P, _P, _P]
        L.kdo_digest_new.restype = _P
        L.kdo_digest_new.argtypes = [ctypes.c_int, _D, _D]
        L.kdo_digest_clone.restype = _P
        L.kdo_digest_clone.argtypes = [_P]
        L.kdo_digest_free.argtypes = [_P]
        L.kdo_add.argtypes = [_P, _D, _D]
        L.kdo_add_at.argtypes = [_P, _D, _D, _D]
        L.kdo_add_many.argtypes = [_P, _P, ctypes.c_int64]
        L.kdo_merge.argtypes = [_P]
        L.kdo_merge_into.argtypes = [_P, _P]
        L.kdo_add_batch_p.argtypes = [_P, _P, _I64]
        L.kdo_add_batch_p_at.argtypes = [_P, _P, _I64, _D]
        L.kdo_quantile.argtypes = [_P, _D, ctypes.POINTER(_D)]
        L.kdo_cdf.argtypes = [_P, _D, ctypes.POINTER(_D)]
        L.kdo_to_bytes.restype = _I64
        L.kdo_to_bytes.argtypes = [_P, _P, _I64]
        L.kdo_from_bytes.restype = _P
        L.kdo_from_bytes.argtypes = [_P, _I64, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.kdo_len.restype = _I64
        L.kdo_len.argtypes = [_P]
        L.kdo_total_weight.restype = _D
        L.kdo_total_weight.argtypes = [_P]
        L.kdo_state.argtypes = [_P, _P]
        L.kdo_centroids.restype = _I64
        L.kdo_centroids.argtypes = [_P, _P, _P, _I64]
        L.kdo_set_state.argtypes = [_P, _P, _P, _I64, _D, _D, _D, _D, _D]
        L.kdo_grouped_add_batch.argtypes = [_P, _I64, _P, _P, _I64, ctypes.c_int, _D, ctypes.c_int]
        L.kdo_merge_parts_p.argtypes = [_P, _P, _I64]
        L.kdo_query_batch.argtypes = [_P, _I64, _P, _P, _I64, ctypes.c_int, _P, ctypes.c_int]
        for name in ("kdo_log", "kdo_exp", "kdo_asin"):
            getattr(L, name).restype = _D
            getattr(L, name).argtypes = [_D]
        L.kdo_normalizer.restype = _D
        L.kdo_normalizer.argtypes = [ctypes.c_int, _D, _D]
        L.kdo_k.restype = _D
        L.kdo_k.argtypes = [ctypes.c_int, _D, _D]
        L.kdo_bucket.restype = ctypes.c_int32
        L.kdo_bucket.argtypes = [ctypes.c_int, _D, _D, _D]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        super().__init__(f"oracle error {code} {what}")
        self.code = code


MATH_SHARED, MATH_LIBM = 0, 1


class math_mode:
    """Context manager: evaluate the scale functions with the shared FP64
    functions (MATH_SHARED, what the kernels compute) or with the C library's
    log / asin (MATH_LIBM) inside the block."""

    def __init__(self, mode: int):
        self.mode = mode

    def __enter__(self):
        self.prev = lib().kdo_get_math()
        lib().kdo_set_math(self.mode)
        return self

    def __exit__(self, *exc):
        lib().kdo_set_math(self.prev)
        return False


SUMS_BUILD, SUMS_REFERENCE = 0, 1


class sums_mode:
    """Context manager: segment sums of w*x in the kernels' association
    (SUMS_BUILD) or in the reference's Hillis-Steele tree (SUMS_REFERENCE)
    inside the block.  Prefix sums, totals and weights never change."""

    def __init__(self, mode: int):
        self.mode = mode

    def __enter__(self):
        self.prev = lib().kdo_get_sums()
        lib().kdo_set_sums(self.mode)
        return self

    def __exit__(self, *exc):
        lib().kdo_set_sums(self.prev)
        return False


def _tile(fn, scale, compression, x, w):
    x = np.ascontiguousarray(x, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    n = len(x)
    om = np.empty(max(n, 1)); ow = np.empty(max(n, 1)); ids = np.empty(max(n, 1), np.int32)
    c = fn(scale, compression, _ptr(x), _ptr(w), n, _ptr(om), _ptr(ow), _ptr(ids))
    return om[:c].copy(), ow[:c].copy(), ids[:n].copy()


def tile_compress(scale: int, compression: float, x, w):
    """One P-path tile in the reference's Hillis-Steele association."""
    return _tile(lib().kdo_tile_compress, scale, compression, x, w)


def tile_compress_literal(scale: int, compression: float, x, w):
    """The same tile through the reference kernel's 1024-lane loops."""
    return _tile(lib().kdo_tile_compress_literal, scale, compression, x, w)


def ppath_compress(scale: int, compression: float, means, weights, want_perm: bool = False):
    m = np.ascontiguousarray(means, dtype=np.float64)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    n = len(m)
    om = np.empty(max(n, 1)); ow = np.empty(max(n, 1))
    perm = np.empty(max(n, 1), np.int64) if want_perm else None
    c = lib().kdo_ppath_compress(scale, compression, _ptr(m), _ptr(w), n, _ptr(om), _ptr(ow),
                                 _ptr(perm) if want_perm else None)
    if c < 0:
        raise OracleError(-c, "ppath")
    if want_perm:
        return om[:c].copy(), ow[:c].copy(), perm[:n].copy()
    return om[:c].copy(), ow[:c].copy()


class Digest:
    """One oracle TDigest (tdigest.mojo) with FP64 state."""

    def __init__(self, scale: int = K1, compression: float = 100.0, decay_lambda: float = 0.0,
                 _handle=None):
        self.scale = scale
        self._h = _handle if _handle is not None else lib().kdo_digest_new(scale, compression, decay_lambda)

    def __del__(self):
        try:
            if self._h:
                lib().kdo_digest_free(self._h)
                self._h = None
        except Exception:
            pass

    def clone(self) -> "Digest":
        return Digest(self.scale, _handle=lib().kdo_digest_clone(self._h))

    def _check(self, rc, what=""):
        if rc:
            raise OracleError(rc, what)

    def add(self, v: float, w: float = 1.0):
        self._check(lib().kdo_add(self._h, v, w), "add")

    def add_many(self, values):
        """The sequential add loop over unit-weight samples, in C."""
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._check(lib().kdo_add_many(self._h, v.ctypes.data_as(ctypes.c_void_p), len(v)), "add_many")

    def add_at(self, v: float, t: float, w: float = 1.0):
        self._check(lib().kdo_add_at(self._h, v, t, w), "add_at")

    def merge(self):
        lib().kdo_merge(self._h)

    def merge_into(self, other: "Digest"):
        self._check(lib().kdo_merge_into(self._h, other._h), "merge_into")

    def add_batch_p(self, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._check(lib().kdo_add_batch_p(self._h, _ptr(v), len(v)), "add_batch_p")

    def add_batch_p_at(self, values, t: float):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._check(lib().kdo_add_batch_p_at(self._h, _ptr(v), len(v), t), "add_batch_p_at")

    def quantile(self, q: float) -> float:
        out = _D()
        self._check(lib().kdo_quantile(self._h, q, ctypes.byref(out)), "quantile")
        return out.value

    def cdf(self, x: float) -> float:
        out = _D()
        self._check(lib().kdo_cdf(self._h, x, ctypes.byref(out)), "cdf")
        return out.value

    def to_bytes(self) -> bytes:
        n = lib().kdo_to_bytes(self._h, None, 0)
        buf = np.empty(n, np.uint8)
        lib().kdo_to_bytes(self._h, _ptr(buf), n)
        return buf.tobytes()

    @staticmethod
    def from_bytes(data: bytes, scale: int) -> "Digest":
        buf = np.frombuffer(data, np.uint8).copy() if len(data) else np.zeros(1, np.uint8)
        err = ctypes.c_int(0)
        h = lib().kdo_from_bytes(_ptr(buf), len(data), scale, ctypes.byref(err))
        if not h:
            raise OracleError(err.value, "from_bytes")
        return Digest(scale, _handle=h)

    def __len__(self):
        return int(lib().kdo_len(self._h))

    def total_weight(self) -> float:
        return lib().kdo_total_weight(self._h)

    def state(self) -> dict:
        s = np.empty(8)
        lib().kdo_state(self._h, _ptr(s))
        keys = ("compression", "lambda", "log_scale", "clock", "stored_total", "min", "max", "count")
        return dict(zip(keys, s.tolist()))

    def centroids(self):
        n = len(self)
        m = np.empty(max(n, 1)); w = np.empty(max(n, 1))
        lib().kdo_centroids(self._h, _ptr(m), _ptr(w), n)
        return m[:n].copy(), w[:n].copy()

    def set_state(self, means, weights, stored_total, log_scale, clock, min_v, max_v):
        m = np.ascontiguousarray(means, dtype=np.float64)
        w = np.ascontiguousarray(weights, dtype=np.float64)
        lib().kdo_set_state(self._h, _ptr(m), _ptr(w), len(m), stored_total, log_scale, clock,
                            min_v, max_v)


def grouped_add_batch(digests, keys, values, mode: int = 0, timestamp: float = 0.0,
                      threads: int = 1):
    k = np.ascontiguousarray(keys, dtype=np.uint32)
    v = np.ascontiguousarray(values, dtype=np.float64)
    arr = (ctypes.c_void_p * len(digests))(*[d._h for d in digests])
    rc = lib().kdo_grouped_add_batch(arr, len(digests), _ptr(k), _ptr(v), len(v), mode, timestamp,
                                     threads)
    if rc:
        raise OracleError(rc, "grouped_add_batch")


def merge_parts(dst: Digest, parts):
    arr = (ctypes.c_void_p * len(parts))(*[p._h for p in parts])
    rc = lib().kdo_merge_parts_p(dst._h, arr, len(parts))
    if rc:
        raise OracleError(rc, "merge_parts")


def query_batch(digests, ids, xs, is_cdf: bool, threads: int = 1):
    """Batched quantile / cdf over digests[ids[i]] at xs[i] (NaN where a query fails)."""
    arr = (ctypes.c_void_p * len(digests))(*[d._h for d in digests])
    k = np.ascontiguousarray(ids, dtype=np.int32)
    x = np.ascontiguousarray(xs, dtype=np.float64)
    out = np.empty(len(x))
    lib().kdo_query_batch(arr, len(digests), _ptr(k), _ptr(x), len(x), int(is_cdf), _ptr(out),
                          threads)
    return out


def log(x): return lib().kdo_log(x)
def exp(x): return lib().kdo_exp(x)
def asin(x): return lib().kdo_asin(x)
def normalizer(scale, compression, n): return lib().kdo_normalizer(scale, compression, n)
def k(scale, q, nrm): return lib().kdo_k(scale, q, nrm)
def bucket(scale, cum, tot, nrm): return lib().kdo_bucket(scale, cum, tot, nrm)
