"""Host mirror of the reference kdigest API over the GB300 engine.

Names, argument meaning and error behaviour follow the reference
(src/kdigest/tdigest.mojo, grouped.mojo, decay.mojo, gpu/session.mojo):

  * ``Decay.none / rate / half_life``           (decay.mojo:24-51)
  * ``TDigest(compression, scale, decay)``       (tdigest.mojo:135-151)
      add_batch / add_batch_at / add / add_at, quantile, cdf, merge_into,
      to_bytes / from_bytes, total_weight, min, max, len
  * ``GroupedTDigest(num_keys, compression, decay)`` (grouped.mojo:30-190)
  * ``GpuSession``                                (gpu/session.mojo:19-27)

Every batch takes the reference's GPU route (the P-path: parallel
k-bucketing over 1024-element tiles), in FP64.  Errors the reference raises
surface as ``ValueError`` (invalid input), ``IndexError`` (key out of range)
or ``KdError`` (engine status), and a rejected batch leaves every digest
unchanged.
"""
from __future__ import annotations

import ctypes
import math
import sys

import numpy as np

from . import _native as N
from ._native import KdError

K0, K1, K2, K3 = N.KD_K0, N.KD_K1, N.KD_K2, N.KD_K3
SCALES = {"K0": K0, "K1": K1, "K2": K2, "K3": K3}


def _check(sess_handle, rc: int):
    if rc == N.KD_OK:
        return
    msg = N.load().kd_last_error(sess_handle).decode(errors="replace")
    if rc == N.KD_EINVAL:
        raise ValueError(msg)
    if rc == N.KD_EEMPTY:
        raise ValueError(msg)
    raise KdError(rc, msg)


class Decay:
    """Exponential decay rate lambda per unit of the digest's clock."""

    def __init__(self, rate_lambda: float = 0.0):
        self.rate_lambda = float(rate_lambda)

    @staticmethod
    def none() -> "Decay":
        return Decay(0.0)

    @staticmethod
    def rate(lambda_: float) -> "Decay":
        return Decay(lambda_)

    @staticmethod
    def half_life(h: float) -> "Decay":
        if not h > 0.0:
            raise ValueError("half_life must be positive")
        return Decay(math.log(2.0) / h)

    def is_active(self) -> bool:
        return self.rate_lambda > 0.0

    def __repr__(self):
        return f"Decay(lambda={self.rate_lambda})"


class GpuSession:
    """One device, one CUDA stream, reusable workspaces (gpu/session.mojo)."""

    def __init__(self, device: int = 0, mem_budget: int = 0, tuned: bool = True):
        L = N.load()
        h = ctypes.c_void_p()
        rc = L.kd_session_create(device, mem_budget, ctypes.byref(h))
        if rc != N.KD_OK:
            raise KdError(rc, f"kd_session_create failed ({L.kd_status_string(rc).decode()})")
        self._h = h.value
        self.device = device
        if tuned:  # launch parameters chosen by the committed autotuner run
            from .tune import apply_tuning, load_tuning

            apply_tuning(self, load_tuning())

    @property
    def handle(self):
        return self._h

    def set_option(self, option: int, value: int):
        _check(self._h, N.load().kd_session_set_option(self._h, option, value))

    def sync(self):
        _check(self._h, N.load().kd_session_sync(self._h))

    def stats(self) -> dict:
        ms = np.zeros(8)
        launches = ctypes.c_int64(0)
        ingests = ctypes.c_int64(0)
        n = N.load().kd_session_stats(self._h, N.ptr(ms), 8, ctypes.byref(launches),
                                      ctypes.byref(ingests))
        return {"stage_ms": dict(zip(N.STAGES, ms[:n].tolist())), "launches": launches.value,
                "ingests": ingests.value}

    def reset_stats(self):
        N.load().kd_session_reset_stats(self._h)

    def alloc_stats(self) -> dict:
        """Ingest workspace (re)allocations so far and the host seconds they took."""
        grows = ctypes.c_int64(0)
        sec = ctypes.c_double(0.0)
        N.load().kd_session_alloc_stats(self._h, ctypes.byref(grows), ctypes.byref(sec))
        return {"workspace_growths": grows.value, "workspace_growth_s": sec.value}

    @property
    def stream(self) -> int:
        return N.load().kd_session_stream(self._h) or 0

    def close(self):
        if getattr(self, "_h", None):
            N.load().kd_session_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            if not sys.is_finalizing():  # process exit releases everything
                self.close()
        except Exception:
            pass


_default_session = None


def default_session() -> GpuSession:
    global _default_session
    if _default_session is None:
        _default_session = GpuSession()
    return _default_session


def compress(means, weights, compression: float = 100.0, scale: int = K1,
             session: GpuSession | None = None):
    """gpu_compress_batch (gpu/add_batch.mojo:629-663): P-path compress of an
    arbitrary (mean, weight) set.  Returns (means, weights) as float64 arrays."""
    s = session or default_session()
    m = np.ascontiguousarray(means, dtype=np.float64)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    if m.shape != w.shape:
        raise ValueError("means and weights must have equal length")
    n = len(m)
    cap = min(max(n, 1), 1024)
    om = np.empty(cap)
    ow = np.empty(cap)
    out_n = ctypes.c_int64(0)
    rc = N.load().kd_compress(s.handle, scale, compression, N.ptr(m), N.ptr(w), n, 0, N.ptr(om),
                              N.ptr(ow), cap, ctypes.byref(out_n))
    _check(s.handle, rc)
    return om[:out_n.value].copy(), ow[:out_n.value].copy()


class _Store:
    """A resident store of num_keys digests on the device."""

    def __init__(self, num_keys: int, compression: float, scale: int, decay: Decay,
                 session: GpuSession | None):
        self.session = session or default_session()
        self.num_keys = int(num_keys)
        self.compression = float(compression)
        self.scale = int(scale)
        self.decay = decay if decay is not None else Decay.none()
        h = ctypes.c_void_p()
        rc = N.load().kd_store_create(self.session.handle, self.num_keys, self.scale,
                                      self.compression, self.decay.rate_lambda, ctypes.byref(h))
        _check(self.session.handle, rc)
        self._h = h.value

    def __del__(self):
        try:
            if getattr(self, "_h", None) and not sys.is_finalizing():
                N.load().kd_store_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def _chk(self, rc):
        _check(self.session.handle, rc)

    def ingest(self, keys, values, clock_mode=N.KD_CLOCK_COUNT, timestamp=0.0):
        v = np.ascontiguousarray(values, dtype=np.float64)
        k = None
        if keys is not None:
            k = np.asarray(keys)
            if len(k) != len(v):
                raise ValueError("keys and values must have equal length")
            if k.dtype.kind == "i" and len(k) and (k.min() < 0):
                raise IndexError("key out of range [0, num_keys)")
            k = np.ascontiguousarray(k, dtype=np.uint32)
        rc = N.load().kd_store_ingest(self._h, N.ptr(k), N.ptr(v), len(v), clock_mode, timestamp, 0)
        if rc == N.KD_EINVAL and k is not None and len(k) and int(k.max()) >= self.num_keys:
            raise IndexError("key out of range [0, num_keys)")
        self._chk(rc)

    def ingest_many(self, keys: list, values: list, device: bool):
        """kd_store_ingest_many over arrays that stay alive for the call:
        numpy arrays (host) or CUDA tensors (device, read in place)."""
        nb = len(values)
        if nb == 0:
            return
        addr = (lambda a: a.data_ptr()) if device else (lambda a: a.ctypes.data)
        kp = (ctypes.c_void_p * nb)(*[addr(k) if k is not None else None for k in keys])
        vp = (ctypes.c_void_p * nb)(*[addr(v) for v in values])
        ns = (ctypes.c_int64 * nb)(*[len(v) for v in values])
        done = ctypes.c_int64(0)
        rc = N.load().kd_store_ingest_many(self._h, nb, kp, vp, ns, N.KD_CLOCK_COUNT, None,
                                           N.KD_PTR_DEVICE if device else 0, ctypes.byref(done))
        self._chk(rc)

    def query(self, keys, xs, is_cdf: bool):
        x = np.ascontiguousarray(xs, dtype=np.float64)
        k = None if keys is None else np.ascontiguousarray(keys, dtype=np.uint32)
        out = np.empty(len(x))
        fn = N.load().kd_store_cdf if is_cdf else N.load().kd_store_quantile
        self._chk(fn(self._h, N.ptr(k), N.ptr(x), len(x), N.ptr(out), 0))
        return out

    def digest(self, key: int):
        hdr = np.empty(8)
        cnt = ctypes.c_int64(0)
        self._chk(N.load().kd_store_get_digest(self._h, key, N.ptr(hdr), None, None, 0,
                                               ctypes.byref(cnt)))
        m = np.empty(max(cnt.value, 1))
        w = np.empty(max(cnt.value, 1))
        self._chk(N.load().kd_store_get_digest(self._h, key, N.ptr(hdr), N.ptr(m), N.ptr(w),
                                               cnt.value, ctypes.byref(cnt)))
        return hdr, m[:cnt.value].copy(), w[:cnt.value].copy()

    def set_digest(self, key: int, hdr, means, weights):
        hdr = np.ascontiguousarray(hdr, dtype=np.float64)
        m = np.ascontiguousarray(means, dtype=np.float64)
        w = np.ascontiguousarray(weights, dtype=np.float64)
        self._chk(N.load().kd_store_set_digest(self._h, key, N.ptr(hdr), N.ptr(m), N.ptr(w), len(m)))

    def to_bytes(self, key: int) -> bytes:
        n = ctypes.c_int64(0)
        self._chk(N.load().kd_store_to_bytes(self._h, key, None, 0, ctypes.byref(n)))
        buf = np.empty(n.value, np.uint8)
        self._chk(N.load().kd_store_to_bytes(self._h, key, N.ptr(buf), n.value, ctypes.byref(n)))
        return buf.tobytes()

    def from_bytes(self, key: int, data: bytes):
        buf = np.frombuffer(bytes(data), np.uint8).copy() if len(data) else np.zeros(1, np.uint8)
        rc = N.load().kd_store_from_bytes(self._h, key, N.ptr(buf), len(data))
        self._chk(rc)

    def merge_from(self, src: "_Store", group_offsets, parts):
        go = np.ascontiguousarray(group_offsets, dtype=np.int64)
        pa = np.ascontiguousarray(parts, dtype=np.uint32)
        self._chk(N.load().kd_store_merge(self._h, src._h, N.ptr(go), N.ptr(pa), len(go) - 1))


def _validate_values(values) -> np.ndarray:
    v = np.ascontiguousarray(values, dtype=np.float64)
    if v.size and not np.all(np.isfinite(v)):
        raise ValueError("value must be finite (got NaN or inf)")
    return v


# add_batch takes the batch path from these sizes up, the single-sample loop
# below them (tdigest.mojo:49-58, 199, 215).
GPU_CROSSOVER = 60_000
GPU_CROSSOVER_SESSION = 40_000
_ADD_QUEUE = 4096  # single adds queued on the host before one device call


class TDigest:
    """One t-digest on the device (tdigest.mojo:97-726) — a one-key store.

    ``add`` / ``add_at`` and ``add_batch`` below the crossover run the
    reference's single-sample loop on the device (buffer, sequential merge
    pass); ``add_batch`` from the crossover up runs the batch path with the
    buffer folded in, as the reference does.  Single adds are validated at once
    and queued on the host; every other call first sends the queue, in order,
    so results are those of the reference's loop."""

    def __init__(self, compression: float = 100.0, scale: int = K1, decay: Decay | None = None,
                 session: GpuSession | None = None, _store: _Store | None = None):
        self.compression = float(compression)
        self.scale = scale
        self._decay = decay if decay is not None else Decay.none()
        self._store = _store or _Store(1, compression, scale, self._decay, session)
        self._qv: list[float] = []
        self._qw: list[float] = []
        self._qt: list[float] | None = None  # timestamps when the queue holds add_at

    @property
    def session(self) -> GpuSession:
        return self._store.session

    # -- ingest ---------------------------------------------------------------
    def _add_many(self, values, weights=None, timestamps=None):
        v = np.ascontiguousarray(values, dtype=np.float64)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        t = None if timestamps is None else np.ascontiguousarray(timestamps, dtype=np.float64)
        rc = N.load().kd_store_add(self._store._h, N.ptr(v), N.ptr(w), N.ptr(t), len(v), 0)
        self._store._chk(rc)

    def _sync(self):
        """Send the queued single adds (in order) to the device."""
        if not self._qv:
            return
        v, w, t = self._qv, self._qw, self._qt
        self._qv, self._qw, self._qt = [], [], None
        weights = None if all(x == 1.0 for x in w) else w
        self._add_many(v, weights, t)

    def _queue(self, value, weight, timestamp):
        timed = timestamp is not None
        if self._qv and (self._qt is not None) != timed:
            self._sync()
        self._qv.append(float(value))
        self._qw.append(float(weight))
        if timed:
            if self._qt is None:
                self._qt = []
            self._qt.append(float(timestamp))
        if len(self._qv) >= _ADD_QUEUE:
            self._sync()

    def add(self, value: float, weight: float = 1.0):
        """One sample, one clock tick (tdigest.mojo:153-161)."""
        _validate_sample(value, weight)
        self._queue(value, weight, None)

    def add_at(self, value: float, timestamp: float, weight: float = 1.0):
        """One sample at `timestamp` (tdigest.mojo:163-175)."""
        _validate_sample(value, weight)
        self._queue(value, weight, timestamp)

    def add_batch(self, values, session: GpuSession | None = None):
        """Fold a batch of unit-weight samples in (tdigest.mojo:177-234); the
        clock advances by len(values) ticks.  Below the crossover (60,000, or
        40,000 with a session) this is the reference's add loop, which stops at
        the first invalid value; from it up the batch path validates first."""
        self._sync()
        v = np.ascontiguousarray(values, dtype=np.float64)
        if v.size == 0:
            return
        crossover = GPU_CROSSOVER if session is None else GPU_CROSSOVER_SESSION
        if v.size < crossover:
            self._add_many(v)
            return
        v = _validate_values(v)
        self._store.ingest(None, v, N.KD_CLOCK_COUNT, 0.0)

    def add_batch_p(self, values):
        """The batch path at any size (the reference's _add_batch_gpu,
        tdigest.mojo:223-234)."""
        self._sync()
        v = _validate_values(values)
        if v.size == 0:
            return
        self._store.ingest(None, v, N.KD_CLOCK_COUNT, 0.0)

    def add_batches(self, batches):
        """A sequence of add_batch_p calls in one (the batch path for every
        batch, as add_batch takes from the crossover up): the results are those
        of the calls one by one, in order, while the sort of each batch overlaps
        the compress of the one before.  `batches` holds numpy arrays (checked
        on the host) or CUDA float64 tensors (read in place, checked on the
        device).  A failing batch raises; the batches before it stay applied."""
        self._sync()
        batches = list(batches)
        if not batches:
            return
        if any(getattr(v, "is_cuda", False) for v in batches):
            if not all(getattr(v, "is_cuda", False) for v in batches):
                raise ValueError("batches must be all host arrays or all CUDA tensors")
            if any(str(v.dtype) != "torch.float64" for v in batches):
                raise TypeError("CUDA batches need float64 values")
            vs = [v.contiguous() for v in batches]
            self._store.ingest_many([None] * len(vs), vs, device=True)
            return
        vs, err = [], None
        for v in batches:
            try:
                vs.append(_validate_values(v))
            except ValueError as e:
                err = e
                break
        self._store.ingest_many([None] * len(vs), vs, device=False)
        if err is not None:
            raise err

    def add_batch_at(self, values, timestamp: float):
        """Batch form of add_at on the batch path: the clock moves to
        `timestamp` once when later, then every sample is inserted."""
        self._sync()
        v = _validate_values(values)
        if v.size == 0:
            return
        self._store.ingest(None, v, N.KD_CLOCK_TIME, float(timestamp))

    def merge(self):
        """Merge the buffered samples (tdigest.mojo:391-439)."""
        self._sync()
        self._store._chk(N.load().kd_store_flush(self._store._h))

    # -- queries --------------------------------------------------------------
    def quantile(self, q: float) -> float:
        if not (0.0 <= q <= 1.0):
            raise ValueError("quantile q must be in [0, 1]")
        self._sync()
        return float(self._store.query(None, [q], False)[0])

    def cdf(self, x: float) -> float:
        self._sync()
        return float(self._store.query(None, [x], True)[0])

    def quantiles(self, qs) -> np.ndarray:
        self._sync()
        return self._store.query(None, qs, False)

    def cdfs(self, xs) -> np.ndarray:
        self._sync()
        return self._store.query(None, xs, True)

    # -- state ----------------------------------------------------------------
    def _state(self):
        self._sync()
        return self._store.digest(0)

    def centroids(self):
        """The merged centroids (buffered samples not included, as len())."""
        _, m, w = self._state()
        return m, w

    def __len__(self) -> int:
        return int(self._state()[0][7])

    def total_weight(self) -> float:
        hdr = self._state()[0]
        if self._decay.is_active():
            return float(hdr[4] * math.exp(-hdr[2]))
        return float(hdr[4])

    def min(self) -> float:
        return float(self._state()[0][5])

    def max(self) -> float:
        return float(self._state()[0][6])

    def state(self) -> dict:
        hdr = self._state()[0]
        keys = ("compression", "lambda", "log_scale", "clock", "stored_total", "min", "max", "count")
        return dict(zip(keys, hdr.tolist()))

    # -- merge / serde --------------------------------------------------------
    def merge_into(self, other: "TDigest"):
        """Fold `other` into this digest (tdigest.mojo:589-623): both merged,
        both rebased to effective weights when decaying, other's centroids
        through this digest's merge pass."""
        if other is self:
            raise ValueError("cannot merge a digest into itself")
        self._sync()
        other._sync()
        rc = N.load().kd_store_merge_into(self._store._h, other._store._h)
        self._store._chk(rc)

    def to_bytes(self) -> bytes:
        self._sync()
        return self._store.to_bytes(0)

    @staticmethod
    def from_bytes(data: bytes, scale: int = K1, session: GpuSession | None = None) -> "TDigest":
        if len(data) == 0 or data[0] != 1:
            raise ValueError("unrecognized digest serialization version")
        if len(data) < 65:
            raise ValueError("truncated digest: not enough bytes for a Float64")
        hdr = np.frombuffer(bytes(data[1:65]), dtype="<f8")
        d = TDigest(compression=float(hdr[0]), scale=scale, decay=Decay.rate(float(hdr[1])),
                    session=session)
        try:
            d._store.from_bytes(0, data)
        except KdError as e:
            if e.code == N.KD_ERANGE:
                raise ValueError(e.message) from None
            raise
        return d


def _validate_sample(value: float, weight: float):
    """TDigest._validate (tdigest.mojo:317-322)."""
    if not math.isfinite(value):
        raise ValueError("value must be finite (got NaN or inf)")
    if not (weight > 0.0) or not math.isfinite(weight):
        raise ValueError("weight must be positive and finite")


def merge_digests(dst: TDigest, parts) -> None:
    """Replace `dst` by the P-path merge of `parts` (gpu_merge_digests); each
    part is merged first, as reading its centroids requires."""
    sess = dst.session
    dst._sync()
    tmp = _Store(len(parts), parts[0].compression, parts[0].scale, parts[0]._decay, sess)
    for i, p in enumerate(parts):
        p.merge()
        hdr, m, w = p._state()
        tmp.set_digest(i, hdr, m, w)
    dst._store.merge_from(tmp, [0, len(parts)], np.arange(len(parts), dtype=np.uint32))


# ---------------------------------------------------------------------------
# Stateless calls over caller-held centroid arrays (the reference's GPU entry
# points, which its host-side digests call with their centroids)
# ---------------------------------------------------------------------------
def _csr(parts):
    offs = np.zeros(len(parts) + 1, np.int64)
    offs[1:] = np.cumsum([len(p) for p in parts])
    cat = np.concatenate([np.asarray(p, np.float64) for p in parts]) if offs[-1] else np.zeros(1)
    return offs, np.ascontiguousarray(cat)


def _split(offs, m, w):
    return ([m[offs[k]:offs[k + 1]].copy() for k in range(len(offs) - 1)],
            [w[offs[k]:offs[k + 1]].copy() for k in range(len(offs) - 1)])


def gpu_grouped_compress_weighted(keys, values, new_weights, prior_means, prior_weights,
                                  num_keys: int, compression: float, scale: int = K2,
                                  session: GpuSession | None = None):
    """gpu_grouped_compress_weighted (gpu/grouped.mojo:415-643): per key, the
    P-path compress of its prior centroids followed by its new samples (weight
    new_weights[k]).  Returns (means per key, weights per key, mins, maxs), the
    ranges over each key's new samples only, like GroupedResult."""
    s = session or default_session()
    k = np.ascontiguousarray(keys, dtype=np.uint32)
    v = np.ascontiguousarray(values, dtype=np.float64)
    nw = None if new_weights is None else np.ascontiguousarray(new_weights, dtype=np.float64)
    po, pm = _csr(prior_means)
    _, pw = _csr(prior_weights)
    out_off = np.zeros(num_keys + 1, np.int64)
    mins = np.zeros(num_keys)
    maxs = np.zeros(num_keys)
    cap = int(po[-1] + len(v))
    om = np.empty(max(cap, 1))
    ow = np.empty(max(cap, 1))
    out_n = ctypes.c_int64(0)
    rc = N.load().kd_grouped_compress(s.handle, scale, compression, num_keys, N.ptr(k), N.ptr(v),
                                      len(v), N.ptr(nw) if nw is not None else None, N.ptr(po),
                                      N.ptr(pm), N.ptr(pw), N.ptr(out_off), N.ptr(om), N.ptr(ow),
                                      cap, ctypes.byref(out_n), N.ptr(mins), N.ptr(maxs))
    _check(s.handle, rc)
    means, weights = _split(out_off, om, ow)
    return means, weights, mins, maxs


def _digest_query(fn, means, weights, mins, maxs, ids, xs, session):
    s = session or default_session()
    offs, m = _csr(means)
    _, w = _csr(weights)
    mn = np.ascontiguousarray(mins, dtype=np.float64)
    mx = np.ascontiguousarray(maxs, dtype=np.float64)
    x = np.ascontiguousarray(xs, dtype=np.float64)
    k = None if ids is None else np.ascontiguousarray(ids, dtype=np.uint32)
    out = np.empty(len(x))
    rc = fn(s.handle, N.ptr(offs), len(means), N.ptr(m), N.ptr(w), N.ptr(mn), N.ptr(mx),
            N.ptr(k) if k is not None else None, N.ptr(x), len(x), N.ptr(out), 0)
    _check(s.handle, rc)
    return out


def gpu_quantile(means, weights, qs, min_v: float, max_v: float,
                 session: GpuSession | None = None) -> np.ndarray:
    """gpu_quantile (gpu/query.mojo:320-330): every q against one digest."""
    return _digest_query(N.load().kd_quantile, [means], [weights], [min_v], [max_v], None, qs, session)


def gpu_cdf(means, weights, xs, min_v: float, max_v: float,
            session: GpuSession | None = None) -> np.ndarray:
    """gpu_cdf (gpu/query.mojo:333-342): every x against one digest."""
    return _digest_query(N.load().kd_cdf, [means], [weights], [min_v], [max_v], None, xs, session)


def gpu_quantile_many(means, weights, mins, maxs, ids, qs, session: GpuSession | None = None):
    """gpu_quantile for many caller-held digests in one call: query i against
    digest ids[i]."""
    return _digest_query(N.load().kd_quantile, means, weights, mins, maxs, ids, qs, session)


def gpu_cdf_many(means, weights, mins, maxs, ids, xs, session: GpuSession | None = None):
    return _digest_query(N.load().kd_cdf, means, weights, mins, maxs, ids, xs, session)


def gpu_merge_digests(part_means, part_weights, compression: float, scale: int = K2,
                      group_offsets=None, session: GpuSession | None = None):
    """gpu_merge_digests (gpu/query.mojo:348-369): the parts' centroids
    concatenated in order and compressed once.  With group_offsets, each group
    of consecutive parts is merged on its own and a list per group returned."""
    s = session or default_session()
    po, m = _csr(part_means)
    _, w = _csr(part_weights)
    go = np.array([0, len(part_means)] if group_offsets is None else group_offsets, np.int64)
    ng = len(go) - 1
    out_off = np.zeros(ng + 1, np.int64)
    cap = max(int(po[-1]), 1)
    om = np.empty(cap)
    ow = np.empty(cap)
    out_n = ctypes.c_int64(0)
    rc = N.load().kd_merge(s.handle, scale, compression, N.ptr(po), len(part_means), N.ptr(m),
                           N.ptr(w), N.ptr(go), ng, None, N.ptr(out_off), N.ptr(om), N.ptr(ow),
                           cap, ctypes.byref(out_n))
    _check(s.handle, rc)
    means, weights = _split(out_off, om, ow)
    if group_offsets is None:
        return means[0], weights[0]
    return means, weights


class GroupedTDigest:
    """num_keys independent digests updated together (grouped.mojo:30-190)."""

    def __init__(self, num_keys: int, compression: float = 100.0, decay: Decay | None = None,
                 scale: int = K2, session: GpuSession | None = None):
        self.num_keys = int(num_keys)
        self.compression = float(compression)
        self.decay = decay if decay is not None else Decay.none()
        self.scale = scale
        self._store = _Store(num_keys, compression, scale, self.decay, session)

    @property
    def session(self) -> GpuSession:
        return self._store.session

    def _check_keys(self, keys) -> np.ndarray:
        k = np.asarray(keys)
        if k.size and (k.min() < 0 or k.max() >= self.num_keys):
            raise IndexError("key out of range [0, num_keys)")
        return np.ascontiguousarray(k, dtype=np.uint32)

    def add_batch(self, keys, values):
        """Fold (key, value) samples into their per-key digests; every key's
        clock advances by its own sample count.  Validated before mutation."""
        k = np.asarray(keys)
        v = np.asarray(values)
        if len(k) != len(v):
            raise ValueError("keys and values must have equal length")
        if len(v) == 0:
            return
        k = self._check_keys(k)
        v = _validate_values(v)
        self._store.ingest(k, v, N.KD_CLOCK_COUNT, 0.0)

    def add_batch_at(self, keys, values, timestamp: float):
        k = np.asarray(keys)
        v = np.asarray(values)
        if len(k) != len(v):
            raise ValueError("keys and values must have equal length")
        if len(v) == 0:
            return
        k = self._check_keys(k)
        v = _validate_values(v)
        self._store.ingest(k, v, N.KD_CLOCK_TIME, float(timestamp))

    def add_batches(self, batches):
        """A sequence of add_batch calls in one: the results are those of the
        calls one by one, in order, while the sort of each batch overlaps the
        compress of the one before.  `batches` holds (keys, values) pairs,
        either numpy arrays (checked on the host) or CUDA tensors (uint32 or
        int32 keys, float64 values; read in place, checked on the device).  A
        failing batch raises; the batches before it stay applied."""
        batches = list(batches)
        if not batches:
            return
        dev = [getattr(v, "is_cuda", False) for _, v in batches]
        if any(dev):
            if not all(dev) or not all(getattr(k, "is_cuda", False) for k, _ in batches):
                raise ValueError("batches must be all host arrays or all CUDA tensors")
            ks, vs = [], []
            for k, v in batches:
                if len(k) != len(v):
                    raise ValueError("keys and values must have equal length")
                if str(v.dtype) != "torch.float64" or str(k.dtype) not in ("torch.int32", "torch.uint32"):
                    raise TypeError("CUDA batches need int32/uint32 keys and float64 values")
                ks.append(k.contiguous())
                vs.append(v.contiguous())
            self._store.ingest_many(ks, vs, device=True)
            return
        ks, vs, err = [], [], None
        for k, v in batches:  # host checks, in batch order: apply what precedes a bad batch
            try:
                k = np.asarray(k)
                v = np.asarray(v)
                if len(k) != len(v):
                    raise ValueError("keys and values must have equal length")
                ks.append(self._check_keys(k))
                vs.append(_validate_values(v))
            except (ValueError, IndexError) as e:
                err = e
                break
        self._store.ingest_many(ks, vs, device=False)
        if err is not None:
            raise err

    def _key(self, key: int) -> int:
        if key < 0 or key >= self.num_keys:
            raise IndexError("key out of range [0, num_keys)")
        return int(key)

    def quantile(self, key: int, q: float) -> float:
        self._key(key)
        if not (0.0 <= q <= 1.0):
            raise ValueError("quantile q must be in [0, 1]")
        return float(self._store.query([key], [q], False)[0])

    def cdf(self, key: int, x: float) -> float:
        self._key(key)
        return float(self._store.query([key], [x], True)[0])

    def quantiles(self, keys, qs) -> np.ndarray:
        return self._store.query(self._check_keys(keys), qs, False)

    def cdfs(self, keys, xs) -> np.ndarray:
        return self._store.query(self._check_keys(keys), xs, True)

    def query_batch(self, qkeys, qs, ckeys, xs):
        """quantiles(qkeys, qs) and cdfs(ckeys, xs) in one kernel launch.
        Host arrays return numpy arrays; CUDA tensors (uint32 / int32 keys,
        float64 values) are read and written in place, returning two CUDA
        tensors, and a repeated call with the same tensors replays a captured
        CUDA graph."""
        L = N.load()
        h = self._store._h
        if getattr(qs, "is_cuda", False):
            import torch

            qo = torch.empty_like(qs)
            co = torch.empty_like(xs)
            torch.cuda.current_stream(qs.device).synchronize()
            rc = L.kd_store_query_batch(h, qkeys.data_ptr(), qs.data_ptr(), qs.numel(), qo.data_ptr(),
                                        ckeys.data_ptr(), xs.data_ptr(), xs.numel(), co.data_ptr(),
                                        N.KD_PTR_DEVICE)
            _check(self.session.handle, rc)
            return qo, co
        qk = self._check_keys(qkeys)
        ck = self._check_keys(ckeys)
        q = np.ascontiguousarray(qs, dtype=np.float64)
        x = np.ascontiguousarray(xs, dtype=np.float64)
        qo = np.empty(len(q))
        co = np.empty(len(x))
        rc = L.kd_store_query_batch(h, N.ptr(qk), N.ptr(q), len(q), N.ptr(qo), N.ptr(ck), N.ptr(x),
                                    len(x), N.ptr(co), 0)
        _check(self.session.handle, rc)
        return qo, co

    def to_bytes(self, key: int) -> bytes:
        return self._store.to_bytes(self._key(key))

    def from_bytes(self, key: int, data: bytes):
        self._store.from_bytes(self._key(key), data)

    def centroid_count(self, key: int) -> int:
        return int(self._store.digest(self._key(key))[0][7])

    def centroid_counts(self) -> np.ndarray:
        out = np.empty(self.num_keys, np.int32)
        self._store._chk(N.load().kd_store_counts(self._store._h, N.ptr(out), 0))
        return out

    def centroids(self, key: int):
        _, m, w = self._store.digest(self._key(key))
        return m, w

    def state(self, key: int) -> dict:
        hdr = self._store.digest(self._key(key))[0]
        keys = ("compression", "lambda", "log_scale", "clock", "stored_total", "min", "max", "count")
        return dict(zip(keys, hdr.tolist()))

    def total_weight(self, key: int) -> float:
        hdr = self._store.digest(self._key(key))[0]
        if self.decay.is_active():
            return float(hdr[4] * math.exp(-hdr[2]))
        return float(hdr[4])

    # -- checkpoint ------------------------------------------------------------
    def export(self, keys=None):
        """to_bytes of many keys at once: (records as one bytes buffer, int64
        offsets with one entry more than keys)."""
        k = None if keys is None else np.ascontiguousarray(keys, dtype=np.uint32)
        nk = self.num_keys if k is None else len(k)
        offs = np.zeros(nk + 1, dtype=np.int64)
        L = N.load()
        h = self._store._h
        self._store._chk(L.kd_store_export(h, N.ptr(k), nk, None, 0, N.ptr(offs), 0))
        buf = np.empty(int(offs[-1]), dtype=np.uint8)
        self._store._chk(L.kd_store_export(h, N.ptr(k), nk, N.ptr(buf), len(buf), N.ptr(offs), 0))
        return buf.tobytes(), offs

    def import_records(self, data: bytes, offsets, keys=None):
        """from_bytes of many keys; every record is validated before any key changes."""
        buf = np.frombuffer(data, dtype=np.uint8)
        offs = np.ascontiguousarray(offsets, dtype=np.int64)
        k = None if keys is None else np.ascontiguousarray(keys, dtype=np.uint32)
        nk = len(offs) - 1
        self._store._chk(N.load().kd_store_import(self._store._h, N.ptr(k), nk, N.ptr(buf),
                                                  N.ptr(offs), 0))

    _SNAP_MAGIC = b"KDGB300S"

    def snapshot(self, path: str):
        """Write every key's record (the to_bytes wire format) with the store's
        shape to a file."""
        data, offs = self.export()
        head = np.array([self.num_keys, self.scale], dtype=np.int64)
        par = np.array([self.compression, self.decay.rate_lambda], dtype=np.float64)
        with open(path, "wb") as f:
            f.write(self._SNAP_MAGIC)
            f.write(head.tobytes())
            f.write(par.tobytes())
            f.write(offs.tobytes())
            f.write(data)

    @classmethod
    def restore(cls, path: str, session: GpuSession | None = None) -> "GroupedTDigest":
        """A store rebuilt from a snapshot file."""
        with open(path, "rb") as f:
            if f.read(8) != cls._SNAP_MAGIC:
                raise ValueError("not a grouped digest snapshot")
            num_keys, scale = np.frombuffer(f.read(16), dtype=np.int64)
            compression, lam = np.frombuffer(f.read(16), dtype=np.float64)
            offs = np.frombuffer(f.read(8 * (int(num_keys) + 1)), dtype=np.int64)
            data = f.read(int(offs[-1]))
        g = cls(int(num_keys), float(compression), decay=Decay.rate(float(lam)), scale=int(scale),
                session=session)
        g.import_records(data, offs)
        return g

    def merge_groups(self, src: "GroupedTDigest", group_offsets, parts):
        """Batched merge_into: key g of this store becomes the P-path merge of
        src keys parts[group_offsets[g]:group_offsets[g+1]] (in order)."""
        self._store.merge_from(src._store, group_offsets, parts)


class KeyDictionary:
    """Device-resident map from arbitrary 64-bit keys to dense ids [0, capacity)
    (no reference counterpart: GroupedTDigest.add_batch takes dense ids,
    grouped.mojo:60-63).  Ids are stable once given; keys first seen in the
    same call get theirs in an unspecified order.  2**64 - 1 is reserved.

    ``map`` / ``lookup`` take a host array (returning a numpy uint32 array) or a
    CUDA tensor with ``data_ptr()`` (returning a CUDA int32 tensor of the ids'
    bit patterns, ready for a device-pointer ingest)."""

    def __init__(self, capacity: int, session: GpuSession | None = None):
        self.session = session or default_session()
        self.capacity = int(capacity)
        h = ctypes.c_void_p()
        rc = N.load().kd_keymap_create(self.session.handle, self.capacity, ctypes.byref(h))
        _check(self.session.handle, rc)
        self._h = h.value

    def _run(self, fn, keys):
        if hasattr(keys, "data_ptr") and getattr(keys, "is_cuda", False):
            import torch

            k = keys.contiguous()
            if k.element_size() != 8:
                raise ValueError("device keys must be a 64-bit integer tensor")
            out = torch.empty(k.numel(), dtype=torch.int32, device=k.device)
            torch.cuda.current_stream(k.device).synchronize()
            rc = fn(self._h, k.data_ptr(), k.numel(), out.data_ptr(), N.KD_PTR_DEVICE)
            _check(self.session.handle, rc)
            return out
        k = np.ascontiguousarray(np.asarray(keys).astype(np.uint64, copy=False))
        out = np.empty(len(k), np.uint32)
        rc = fn(self._h, N.ptr(k), len(k), N.ptr(out), 0)
        _check(self.session.handle, rc)
        return out

    def map(self, keys):
        """Ids of keys, inserting unknown keys (KdError when the map is full)."""
        return self._run(N.load().kd_keymap_map, keys)

    def lookup(self, keys):
        """Ids of keys; unknown keys give 2**32 - 1 (-1 in a device tensor)."""
        return self._run(N.load().kd_keymap_lookup, keys)

    def __len__(self) -> int:
        return int(N.load().kd_keymap_size(self._h))

    def close(self):
        if getattr(self, "_h", None):
            N.load().kd_keymap_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            if not sys.is_finalizing():  # process exit releases everything
                self.close()
        except Exception:
            pass


class Server:
    """Serving loop over a resident digest store (no reference counterpart):
    requests with non-decreasing timestamps are batched per window of the
    timestamp axis by a native worker thread.  A window's queries see the store
    before the window's ingests; the window's ingests are one grouped batch.
    The store's session belongs to the server until close()."""

    def __init__(self, digests, window: float = 1e-3, budget_bytes: int = 0):
        self._digests = digests
        store = digests._store
        self.session = store.session
        h = ctypes.c_void_p()
        rc = N.load().kd_server_create(store._h, float(window), int(budget_bytes), ctypes.byref(h))
        _check(self.session.handle, rc)
        self._h = h.value
        self._outs = {}  # ticket -> output array kept alive until waited

    def _submit(self, kind, timestamp, keys, vals, out=None):
        v = np.ascontiguousarray(vals, dtype=np.float64)
        k = None if keys is None else np.ascontiguousarray(keys, dtype=np.uint32)
        if k is not None and len(k) != len(v):
            raise ValueError("keys and values must have equal length")
        t = ctypes.c_int64(0)
        rc = N.load().kd_server_submit(self._h, kind, float(timestamp), N.ptr(k), N.ptr(v), len(v),
                                       N.ptr(out), ctypes.byref(t))
        if rc:
            raise KdError(rc, "request rejected (invalid input, closed window or over budget)")
        return t.value

    def submit_ingest(self, timestamp: float, keys, values) -> int:
        return self._submit(N.KD_REQ_INGEST, timestamp, keys, values)

    def submit_quantiles(self, timestamp: float, keys, qs) -> int:
        out = np.empty(len(qs))
        t = self._submit(N.KD_REQ_QUANTILE, timestamp, keys, qs, out)
        self._outs[t] = out
        return t

    def submit_cdfs(self, timestamp: float, keys, xs) -> int:
        out = np.empty(len(xs))
        t = self._submit(N.KD_REQ_CDF, timestamp, keys, xs, out)
        self._outs[t] = out
        return t

    def advance(self, now: float):
        N.load().kd_server_advance(self._h, float(now))

    def wait(self, ticket: int, timeout: float = -1.0):
        """(status, outputs or None) of a request."""
        st = ctypes.c_int(0)
        rc = N.load().kd_server_wait(self._h, int(ticket), float(timeout), ctypes.byref(st))
        if rc:
            raise KdError(rc, "wait failed (unknown ticket or timeout)")
        return st.value, self._outs.pop(ticket, None)

    def flush(self):
        N.load().kd_server_flush(self._h)

    def latency(self, ticket: int) -> float:
        """Submit-to-completion seconds of a completed request not yet waited
        for (-1 while pending)."""
        sec = ctypes.c_double(0.0)
        rc = N.load().kd_server_latency(self._h, int(ticket), ctypes.byref(sec))
        if rc:
            raise KdError(rc, "unknown ticket")
        return sec.value

    def memory(self) -> dict:
        """Device bytes counted against the admission budget (now, peak), the
        budget, and the device memory measured after the last window."""
        a, b, c, d = (ctypes.c_size_t(0) for _ in range(4))
        N.load().kd_server_memory(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                  ctypes.byref(d))
        return {"in_use_bytes": a.value, "peak_bytes": b.value, "budget_bytes": c.value,
                "measured_bytes": d.value}

    def stats(self) -> dict:
        lat = np.zeros(3)
        done = ctypes.c_int64(0)
        wins = ctypes.c_int64(0)
        busy = ctypes.c_double(0.0)
        groups = ctypes.c_int64(0)
        grouped = ctypes.c_int64(0)
        gmax = ctypes.c_double(0.0)
        slow = ctypes.c_int64(0)
        stage = ctypes.c_double(0.0)
        L = N.load()
        L.kd_server_stats(self._h, N.ptr(lat), ctypes.byref(done), ctypes.byref(wins),
                          ctypes.byref(busy))
        L.kd_server_groups(self._h, ctypes.byref(groups), ctypes.byref(grouped), ctypes.byref(gmax),
                           ctypes.byref(slow), ctypes.byref(stage))
        return {"p50_s": lat[0], "p99_s": lat[1], "p999_s": lat[2], "completed": done.value,
                "windows": wins.value, "busy_s": busy.value, "groups": groups.value,
                "windows_grouped": grouped.value, "max_group_s": gmax.value,
                "slow_groups": slow.value, "stage_s": stage.value}

    def close(self):
        if getattr(self, "_h", None):
            N.load().kd_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            if not sys.is_finalizing():  # process exit releases everything
                self.close()
        except Exception:
            pass
