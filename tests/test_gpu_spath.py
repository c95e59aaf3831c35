"""Single-sample path of a one-key store against the oracle's add loop.

The reference runs TDigest.add / add_at, and add_batch below its GPU crossover,
as a sequential loop: buffer, then a merge pass when the buffer fills
(src/kdigest/tdigest.mojo:153-221, 324-458); merge_into is the same pass over
the other digest's centroids (:589-623).  The oracle restates that loop in C
(pinned to the reference's own known answers in test_oracle.py), so every
check here is bit-exact: header, centroids, queries and bytes."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QS = [0.0, 1e-4, 0.001, 0.01, 0.1, 0.25, 0.5, 0.75, 0.9, 0.99, 0.999, 1.0]


def _same(d, od):
    """Header and merged centroids equal bit for bit (buffer not merged)."""
    st, ost = d.state(), od.state()
    for f in ("log_scale", "clock", "stored_total", "min", "max", "count"):
        a, b = st[f], ost[f]
        assert a == b or (math.isnan(a) and math.isnan(b)), (f, a, b)
        assert math.copysign(1.0, a) == math.copysign(1.0, b), f
    m, w = d.centroids()
    om, ow = od.centroids()
    assert np.array_equal(m.view(np.uint64), om.view(np.uint64))
    assert np.array_equal(w.view(np.uint64), ow.view(np.uint64))


def _same_queries(d, od, xs=(-3.0, -1.0, 0.0, 0.5, 1.0, 3.0)):
    for q in QS:
        assert d.quantile(q) == od.quantile(q), q
    for x in xs:
        assert d.cdf(x) == od.cdf(x), x
    _same(d, od)  # both merged by the queries


@pytest.mark.parametrize("scale", [0, 1, 2, 3])
@pytest.mark.parametrize("compression", [100.0, 37.5, 200.0])
def test_add_batch_below_crossover_is_the_add_loop(kd, oracle, scale, compression):
    d = kd.TDigest(compression, scale)
    od = oracle.Digest(scale, compression, 0.0)
    rng = np.random.default_rng(scale * 1000 + int(compression))
    for n in (1, 2, 499, 500, 501, 4096, 4096, 12345, 7):
        v = rng.standard_normal(n)
        d.add_batch(v)
        od.add_many(v)
        _same(d, od)
    _same_queries(d, od)
    assert d.to_bytes() == od.to_bytes()


def test_config1_stream(kd, oracle):
    """1e6 N(0,1) samples in batches of 4096 into one K1 digest, compression 100."""
    d = kd.TDigest(100.0, kd.K1)
    od = oracle.Digest(oracle.K1, 100.0, 0.0)
    rng = np.random.default_rng(0)
    vals = rng.standard_normal(1_000_000)
    for b in range(0, len(vals), 4096):
        d.add_batch(vals[b:b + 4096])
        od.add_many(vals[b:b + 4096])
    _same(d, od)
    _same_queries(d, od)


@pytest.mark.parametrize("half_life", [50.0, 3000.0])
def test_count_decay_renormalise_and_prune(kd, oracle, half_life):
    """lambda * count passes 400 inside a batch: the loop renormalises between
    two samples; prune drops decayed centroids."""
    dec = kd.Decay.half_life(half_life)
    d = kd.TDigest(100.0, kd.K2, decay=dec)
    od = oracle.Digest(oracle.K2, 100.0, dec.rate_lambda)
    rng = np.random.default_rng(7)
    for n in (20000, 20000, 333, 20000):
        v = rng.lognormal(0, 1, n)
        d.add_batch(v)
        od.add_many(v)
        _same(d, od)
    _same_queries(d, od, xs=(0.1, 0.5, 1.0, 2.0, 10.0))


@pytest.mark.parametrize("scale", [0, 1])
def test_count_decay_unclamped_scales(kd, oracle, scale):
    """K0 and K1 do not clamp q (scale.mojo:91-118): with decayed weights the
    chain's sum can round above the stored total, so K1 meets asin just above
    1 (NaN: the candidate does not fit) at the end of a merge pass, where the
    parallel sweep's speculation assumed the end value; the pass then resumes
    the reference loop at the overturned candidate.  Config 1's stream with a
    10^5-sample half-life, a quarter of it."""
    dec = kd.Decay.half_life(1e5)
    d = kd.TDigest(100.0, scale, decay=dec)
    od = oracle.Digest(scale, 100.0, dec.rate_lambda)
    rng = np.random.default_rng(31 + scale)
    vals = rng.standard_normal(250_000)
    for b in range(0, len(vals), 4096):
        d.add_batch(vals[b:b + 4096])
        od.add_many(vals[b:b + 4096])
        if b % (16 * 4096) == 0:
            _same(d, od)
    _same(d, od)
    _same_queries(d, od)


def test_add_at_weighted_and_time_decay(kd, oracle):
    dec = kd.Decay.half_life(10.0)
    d = kd.TDigest(100.0, kd.K3, decay=dec)
    od = oracle.Digest(oracle.K3, 100.0, dec.rate_lambda)
    rng = np.random.default_rng(8)
    t = 0.0
    for i in range(9000):
        t += float(rng.exponential(0.5)) if i % 7 else 0.0  # equal stamps too
        ts = t - 1.0 if i % 97 == 0 else t  # an earlier stamp does not move the clock
        v = float(rng.standard_normal())
        w = float(rng.uniform(0.1, 3.0))
        d.add_at(v, ts, w)
        od.add_at(v, ts, w)
    _same(d, od)
    _same_queries(d, od)


def test_weighted_adds_without_decay(kd, oracle):
    """Non-integral weights: the sweep's chain is speculated, then re-checked."""
    d = kd.TDigest(100.0, kd.K1)
    od = oracle.Digest(oracle.K1, 100.0, 0.0)
    rng = np.random.default_rng(9)
    for i in range(6000):
        v, w = float(rng.standard_normal()), float(rng.uniform(0.01, 5.0))
        d.add(v, w)
        od.add(v, w)
    _same(d, od)
    _same_queries(d, od)


@pytest.mark.parametrize("kind", ["integers", "identical", "zeros"])
def test_ties_and_signed_zeros(kd, oracle, kind):
    """Exact mean ties coalesce across the k limit (tdigest.mojo:431)."""
    rng = np.random.default_rng(10)
    if kind == "integers":
        v = rng.integers(0, 7, 30000).astype(np.float64)
    elif kind == "identical":
        v = np.full(30000, 2.5)
    else:
        v = np.where(rng.random(30000) < 0.5, -0.0, 0.0)
        v[::11] = rng.standard_normal(len(v[::11]))
    for scale in (1, 2):
        d = kd.TDigest(100.0, scale)
        od = oracle.Digest(scale, 100.0, 0.0)
        for b in range(0, len(v), 5000):
            d.add_batch(v[b:b + 5000])
            od.add_many(v[b:b + 5000])
        _same(d, od)
        _same_queries(d, od)


def test_large_compression_uses_global_scratch(kd, oracle):
    d = kd.TDigest(400.0, kd.K2)
    od = oracle.Digest(oracle.K2, 400.0, 0.0)
    rng = np.random.default_rng(11)
    for _ in range(5):
        v = rng.standard_normal(9000)
        d.add_batch(v)
        od.add_many(v)
    _same(d, od)
    _same_queries(d, od)


def test_batch_path_folds_the_buffer(kd, oracle):
    """Small batches leave a buffer; a batch above the crossover compresses
    centroids ++ buffer ++ batch (tdigest.mojo:236-315)."""
    dec = kd.Decay.half_life(1e5)
    d = kd.TDigest(200.0, kd.K2, decay=dec)
    od = oracle.Digest(oracle.K2, 200.0, dec.rate_lambda)
    rng = np.random.default_rng(12)
    for n, big in ((777, False), (1500, False), (70000, True), (123, False), (65000, True),
                   (4096, False)):
        v = rng.lognormal(0, 1.5, n)
        d.add_batch(v)
        if big:
            od.add_batch_p(v)
        else:
            od.add_many(v)
        _same(d, od)
    _same_queries(d, od, xs=(0.2, 1.0, 5.0))


def test_merge_into(kd, oracle):
    rng = np.random.default_rng(13)
    for lam in (0.0, 1e-3):
        dec = kd.Decay.rate(lam)
        a, b = kd.TDigest(100.0, kd.K1, decay=dec), kd.TDigest(100.0, kd.K1, decay=dec)
        oa, ob = oracle.Digest(oracle.K1, 100.0, lam), oracle.Digest(oracle.K1, 100.0, lam)
        va, vb = rng.standard_normal(3210), rng.standard_normal(2345) + 1.0
        a.add_batch(va)
        oa.add_many(va)
        b.add_batch(vb)
        ob.add_many(vb)
        a.merge_into(b)
        oa.merge_into(ob)
        _same(a, oa)
        _same(b, ob)  # merged and renormalised in place
        _same_queries(a, oa)
    e = kd.TDigest(100.0, kd.K1)
    with pytest.raises(ValueError):
        e.merge_into(e)
    a.merge_into(kd.TDigest(100.0, kd.K1))  # an empty digest changes nothing
    _same(a, oa)


def test_invalid_sample_stops_the_loop(kd, oracle):
    d = kd.TDigest(100.0, kd.K1)
    od = oracle.Digest(oracle.K1, 100.0, 0.0)
    v = np.arange(1000, dtype=np.float64)
    v[700] = np.nan
    with pytest.raises(ValueError):
        d.add_batch(v)
    with pytest.raises(Exception):
        od.add_many(v)
    _same(d, od)  # the first 700 samples stay applied, as in the loop
    with pytest.raises(ValueError):
        d.add(float("inf"))
    with pytest.raises(ValueError):
        d.add(1.0, 0.0)
    _same(d, od)


def test_pending_buffer_reads(kd, oracle):
    """len() and total_weight() see the buffer unmerged; queries, to_bytes and
    export merge it first."""
    d = kd.TDigest(100.0, kd.K2)
    od = oracle.Digest(oracle.K2, 100.0, 0.0)
    rng = np.random.default_rng(14)
    v = rng.standard_normal(1234)
    d.add_batch(v)
    od.add_many(v)
    assert len(d) == len(od)
    assert d.total_weight() == od.total_weight()
    assert d.min() == float(v.min()) and d.max() == float(v.max())
    assert d.to_bytes() == od.to_bytes()
    d.add(0.25)
    od.add(0.25)
    assert d.quantile(0.5) == od.quantile(0.5)
    r = kd.TDigest.from_bytes(d.to_bytes(), scale=kd.K2)
    orr = oracle.Digest.from_bytes(od.to_bytes(), oracle.K2)
    w = rng.standard_normal(900)
    r.add_batch(w)
    orr.add_many(w)
    _same(r, orr)
    big = rng.standard_normal(61000)
    r.add_batch(big)
    orr.add_batch_p(big)
    _same(r, orr)


@pytest.mark.parametrize("scale", [2, 3])
def test_long_streams_k2_k3(kd, oracle, scale):
    """Normalisers that grow with the total (K2, K3) over 600,000 samples."""
    d = kd.TDigest(150.0, scale)
    od = oracle.Digest(scale, 150.0, 0.0)
    rng = np.random.default_rng(20 + scale)
    v = rng.lognormal(0, 2.0, 600_000)
    for b in range(0, len(v), 5000):
        d.add_batch(v[b:b + 5000])
        od.add_many(v[b:b + 5000])
    _same(d, od)
    _same_queries(d, od, xs=(0.01, 0.5, 1.0, 4.0, 100.0))


def test_tiny_compression_merges_every_sample(kd, oracle):
    """int(compression) * 5 below 1: the buffer limit is one sample."""
    d = kd.TDigest(0.15, kd.K1)
    od = oracle.Digest(oracle.K1, 0.15, 0.0)
    rng = np.random.default_rng(30)
    v = rng.standard_normal(300)
    d.add_batch(v)
    od.add_many(v)
    _same(d, od)
    _same_queries(d, od)


def test_server_over_single_digest_merges_the_buffer(kd, oracle):
    """A serving loop takes the store over: buffered samples are merged first."""
    d = kd.TDigest(100.0, kd.K2)
    od = oracle.Digest(oracle.K2, 100.0, 0.0)
    v = np.random.default_rng(31).standard_normal(777)
    d.add_batch(v)
    od.add_many(v)
    srv = kd.Server(d, window=1e-3)
    srv.close()
    od.merge()
    _same(d, od)


def test_one_call_many_merges_below_crossover(kd, oracle):
    """59,999 samples (just below the crossover) in one call: 119 merge passes."""
    d = kd.TDigest(100.0, kd.K3)
    od = oracle.Digest(oracle.K3, 100.0, 0.0)
    v = np.random.default_rng(40).standard_cauchy(59_999)
    d.add_batch(v)
    od.add_many(v)
    _same(d, od)
    _same_queries(d, od, xs=(-10.0, 0.0, 0.1, 10.0))


def test_add_at_odd_timestamps_and_renormalisation(kd, oracle):
    """NaN stamps never move the clock; a long gap renormalises (time decay)."""
    dec = kd.Decay.rate(0.9)
    d = kd.TDigest(50.0, kd.K2, decay=dec)
    od = oracle.Digest(oracle.K2, 50.0, dec.rate_lambda)
    rng = np.random.default_rng(41)
    t = 0.0
    for i in range(5000):
        if i == 2500:
            t += 600.0  # lambda * gap > 400: renormalise inside the loop
        elif i % 50 == 7:
            ts = float("nan")
        else:
            t += float(rng.exponential(0.01))
        ts = float("nan") if i % 50 == 7 else t
        v = float(rng.normal())
        d.add_at(v, ts)
        od.add_at(v, ts)
    _same(d, od)
    _same_queries(d, od)


def test_time_clock_without_decay(kd, oracle):
    d = kd.TDigest(100.0, kd.K1)
    od = oracle.Digest(oracle.K1, 100.0, 0.0)
    rng = np.random.default_rng(42)
    ts = np.cumsum(rng.exponential(1.0, 3000))
    ts[::17] = ts[::17] - 5.0  # late stamps
    for v, t in zip(rng.normal(size=3000), ts):
        d.add_at(float(v), float(t))
        od.add_at(float(v), float(t))
    _same(d, od)


def test_restore_then_single_samples(kd, oracle):
    """A digest restored from bytes continues on the single-sample path."""
    rng = np.random.default_rng(43)
    od = oracle.Digest(oracle.K1, 100.0, 0.0)
    od.add_many(rng.normal(size=7000))
    d = kd.TDigest.from_bytes(od.to_bytes(), scale=kd.K1)
    v = rng.normal(size=3333)
    d.add_batch(v)
    od.add_many(v)
    _same(d, od)
    _same_queries(d, od)
