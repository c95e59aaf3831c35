"""The CPU oracle pinned against the reference's own known-answer tests.

The reference (Mojo, osx-arm64 only) cannot run here, and it stores no golden
vectors; its tests pin behaviour through known answers and accuracy bands on
deterministic generators.  Each test below restates one of them against the
oracle (file:line of the reference test in each docstring).
"""
import math

import numpy as np
import pytest

from oracle import pyoracle as o


# ---------------------------------------------------------------------------
# Deterministic generators of the reference tests
# ---------------------------------------------------------------------------
class XorShift:
    """xorshift64* -> (0, 1) (test/test_gpu_add_batch.mojo:58-82)."""

    def __init__(self, seed):
        self.s = seed & 0xFFFFFFFFFFFFFFFF

    def unit(self):
        s = self.s
        s ^= s >> 12
        s ^= (s << 25) & 0xFFFFFFFFFFFFFFFF
        s ^= s >> 27
        self.s = s
        x = ((s * 0x2545F4914F6CDD1D) & 0xFFFFFFFFFFFFFFFF) >> 11
        return (float(x) + 0.5) / float(1 << 53)

    def normal(self):
        u1, u2 = self.unit(), self.unit()
        return math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)


def _data(kind, n, seed):
    r = XorShift(seed)
    if kind == "uniform":
        return np.array([r.unit() for _ in range(n)])
    if kind == "normal":
        return np.array([r.normal() for _ in range(n)])
    if kind == "exponential":
        return np.array([-math.log(r.unit()) for _ in range(n)])
    return np.array([r.unit() ** (-1.0 / 2.5) for _ in range(n)])


def _truth(data, qs):
    s = np.sort(data)
    n = len(s)
    return [s[min(max(int(q * n), 0), n - 1)] for q in qs]


# ---------------------------------------------------------------------------
# Shared FP64 scale arithmetic
# ---------------------------------------------------------------------------
def test_kscale_math_accuracy():
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 120
    rng = np.random.default_rng(1)
    for x in np.exp(rng.uniform(-700, 700, 3000)):
        y = o.log(float(x))
        assert abs((mp.mpf(y) - mp.log(mp.mpf(float(x)))) / mp.log(mp.mpf(float(x)))) < 4 * 2.0 ** -52 or abs(float(x) - 1) < 1e-3
    for x in rng.uniform(-700, 700, 3000):
        r = mp.exp(mp.mpf(float(x)))
        assert abs((mp.mpf(o.exp(float(x))) - r) / r) < 4 * 2.0 ** -52
    for x in np.concatenate([rng.uniform(-1, 1, 3000), 1 - 10 ** rng.uniform(-16, -1, 500)]):
        r = mp.asin(mp.mpf(float(x)))
        if r != 0:
            assert abs((mp.mpf(o.asin(float(x))) - r) / r) < 8 * 2.0 ** -52


def test_scale_functions_known_values():
    """scale.mojo:78-192 restated: K0 linear, K1 asin, K2 logit, K3 piecewise log."""
    d = 100.0
    assert o.normalizer(o.K0, d, 1000) == 50.0
    assert abs(o.normalizer(o.K1, d, 1000) - d / (2 * math.pi)) < 1e-12
    assert abs(o.normalizer(o.K2, d, 1000) - d / (4 * math.log(10) + 24)) < 1e-12
    assert abs(o.normalizer(o.K3, d, 1000) - d / (4 * math.log(10) + 21)) < 1e-12
    for q in (0.001, 0.3, 0.5, 0.77, 0.999):
        assert abs(o.k(o.K1, q, 1.0) - math.asin(2 * q - 1)) < 1e-14
        assert abs(o.k(o.K2, q, 1.0) - math.log(q / (1 - q))) < 1e-13
        k3 = math.log(2 * q) if q <= 0.5 else -math.log(2 * (1 - q))
        assert abs(o.k(o.K3, q, 1.0) - k3) < 1e-13
    # clamp (scale.mojo:41-47): q = 0 and q = 1 stay finite for K2/K3
    assert math.isfinite(o.k(o.K2, 0.0, 1.0)) and math.isfinite(o.k(o.K3, 1.0, 1.0))
    # strict monotonicity on a dense grid (test/test_scale.mojo:29-64)
    for sc in (o.K0, o.K1, o.K2, o.K3):
        ks = [o.k(sc, q, 5.0) for q in np.linspace(1e-6, 1 - 1e-6, 4001)]
        assert all(b > a for a, b in zip(ks, ks[1:]))


# ---------------------------------------------------------------------------
# S-path, decay, edge cases, serde (tdigest.mojo) — known answers
# ---------------------------------------------------------------------------
def test_half_life_seed_contribution_exactly_half():
    """test/test_decay.mojo:137-160."""
    h = 2000.0
    lam = o.log(2.0) / h
    a = o.Digest(o.K1, 100.0, lam)
    b = o.Digest(o.K1, 100.0, lam)
    a.add_at(1000.0, 0.0)
    a.add_at(0.0, h)
    b.add_at(0.0, h)
    assert abs((a.total_weight() - b.total_weight()) - 0.5) < 1e-6


def test_add_at_time_based_decay_total():
    """test/test_decay.mojo:203-211: effective total 1.5."""
    d = o.Digest(o.K1, 100.0, o.log(2.0) / 100.0)
    d.add_at(0.0, 0.0)
    d.add_at(0.0, 100.0)
    assert abs(d.total_weight() - 1.5) < 1e-6


def test_steady_state_total_weight():
    """test/test_decay.mojo:108-134: steady state 1/(1-e^-lambda) within 5%."""
    h = 1000
    lam = o.log(2.0) / h
    d = o.Digest(o.K1, 100.0, lam)
    r = XorShift(7)
    for _ in range(12 * h):
        d.add(r.normal())
    steady = 1.0 / (1.0 - math.exp(-lam))
    assert abs(d.total_weight() - steady) / steady < 0.05


def test_memory_bounded_with_pruning():
    """test/test_decay.mojo:166-178: <= 6 * compression centroids."""
    d = o.Digest(o.K1, 100.0, o.log(2.0) / 5000.0)
    rng = np.random.default_rng(3)
    for v in rng.standard_normal(150_000):
        d.add(float(v))
    d.merge()
    assert len(d) <= 600


def test_drift_tracking():
    """test/test_decay.mojo:69-102."""
    rng = np.random.default_rng(1)
    dec = o.Digest(o.K1, 100.0, o.log(2.0) / 2000.0)
    plain = o.Digest(o.K1, 100.0, 0.0)
    a = rng.standard_normal(20000)
    b = rng.standard_normal(20000) + 10.0
    for v in a:
        dec.add(float(v))
        plain.add(float(v))
    assert abs(dec.quantile(0.5)) < 0.5
    for v in b:
        dec.add(float(v))
        plain.add(float(v))
    assert abs(dec.quantile(0.5) - 10.0) < 1.0
    assert abs(plain.quantile(0.5) - 10.0) > 2.0


def test_zero_decay_matches_undecayed():
    """test/test_decay.mojo:183-200."""
    rng = np.random.default_rng(4)
    a = o.Digest(o.K1, 100.0, 0.0)
    b = o.Digest(o.K1, 100.0, 0.0)
    for v in rng.random(20000):
        a.add(float(v))
        b.add(float(v))
    for q in (0.001, 0.01, 0.5, 0.99, 0.999):
        assert abs(a.quantile(q) - b.quantile(q)) < 1e-12


def test_edge_cases():
    """test/test_edge.mojo:40-135."""
    d = o.Digest(o.K1)
    with pytest.raises(o.OracleError):
        d.quantile(0.5)
    with pytest.raises(o.OracleError):
        d.cdf(0.0)
    assert d.total_weight() == 0.0 and len(d) == 0
    d.add(7.0)
    assert [d.quantile(q) for q in (0.0, 0.5, 1.0)] == [7.0, 7.0, 7.0]
    assert (d.cdf(6.0), d.cdf(8.0), d.cdf(7.0)) == (0.0, 1.0, 0.5)
    same = o.Digest(o.K1, 100.0)
    for _ in range(10_000):
        same.add(3.0)
    same.merge()
    assert len(same) == 1 and same.quantile(0.999) == 3.0 and same.state()["min"] == 3.0
    e = o.Digest(o.K1)
    e.add(5.0)
    before = e.total_weight()
    for bad in (float("nan"), float("inf"), -float("inf")):
        with pytest.raises(o.OracleError):
            e.add(bad)
    for w in (0.0, -2.0):
        with pytest.raises(o.OracleError):
            e.add(1.0, w)
    assert e.total_weight() == before
    with pytest.raises(o.OracleError):
        e.quantile(-0.001)
    with pytest.raises(o.OracleError):
        e.quantile(1.001)


def test_serialization():
    """test/test_edge.mojo:139-217."""
    rng = np.random.default_rng(1)
    d = o.Digest(o.K2, 100.0, o.log(2.0) / 5000.0)
    for v in rng.random(20000):
        d.add(float(v))
    b = d.to_bytes()
    assert b[0] == 1 and len(b) == 65 + 16 * len(d)
    r = o.Digest.from_bytes(b, o.K2)
    assert len(r) == len(d) and abs(r.total_weight() - d.total_weight()) < 1e-9
    for q in (0.001, 0.01, 0.5, 0.99, 0.999):
        assert abs(r.quantile(q) - d.quantile(q)) < 1e-12
    with pytest.raises(o.OracleError):
        o.Digest.from_bytes(bytes([99]), o.K1)
    with pytest.raises(o.OracleError):
        o.Digest.from_bytes(b[:-16], o.K2)
    # cross-process merge
    data = rng.random(20000)
    da, db, comb = o.Digest(o.K1), o.Digest(o.K1), o.Digest(o.K1)
    for i, v in enumerate(data):
        (da if i % 2 == 0 else db).add(float(v))
        comb.add(float(v))
    ra = o.Digest.from_bytes(da.to_bytes(), o.K1)
    rb = o.Digest.from_bytes(db.to_bytes(), o.K1)
    ra.merge_into(rb)
    for q in (0.01, 0.1, 0.5, 0.9, 0.99):
        assert abs(ra.quantile(q) - comb.quantile(q)) < 0.03
    assert abs(ra.total_weight() - 20000) < 1e-6


def test_accuracy_and_compression_bound_spath():
    """test/test_tdigest.mojo:109-163, 231-243."""
    rng = np.random.default_rng(5)
    data = rng.standard_normal(50_000)
    d = o.Digest(o.K1, 100.0)
    for v in data:
        d.add(float(v))
    d.merge()
    s = np.sort(data)
    for q, tol in ((0.001, 0.003), (0.01, 0.003), (0.5, 0.01), (0.99, 0.003), (0.999, 0.003)):
        est = d.quantile(q)
        rank = np.searchsorted(s, est) / len(s)
        assert abs(rank - q) <= tol
    assert len(d) <= 600


# ---------------------------------------------------------------------------
# P-path (the GPU algorithm) — reference accuracy bands and self-consistency
# ---------------------------------------------------------------------------
BANDS = {0: (0.30, 0.10), 1: (0.30, 0.40), 2: (0.25, 0.20), 3: (0.25, 0.20)}


@pytest.mark.parametrize("scale", [0, 1, 2, 3])
def test_ppath_accuracy_bands(scale):
    """test/test_gpu_add_batch.mojo:138-251: P-path estimates within the
    reference's per-rank bands of the true quantile (N=200k, compression 100)."""
    kinds = ["uniform"] if scale == 0 else ["uniform", "normal", "exponential", "pareto"]
    seeds = {"uniform": 0xA1, "normal": 0xB2, "exponential": 0xC3, "pareto": 0xD4}
    low, high = BANDS[scale]
    for kind in kinds:
        data = _data(kind, 200_000, seeds[kind])
        d = o.Digest(scale, 100.0, 0.0)
        d.add_batch_p(data)
        qs = [0.001, 0.5, 0.999]
        for q, t, band in zip(qs, _truth(data, qs), (low, 0.05, high)):
            assert abs(d.quantile(q) - t) <= band * max(1.0, abs(t)), (kind, q)
        cpu = o.Digest(scale, 100.0, 0.0)
        for v in data[:20000]:
            cpu.add(float(v))
        assert d.total_weight() == 200_000


def test_ppath_single_tile_is_one_compress():
    rng = np.random.default_rng(2)
    for n in (1, 2, 17, 1000, 1024):
        m = rng.standard_normal(n)
        w = rng.random(n) + 1
        om, ow = o.ppath_compress(o.K2, 100.0, m, w)
        order = np.argsort(m, kind="stable")
        tm, tw, _ = o.tile_compress(o.K2, 100.0, m[order], w[order])
        assert np.array_equal(om, tm) and np.array_equal(ow, tw)


def test_ppath_hierarchy_restated():
    """gpu_compress_batch_host_tiled (add_batch.mojo:308-347): tile, compress,
    concatenate, repeat while the pass input exceeded one tile."""
    rng = np.random.default_rng(3)
    m = rng.standard_normal(70_001)
    w = rng.random(70_001) + 1
    om, ow = o.ppath_compress(o.K2, 100.0, m, w)
    order = np.argsort(m, kind="stable")
    cm, cw = m[order], w[order]
    while True:
        nm, nw = [], []
        for p in range(0, len(cm), 1024):
            a, b, _ = o.tile_compress(o.K2, 100.0, cm[p:p + 1024], cw[p:p + 1024])
            nm.append(a)
            nw.append(b)
        done = len(cm) <= 1024
        cm, cw = np.concatenate(nm), np.concatenate(nw)
        assert np.all(np.diff(cm) >= 0)  # survivors stay sorted (clamped means)
        if done:
            break
    assert np.array_equal(om, cm) and np.array_equal(ow, cw)


def _hillis_steele_ids(scale, compression, w):
    """Literal FP64 restatement of the reference's 1024-wide Hillis-Steele
    inclusive scan + bucket ids (add_batch.mojo:79-112), in numpy."""
    n = len(w)
    cum = np.zeros(1024)
    cum[:n] = w
    off = 1
    while off < 1024:
        nxt = cum.copy()
        nxt[off:] = cum[off:] + cum[:-off]
        cum = nxt
        off *= 2
    total = cum[1023]
    if total <= 0:
        total = 1.0
    nrm = o.normalizer(scale, compression, total)
    return [o.bucket(scale, float(cum[i]), float(total), nrm) for i in range(n)]


def _tile_cases(rng, count):
    """Sorted tiles of every size class with integral, fractional, equal
    decayed and mixed prior/new weights, with and without ties."""
    for i in range(count):
        n = int(rng.integers(1, 1025)) if i % 5 else int(rng.choice([1, 2, 3, 31, 32, 33, 127, 128, 129, 1023, 1024]))
        x = np.sort(rng.standard_normal(n))
        kind = i % 4
        if kind == 0:
            w = rng.integers(1, 50, n).astype(np.float64)
        elif kind == 1:
            w = rng.random(n) + 0.5
        elif kind == 2:  # one batch's samples at a decay factor e^{log_scale}
            w = np.full(n, np.exp(rng.uniform(0, 40)))
        else:  # prior centroids (fractional weights) merged with new samples, ties
            w = np.full(n, 1.37)
            k = int(rng.integers(0, n))
            w[:k] = rng.random(k) * 100
            x = np.sort(np.round(x * 3) / 3)
        yield int(rng.integers(0, 4)), float(rng.choice([50.0, 100.0, 200.0])), x, w


def test_tile_compress_equals_reference_lane_loops():
    """In the reference association, the oracle's tile (Hillis-Steele prefix,
    balanced-tree total, right-aligned segment trees) equals the reference
    kernel's 1024-lane loops run literally, bit for bit: ids, centroid means
    and weights."""
    rng = np.random.default_rng(2024)
    with o.sums_mode(o.SUMS_REFERENCE):
        for scale, comp, x, w in _tile_cases(rng, 600):
            a = o.tile_compress(scale, comp, x, w)
            b = o.tile_compress_literal(scale, comp, x, w)
            for u, v in zip(a, b):
                assert np.array_equal(u, v), (scale, comp, len(x))


def test_build_sums_differ_from_reference_in_means_only():
    """The kernels' association of sum(w*x) changes the means by rounding only:
    bucket ids, centroid counts and weights are identical to the reference's,
    and every mean agrees within 1e-12 relative (the bound set for summation
    order)."""
    rng = np.random.default_rng(77)
    worst = 0.0
    for scale, comp, x, w in _tile_cases(rng, 600):
        x = x * 10.0 ** rng.uniform(-3, 3) + rng.uniform(-50, 50)
        a = o.tile_compress(scale, comp, x, w)
        with o.sums_mode(o.SUMS_REFERENCE):
            b = o.tile_compress(scale, comp, x, w)
        assert np.array_equal(a[2], b[2]) and np.array_equal(a[1], b[1])
        scale_m = np.maximum(np.abs(b[0]), np.max(np.abs(x)))  # relative to the tile's magnitude
        worst = max(worst, float(np.max(np.abs(a[0] - b[0]) / scale_m)))
    assert worst < 1e-12, worst


@pytest.mark.parametrize("scale", [0, 1, 2, 3])
def test_tile_ids_equal_numpy_hillis_steele(scale):
    """The C lane loops and an independent numpy statement of the reference's
    scan give the same bucket ids, for integral and fractional weights."""
    rng = np.random.default_rng(9 + scale)
    for n in (1, 5, 32, 33, 100, 777, 1024):
        for w in (rng.integers(1, 50, n).astype(np.float64), rng.random(n) * 3 + 0.01):
            x = np.sort(rng.standard_normal(n))
            _, _, ids = o.tile_compress(scale, 100.0, x, w)
            assert list(ids) == _hillis_steele_ids(scale, 100.0, w)


def test_k1_prefix_above_total_maps_to_id_zero():
    """A fractional tile whose last prefix sum rounds above the balanced-tree
    total: K1 evaluates asin slightly above 1 (scale.mojo:114-118 does not
    clamp q), gets NaN and int32 id 0, as the reference's platform converts."""
    rng = np.random.default_rng(5)
    hits = 0
    for _ in range(4000):
        n = int(rng.integers(3, 40))
        w = rng.random(n) + 0.1
        x = np.sort(rng.standard_normal(n))
        _, _, ids = o.tile_compress(o.K1, 100.0, x, w)
        lit = o.tile_compress_literal(o.K1, 100.0, x, w)[2]
        assert list(ids) == list(lit)
        hits += int(ids[-1] == 0)
    assert hits > 0


def test_grouped_equals_per_key_single_digest():
    """test/test_gpu_grouped.mojo:241-311 as an oracle property."""
    rng = np.random.default_rng(0xACC0)
    nk = 5
    g = [o.Digest(o.K2, 100.0, 0.0) for _ in range(nk)]
    r = [o.Digest(o.K2, 100.0, 0.0) for _ in range(nk)]
    for _ in range(3):
        keys = rng.integers(0, nk, 3000)
        vals = rng.random(3000)
        o.grouped_add_batch(g, keys, vals, threads=2)
        for k in range(nk):
            r[k].add_batch_p(vals[keys == k])
    for k in range(nk):
        a, b = g[k].centroids(), r[k].centroids()
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_grouped_rejects_bad_batch_before_mutation():
    g = [o.Digest(o.K2) for _ in range(2)]
    o.grouped_add_batch(g, [0, 1, 0], [1.0, 2.0, 3.0])
    before = [d.total_weight() for d in g]
    with pytest.raises(o.OracleError):
        o.grouped_add_batch(g, [0, 1], [1.0, float("inf")])
    with pytest.raises(o.OracleError):
        o.grouped_add_batch(g, [0, 5], [1.0, 2.0])
    assert [d.total_weight() for d in g] == before


def test_add_many_is_the_add_loop(oracle):
    """The C add loop equals one add() per sample (tdigest.mojo:199-202)."""
    v = np.random.default_rng(9).standard_normal(5000)
    a = oracle.Digest(oracle.K2, 100.0, 0.0)
    b = oracle.Digest(oracle.K2, 100.0, 0.0)
    a.add_many(v)
    for x in v:
        b.add(float(x))
    a.merge()
    b.merge()
    for ca, cb in zip(a.centroids(), b.centroids()):
        assert np.array_equal(ca, cb)
