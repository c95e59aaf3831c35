"""Ingest steps replayed from captured CUDA graphs give exactly the eager
results: a step shape seen twice is captured, later steps replay it with new
input pointers, timestamps and host-staged inputs; a replay whose keys need
more hierarchy levels than were captured continues eagerly; the sort's
look-back epochs advance on every replay."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair(kd, num_keys, scale, compression=100.0, decay=None):
    a = kd.GpuSession()
    b = kd.GpuSession()
    b.set_option(4, 0)  # KD_OPT_GRAPHS off: eager reference
    ga = kd.GroupedTDigest(num_keys, compression, decay=decay, scale=scale, session=a)
    gb = kd.GroupedTDigest(num_keys, compression, decay=decay, scale=scale, session=b)
    return ga, gb


def _same(ga, gb, num_keys):
    assert np.array_equal(ga.centroid_counts(), gb.centroid_counts())
    for k in range(0, num_keys, max(1, num_keys // 37)):
        ma, wa = ga.centroids(k)
        mb, wb = gb.centroids(k)
        assert np.array_equal(ma, mb) and np.array_equal(wa, wb)
        assert ga.state(k) == gb.state(k)


def test_replays_match_eager_count_clock(kd):
    nk, n = 300, 20000
    ga, gb = _pair(kd, nk, kd.K3)
    rng = np.random.default_rng(1)
    for step in range(12):
        keys = rng.zipf(1.3, n) % nk
        vals = rng.standard_normal(n) * (1 + keys % 7) + keys
        ga.add_batch(keys, vals)  # fresh arrays each step: new input pointers
        gb.add_batch(keys, vals)
        _same(ga, gb, nk)
    qk = np.arange(nk).repeat(3)
    qs = np.tile([0.01, 0.5, 0.99], nk)
    assert np.array_equal(ga.quantiles(qk, qs), gb.quantiles(qk, qs))


def test_replays_match_eager_time_clock_with_decay(kd):
    nk, n = 64, 5000
    ga, gb = _pair(kd, nk, kd.K2, 200.0, decay=kd.Decay.half_life(3.0))
    rng = np.random.default_rng(2)
    for step in range(10):
        keys = rng.integers(0, nk, n)
        vals = rng.lognormal(0.0, 1.5, n)
        ts = 1.5 * step + rng.random()  # a new timestamp every replay
        ga.add_batch_at(keys, vals, ts)
        gb.add_batch_at(keys, vals, ts)
        _same(ga, gb, nk)


def test_replay_needing_more_levels_continues(kd):
    nk, n = 16, 200000
    ga, gb = _pair(kd, nk, kd.K1)
    rng = np.random.default_rng(3)
    for step in range(6):
        if step < 4:
            keys = rng.integers(0, nk, n)  # ~12.5k per key
        else:
            keys = np.zeros(n, dtype=np.int64)  # one key takes the whole batch
        vals = rng.standard_normal(n)
        ga.add_batch(keys, vals)
        gb.add_batch(keys, vals)
        _same(ga, gb, nk)


def test_single_digest_and_compress_replays(kd, oracle):
    sess = kd.GpuSession()
    d = kd.TDigest(100.0, kd.K1, session=sess)
    ref = oracle.Digest(oracle.K1, 100.0, 0.0)
    rng = np.random.default_rng(4)
    for step in range(8):
        v = rng.standard_normal(4096)
        d.add_batch_p(v)
        ref.add_batch_p(v)
    m, w = d.centroids()
    om, ow = ref.centroids()
    assert np.array_equal(m, om) and np.array_equal(w, ow)
    for step in range(6):
        m = rng.standard_normal(3000)
        w = rng.random(3000) + 0.5
        gm, gw = kd.compress(m, w, 100.0, kd.K2, session=sess)
        om, ow = oracle.ppath_compress(oracle.K2, 100.0, m, w)
        assert np.array_equal(gm, om) and np.array_equal(gw, ow)


def test_many_replays_keep_sorting(kd):
    nk, n = 1000, 1 << 14
    ga, gb = _pair(kd, nk, kd.K3)
    rng = np.random.default_rng(5)
    for step in range(60):
        keys = rng.integers(0, nk, n)
        vals = rng.standard_normal(n)
        ga.add_batch(keys, vals)
        gb.add_batch(keys, vals)
    _same(ga, gb, nk)


def test_replays_with_stage_timing(kd):
    """Stage events are recorded inside captured graphs too."""
    nk, n = 200, 30000
    sess = kd.GpuSession()
    sess.set_option(3, 1)  # KD_OPT_STAGE_TIMING
    g = kd.GroupedTDigest(nk, 100.0, scale=kd.K3, session=sess)
    e = kd.GroupedTDigest(nk, 100.0, scale=kd.K3, session=kd.GpuSession())
    rng = np.random.default_rng(6)
    for step in range(6):
        keys = rng.integers(0, nk, n)
        vals = rng.standard_normal(n)
        g.add_batch(keys, vals)
        e.add_batch(keys, vals)
    st = sess.stats()
    # every ingest: prep, histogram, the radix passes, unpack, repair, two
    # one-block scans, prepare, level plan, tiles and commit
    assert st["ingests"] == 6 and st["launches"] >= 6 * 15
    assert all(v > 0.0 for v in st["stage_ms"].values()), st
    _same(g, e, nk)


def test_launch_tuning_never_changes_results(kd):
    """Every tile-kernel split and grid, serial or on two streams, eager or
    replayed, gives the same digests."""
    nk, n = 500, 60000
    rng = np.random.default_rng(7)
    batches = [(rng.zipf(1.2, n) % nk, rng.standard_normal(n) * 3.0) for _ in range(4)]
    ref = None
    for cap, lb, sb, cc in ((128, 6, 8, 0), (32, 4, 16, 0), (64, 8, 4, 0), (1, 1, 1, 0),
                            (128, 6, 8, 1), (64, 4, 16, 1)):
        s = kd.GpuSession(tuned=False)
        s.set_option(5, cap)
        s.set_option(6, lb)
        s.set_option(7, sb)
        s.set_option(8, cc)  # KD_OPT_CONCURRENT_TILES: the two tile kernels on two streams
        g = kd.GroupedTDigest(nk, 100.0, scale=kd.K3, session=s)
        for k, v in batches:
            g.add_batch(k, v)
        if ref is None:
            ref = g
        else:
            _same(g, ref, nk)
