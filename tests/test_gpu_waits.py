"""Bounded device waits run out cleanly.

With the test-only session option KD_OPT_TEST_WAIT, one wait per radix pass
(the decoupled look-back of the sort) and one per key-map call (an id that is
never published) wait on a word that nothing writes, with a short poll limit.
The call must come back with KD_ETIMEOUT, leave every digest as it was, and the
session must serve the next call normally.  No wait is removed or unbounded:
the option only makes a bounded wait's flag stay unset.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _snapshot(g):
    return [g.to_bytes(k) if g.centroid_count(k) else b"" for k in range(g.num_keys)]


def test_sort_lookback_timeout_changes_nothing(kd, oracle):
    from kdigest_gb300 import _native as N

    sess = kd.GpuSession()
    sess.set_option(N.KD_OPT_GRAPHS, 0)
    nk = 64
    g = kd.GroupedTDigest(nk, 100.0, scale=kd.K2, session=sess)
    refs = [oracle.Digest(oracle.K2, 100.0, 0.0) for _ in range(nk)]
    rng = np.random.default_rng(5)
    keys = rng.integers(0, nk, 50000).astype(np.uint32)  # several sort tiles
    vals = rng.standard_normal(50000)
    g.add_batch(keys, vals)
    oracle.grouped_add_batch(refs, keys, vals)
    before = _snapshot(g)
    sess.set_option(N.KD_OPT_TEST_WAIT, 2000)
    keys2 = rng.integers(0, nk, 50000).astype(np.uint32)
    vals2 = rng.standard_normal(50000)
    with pytest.raises(N.KdError) as ei:
        g.add_batch(keys2, vals2)
    assert ei.value.code == N.KD_ETIMEOUT
    assert _snapshot(g) == before
    sess.set_option(N.KD_OPT_TEST_WAIT, 0)
    g.add_batch(keys2, vals2)
    oracle.grouped_add_batch(refs, keys2, vals2)
    for k in range(nk):
        m, w = g.centroids(k)
        rm, rw = refs[k].centroids()
        assert np.array_equal(m, rm) and np.array_equal(w, rw), k


def test_keymap_publish_wait_timeout(kd):
    from kdigest_gb300 import _native as N

    sess = kd.GpuSession()
    m = kd.KeyDictionary(1000, session=sess)
    base = np.arange(1, 101, dtype=np.uint64) * 7919
    ids = m.map(base)
    assert sorted(ids.tolist()) == list(range(100))
    sess.set_option(N.KD_OPT_TEST_WAIT, 500)
    k0 = np.uint64(123456789)
    keys = np.array([k0, 5, 6, k0, k0, 9], dtype=np.uint64)
    with pytest.raises(N.KdError) as ei:
        m.map(keys)
    assert ei.value.code == N.KD_ETIMEOUT
    sess.set_option(N.KD_OPT_TEST_WAIT, 0)
    # keys that got ids before keep them, and the session keeps serving
    assert np.array_equal(m.lookup(base), ids)
    fresh = np.array([11, 12, 13], dtype=np.uint64) * 104729
    got = m.map(fresh)
    assert len(set(got.tolist())) == 3 and all(int(i) < 1000 for i in got)
