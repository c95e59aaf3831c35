"""Device key dictionary: arbitrary 64-bit keys to the dense ids a grouped
store is indexed by (grouped.mojo:60-63 requires ids in [0, num_keys)).

The map's contract is checked against numpy set arithmetic: a bijection from
the distinct keys seen so far onto [0, len), ids stable across calls, new keys
numbered after old ones, lookups that insert nothing, and a clean error when
the map is full.  Ingest through the map must give every key exactly the digest
it gets under any other dense numbering."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NOID = np.uint32(0xFFFFFFFF)


def _keys(rng, n, distinct):
    pool = rng.integers(0, 2**64 - 1, distinct, dtype=np.uint64)
    pool = np.unique(pool)
    return pool, pool[rng.integers(0, len(pool), n)]


def _check_bijection(keys, ids, size):
    u, inv = np.unique(keys, return_inverse=True)
    first = np.zeros(len(u), np.int64)
    first[inv[::-1]] = np.arange(len(keys))[::-1]  # an occurrence of each key
    per_key = ids[first]
    assert np.array_equal(ids, per_key[inv]), "a key got two ids"
    assert len(np.unique(per_key)) == len(u), "two keys share an id"
    assert per_key.max() < size
    return dict(zip(u.tolist(), per_key.tolist()))


def test_dense_stable_ids(kd):
    rng = np.random.default_rng(1)
    m = kd.KeyDictionary(100000)
    pool, k1 = _keys(rng, 300000, 40000)
    ids1 = m.map(k1)
    n1 = len(np.unique(k1))
    assert len(m) == n1
    assert np.array_equal(np.unique(ids1), np.arange(n1, dtype=np.uint32))
    before = _check_bijection(k1, ids1, n1)
    # a second call: old keys keep their ids, new keys take ids n1, n1+1, ...
    _, k2 = _keys(rng, 200000, 30000)
    k2 = np.concatenate([k2, k1[:50000]])
    ids2 = m.map(k2)
    n2 = len(np.unique(np.concatenate([k1, k2])))
    assert len(m) == n2
    after = _check_bijection(k2, ids2, n2)
    for k, i in after.items():
        if k in before:
            assert before[k] == i
        else:
            assert n1 <= i < n2
    assert np.array_equal(m.map(k1), ids1)


def test_one_hot_key_many_threads(kd):
    """Every thread of the grid races for the same few new keys."""
    m = kd.KeyDictionary(64)
    keys = np.full(1 << 20, 12345, np.uint64)
    keys[::1000] = 777
    keys[5::1000] = 2**63
    ids = m.map(keys)
    assert len(m) == 3
    _check_bijection(keys, ids, 3)


def test_lookup_inserts_nothing(kd):
    rng = np.random.default_rng(2)
    m = kd.KeyDictionary(5000)
    pool, k = _keys(rng, 20000, 3000)
    ids = m.map(k)
    unknown = np.setdiff1d(rng.integers(0, 2**64 - 1, 5000, dtype=np.uint64), pool)
    q = np.concatenate([k[:1000], unknown])
    got = m.lookup(q)
    assert np.array_equal(got[:1000], ids[:1000])
    assert np.all(got[1000:] == NOID)
    assert len(m) == len(np.unique(k))
    assert np.array_equal(m.lookup(np.zeros(0, np.uint64)), np.zeros(0, np.uint32))


def test_full_map_and_reserved_key(kd):
    m = kd.KeyDictionary(1000)
    keys = np.arange(1, 1501, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
    with pytest.raises(kd.KdError) as e:
        m.map(keys)
    assert e.value.code == 5  # KD_ENOMEM
    assert len(m) == 1000
    got = m.lookup(keys)
    have = got != NOID
    assert have.sum() == 1000
    assert np.array_equal(np.sort(got[have]), np.arange(1000, dtype=np.uint32))
    assert np.array_equal(m.map(keys[have]), got[have])  # keys with ids still map
    with pytest.raises(kd.KdError):
        m.map(keys[~have][:1])  # a key stored when the map was full has no id
    with pytest.raises(ValueError):
        kd.KeyDictionary(10).map(np.array([2**64 - 1], np.uint64))


def test_ingest_through_dictionary(kd):
    """A key's digest does not depend on its dense number."""
    rng = np.random.default_rng(3)
    pool, k = _keys(rng, 400000, 20000)
    vals = rng.lognormal(0, 1.0, len(k))
    m = kd.KeyDictionary(len(pool))
    ids = m.map(k)
    a = kd.GroupedTDigest(len(pool), 100.0, scale=kd.K3)
    a.add_batch(ids, vals)
    u, inv = np.unique(k, return_inverse=True)
    b = kd.GroupedTDigest(len(u), 100.0, scale=kd.K3)
    b.add_batch(inv.astype(np.uint32), vals)
    by_key = m.lookup(u)
    for j in range(0, len(u), 397):
        ma, wa = a.centroids(int(by_key[j]))
        mb, wb = b.centroids(j)
        assert np.array_equal(ma, mb) and np.array_equal(wa, wb)


def test_device_keys_to_device_ingest(kd):
    torch = pytest.importorskip("torch")
    from kdigest_gb300 import _native as N

    rng = np.random.default_rng(4)
    pool, k = _keys(rng, 1 << 20, 50000)
    vals = rng.standard_normal(len(k))
    m = kd.KeyDictionary(len(pool))
    dk = torch.from_numpy(k.view(np.int64)).cuda()
    dids = m.map(dk)
    assert dids.dtype == torch.int32 and dids.is_cuda
    ids = dids.cpu().numpy().view(np.uint32)
    assert np.array_equal(m.lookup(k), ids)
    g = kd.GroupedTDigest(len(pool), 100.0, scale=kd.K2)
    dv = torch.from_numpy(vals).cuda()
    torch.cuda.synchronize()
    L = N.load()
    rc = L.kd_store_ingest(g._store._h, dids.data_ptr(), dv.data_ptr(), len(k), N.KD_CLOCK_COUNT,
                           0.0, N.KD_PTR_DEVICE)
    assert rc == 0
    h = kd.GroupedTDigest(len(pool), 100.0, scale=kd.K2)
    h.add_batch(ids, vals)
    assert np.array_equal(g.centroid_counts(), h.centroid_counts())
    for j in range(0, len(pool), 4999):
        assert np.array_equal(g.centroids(j)[0], h.centroids(j)[0])


def test_session_destroyed_before_map(kd):
    sess = kd.GpuSession()
    m = kd.KeyDictionary(10, session=sess)
    m.map(np.array([1, 2, 3], np.uint64))
    sess.close()
    with pytest.raises(ValueError):
        m.map(np.array([4], np.uint64))
    from kdigest_gb300 import _native as N

    assert N.load().kd_keymap_size(m._h) == -1
    m.close()
