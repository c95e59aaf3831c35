"""Batched to_bytes / from_bytes (checkpoint and restore of a resident store).

Each record is the reference's wire format (test/test_edge.mojo:139-217 pins it
per digest through the oracle): the batched export must equal the per-key
to_bytes byte for byte, and an import must reproduce every digest exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _filled(kd, nk, seed, decay=None, scale=None, batches=3, n=200000):
    g = kd.GroupedTDigest(nk, 100.0, decay=decay, scale=kd.K2 if scale is None else scale)
    rng = np.random.default_rng(seed)
    for b in range(batches):
        keys = rng.zipf(1.2, n) % nk
        vals = rng.lognormal(0, 1.5, n)
        if decay is not None:
            g.add_batch_at(keys, vals, float(b + 1))
        else:
            g.add_batch(keys, vals)
    return g


def _same_state(a, b, keys):
    for k in keys:
        ma, wa = a.centroids(int(k))
        mb, wb = b.centroids(int(k))
        assert np.array_equal(ma, mb) and np.array_equal(wa, wb)
        assert a.state(int(k)) == b.state(int(k))


def test_export_equals_per_key_to_bytes(kd):
    nk = 3000
    g = _filled(kd, nk, 1)
    data, offs = g.export()
    assert len(offs) == nk + 1 and offs[0] == 0 and offs[-1] == len(data)
    for k in list(range(0, nk, 97)) + [nk - 1]:
        assert data[offs[k]:offs[k + 1]] == g.to_bytes(k)
    sub = np.array([5, 2999, 5, 17, 0], dtype=np.uint32)
    d2, o2 = g.export(sub)
    for i, k in enumerate(sub):
        assert d2[o2[i]:o2[i + 1]] == g.to_bytes(int(k))


def test_import_reproduces_every_digest(kd):
    nk = 2000
    g = _filled(kd, nk, 2)
    data, offs = g.export()
    h = kd.GroupedTDigest(nk, 100.0, scale=kd.K2)
    h.import_records(data, offs)
    _same_state(g, h, range(0, nk, 13))
    qk = np.repeat(np.arange(nk), 3)
    qs = np.tile([0.01, 0.5, 0.99], nk)
    assert np.array_equal(g.quantiles(qk, qs), h.quantiles(qk, qs))
    # a key list places records anywhere
    h2 = kd.GroupedTDigest(nk, 100.0, scale=kd.K2)
    keys = np.array([7, 1999, 0], dtype=np.uint32)
    d3, o3 = g.export(keys[::-1])
    h2.import_records(d3, o3, keys[::-1])
    _same_state(g, h2, keys)


def test_import_validates_before_any_change(kd):
    nk = 500
    g = _filled(kd, nk, 3, n=50000)
    data, offs = g.export()
    h = _filled(kd, nk, 4, n=50000)
    before, boffs = h.export()
    bad = bytearray(data)
    bad[offs[nk // 2]] = 2  # version byte of one record in the middle
    with pytest.raises(ValueError):
        h.import_records(bytes(bad), offs)
    after, _ = h.export()
    assert after == before
    trunc = offs.copy()
    trunc[nk // 3 + 1] = trunc[nk // 3] + 40  # a record shorter than its header
    with pytest.raises(Exception):
        h.import_records(data, trunc)
    assert h.export()[0] == before


def test_snapshot_restore_resumes_exactly(kd, tmp_path):
    nk = 1500
    dec = kd.Decay.half_life(2.0)
    g = _filled(kd, nk, 5, decay=dec, scale=kd.K3)
    path = str(tmp_path / "store.snap")
    g.snapshot(path)
    h = kd.GroupedTDigest.restore(path)
    assert h.num_keys == nk and h.scale == g.scale
    _same_state(g, h, range(0, nk, 11))
    rng = np.random.default_rng(6)
    keys = rng.integers(0, nk, 100000)
    vals = rng.standard_normal(100000)
    g.add_batch_at(keys, vals, 9.5)
    h.add_batch_at(keys, vals, 9.5)
    _same_state(g, h, range(0, nk, 11))


def test_export_import_across_chunks(kd):
    """More than one 256 MB staging round trip each way."""
    nk = 400000
    g = kd.GroupedTDigest(nk, 100.0, scale=kd.K1)
    rng = np.random.default_rng(8)
    for _ in range(5):
        n = 1 << 23
        g.add_batch(rng.integers(0, nk, n), rng.standard_normal(n))
    data, offs = g.export()
    assert len(data) > (256 << 20)
    h = kd.GroupedTDigest(nk, 100.0, scale=kd.K1)
    h.import_records(data, offs)
    assert np.array_equal(g.centroid_counts(), h.centroid_counts())
    _same_state(g, h, range(0, nk, 9973))
    d2, _ = h.export()
    assert d2 == data


def test_session_destroyed_before_its_store_and_server(kd):
    """Any destruction order is safe: a session destroyed first stops its
    servers and frees its stores' device memory; the handles then fail cleanly."""
    sess = kd.GpuSession()
    g = kd.GroupedTDigest(100, 100.0, scale=kd.K2, session=sess)
    g.add_batch(np.arange(100), np.ones(100))
    srv = kd.Server(g, window=1e-3)
    t = srv.submit_ingest(0.5, np.array([1, 2], np.uint32), [2.0, 3.0])
    sess.close()  # drains the server, orphans the store
    assert srv.wait(t, 10.0)[0] == 0
    with pytest.raises(ValueError):
        g.centroid_counts()
    srv.close()
    del g


@pytest.mark.parametrize("clock", ["count", "time"])
def test_export_equals_oracle_records_with_decay(kd, oracle, clock):
    """Every record of a multi-key decayed store's batched export equals, byte
    for byte, the oracle's to_bytes of that key's digest fed the same batches
    (decayed weights, log-scale, clock and stored total in the header; keys
    never ingested as empty records)."""
    nk = 48
    rng = np.random.default_rng(41 if clock == "count" else 42)
    if clock == "count":
        lam = oracle.log(2.0) / 5000.0
        g = kd.GroupedTDigest(nk, 100.0, kd.Decay.rate(lam), scale=kd.K3)
        refs = [oracle.Digest(oracle.K3, 100.0, lam) for _ in range(nk)]
    else:
        lam = oracle.log(2.0) / 60.0
        g = kd.GroupedTDigest(nk, 200.0, kd.Decay.rate(lam), scale=kd.K2)
        refs = [oracle.Digest(oracle.K2, 200.0, lam) for _ in range(nk)]
    t = 0.0
    for step in range(8):
        n = int(rng.integers(2000, 30000))
        keys = (rng.zipf(1.3, n) - 1) % (nk - 3)  # the last three keys stay empty
        vals = rng.lognormal(0.0, 2.0, n)
        if clock == "count":
            g.add_batch(keys.astype(np.uint32), vals)
            oracle.grouped_add_batch(refs, keys, vals)
        else:
            t += rng.exponential(30.0)
            g.add_batch_at(keys.astype(np.uint32), vals, t)
            for k in range(nk):
                sel = vals[keys == k]
                if len(sel):
                    refs[k].add_batch_p_at(sel, t)
    data, offs = g.export()
    for k in range(nk):
        assert data[offs[k]:offs[k + 1]] == refs[k].to_bytes(), k
