"""GPU parity of grouped ingest, queries and merges against the CPU oracle.

Restates test/test_gpu_grouped.mojo: grouped == per-key reference
(:188-238), accumulation over batches with keys coming and going and a key
crossing 1024, with and without decay (:241-311), untouched keys unchanged
(:314-339), an invalid batch leaves state unchanged (:342-365), prior
centroids folded with new samples (:368-429).  Tolerance 0: the GPU state
must equal the oracle state bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _assert_same(g, refs, keys, tag=""):
    for k in keys:
        m, w = g.centroids(k)
        rm, rw = refs[k].centroids()
        assert len(m) == len(rm), f"count {tag} key={k}"
        assert np.array_equal(m, rm), f"means {tag} key={k}"
        assert np.array_equal(w, rw), f"weights {tag} key={k}"
        st, rs = g.state(k), refs[k].state()
        for f in ("stored_total", "log_scale", "clock", "min", "max", "count"):
            assert st[f] == rs[f], f"{f} {tag} key={k}: {st[f]} vs {rs[f]}"


@pytest.mark.parametrize("cfg", [(50, 300, 0), (40, 1024, 13), (6, 2500, 0), (300, 1, 0)])
def test_grouped_matches_per_key_reference(kd, oracle, cfg):
    nk, per, lev = cfg
    rng = np.random.default_rng(0xBEE + nk)
    keys, vals = [], []
    for i in range(per):
        for k in range(nk):
            if k % 7 == 3:
                continue
            if k % 5 == 1 and i >= per // 3:
                continue
            u = rng.random()
            keys.append(k)
            vals.append(float(int(u * lev)) if lev > 0 else u * (k + 1))
    g = kd.GroupedTDigest(nk, compression=100.0, scale=kd.K2)
    g.add_batch(np.array(keys), np.array(vals))
    refs = [oracle.Digest(oracle.K2, 100.0, 0.0) for _ in range(nk)]
    oracle.grouped_add_batch(refs, np.array(keys), np.array(vals))
    _assert_same(g, refs, range(nk), str(cfg))
    for k in range(nk):
        if k % 7 == 3:
            assert g.centroid_count(k) == 0


@pytest.mark.parametrize("half_life", [0.0, 500.0, 37.0])
@pytest.mark.parametrize("scale", [1, 2, 3])
def test_grouped_accumulates_across_batches(kd, oracle, half_life, scale):
    lam = 0.0 if half_life == 0.0 else oracle.log(2.0) / half_life
    nk = 6
    g = kd.GroupedTDigest(nk, 100.0, kd.Decay.rate(lam), scale=scale)
    refs = [oracle.Digest(scale, 100.0, lam) for _ in range(nk)]
    rng = np.random.default_rng(0xACC0)
    for batch in range(5):
        keys, vals = [], []
        for i in range(400):
            for k in range(nk):
                if k == 1 and batch % 2 == 1:
                    continue
                if k == 2 and batch >= 2:
                    continue
                if k == 4 and i >= 10:
                    continue
                if k == 5 and batch == 3 and i >= 300:
                    continue
                keys.append(k)
                vals.append(rng.random() * (k + 1) + batch)
        if batch == 4:
            for _ in range(800):
                keys.append(3)
                vals.append(rng.random() * 4.0 + 4.0)
        g.add_batch(np.array(keys), np.array(vals))
        oracle.grouped_add_batch(refs, np.array(keys), np.array(vals))
        _assert_same(g, refs, range(nk), f"batch={batch}")
    qs = [0.0, 0.001, 0.01, 0.25, 0.5, 0.75, 0.99, 0.999, 1.0]
    for k in range(nk):
        got = g.quantiles(np.full(len(qs), k), qs)
        want = [refs[k].quantile(q) for q in qs]
        assert np.array_equal(got, np.array(want))


def test_untouched_key_and_total_weight(kd):
    g = kd.GroupedTDigest(3, 100.0, scale=kd.K2)
    k1 = np.repeat(np.arange(3)[None, :], 500, axis=0).ravel()
    v1 = np.repeat(np.arange(500.0)[:, None], 3, axis=1).ravel()
    g.add_batch(k1, v1)
    before_c = g.centroid_count(2)
    before_q = g.quantile(2, 0.5)
    g.add_batch(np.zeros(300, np.int64), 1000.0 + np.arange(300.0))
    assert g.total_weight(0) == 800.0
    assert g.total_weight(2) == 500.0
    assert g.centroid_count(2) == before_c
    assert g.quantile(2, 0.5) == before_q
    p50 = g.quantile(0, 0.5)
    assert 300.0 < p50 < 1100.0


def test_invalid_batch_leaves_state_unchanged(kd):
    g = kd.GroupedTDigest(2, 100.0, scale=kd.K2)
    g.add_batch(np.arange(200) % 2, np.arange(200.0))
    w0, w1 = g.total_weight(0), g.total_weight(1)
    m0 = g.centroids(0)
    bad_v = np.arange(100.0)
    bad_v[57] = np.inf
    with pytest.raises(ValueError):
        g.add_batch(np.arange(100) % 2, bad_v)
    with pytest.raises(IndexError):
        g.add_batch(np.array([0, 1, 2]), np.array([1.0, 2.0, 3.0]))
    assert g.total_weight(0) == w0 and g.total_weight(1) == w1
    assert np.array_equal(g.centroids(0)[0], m0[0])


def test_device_side_validation_leaves_state_unchanged(kd):
    """The native entry point validates on the device too (keys bypassing the
    host check): nothing is committed."""
    import kdigest_gb300._native as N
    g = kd.GroupedTDigest(4, 100.0, scale=kd.K3)
    g.add_batch(np.arange(400) % 4, np.arange(400.0))
    before = [g.centroids(k) for k in range(4)]
    keys = np.array([0, 1, 7, 2], np.uint32)
    vals = np.array([1.0, 2.0, 3.0, 4.0])
    rc = N.load().kd_store_ingest(g._store._h, N.ptr(keys), N.ptr(vals), 4, 0, 0.0, 0)
    assert rc == N.KD_EINVAL
    for k in range(4):
        assert np.array_equal(g.centroids(k)[0], before[k][0])


def test_touched_keys_key_level_and_element_level(kd, oracle):
    """Batches with at least as many samples as keys list their touched keys
    from per-key stamps, smaller ones by a scan over the samples.  Two stores
    of one session alternate (their steps share the stamp array), a batch
    holds a key in [K, 2^ceil(log2 K)) that only the device check sees, and
    every store still equals the oracle bit for bit."""
    import kdigest_gb300._native as N
    sess = kd.GpuSession()
    sizes = (1000, 50)
    stores = [kd.GroupedTDigest(k, 100.0, scale=kd.K1, session=sess) for k in sizes]
    refs = [[oracle.Digest(oracle.K1, 100.0, 0.0) for _ in range(k)] for k in sizes]
    rng = np.random.default_rng(0x70C)
    for step in range(6):
        for g, r, nk in zip(stores, refs, sizes):
            n = 3000 if step % 2 == 0 else 400  # above / below the key count of the first store
            keys = (rng.zipf(1.3, n) - 1) % nk
            vals = rng.standard_normal(n) + keys % 11
            g.add_batch(keys, vals)
            oracle.grouped_add_batch(r, keys, vals)
        if step == 2:
            before = stores[0].centroid_counts().copy()
            keys = (np.arange(2000) % 1000).astype(np.uint32)
            keys[1234] = 1010  # below 2^10, above the store's 1000 keys
            vals = rng.standard_normal(2000)
            rc = N.load().kd_store_ingest(stores[0]._store._h, N.ptr(keys), N.ptr(vals), 2000, 0,
                                          0.0, 0)
            assert rc == N.KD_EINVAL
            assert np.array_equal(stores[0].centroid_counts(), before)
    for g, r, nk in zip(stores, refs, sizes):
        _assert_same(g, r, range(nk), f"K={nk}")


def test_time_clock_decay(kd, oracle):
    lam = oracle.log(2.0) / 60.0
    nk = 20
    g = kd.GroupedTDigest(nk, 200.0, kd.Decay.rate(lam), scale=kd.K2)
    refs = [oracle.Digest(oracle.K2, 200.0, lam) for _ in range(nk)]
    rng = np.random.default_rng(5)
    t = 0.0
    for step in range(12):
        t += rng.exponential(30.0)
        n = int(rng.integers(1, 3000))
        keys = rng.integers(0, nk, n)
        vals = rng.lognormal(0.0, 2.0, n)
        g.add_batch_at(keys, vals, t)
        # oracle: per key add_batch_p_at with the shared timestamp
        for k in range(nk):
            sel = vals[keys == k]
            if len(sel):
                refs[k].add_batch_p_at(sel, t)
        _assert_same(g, refs, range(nk), f"step={step}")


def test_renormalisation_and_prune(kd, oracle):
    """Decay fast enough to cross the 400 renormalisation threshold and to
    prune centroids below the 1e-6 effective-weight floor."""
    lam = 0.05
    g = kd.GroupedTDigest(3, 100.0, kd.Decay.rate(lam), scale=kd.K1)
    refs = [oracle.Digest(oracle.K1, 100.0, lam) for _ in range(3)]
    rng = np.random.default_rng(11)
    for b in range(30):
        n = 1500
        keys = rng.integers(0, 3, n)
        vals = rng.standard_normal(n) + b
        g.add_batch(keys, vals)
        oracle.grouped_add_batch(refs, keys, vals)
        _assert_same(g, refs, range(3), f"b={b}")


def test_queries_match_oracle(kd, oracle):
    nk = 64
    g = kd.GroupedTDigest(nk, 100.0, scale=kd.K3)
    refs = [oracle.Digest(oracle.K3, 100.0, 0.0) for _ in range(nk)]
    rng = np.random.default_rng(3)
    for _ in range(3):
        keys = rng.integers(0, nk, 50000)
        vals = rng.standard_normal(50000) * (1 + keys)
        g.add_batch(keys, vals)
        oracle.grouped_add_batch(refs, keys, vals)
    qk = rng.integers(0, nk, 20000)
    qs = np.concatenate([rng.random(10000), 10 ** rng.uniform(-6, -2, 5000),
                         1 - 10 ** rng.uniform(-6, -2, 5000)])
    got = g.quantiles(qk, qs)
    want = np.array([refs[k].quantile(q) for k, q in zip(qk, qs)])
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=0)
    assert np.array_equal(got, want)
    xs = rng.standard_normal(20000) * 40
    got = g.cdfs(qk, xs)
    want = np.array([refs[k].cdf(x) for k, x in zip(qk, xs)])
    assert np.array_equal(got, want)


def test_query_errors(kd):
    g = kd.GroupedTDigest(3, 100.0)
    g.add_batch([0, 0, 1], [1.0, 2.0, 3.0])
    with pytest.raises(ValueError):
        g.quantile(2, 0.5)  # empty digest
    with pytest.raises(ValueError):
        g.quantile(0, 1.5)
    with pytest.raises(IndexError):
        g.quantile(5, 0.5)


def test_merge_groups_matches_oracle(kd, oracle):
    nparts, per_group = 64, 8
    src = kd.GroupedTDigest(nparts, 50.0, scale=kd.K2)
    refs = [oracle.Digest(oracle.K2, 50.0, 0.0) for _ in range(nparts)]
    rng = np.random.default_rng(21)
    keys = np.repeat(np.arange(nparts), rng.integers(64, 4096, nparts))
    vals = rng.standard_normal(len(keys)) * rng.uniform(0.1, 5, nparts)[keys] + \
        rng.uniform(-10, 10, nparts)[keys]
    src.add_batch(keys, vals)
    oracle.grouped_add_batch(refs, keys, vals)
    ngroups = nparts // per_group
    dst = kd.GroupedTDigest(ngroups, 200.0, scale=kd.K2)
    go = np.arange(0, nparts + 1, per_group)
    dst.merge_groups(src, go, np.arange(nparts))
    for gi in range(ngroups):
        d = oracle.Digest(oracle.K2, 200.0, 0.0)
        oracle.merge_parts(d, refs[gi * per_group:(gi + 1) * per_group])
        m, w = dst.centroids(gi)
        rm, rw = d.centroids()
        assert np.array_equal(m, rm) and np.array_equal(w, rw)
        st, rs = dst.state(gi), d.state()
        for f in ("stored_total", "min", "max", "clock"):
            assert st[f] == rs[f]


def test_serde_round_trip(kd, oracle):
    d = kd.TDigest(100.0, kd.K2, kd.Decay.half_life(5000.0))
    rng = np.random.default_rng(1)
    d.add_batch(rng.random(20000))
    b = d.to_bytes()
    r = kd.TDigest.from_bytes(b, scale=kd.K2)
    assert len(r) == len(d)
    assert r.total_weight() == d.total_weight()
    for q in (0.001, 0.01, 0.5, 0.99, 0.999):
        assert r.quantile(q) == d.quantile(q)
    # the oracle reads the same bytes
    od = oracle.Digest.from_bytes(b, oracle.K2)
    assert od.centroids()[0].tolist() == d.centroids()[0].tolist()
    with pytest.raises(ValueError):
        kd.TDigest.from_bytes(bytes([99]))
    with pytest.raises(ValueError):
        kd.TDigest.from_bytes(b[:-16], scale=kd.K2)


@pytest.mark.parametrize("num_keys", [300, 70000])
def test_packed_sort_inversion_falls_back_to_full_sort(kd, oracle, num_keys):
    """Samples of one key whose order keys differ only in the bits the packed
    sort leaves out arrive larger-first: the step must detect the inversion,
    commit nothing from the packed order, and sort in full."""
    rng = np.random.default_rng(17)
    base = rng.standard_normal(2000) * 10
    ulp = np.spacing(np.abs(base))
    keys = np.repeat(rng.integers(0, num_keys, 2000), 2)
    vals = np.stack([base + 3 * ulp, base], axis=1).reshape(-1)  # larger first, same top bits
    more_k = rng.integers(0, num_keys, 30000)
    more_v = rng.standard_normal(30000)
    keys = np.concatenate([keys, more_k])
    vals = np.concatenate([vals, more_v])
    g = kd.GroupedTDigest(num_keys, 100.0, scale=kd.K2)
    for step in range(2):
        g.add_batch(keys, vals)
    used = np.unique(keys)
    ref = [oracle.Digest(oracle.K2, 100.0, 0.0) for _ in range(len(used))]
    pos = {k: i for i, k in enumerate(used)}
    sub = np.array([pos[k] for k in keys])
    for step in range(2):
        oracle.grouped_add_batch(ref, sub, vals)
    for k in used[:: max(1, len(used) // 50)]:
        gm, gw = g.centroids(int(k))
        om, ow = ref[pos[k]].centroids()
        assert np.array_equal(gm, om) and np.array_equal(gw, ow)


def test_packed_sort_long_run_falls_back(kd, oracle):
    """200 samples of one key equal in their packed bits (1 + j ulp, shuffled):
    a run too long to repair in place, so the step sorts in full."""
    rng = np.random.default_rng(23)
    nk = 1000
    vals = 1.0 + rng.permutation(200) * np.spacing(1.0)
    keys = np.full(200, 7)
    keys = np.concatenate([keys, rng.integers(0, nk, 5000)])
    vals = np.concatenate([vals, rng.standard_normal(5000)])
    g = kd.GroupedTDigest(nk, 100.0, scale=kd.K1)
    g.add_batch(keys, vals)
    refs = [oracle.Digest(oracle.K1, 100.0, 0.0) for _ in range(nk)]
    oracle.grouped_add_batch(refs, keys, vals)
    for k in [7] + list(range(0, nk, 97)):
        gm, gw = g.centroids(k)
        om, ow = refs[k].centroids()
        assert np.array_equal(gm, om) and np.array_equal(gw, ow)


@pytest.mark.parametrize("scale", [0, 1, 2, 3])
def test_grouped_filter_matches_exact_path(kd, scale):
    """Grouped ingest (integral weights) with the FP32 bucket filter gives the
    same digests as every id evaluated in FP64."""
    nk, n = 3000, 200000
    rng = np.random.default_rng(31 + scale)
    batches = [(rng.zipf(1.15, n) % nk, rng.standard_normal(n) * 5 + rng.integers(0, 3, n))
               for _ in range(3)]
    out = []
    for exact in (0, 1):
        s = kd.GpuSession()
        s.set_option(1, exact)  # KD_OPT_FORCE_EXACT_K
        g = kd.GroupedTDigest(nk, 100.0, scale=scale, session=s)
        for k, v in batches:
            g.add_batch(k, v)
        out.append(g)
    assert np.array_equal(out[0].centroid_counts(), out[1].centroid_counts())
    for k in range(0, nk, 41):
        ma, wa = out[0].centroids(k)
        mb, wb = out[1].centroids(k)
        assert np.array_equal(ma, mb) and np.array_equal(wa, wb)


def test_ingest_from_pinned_host_buffers(kd):
    """Pinned host inputs are read in place by the kernels; pageable ones are
    staged; device pointers are used as they are: the same digests."""
    torch = pytest.importorskip("torch")
    from kdigest_gb300 import _native as N

    nk, n = 777, 300000
    rng = np.random.default_rng(41)
    k = (rng.zipf(1.2, n) % nk).astype(np.uint32)
    v = rng.standard_normal(n) * 4
    pk = torch.from_numpy(k.view(np.int32)).pin_memory()
    pv = torch.from_numpy(v).pin_memory()
    dk = pk.cuda()
    dv = pv.cuda()
    L = N.load()
    stores = []
    for mode in ("pinned", "pageable", "device"):
        g = kd.GroupedTDigest(nk, 100.0, scale=kd.K2)
        for _ in range(2):
            if mode == "pinned":
                rc = L.kd_store_ingest(g._store._h, pk.data_ptr(), pv.data_ptr(), n, 0, 0.0, 0)
            elif mode == "pageable":
                rc = L.kd_store_ingest(g._store._h, N.ptr(k), N.ptr(v), n, 0, 0.0, 0)
            else:
                torch.cuda.synchronize()
                rc = L.kd_store_ingest(g._store._h, dk.data_ptr(), dv.data_ptr(), n, 0, 0.0,
                                       N.KD_PTR_DEVICE)
            assert rc == 0
        stores.append(g)
    for g in stores[1:]:
        assert np.array_equal(g.centroid_counts(), stores[0].centroid_counts())
        for key in range(0, nk, 37):
            ma, wa = g.centroids(key)
            mb, wb = stores[0].centroids(key)
            assert np.array_equal(ma, mb) and np.array_equal(wa, wb)
