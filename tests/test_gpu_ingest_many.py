"""Multi-batch ingest (kd_store_ingest_many / GroupedTDigest.add_batches): the
sort of each batch overlaps the compress of the one before, and the store
must end exactly as after one add_batch per batch, in order.  Covered: device
tensors, pinned and pageable host arrays, decay, batches that need the full
sort or more hierarchy levels in the middle of a sequence (retried one call
at a time), a failing batch (earlier batches stay applied, later ones do not),
the time clock through the C ABI, and parity with the oracle."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b, nk, keys=None):
    assert np.array_equal(a.centroid_counts(), b.centroid_counts())
    for k in keys if keys is not None else range(0, nk, max(1, nk // 41)):
        ma, wa = a.centroids(k)
        mb, wb = b.centroids(k)
        assert np.array_equal(ma, mb) and np.array_equal(wa, wb), f"key {k}"
        assert a.state(k) == b.state(k), f"key {k}"


def _batches(nk, sizes, seed, zipf=1.2):
    rng = np.random.default_rng(seed)
    out = []
    for n in sizes:
        k = ((rng.zipf(zipf, n) - 1) % nk).astype(np.uint32)
        v = rng.standard_normal(n) * (1 + k % 5) + k % 13
        out.append((k, v))
    return out


def _pair(kd, nk, decay=None, scale=None):
    scale = kd.K3 if scale is None else scale
    a = kd.GroupedTDigest(nk, 100.0, decay=decay, scale=scale, session=kd.GpuSession())
    b = kd.GroupedTDigest(nk, 100.0, decay=decay, scale=scale, session=kd.GpuSession())
    return a, b


@pytest.mark.parametrize("decay", [None, 2000.0])
def test_device_batches_equal_one_call_each(kd, decay):
    import torch

    nk = 3000
    dec = None if decay is None else kd.Decay.half_life(decay)
    a, b = _pair(kd, nk, dec)
    batches = _batches(nk, [50000, 20000, 0, 70000, 1000, 50000, 33333, 2], 5)
    dev = [(torch.from_numpy(k).cuda(), torch.from_numpy(v).cuda()) for k, v in batches]
    a.add_batches(dev)
    for k, v in batches:
        if len(v):
            b.add_batch(k, v)
    _same(a, b, nk)
    a.add_batches(dev[:3])  # a second call on the same store and session
    for k, v in batches[:3]:
        if len(v):
            b.add_batch(k, v)
    _same(a, b, nk)


def test_host_batches_pinned_and_pageable(kd):
    import torch

    nk = 500
    a, b = _pair(kd, nk)
    batches = _batches(nk, [8000, 9000, 7000, 12000], 9)
    pinned = [(torch.from_numpy(k.astype(np.int32)).pin_memory().numpy().view(np.uint32),
               torch.from_numpy(v).pin_memory().numpy()) for k, v in batches]
    a.add_batches(pinned)
    a.add_batches(batches)  # pageable: staged by the copy engine too
    for _ in range(2):
        for k, v in batches:
            b.add_batch(k, v)
    _same(a, b, nk)


def test_matches_oracle(kd, oracle):
    import torch

    nk = 40
    g = kd.GroupedTDigest(nk, 100.0, scale=kd.K2)
    refs = [oracle.Digest(oracle.K2, 100.0, 0.0) for _ in range(nk)]
    batches = _batches(nk, [3000, 5000, 4000, 6000, 2500], 13, zipf=1.5)
    g.add_batches([(torch.from_numpy(k).cuda(), torch.from_numpy(v).cuda()) for k, v in batches])
    for k, v in batches:
        oracle.grouped_add_batch(refs, k, v)
    for k in range(nk):
        m, w = g.centroids(k)
        rm, rw = refs[k].centroids()
        assert np.array_equal(m, rm) and np.array_equal(w, rw), f"key {k}"


def test_full_sort_and_more_levels_in_the_middle(kd):
    """Batch 2 holds an inversion the packed sort leaves (full sort), and a
    fresh store's first heavy batches need more levels than planned: those
    batches are retried one call at a time and the rest stay pipelined."""
    import torch

    nk = 64
    a, b = _pair(kd, nk, scale=kd.K2)
    rng = np.random.default_rng(17)
    base = rng.standard_normal(2000) * 10
    ulp = np.spacing(np.abs(base))
    inv_k = np.repeat(rng.integers(0, nk, 2000), 2).astype(np.uint32)
    inv_v = np.stack([base + 3 * ulp, base], axis=1).reshape(-1)
    heavy = [(np.zeros(300000, np.uint32), rng.standard_normal(300000)),
             ((np.arange(200000) % 3).astype(np.uint32), rng.standard_normal(200000))]
    batches = heavy + [(inv_k, inv_v)] + _batches(nk, [40000, 40000], 3)
    a.add_batches([(torch.from_numpy(k).cuda(), torch.from_numpy(v).cuda()) for k, v in batches])
    for k, v in batches:
        b.add_batch(k, v)
    _same(a, b, nk, keys=range(nk))


def test_failing_batch_keeps_earlier_ones(kd):
    import torch

    nk = 1000
    a, b = _pair(kd, nk)
    batches = _batches(nk, [20000, 20000, 20000, 20000], 21)
    bad_k = batches[2][0].copy()
    bad_k[777] = 1010  # above the store's keys, below 2^10: only the device sees it
    dev = [(torch.from_numpy(k).cuda(), torch.from_numpy(v).cuda()) for k, v in batches]
    dev[2] = (torch.from_numpy(bad_k).cuda(), dev[2][1])
    with pytest.raises(Exception) as ei:
        a.add_batches(dev)
    assert "batch 2" in str(ei.value)
    for k, v in batches[:2]:
        b.add_batch(k, v)
    _same(a, b, nk)
    # host arrays: the bad batch is caught on the host, the ones before it apply
    host = list(batches)
    host[1] = (bad_k, batches[1][1])
    with pytest.raises(IndexError):
        a.add_batches(host)
    b.add_batch(*batches[0])
    _same(a, b, nk)


def test_time_clock_through_the_c_abi(kd):
    import kdigest_gb300._native as N
    import torch

    nk = 200
    lam = np.log(2.0) / 50.0
    a, b = _pair(kd, nk, kd.Decay.rate(lam))
    batches = _batches(nk, [5000, 6000, 7000], 31)
    ts = [10.0, 10.0, 42.5]
    keep = [(torch.from_numpy(k).cuda(), torch.from_numpy(v).cuda()) for k, v in batches]
    nb = len(keep)
    kp = (ctypes.c_void_p * nb)(*[k.data_ptr() for k, _ in keep])
    vp = (ctypes.c_void_p * nb)(*[v.data_ptr() for _, v in keep])
    ns = (ctypes.c_int64 * nb)(*[len(v) for _, v in keep])
    tsa = (ctypes.c_double * nb)(*ts)
    done = ctypes.c_int64(-1)
    rc = N.load().kd_store_ingest_many(a._store._h, nb, kp, vp, ns, N.KD_CLOCK_TIME, tsa,
                                       N.KD_PTR_DEVICE, ctypes.byref(done))
    assert rc == 0 and done.value == nb
    for (k, v), t in zip(batches, ts):
        b.add_batch_at(k, v, t)
    _same(a, b, nk)


def test_single_digest_batches(kd):
    """TDigest.add_batches equals add_batch_p per batch, with decay, and after
    single-sample adds (the buffer is carried into the first batch)."""
    import torch

    rng = np.random.default_rng(41)
    vals = [rng.lognormal(0.0, 1.5, n) for n in (70000, 65536, 100000, 80000)]
    for pre in (0, 300):
        a = kd.TDigest(200.0, kd.K2, decay=kd.Decay.half_life(1e5), session=kd.GpuSession())
        b = kd.TDigest(200.0, kd.K2, decay=kd.Decay.half_life(1e5), session=kd.GpuSession())
        if pre:
            head = rng.standard_normal(pre)
            a.add_batch(head)
            b.add_batch(head)
        a.add_batches([torch.from_numpy(v).cuda() for v in vals])
        for v in vals:
            b.add_batch_p(v)
        ma, wa = a.centroids()
        mb, wb = b.centroids()
        assert np.array_equal(ma, mb) and np.array_equal(wa, wb), f"pre={pre}"
        assert a.state() == b.state()
        assert a.to_bytes() == b.to_bytes()


def test_two_stores_share_the_pipeline(kd):
    """Stores of one session take turns (they share the workspaces and the
    streams, each keeps its own graphs), with batch sizes that change between
    calls; every store equals its one-call-per-batch twin."""
    import torch

    sess = kd.GpuSession()
    ref_sess = kd.GpuSession()
    sizes = (700, 5000)
    stores = [kd.GroupedTDigest(k, 100.0, scale=kd.K1, session=sess) for k in sizes]
    refs = [kd.GroupedTDigest(k, 100.0, scale=kd.K1, session=ref_sess) for k in sizes]
    for rnd in range(3):
        for j, nk in enumerate(sizes):
            n = (30000, 8000, 30000)[rnd] + j
            batches = _batches(nk, [n] * (2 + rnd), 100 * rnd + j)
            stores[j].add_batches([(torch.from_numpy(k).cuda(), torch.from_numpy(v).cuda())
                                   for k, v in batches])
            for k, v in batches:
                refs[j].add_batch(k, v)
    for g, r, nk in zip(stores, refs, sizes):
        _same(g, r, nk)


@pytest.mark.parametrize("graphs,fronts", [(0, 2), (1, 1), (0, 1)])
def test_eager_and_one_front_stream(kd, graphs, fronts):
    """Graphs off (every part enqueued eagerly) and a single front stream give
    the same store as one call per batch."""
    import torch

    import kdigest_gb300._native as N

    nk = 900
    a, b = _pair(kd, nk)
    a._store.session.set_option(N.KD_OPT_GRAPHS, graphs)
    a._store.session.set_option(N.KD_OPT_FRONT_STREAMS, fronts)
    batches = _batches(nk, [20000] * 5, 77 + graphs + 2 * fronts)
    a.add_batches([(torch.from_numpy(k).cuda(), torch.from_numpy(v).cuda()) for k, v in batches])
    for k, v in batches:
        b.add_batch(k, v)
    _same(a, b, nk)


def _min_budget(kd, nk, batch):
    """The smallest session budget (to 1 MiB) that holds a store of nk keys
    and one ingest of `batch`."""
    from kdigest_gb300 import _native as N

    lo, hi = 1 << 20, 8 << 30
    while hi - lo > (1 << 20):
        mid = (lo + hi) // 2
        try:
            g = kd.GroupedTDigest(nk, 100.0, scale=kd.K3, session=kd.GpuSession(mem_budget=mid))
            g.add_batch(*batch)
            hi = mid
        except (N.KdError, MemoryError):
            lo = mid
        finally:
            g = None
    return hi


def test_budget_without_room_for_the_pipeline(kd):
    """A session budget that fits the store and one ingest workspace but not
    the pipeline's two extra workspaces and staging buffers: add_batches falls
    back to one call per batch (device tensors, and host arrays) and ends
    exactly where one add_batch per batch ends."""
    import torch

    nk = 500
    batches = _batches(nk, [120000] * 4, 77)
    budget = _min_budget(kd, nk, batches[0]) + (2 << 20)
    b = kd.GroupedTDigest(nk, 100.0, scale=kd.K3, session=kd.GpuSession())
    for k, v in batches:
        b.add_batch(k, v)
    a = kd.GroupedTDigest(nk, 100.0, scale=kd.K3, session=kd.GpuSession(mem_budget=budget))
    dev = [(torch.from_numpy(k).cuda(), torch.from_numpy(v).cuda()) for k, v in batches]
    a.add_batches(dev)
    _same(a, b, nk, keys=range(nk))
    c = kd.GroupedTDigest(nk, 100.0, scale=kd.K3, session=kd.GpuSession(mem_budget=budget))
    c.add_batches(batches)
    _same(c, b, nk, keys=range(nk))
