"""Serving loop: every request's result is the same alone and in the mix.

"In the mix": the requests are submitted back to back by a client while the
server batches them per window, runs the windows that closed together as one
group (one window's prep and sort beside the previous window's queries,
compress and commit) and overlaps the next group's copy with the current
group's compute.  "Alone": each query request is evaluated by itself
against the state its window defines, and each window's ingests are applied
as one batch, one step at a time with no server.  Results are compared bit for
bit (tolerance 0, inside the 1e-9 quantile/cdf tolerance), as is the final
state of every digest.
"""
import math
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NK = 400
LAMBDA = math.log(2.0) / 60.0  # 60 s half-life on the timestamp axis


def _trace(seed, n_req, gap, nk=NK):
    rng = np.random.default_rng(seed)
    ts = 0.002 + np.cumsum(rng.exponential(gap, n_req))
    reqs = []
    # the first request, alone in the first window, touches every key so that
    # no later query meets an empty digest
    reqs.append(("ingest", 0.0, np.arange(nk, dtype=np.uint32), rng.lognormal(0, 2, nk)))
    for t in ts:
        u = rng.random()
        if u < 0.7:
            n = int(min(2000, rng.lognormal(math.log(200), 1.0))) + 1
            keys = (rng.zipf(1.2, n) - 1) % nk
            reqs.append(("ingest", float(t), keys.astype(np.uint32), rng.lognormal(0, 2, n)))
        elif u < 0.85:
            n = int(rng.integers(1, 40))
            qs = np.where(rng.random(n) < 0.5, rng.random(n), 10 ** rng.uniform(-6, -2, n))
            reqs.append(("quantile", float(t), rng.integers(0, nk, n).astype(np.uint32), qs))
        else:
            n = int(rng.integers(1, 40))
            reqs.append(("cdf", float(t), rng.integers(0, nk, n).astype(np.uint32),
                         rng.lognormal(0, 2, n)))
    return reqs


def _store(kd):
    return kd.GroupedTDigest(NK, 200.0, decay=kd.Decay.rate(LAMBDA), scale=kd.K2,
                             session=kd.GpuSession())


def _device_budget(kd, g, extra):
    """A budget of `extra` bytes above the device memory the store's session
    holds when a server starts."""
    probe = kd.Server(g, window=1e-3)
    used = probe.memory()["in_use_bytes"]
    probe.close()
    return used + extra


def _serve(kd, reqs, window, budget=0):
    g = _store(kd)
    if budget:
        budget = _device_budget(kd, g, budget)
    srv = kd.Server(g, window=window, budget_bytes=budget)
    tickets = []
    for kind, t, k, v in reqs:
        if kind == "ingest":
            tickets.append(srv.submit_ingest(t, k, v))
        elif kind == "quantile":
            tickets.append(srv.submit_quantiles(t, k, v))
        else:
            tickets.append(srv.submit_cdfs(t, k, v))
    srv.flush()
    res = [srv.wait(tk, 30.0) for tk in tickets]
    stats = srv.stats()
    srv.close()
    return g, res, stats


def _alone(kd, reqs, window):
    """Window semantics executed step by step, each query request by itself."""
    g = _store(kd)
    res = []
    i = 0
    while i < len(reqs):
        w = math.floor(reqs[i][1] / window)
        j = i
        while j < len(reqs) and math.floor(reqs[j][1] / window) == w:
            j += 1
        ing_k, ing_v, ts = [], [], None
        for kind, t, k, v in reqs[i:j]:
            if kind == "ingest":
                ing_k.append(k)
                ing_v.append(v)
                ts = t
                res.append((0, None))
            else:
                out = g.quantiles(k, v) if kind == "quantile" else g.cdfs(k, v)
                res.append((0, out))
        if ing_k:
            g.add_batch_at(np.concatenate(ing_k), np.concatenate(ing_v), ts)
        i = j
    return g, res


def _compare(kd, ga, ra, gb, rb):
    assert len(ra) == len(rb)
    for (sa, oa), (sb, ob) in zip(ra, rb):
        assert sa == sb == 0
        if oa is None:
            assert ob is None
        else:
            assert np.array_equal(oa, ob)
    assert np.array_equal(ga.centroid_counts(), gb.centroid_counts())
    for k in range(0, NK, 7):
        ma, wa = ga.centroids(k)
        mb, wb = gb.centroids(k)
        assert np.array_equal(ma, mb) and np.array_equal(wa, wb)
        assert ga.state(k) == gb.state(k)


def test_results_same_alone_and_in_the_mix(kd):
    reqs = _trace(11, 600, 2e-4)
    window = 1e-3
    ga, ra, st = _serve(kd, reqs, window)
    gb, rb = _alone(kd, reqs, window)
    _compare(kd, ga, ra, gb, rb)
    assert st["completed"] == len(reqs)
    assert st["windows"] < len(reqs) // 2  # requests were batched
    # the client submits far faster than the windows are served, so closed
    # windows queue up and run in groups
    assert st["windows_grouped"] > 0 and st["groups"] < st["windows"]
    assert 0.0 < st["p50_s"] <= st["p99_s"] <= st["p999_s"]


def test_one_request_per_window_is_request_by_request(kd):
    reqs = _trace(12, 150, 1e-3)
    window = 1e-7  # gaps of ~1 ms: every request is alone in its window
    assert len({math.floor(t / window) for _, t, _, _ in reqs}) == len(reqs)
    ga, ra, _ = _serve(kd, reqs, window)
    gb = _store(kd)
    rb = []
    for kind, t, k, v in reqs:
        if kind == "ingest":
            gb.add_batch_at(k, v, t)
            rb.append((0, None))
        else:
            rb.append((0, gb.quantiles(k, v) if kind == "quantile" else gb.cdfs(k, v)))
    _compare(kd, ga, ra, gb, rb)


def test_budget_backpressure_keeps_results(kd):
    reqs = _trace(13, 300, 2e-4)
    window = 1e-3
    # the largest window's footprint is about 0.32 MB: at most two windows at a time
    ga, ra, _ = _serve(kd, reqs, window, budget=500_000)
    gb, rb = _alone(kd, reqs, window)
    _compare(kd, ga, ra, gb, rb)


def test_retry_inside_a_window_group(kd):
    """A window whose batch needs the full sort (more than 64 values of one key
    that agree in every sorted bit, out of order) is retried by itself inside
    its group; the later windows of the group run again, queries included, on
    the retried store.  Every result is still the same as alone."""
    rng = np.random.default_rng(15)
    reqs = [("ingest", 0.0, np.arange(NK, dtype=np.uint32), rng.lognormal(0, 2, NK))]
    for w in range(40):
        t = 0.0021 + w * 1e-3
        k = int(rng.integers(0, NK))
        base = 1.0 + float(rng.integers(0, 1 << 20)) * 2.0 ** -20  # low 32 significand bits zero
        tied = base + rng.permutation(100) * 2.0 ** -52              # differ in the lowest 7 bits
        reqs.append(("ingest", t, np.full(100, k, np.uint32), tied))
        reqs.append(("ingest", t + 1e-5, rng.integers(0, NK, 500).astype(np.uint32),
                     rng.lognormal(0, 2, 500)))
        reqs.append(("quantile", t + 2e-5, rng.integers(0, NK, 20).astype(np.uint32), rng.random(20)))
        reqs.append(("cdf", t + 3e-5, rng.integers(0, NK, 20).astype(np.uint32),
                     rng.lognormal(0, 2, 20)))
    window = 1e-3
    ga, ra, st = _serve(kd, reqs, window)
    gb, rb = _alone(kd, reqs, window)
    _compare(kd, ga, ra, gb, rb)
    assert st["windows_grouped"] > 0  # full-sort windows keep the worker behind the client


def test_failed_windows_report_and_the_server_recovers(kd):
    """With every sort's look-back made to run out (the test-only session
    option), each window's ingest fails with KD_ETIMEOUT: every request of
    those windows completes with that status (none hangs), whether the
    windows ran alone or grouped, and the store stays as the last good window
    left it.  With the option cleared the server serves new windows, and the
    store equals one that never saw the failed windows."""
    from kdigest_gb300 import _native as N

    rng = np.random.default_rng(21)
    g = _store(kd)
    sess = g.session
    srv = kd.Server(g, window=1e-3)
    first = rng.lognormal(0, 2, NK)
    t0 = srv.submit_ingest(0.0, np.arange(NK, dtype=np.uint32), first)
    srv.flush()
    assert srv.wait(t0, 30.0)[0] == 0
    sess.set_option(N.KD_OPT_TEST_WAIT, 2000)
    tickets = []
    for w in range(6):
        t = 0.0105 + w * 1e-3
        keys = rng.integers(0, NK, 20000).astype(np.uint32)  # several sort tiles
        tickets.append(srv.submit_ingest(t, keys, rng.lognormal(0, 2, 20000)))
        tickets.append(srv.submit_quantiles(t + 1e-4, keys[:10], rng.random(10)))
    srv.flush()
    assert [srv.wait(tk, 60.0)[0] for tk in tickets] == [N.KD_ETIMEOUT] * len(tickets)
    sess.set_option(N.KD_OPT_TEST_WAIT, 0)
    keys = rng.integers(0, NK, 20000).astype(np.uint32)
    vals = rng.lognormal(0, 2, 20000)
    t1 = srv.submit_ingest(0.05, keys, vals)
    srv.flush()
    assert srv.wait(t1, 30.0)[0] == 0
    srv.close()
    ref = _store(kd)
    ref.add_batch_at(np.arange(NK, dtype=np.uint32), first, 0.0)
    ref.add_batch_at(keys, vals, 0.05)
    assert np.array_equal(g.centroid_counts(), ref.centroid_counts())
    for k in range(0, NK, 5):
        ma, wa = g.centroids(k)
        mb, wb = ref.centroids(k)
        assert np.array_equal(ma, mb) and np.array_equal(wa, wb), k
        assert g.state(k) == ref.state(k)


def test_concurrent_waiters(kd):
    """Waiters on other threads see their own results while the client submits."""
    reqs = _trace(14, 200, 2e-4)
    window = 1e-3
    g = _store(kd)
    srv = kd.Server(g, window=window)
    results = {}

    def waiter(tk):
        results[tk] = srv.wait(tk, 30.0)

    threads = []
    for kind, t, k, v in reqs:
        if kind == "ingest":
            tk = srv.submit_ingest(t, k, v)
        elif kind == "quantile":
            tk = srv.submit_quantiles(t, k, v)
        else:
            tk = srv.submit_cdfs(t, k, v)
        th = threading.Thread(target=waiter, args=(tk,))
        th.start()
        threads.append(th)
    srv.advance(reqs[-1][1] + 1.0)
    for th in threads:
        th.join(60)
    srv.close()
    assert len(results) == len(reqs) and all(s == 0 for s, _ in results.values())


def test_rejections_and_empty_digest(kd):
    from kdigest_gb300 import KdError

    g = _store(kd)
    srv = kd.Server(g, window=1e-3, budget_bytes=_device_budget(kd, g, 10_000))
    k = np.array([1, 2], dtype=np.uint32)
    with pytest.raises(KdError):
        srv.submit_ingest(0.5, np.array([NK], dtype=np.uint32), [1.0])  # key out of range
    with pytest.raises(KdError):
        srv.submit_ingest(0.5, k, [1.0, float("nan")])
    with pytest.raises(KdError):
        srv.submit_quantiles(0.5, k, [0.5, 1.5])
    with pytest.raises(KdError):
        srv.submit_ingest(0.5, np.zeros(2000, np.uint32), np.ones(2000))  # could not fit alone
    t0 = srv.submit_quantiles(0.5, k, [0.5, 0.5])  # empty digests
    t1 = srv.submit_ingest(0.6, k, [3.0, 4.0])
    with pytest.raises(KdError):
        srv.submit_ingest(0.4, k, [1.0, 1.0])  # timestamps must not decrease
    srv.advance(0.7)
    with pytest.raises(KdError):
        srv.submit_ingest(0.65, k, [1.0, 1.0])  # its window [0.650, 0.651) closed
    st0, out0 = srv.wait(t0, 30.0)
    st1, _ = srv.wait(t1, 30.0)
    assert st0 == 2 and np.isnan(out0).all()  # KD_EEMPTY
    assert st1 == 0
    t2 = srv.submit_quantiles(0.8, k, [0.5, 0.5])
    srv.flush()
    st2, out2 = srv.wait(t2, 30.0)
    assert st2 == 0 and np.array_equal(out2, [3.0, 4.0])
    # A window whose own requests fill the budget: the next request of that
    # window is refused (waiting could not help: the window closes only on a
    # later request); a request of a later window closes it and is admitted
    # once it drained.
    big = np.ones(60)
    t3 = srv.submit_ingest(0.9, np.zeros(60, np.uint32), big)
    with pytest.raises(KdError) as ei:
        srv.submit_ingest(0.9, np.ones(60, np.uint32), big)
    assert ei.value.code == 5  # KD_ENOMEM
    t4 = srv.submit_ingest(0.95, np.ones(60, np.uint32), big)
    srv.flush()
    assert srv.wait(t3, 30.0)[0] == 0 and srv.wait(t4, 30.0)[0] == 0
    srv.close()
