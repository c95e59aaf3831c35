"""The stateless entry points over caller-held centroid arrays against the
oracle and a literal statement of the reference's query kernels:

- kd_grouped_compress == per key, the oracle's P-path of (priors ++ new
  samples at the key's weight) (gpu/grouped.mojo:415-643), bit for bit, with
  the new samples' ranges;
- kd_quantile / kd_cdf == the reference kernels' serial walk
  (gpu/query.mojo:45-231), bit for bit, plus their error cases;
- kd_merge == the oracle's P-path of the concatenated parts
  (gpu/query.mojo:348-369);
- kd_store_query_batch == kd_store_quantile + kd_store_cdf, eager and replayed
  from its graph."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ref_quantile(m, w, q, mn, mx):
    """gpu/query.mojo:45-135 in float64, operation by operation."""
    nc = len(m)
    n = 0.0
    for x in w:
        n += x
    if n <= 0.0:
        n = 1.0
    if nc == 1:
        return m[0]
    if q <= 0.0:
        return mn
    if q >= 1.0:
        return mx
    target = q * n
    first_half = w[0] / 2.0
    if target < first_half:
        return mn if w[0] <= 1.0 + 1e-6 else mn + (m[0] - mn) * (target / first_half)
    last_half = w[-1] / 2.0
    if target > n - last_half:
        if w[-1] <= 1.0 + 1e-6:
            return mx
        return m[-1] + (mx - m[-1]) * ((target - (n - last_half)) / last_half)
    wsf = w[0] / 2.0
    for j in range(nc - 1):
        dw = (w[j] + w[j + 1]) / 2.0
        if target <= wsf + dw:
            return m[j] + (m[j + 1] - m[j]) * ((target - wsf) / dw)
        wsf += dw
    return m[-1]


def _ref_cdf(m, w, x, mn, mx):
    """gpu/query.mojo:138-231 in float64."""
    nc = len(m)
    n = 0.0
    for v in w:
        n += v
    if n <= 0.0:
        n = 1.0
    if x < mn:
        return 0.0
    if x > mx:
        return 1.0
    if nc == 1:
        return 0.0 if x < m[0] else (1.0 if x > m[0] else 0.5)
    if x < m[0]:
        if mn == m[0]:
            return 0.0
        return (w[0] / 2.0) * ((x - mn) / (m[0] - mn)) / n
    if x > m[-1]:
        if mx == m[-1]:
            return 1.0
        frac = (x - m[-1]) / (mx - m[-1])
        return (n - w[-1] / 2.0 + (w[-1] / 2.0) * frac) / n
    wsf = w[0] / 2.0
    for j in range(nc - 1):
        if x <= m[j + 1]:
            dw = (w[j] + w[j + 1]) / 2.0
            if m[j + 1] == m[j]:
                return (wsf + dw / 2.0) / n
            return (wsf + dw * ((x - m[j]) / (m[j + 1] - m[j]))) / n
        wsf += (w[j] + w[j + 1]) / 2.0
    return 1.0


def _digests(rng, count):
    ms, ws = [], []
    for i in range(count):
        nc = [1, 2, 3, 50, 300, 1024][i % 6]
        m = np.sort(rng.standard_normal(nc) * 5)
        if i % 4 == 0:
            m = np.round(m)  # equal means
        w = rng.random(nc) * 20 + 0.5 if i % 3 else np.ones(nc)
        if i % 5 == 2:
            w[0] = 1.0 + 5e-7  # a singleton tail by the kernels' raw test
            w[-1] = 1.0
        ms.append(m)
        ws.append(w)
    mins = np.array([m[0] - abs(m[0]) * 0.1 - (0.0 if i % 7 else 0.0) for i, m in enumerate(ms)])
    maxs = np.array([m[-1] + 1.0 for m in ms])
    mins[3] = ms[3][0]  # min equal to the first mean
    return ms, ws, mins, maxs


def test_quantile_and_cdf_match_reference_kernels(kd):
    rng = np.random.default_rng(11)
    ms, ws, mins, maxs = _digests(rng, 30)
    nd = len(ms)
    nq = 6000
    ids = rng.integers(0, nd, nq).astype(np.uint32)
    qs = np.concatenate([rng.random(nq - 40), [0.0, 1.0, -0.5, 1.5], 10 ** rng.uniform(-7, -1, 36)])
    xs = np.array([rng.uniform(mins[i] - 1, maxs[i] + 1) for i in ids])
    xs[:30] = [ms[ids[i]][0] for i in range(30)]  # exactly on centroid means
    got_q = kd.gpu_quantile_many(ms, ws, mins, maxs, ids, qs)
    got_c = kd.gpu_cdf_many(ms, ws, mins, maxs, ids, xs)
    for i in range(nq):
        d = ids[i]
        assert got_q[i] == _ref_quantile(ms[d], ws[d], qs[i], mins[d], maxs[d]), i
        assert got_c[i] == _ref_cdf(ms[d], ws[d], xs[i], mins[d], maxs[d]), i
    # the single-digest forms
    one = kd.gpu_quantile(ms[4], ws[4], qs[:100], mins[4], maxs[4])
    assert all(one[i] == _ref_quantile(ms[4], ws[4], qs[i], mins[4], maxs[4]) for i in range(100))


def test_query_errors(kd):
    ms = [np.array([1.0, 2.0]), np.array([]), np.arange(1025, dtype=np.float64)]
    ws = [np.array([1.0, 1.0]), np.array([]), np.ones(1025)]
    mins, maxs = np.array([0.0, 0.0, 0.0]), np.array([3.0, 3.0, 2000.0])
    with pytest.raises(ValueError, match="empty"):
        kd.gpu_quantile_many(ms, ws, mins, maxs, np.array([0, 1], np.uint32), np.array([0.5, 0.5]))
    with pytest.raises(kd.KdError) as ei:
        kd.gpu_cdf_many(ms, ws, mins, maxs, np.array([2], np.uint32), np.array([3.0]))
    assert ei.value.code == 3
    with pytest.raises(ValueError):
        kd.gpu_quantile_many(ms, ws, mins, maxs, np.array([7], np.uint32), np.array([0.5]))


@pytest.mark.parametrize("scale", [1, 2, 3])
def test_grouped_compress_matches_oracle(kd, oracle, scale):
    rng = np.random.default_rng(100 + scale)
    nk = 40
    n = 30000
    keys = np.minimum(rng.zipf(1.3, n) - 1, nk - 1).astype(np.uint32)
    keys[keys == 7] = 8  # key 7: priors only (re-compressed); key 9: nothing
    keys[keys == 9] = 10
    vals = rng.standard_normal(n) * (1 + keys % 4)
    vals[::50] = np.round(vals[::50])
    new_w = np.exp(rng.uniform(0, 20, nk))
    new_w[::3] = 1.0
    pm, pw = [], []
    for k in range(nk):
        c = 0 if k in (9, 11) else int(rng.integers(1, 300))
        pm.append(np.sort(rng.standard_normal(c) * 2))
        pw.append(rng.random(c) * 50 + 0.1)
    pm[12] = np.round(pm[12])  # priors tied with new samples
    vals[keys == 12] = np.round(vals[keys == 12])
    gm, gw, mins, maxs = kd.gpu_grouped_compress_weighted(keys, vals, new_w, pm, pw, nk, 100.0, scale)
    for k in range(nk):
        nv = vals[keys == k]
        m = np.concatenate([pm[k], nv])
        w = np.concatenate([pw[k], np.full(len(nv), new_w[k])])
        if len(m) == 0:
            assert len(gm[k]) == 0
            continue
        om, ow = oracle.ppath_compress(scale, 100.0, m, w)
        assert np.array_equal(gm[k], om) and np.array_equal(gw[k], ow), k
        if len(nv):
            assert mins[k] == nv.min() and maxs[k] == nv.max()
        else:
            assert mins[k] == 0.0 and maxs[k] == 0.0
    assert len(gm[9]) == 0 and len(gm[7]) > 0


def test_grouped_compress_validates_first(kd):
    with pytest.raises(ValueError):
        kd.gpu_grouped_compress_weighted(np.array([0, 5], np.uint32), np.array([1.0, 2.0]), None,
                                         [[], []], [[], []], 2, 100.0)
    with pytest.raises(ValueError):
        kd.gpu_grouped_compress_weighted(np.array([0, 1], np.uint32), np.array([1.0, math.inf]), None,
                                         [[], []], [[], []], 2, 100.0)


def test_merge_matches_oracle(kd, oracle):
    rng = np.random.default_rng(55)
    parts_m, parts_w = [], []
    for p in range(96):
        c = int(rng.integers(0, 400))
        parts_m.append(np.sort(rng.standard_normal(c) + p % 5))
        parts_w.append(rng.random(c) * 10 + 1)
    go = np.array([0, 32, 33, 33, 96])
    gm, gw = kd.gpu_merge_digests(parts_m, parts_w, 200.0, kd.K2, group_offsets=go)
    for g in range(4):
        m = np.concatenate(parts_m[go[g]:go[g + 1]]) if go[g + 1] > go[g] else np.array([])
        w = np.concatenate(parts_w[go[g]:go[g + 1]]) if go[g + 1] > go[g] else np.array([])
        if len(m) == 0:
            assert len(gm[g]) == 0
            continue
        om, ow = oracle.ppath_compress(oracle.K2, 200.0, m, w)
        assert np.array_equal(gm[g], om) and np.array_equal(gw[g], ow), g
    m1, w1 = kd.gpu_merge_digests(parts_m[:10], parts_w[:10], 100.0, kd.K1)
    om, ow = oracle.ppath_compress(oracle.K1, 100.0, np.concatenate(parts_m[:10]), np.concatenate(parts_w[:10]))
    assert np.array_equal(m1, om) and np.array_equal(w1, ow)


def test_query_batch_one_launch_equals_two_calls(kd):
    import torch

    rng = np.random.default_rng(3)
    nk = 500
    g = kd.GroupedTDigest(nk, 100.0, scale=kd.K2, session=kd.GpuSession())
    keys = rng.integers(0, nk, 200000).astype(np.uint32)
    g.add_batch(keys, rng.standard_normal(200000))
    qk = rng.integers(0, nk, 50000).astype(np.uint32)
    qs = rng.random(50000)
    ck = rng.integers(0, nk, 30000).astype(np.uint32)
    xs = rng.standard_normal(30000)
    eq, ec = g.quantiles(qk, qs), g.cdfs(ck, xs)
    hq, hc = g.query_batch(qk, qs, ck, xs)
    assert np.array_equal(hq, eq) and np.array_equal(hc, ec)
    dev = [torch.from_numpy(a).cuda() for a in (qk.view(np.int32), qs, ck.view(np.int32), xs)]
    qo = torch.empty_like(dev[1])
    co = torch.empty_like(dev[3])
    from kdigest_gb300 import _native as N

    L = N.load()
    for rep in range(4):  # eager, then captured, then replayed
        qo.fill_(np.nan)
        co.fill_(np.nan)
        torch.cuda.synchronize()
        rc = L.kd_store_query_batch(g._store._h, dev[0].data_ptr(), dev[1].data_ptr(), 50000,
                                    qo.data_ptr(), dev[2].data_ptr(), dev[3].data_ptr(), 30000,
                                    co.data_ptr(), N.KD_PTR_DEVICE)
        assert rc == 0
        assert np.array_equal(qo.cpu().numpy(), eq) and np.array_equal(co.cpu().numpy(), ec), rep


@pytest.mark.parametrize("nk,decay", [(1024, False), (300, True)])
def test_query_batch_many_queries_per_digest(kd, nk, decay):
    """A batch of hundreds of queries per digest in one launch gives the same
    bits as the per-call queries, for interior points, both tails, q = 0 and 1,
    x outside the range, ties and decayed (singleton-tested) digests."""
    rng = np.random.default_rng(nk)
    dec = kd.Decay.half_life(5e4) if decay else None
    g = kd.GroupedTDigest(nk, 100.0, scale=kd.K2, decay=dec, session=kd.GpuSession())
    for _ in range(3):
        keys = rng.integers(0, nk, 200000).astype(np.uint32)
        vals = np.round(rng.standard_normal(200000) * 4) / 4  # ties
        g.add_batch(keys, vals)
    g.add_batch(np.arange(nk, dtype=np.uint32), rng.standard_normal(nk) * 10)
    n = 280000
    qk = rng.integers(0, nk, n).astype(np.uint32)
    qs = np.concatenate([rng.random(n - 6), [0.0, 1.0, 1e-12, 1 - 1e-12, 0.5, 5e-7]])
    ck = rng.integers(0, nk, n).astype(np.uint32)
    xs = np.concatenate([rng.standard_normal(n - 4) * 5, [-1e9, 1e9, 0.0, 0.25]])
    hq, hc = g.query_batch(qk, qs, ck, xs)
    eq, ec = g.quantiles(qk, qs), g.cdfs(ck, xs)
    assert np.array_equal(hq.view(np.uint64), eq.view(np.uint64))
    assert np.array_equal(hc.view(np.uint64), ec.view(np.uint64))


def test_query_batch_empty_digest_reported(kd):
    rng = np.random.default_rng(9)
    g = kd.GroupedTDigest(512, 100.0, scale=kd.K1, session=kd.GpuSession())
    g.add_batch(rng.integers(0, 511, 100000).astype(np.uint32), rng.standard_normal(100000))  # key 511 stays empty
    n = 140000
    qk = rng.integers(0, 511, n).astype(np.uint32)
    qk[n // 2] = 511
    with pytest.raises(ValueError, match="empty digest"):  # KD_EEMPTY, at the query that hit it
        g.query_batch(qk, rng.random(n), qk[:0], np.zeros(0))
