"""The GPU path against the committed reference-association fixtures
(tests/golden/reference_order.npz): bucket ids show up as centroid counts and
weights, which must equal the fixtures bit for bit, as must every digest's
state; centroid means agree within 1e-12 relative (summation order of
sum(w * x) only) and quantile / cdf answers within 1e-9 relative."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import gen  # noqa: E402

FIX = os.path.join(HERE, "golden", "reference_order.npz")
STATE = ("log_scale", "clock", "stored_total", "min", "max")


@pytest.fixture(scope="module")
def fx():
    return dict(np.load(FIX))


def _close(a, b, rel, span):
    return np.all(np.abs(a - b) <= rel * np.maximum(np.abs(b), span))


def test_tiles_match_reference_association(kd, fx):
    for i, (scale, comp, kind, x, w) in enumerate(gen.tile_cases()):
        m, cw = kd.compress(x, w, compression=comp, scale=scale)
        assert len(m) == len(fx[f"tile_{i}_m"]), (i, kind, len(x))
        assert np.array_equal(cw, fx[f"tile_{i}_cw"]), (i, kind, len(x))
        assert _close(m, fx[f"tile_{i}_m"], 1e-12, np.max(np.abs(x))), (i, kind, len(x))


@pytest.mark.parametrize("case", range(len(gen.DECAY_DIGESTS)))
def test_decayed_digest_matches_reference_association(kd, fx, case):
    scale, comp, lam, nb, bsz = gen.DECAY_DIGESTS[case]
    d = kd.TDigest(comp, scale, kd.Decay.rate(lam))
    for v in gen.decay_digest_batches(case):
        d.add_batch_p(v)
    t = f"decay_{case}"
    m, w = d.centroids()
    assert len(m) == fx[t + "_counts"][0]
    assert np.array_equal(w, fx[t + "_cw"])
    st = d.state()
    assert np.array_equal(np.array([st[k] for k in STATE]), fx[t + "_state"][0])
    span = np.max(np.abs(fx[t + "_m"]))
    assert _close(m, fx[t + "_m"], 1e-12, 0.0)
    q = np.array([d.quantile(float(v)) for v in gen.QS])
    assert _close(q, fx[t + "_q"][0], 1e-9, span)
    c = np.array([d.cdf(float(v)) for v in fx[t + "_x"]])
    assert np.all(np.abs(c - fx[t + "_cdf"][0]) <= 1e-9)


def _check_grouped(g, fx, t, nk):
    counts = g.centroid_counts()
    assert np.array_equal(counts.astype(np.int64), fx[t + "_counts"])
    ms, ws = [], []
    for k in range(nk):
        m, w = g.centroids(k)
        ms.append(m)
        ws.append(w)
        if counts[k]:
            st = g.state(k)
            assert np.array_equal(np.array([st[f] for f in STATE]), fx[t + "_state"][k]), k
    m, w = np.concatenate(ms), np.concatenate(ws)
    assert np.array_equal(w, fx[t + "_cw"])
    assert _close(m, fx[t + "_m"], 1e-12, 0.0)
    span = np.max(np.abs(fx[t + "_m"]))
    for k in range(nk):
        if counts[k]:
            q = np.array([g.quantile(k, float(v)) for v in gen.QS])
            assert _close(q, fx[t + "_q"][k], 1e-9, span), k


def test_grouped_time_decay_matches_reference_association(kd, fx):
    scale, comp, lam, nk = gen.GROUPED_TIME
    g = kd.GroupedTDigest(nk, comp, kd.Decay.rate(lam), scale=scale)
    for keys, vals, t in gen.grouped_time_batches():
        g.add_batch_at(keys, vals, t)
    _check_grouped(g, fx, "gtime", nk)


def test_grouped_k3_matches_reference_association(kd, fx):
    scale, comp, lam, nk = gen.GROUPED_K3
    g = kd.GroupedTDigest(nk, comp, scale=scale)
    for keys, vals in gen.grouped_k3_batches():
        g.add_batch(keys, vals)
    _check_grouped(g, fx, "gk3", nk)
