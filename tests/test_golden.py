"""The CPU oracle against the committed reference-association fixtures
(tests/golden/reference_order.npz, written by tests/golden/make_golden.py from
the seeded inputs of tests/golden/gen.py).

- In the reference association the oracle reproduces every fixture bit for
  bit (ids, counts, centroids, states, quantiles, cdf).
- In the kernels' association (the default) ids, counts, weights and states
  are identical and means, quantiles and cdf agree within the bounds set for
  summation order: 1e-12 relative for centroids, 1e-9 for queries.
- With the C library's log / asin in place of the shared FP64 functions, the
  bucket ids do not change on these cases.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import gen  # noqa: E402

FIX = os.path.join(HERE, "golden", "reference_order.npz")


@pytest.fixture(scope="module")
def fx():
    return dict(np.load(FIX))


def _rel(a, b, floor):
    return np.abs(a - b) / np.maximum(np.maximum(np.abs(b), floor), 1e-300)


def _digest_outputs(o, xs_by_case=None):
    out = {}
    for c, (scale, comp, lam, nb, bsz) in enumerate(gen.DECAY_DIGESTS):
        d = o.Digest(scale, comp, lam)
        for v in gen.decay_digest_batches(c):
            d.add_batch_p(v)
        xs = xs_by_case[c]
        out[f"decay_{c}"] = ([d], xs)
    scale, comp, lam, nk = gen.GROUPED_TIME
    ds = [o.Digest(scale, comp, lam) for _ in range(nk)]
    for keys, vals, t in gen.grouped_time_batches():
        o.grouped_add_batch(ds, keys, vals, mode=1, timestamp=t)
    out["gtime"] = (ds, None)
    scale, comp, lam, nk = gen.GROUPED_K3
    ds = [o.Digest(scale, comp, lam) for _ in range(nk)]
    for keys, vals in gen.grouped_k3_batches():
        o.grouped_add_batch(ds, keys, vals)
    out["gk3"] = (ds, None)
    return out


def _check_digests(o, fx, exact):
    xs = {c: fx[f"decay_{c}_x"] for c in range(len(gen.DECAY_DIGESTS))}
    for t, (ds, x) in _digest_outputs(o, xs).items():
        counts = np.array([len(d) for d in ds])
        assert np.array_equal(counts, fx[t + "_counts"]), t
        m = np.concatenate([d.centroids()[0] for d in ds])
        w = np.concatenate([d.centroids()[1] for d in ds])
        assert np.array_equal(w, fx[t + "_cw"]), t
        st = np.array([[d.state()[k] for k in ("log_scale", "clock", "stored_total", "min", "max")] for d in ds])
        assert np.array_equal(st, fx[t + "_state"]), t
        q = np.array([[d.quantile(float(v)) if len(d) else np.nan for v in gen.QS] for d in ds])
        if exact:
            assert np.array_equal(m, fx[t + "_m"]), t
            assert np.array_equal(q, fx[t + "_q"], equal_nan=True), t
        else:
            span = np.max(np.abs(fx[t + "_m"]))
            assert np.all(_rel(m, fx[t + "_m"], 0.0) < 1e-12) or np.all(np.abs(m - fx[t + "_m"]) < 1e-12 * span), t
            ok = ~np.isnan(fx[t + "_q"])
            assert np.all(_rel(q[ok], fx[t + "_q"][ok], span) < 1e-9), t
        if x is not None:
            c = np.array([[d.cdf(float(v)) for v in x] for d in ds])
            if exact:
                assert np.array_equal(c, fx[t + "_cdf"]), t
            else:
                assert np.all(np.abs(c - fx[t + "_cdf"]) < 1e-9), t


def test_fixture_cases_are_reproducible():
    a = gen.tile_cases()
    b = gen.tile_cases()
    assert all(np.array_equal(u[3], v[3]) and np.array_equal(u[4], v[4]) for u, v in zip(a, b))


def test_oracle_reference_association_reproduces_fixtures(oracle, fx):
    with oracle.sums_mode(oracle.SUMS_REFERENCE):
        for i, (scale, comp, kind, x, w) in enumerate(gen.tile_cases()):
            m, cw, ids = oracle.tile_compress(scale, comp, x, w)
            assert np.array_equal(ids, fx[f"tile_{i}_ids"]), i
            assert np.array_equal(m, fx[f"tile_{i}_m"]) and np.array_equal(cw, fx[f"tile_{i}_cw"]), i
            lm, lw, lids = oracle.tile_compress_literal(scale, comp, x, w)
            assert np.array_equal(lids, ids) and np.array_equal(lm, m) and np.array_equal(lw, cw), i
        _check_digests(oracle, fx, exact=True)


def test_oracle_kernel_association_within_bounds(oracle, fx):
    for i, (scale, comp, kind, x, w) in enumerate(gen.tile_cases()):
        m, cw, ids = oracle.tile_compress(scale, comp, x, w)
        assert np.array_equal(ids, fx[f"tile_{i}_ids"]) and np.array_equal(cw, fx[f"tile_{i}_cw"]), i
        span = np.max(np.abs(x))
        assert np.all(np.abs(m - fx[f"tile_{i}_m"]) <= 1e-12 * np.maximum(np.abs(fx[f"tile_{i}_m"]), span)), i
    _check_digests(oracle, fx, exact=False)


def test_libm_transcendentals_change_no_bucket_id(oracle, fx):
    with oracle.math_mode(oracle.MATH_LIBM), oracle.sums_mode(oracle.SUMS_REFERENCE):
        for i, (scale, comp, kind, x, w) in enumerate(gen.tile_cases()):
            _, cw, ids = oracle.tile_compress(scale, comp, x, w)
            assert np.array_equal(ids, fx[f"tile_{i}_ids"]), i
        xs = {c: fx[f"decay_{c}_x"] for c in range(len(gen.DECAY_DIGESTS))}
        for t, (ds, _) in _digest_outputs(oracle, xs).items():
            assert np.array_equal(np.array([len(d) for d in ds]), fx[t + "_counts"]), t
            w = np.concatenate([d.centroids()[1] for d in ds])
            assert np.array_equal(w, fx[t + "_cw"]), t
