"""Integer-pipe FP64 helpers (division, halving, order keys) against the FP64
instructions they stand for, bit for bit, on the device.

The quantile and cdf kernels use these helpers in place of FP64 divisions,
multiplications by 0.5 and comparisons; a single differing bit would change a
query answer, so the operands cover the whole exponent range, both signs,
zeros, subnormals, infinities, NaN, powers of two, extreme significands and
quotients next to rounding ties.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def native(kd):
    from kdigest_gb300 import _native

    return _native


def _run(N, op, a, b=None):
    import torch

    da = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).cuda() if b is not None else None
    out = torch.empty_like(da)
    rc = N.load().kd_selftest_fp64(op, da.data_ptr(), db.data_ptr() if db is not None else None,
                                   len(a), out.data_ptr())
    assert rc == 0
    return out.cpu().numpy()


def _bits(x):
    return np.ascontiguousarray(x, dtype=np.float64).view(np.uint64)


def _operands(seed, n):
    rng = np.random.default_rng(seed)
    # uniformly random bit patterns (every exponent, both signs, NaN/inf/subnormal included)
    a = rng.integers(0, 2**64, n, dtype=np.uint64, endpoint=False).view(np.float64)
    b = rng.integers(0, 2**64, n, dtype=np.uint64, endpoint=False).view(np.float64)
    # moderate exponents (the fast path), and ratios as the queries see them
    c = rng.standard_normal(n) * np.exp(rng.uniform(-40, 40, n))
    d = rng.standard_normal(n) * np.exp(rng.uniform(-40, 40, n))
    e = rng.random(n)
    f = rng.random(n) + 1e-300
    special = np.array([0.0, -0.0, 1.0, -1.0, 2.0, 0.5, 3.0, 7.0, np.inf, -np.inf, np.nan,
                        5e-324, -5e-324, 2.2250738585072014e-308, 2.2250738585072009e-308,
                        1.7976931348623157e308, -1.7976931348623157e308, 1e-310, 1e300, 1e-300,
                        np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0), np.nextafter(2.0, 0.0),
                        1.0 + 2.0**-52 * 3, 0.1, 1.0 / 3.0])
    sa, sb = np.meshgrid(special, special)
    # significands at the extremes, and b with a = b * (1 + k ulp): quotients next to ties
    m = rng.integers(0, 2**52, n // 4, dtype=np.uint64)
    ext = np.concatenate([m | np.uint64(0xFFFFFFFFF0000), m & np.uint64(0xFFFF)])
    g = (ext | np.uint64(0x3FF0000000000000)).view(np.float64)
    h = (rng.integers(0, 2**52, len(g), dtype=np.uint64) | np.uint64(0x3FF0000000000000)).view(np.float64)
    k = rng.integers(-4, 5, n // 4)
    bt = 1.0 + rng.random(n // 4)
    at = bt * (1.0 + k * 2.0**-52)
    with np.errstate(over="ignore", under="ignore"):  # quotients past either end of the range
        far = np.ldexp(d, rng.integers(-1000, 1000, n))
    A = np.concatenate([a, c, e, sa.ravel(), g, h, at, c])
    B = np.concatenate([b, d, f, sb.ravel(), h, g, bt, far])
    return A, B


@pytest.mark.parametrize("seed", [1, 2])
def test_division_bit_exact(native, seed):
    N = native
    a, b = _operands(seed, 1 << 20)
    got = _run(N, 0, a, b)
    ref = _run(N, 1, a, b)
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    bad = np.flatnonzero(_bits(got)[~nan] != _bits(ref)[~nan])
    assert len(bad) == 0, (a[~nan][bad[:5]], b[~nan][bad[:5]])


def test_halving_bit_exact(native):
    a, _ = _operands(3, 1 << 20)
    got = _run(native, 2, a)
    ref = _run(native, 3, a)
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(_bits(got)[~nan], _bits(ref)[~nan])


def test_order_keys_match_comparisons(native):
    a, b = _operands(4, 1 << 20)
    keep = ~(np.isnan(a) | np.isnan(b))
    a, b = a[keep], b[keep]
    # equal values (including +0 / -0) must compare equal
    a = np.concatenate([a, [0.0, -0.0, 1.5, -2.0]])
    b = np.concatenate([b, [-0.0, 0.0, 1.5, -2.0]])
    assert np.array_equal(_run(native, 4, a, b), _run(native, 5, a, b))
