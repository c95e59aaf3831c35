"""GPU parity of the single-digest P-path compress against the CPU oracle.

Restates the reference's three-path bit-exactness test
(test/test_gpu_add_batch.mojo:293-333): sizes {1, 2, 1023, 1024, 1025, 2049,
5000, 70001, 300000} x {continuous values, 37-level heavy ties}, random
weights in [1, 2).  Here the GPU kernels must match the FP64 oracle exactly:
same sort order, same bucket ids, same centroid counts, means and weights bit
for bit (tolerance 0).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 31, 32, 33, 1023, 1024, 1025, 2049, 5000, 70001, 300000]


def _lcg_data(n, levels, seed):
    # same generator shape as the reference test (LCG, u in [0,1), w in [1,2))
    state = np.uint64(seed)
    m = np.empty(n)
    w = np.empty(n)
    a = np.uint64(6364136223846793005)
    c = np.uint64(1442695040888963407)
    with np.errstate(over="ignore"):
        for i in range(n):
            state = state * a + c
            u = float(state >> np.uint64(11)) / float(1 << 53)
            state = state * a + c
            u2 = float(state >> np.uint64(11)) / float(1 << 53)
            m[i] = float(int(u * levels)) if levels > 0 else u
            w[i] = 1.0 + u2
    return m, w


def _fast_data(n, levels, seed):
    rng = np.random.default_rng(seed)
    u = rng.random(n)
    m = np.floor(u * levels) if levels > 0 else u
    return m, 1.0 + rng.random(n)


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("levels", [0, 37])
def test_compress_matches_oracle_k2(kd, oracle, n, levels):
    m, w = (_lcg_data if n <= 5000 else _fast_data)(n, levels, 0x51 + n)
    gm, gw = kd.compress(m, w, 100.0, kd.K2)
    om, ow = oracle.ppath_compress(oracle.K2, 100.0, m, w)
    assert len(gm) == len(om)
    assert np.array_equal(gm, om)
    assert np.array_equal(gw, ow)


@pytest.mark.parametrize("scale", [0, 1, 2, 3])
@pytest.mark.parametrize("n", [1000, 4096, 100000])
@pytest.mark.parametrize("compression", [50.0, 100.0, 200.0])
def test_compress_all_scales(kd, oracle, scale, n, compression):
    rng = np.random.default_rng(scale * 1000 + n)
    m = rng.standard_normal(n) * 3.0
    w = rng.random(n) * 5.0 + 1e-3
    gm, gw = kd.compress(m, w, compression, scale)
    om, ow = oracle.ppath_compress(scale, compression, m, w)
    assert np.array_equal(gm, om) and np.array_equal(gw, ow)


@pytest.mark.parametrize("scale", [0, 1, 2, 3])
def test_filter_matches_exact_path(kd, scale):
    """The FP32 bucket filter only chooses which evaluation runs: forcing the
    FP64 path everywhere must give the same centroids."""
    sess = kd.GpuSession()
    rng = np.random.default_rng(99 + scale)
    for n in (777, 20000, 250000):
        m = rng.standard_normal(n)
        w = np.where(rng.random(n) < 0.5, 1.0, rng.random(n) * 3 + 0.01)
        a = kd.compress(m, w, 100.0, scale, session=sess)
        sess.set_option(1, 1)  # KD_OPT_FORCE_EXACT_K
        b = kd.compress(m, w, 100.0, scale, session=sess)
        sess.set_option(1, 0)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_unit_weights_and_ties(kd, oracle):
    for n in (5, 1024, 3000, 65537):
        m = np.round(np.random.default_rng(n).standard_normal(n), 1)
        w = np.ones(n)
        gm, gw = kd.compress(m, w, 100.0, kd.K1)
        om, ow = oracle.ppath_compress(oracle.K1, 100.0, m, w)
        assert np.array_equal(gm, om) and np.array_equal(gw, ow)


def test_negative_zero_canonicalised(kd, oracle):
    m = np.array([0.0, -0.0, 1.0, -0.0, -1.0, 0.0] * 300)
    w = np.ones(len(m))
    gm, gw = kd.compress(m, w, 100.0, kd.K2)
    om, ow = oracle.ppath_compress(oracle.K2, 100.0, m, w)
    assert np.array_equal(gm, om) and np.array_equal(gw, ow)


def test_compress_rejects_bad_input(kd):
    with pytest.raises(ValueError):
        kd.compress([1.0, np.nan], [1.0, 1.0])
    with pytest.raises(ValueError):
        kd.compress([1.0, 2.0], [1.0, 0.0])
    with pytest.raises(ValueError):
        kd.compress([1.0, 2.0], [1.0, -1.0])
