"""kd_compress_noalloc: the allocation-free compress entry point.

It runs on a fixed device array inside the library, which every call shares, so
two calls in a row must each give exactly what kd_compress (the session path)
gives for the same input — the second call must not see the first one's leftover
contents.  Compared bit for bit, the tolerance of every compress parity test.
Collected last so it also runs after every other test in the same process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 16384  # KD_NOALLOC_MAX_N


def _noalloc(N, m, w, compression, scale, cap=1024):
    om = np.full(cap, np.nan)
    ow = np.full(cap, np.nan)
    out_n = ctypes.c_int64(-1)
    msg = ctypes.create_string_buffer(256)
    rc = N.load().kd_compress_noalloc(scale, compression, N.ptr(m), N.ptr(w), len(m), 0,
                                      N.ptr(om), N.ptr(ow), cap, ctypes.byref(out_n), None,
                                      msg, len(msg))
    return rc, om[:max(out_n.value, 0)].copy(), ow[:max(out_n.value, 0)].copy(), msg.value


def _session_compress(N, m, w, compression, scale):
    from kdigest_gb300 import tdigest

    return tdigest.compress(m, w, compression, scale)


def _inputs(seed, n, ties):
    rng = np.random.default_rng(seed)
    m = rng.standard_normal(n) * 4.0
    if ties:
        m = np.floor(m * 3.0)
    return m, rng.random(n) * 3.0 + 0.25


def test_two_calls_in_a_row_match_kd_compress(kd):
    from kdigest_gb300 import _native as N

    # Call 1 fills the array at the maximum size; call 2 is smaller, so stale
    # entries of call 1 would surface in its result if anything were not cleared.
    cases = [(_inputs(7, MAX_N, False), 100.0, kd.K3), (_inputs(8, 3001, True), 50.0, kd.K1)]
    got = []
    for (m, w), comp, scale in cases:
        rc, gm, gw, msg = _noalloc(N, m, w, comp, scale)
        assert rc == N.KD_OK, msg
        got.append((gm, gw))
    for ((m, w), comp, scale), (gm, gw) in zip(cases, got):
        em, ew = _session_compress(N, m, w, comp, scale)
        assert len(gm) == len(em) > 0
        assert np.array_equal(gm, em)
        assert np.array_equal(gw, ew)


def test_device_pointers_two_calls(kd):
    torch = pytest.importorskip("torch")
    from kdigest_gb300 import _native as N

    L = N.load()
    stream = torch.cuda.current_stream().cuda_stream
    for seed, n, comp, scale in ((11, 1500, 200.0, kd.K2), (12, 9000, 100.0, kd.K0)):
        m, w = _inputs(seed, n, seed % 2 == 0)
        dm = torch.from_numpy(m).cuda()
        dw = torch.from_numpy(w).cuda()
        om = torch.full((1024,), float("nan"), dtype=torch.float64, device="cuda")
        ow = torch.full((1024,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        out_n = ctypes.c_int64(-1)
        msg = ctypes.create_string_buffer(256)
        rc = L.kd_compress_noalloc(scale, comp, dm.data_ptr(), dw.data_ptr(), n, N.KD_PTR_DEVICE,
                                   om.data_ptr(), ow.data_ptr(), 1024, ctypes.byref(out_n),
                                   stream, msg, len(msg))
        assert rc == N.KD_OK, msg.value
        k = out_n.value
        em, ew = _session_compress(N, m, w, comp, scale)
        assert k == len(em)
        assert np.array_equal(om[:k].cpu().numpy(), em)
        assert np.array_equal(ow[:k].cpu().numpy(), ew)


def test_rejects_sizes_beyond_the_limit(kd):
    from kdigest_gb300 import _native as N

    m, w = _inputs(3, MAX_N + 1, False)
    rc, gm, _, msg = _noalloc(N, m, w, 100.0, kd.K1)
    assert rc == N.KD_ERANGE
    assert b"no-allocation limit" in msg and str(MAX_N).encode() in msg
    assert len(gm) == 0
    # errors found on the device come back as status and text as well
    w_bad = w[:100].copy()
    w_bad[17] = -1.0
    rc, _, _, msg = _noalloc(N, m[:100], w_bad, 100.0, kd.K1)
    assert rc == N.KD_EINVAL and msg
    # and the array still serves a valid call afterwards
    rc, gm, gw, msg = _noalloc(N, m[:2000], w[:2000], 100.0, kd.K1)
    em, ew = _session_compress(N, m[:2000], w[:2000], 100.0, kd.K1)
    assert rc == N.KD_OK and np.array_equal(gm, em) and np.array_equal(gw, ew)


def _stress(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "equal":
        m = np.full(n, 2.5)
    elif kind == "sorted":
        m = np.sort(rng.standard_normal(n))
    elif kind == "reverse":
        m = np.sort(rng.standard_normal(n))[::-1].copy()
    else:  # heavy ties: eight distinct values
        m = rng.integers(0, 8, n).astype(np.float64) * 0.5
    w = np.ones(n) if seed % 2 == 0 else rng.random(n) * 2.0 + 0.5
    return m, w


@pytest.mark.parametrize("kind", ["equal", "sorted", "reverse", "ties"])
@pytest.mark.parametrize("seed", [0, 1])
def test_stress_inputs_at_the_limit(kd, oracle, kind, seed):
    """Inputs of exactly KD_NOALLOC_MAX_N centroids that stress the fixed
    capacities (one value, already sorted, reverse sorted, few distinct values;
    unit and fractional weights) all succeed and match kd_compress and the
    oracle bit for bit."""
    from kdigest_gb300 import _native as N

    m, w = _stress(kind, MAX_N, seed)
    rc, gm, gw, msg = _noalloc(N, m, w, 100.0, kd.K2)
    assert rc == N.KD_OK, msg
    em, ew = _session_compress(N, m, w, 100.0, kd.K2)
    om, ow = oracle.ppath_compress(oracle.K2, 100.0, m, w)
    assert np.array_equal(gm, em) and np.array_equal(gw, ew)
    assert np.array_equal(gm, om) and np.array_equal(gw, ow)


def test_allocates_nothing(kd):
    """After the calls have run once (so every kernel module is loaded), the
    same calls - host and device pointers, sizes up to the limit - leave the
    device's free memory exactly as it was."""
    torch = pytest.importorskip("torch")
    from kdigest_gb300 import _native as N

    L = N.load()
    stream = torch.cuda.current_stream().cuda_stream
    cases = []
    for i, n in enumerate((1, 100, 1024, 1025, 5000, 16384, 777, 3000, 12000, 64)):
        m, w = _inputs(100 + i, n, i % 3 == 0)
        cases.append((m, w, (50.0, 100.0, 200.0)[i % 3], i % 4))
    dev_in = [(torch.from_numpy(m).cuda(), torch.from_numpy(w).cuda()) for m, w, _, _ in cases]
    om = torch.empty(1024, dtype=torch.float64, device="cuda")
    ow = torch.empty(1024, dtype=torch.float64, device="cuda")
    out_n = ctypes.c_int64(-1)
    msg = ctypes.create_string_buffer(256)
    torch.cuda.synchronize()

    def round_():
        for (m, w, comp, scale), (dm, dw) in zip(cases, dev_in):
            rc, _, _, text = _noalloc(N, m, w, comp, scale)
            assert rc == N.KD_OK, text
            rc = L.kd_compress_noalloc(scale, comp, dm.data_ptr(), dw.data_ptr(), len(m),
                                       N.KD_PTR_DEVICE, om.data_ptr(), ow.data_ptr(), 1024,
                                       ctypes.byref(out_n), stream, msg, len(msg))
            assert rc == N.KD_OK, msg.value

    round_()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    round_()
    round_()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_refuses_a_capturing_stream(kd):
    """A call on a stream that is being captured is refused before it touches
    the stream, and the caller's capture completes normally."""
    torch = pytest.importorskip("torch")
    from kdigest_gb300 import _native as N

    L = N.load()
    m, w = _inputs(21, 500, False)
    dm, dw = torch.from_numpy(m).cuda(), torch.from_numpy(w).cuda()
    om = torch.empty(1024, dtype=torch.float64, device="cuda")
    ow = torch.empty(1024, dtype=torch.float64, device="cuda")
    x = torch.zeros(16, device="cuda")
    out_n = ctypes.c_int64(-1)
    msg = ctypes.create_string_buffer(256)
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            x.add_(1.0)
            rc = L.kd_compress_noalloc(kd.K1, 100.0, dm.data_ptr(), dw.data_ptr(), 500,
                                       N.KD_PTR_DEVICE, om.data_ptr(), ow.data_ptr(), 1024,
                                       ctypes.byref(out_n), s.cuda_stream, msg, len(msg))
    assert rc == N.KD_EINVAL and b"captured" in msg.value
    g.replay()
    torch.cuda.synchronize()
    assert float(x[0]) == 1.0
    rc, gm, gw, text = _noalloc(N, m, w, 100.0, kd.K1)
    em, ew = _session_compress(N, m, w, 100.0, kd.K1)
    assert rc == N.KD_OK and np.array_equal(gm, em) and np.array_equal(gw, ew)
