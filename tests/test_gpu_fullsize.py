"""Size-independent properties at the headline size: 2^27 Zipf(1.1)-keyed
samples into 65,536 K3 digests (compression 100) in 2^22 batches, the
workload of the bench.  The oracle cannot replay this in test time, so every
key is checked against exact facts of its own samples instead."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_full_size_grouped_ingest_properties(kd):
    sys.path.insert(0, ROOT)
    import bench

    torch = pytest.importorskip("torch")
    from kdigest_gb300 import _native as N

    nk, batch, total = bench.NUM_KEYS, bench.BATCH, bench.TOTAL
    keys, vals = bench.make_workload(total=total)
    g = kd.GroupedTDigest(nk, bench.COMPRESSION, scale=kd.K3)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dv = torch.from_numpy(vals).cuda()
    torch.cuda.synchronize()
    L = N.load()
    for b in range(total // batch):
        rc = L.kd_store_ingest(g._store._h, dk.data_ptr() + 4 * b * batch,
                               dv.data_ptr() + 8 * b * batch, batch, N.KD_CLOCK_COUNT, 0.0,
                               N.KD_PTR_DEVICE)
        assert rc == 0
    n_key = np.bincount(keys, minlength=nk)
    kmin = np.full(nk, np.inf)
    kmax = np.full(nk, -np.inf)
    np.minimum.at(kmin, keys, vals)
    np.maximum.at(kmax, keys, vals)
    counts = g.centroid_counts()
    touched = n_key > 0
    assert np.all(counts[touched] >= 1) and np.all(counts <= 1024)
    assert np.all(counts[~touched] == 0)
    data, offs = g.export()  # every key's record: header and centroids
    buf = np.frombuffer(data, dtype=np.uint8)
    for k in np.flatnonzero(touched):
        rec = buf[offs[k]:offs[k + 1]]
        hdr = rec[1:65].view("<f8")
        cw = rec[65:].view("<f8").reshape(-1, 2)
        m, w = cw[:, 0], cw[:, 1]
        assert hdr[7] == counts[k] == len(m)
        # unit weights without decay: every partial sum is an exact integer
        assert hdr[4] == n_key[k] and w.sum() == n_key[k]
        assert np.all(np.diff(m) >= 0)
        assert hdr[5] == kmin[k] and hdr[6] == kmax[k]
        assert m[0] >= kmin[k] and m[-1] <= kmax[k]
    qk = np.repeat(np.flatnonzero(touched)[:: 97], 7)
    qs = np.tile(bench.QUANTILES, len(qk) // 7)
    est = g.quantiles(qk, qs).reshape(-1, 7)
    assert np.all(np.diff(est, axis=1) >= 0)
    sel = np.flatnonzero(touched)[:: 97]
    assert np.all(est[:, 0] >= kmin[sel]) and np.all(est[:, -1] <= kmax[sel])
    h = kd.GroupedTDigest(nk, bench.COMPRESSION, scale=kd.K3)
    h.import_records(data, offs)
    assert h.export()[0] == data


def test_full_size_pipelined_equals_one_call_per_batch(kd):
    """The whole 2^27-sample stream through one pipelined add_batches call ends
    bit for bit where one kd_store_ingest per 2^22 batch ends."""
    sys.path.insert(0, ROOT)
    import bench

    torch = pytest.importorskip("torch")
    from kdigest_gb300 import _native as N

    nk, batch, total = bench.NUM_KEYS, bench.BATCH, bench.TOTAL
    keys, vals = bench.make_workload(total=total)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dv = torch.from_numpy(vals).cuda()
    nb = total // batch
    a = kd.GroupedTDigest(nk, bench.COMPRESSION, scale=kd.K3)
    b = kd.GroupedTDigest(nk, bench.COMPRESSION, scale=kd.K3)
    a.add_batches([(dk[i * batch:(i + 1) * batch], dv[i * batch:(i + 1) * batch]) for i in range(nb)])
    L = N.load()
    for i in range(nb):
        rc = L.kd_store_ingest(b._store._h, dk.data_ptr() + 4 * i * batch, dv.data_ptr() + 8 * i * batch,
                               batch, N.KD_CLOCK_COUNT, 0.0, N.KD_PTR_DEVICE)
        assert rc == 0
    assert a.export()[0] == b.export()[0]  # every key's header and centroids
