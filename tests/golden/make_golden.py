"""Writes tests/golden/reference_order.npz: the outputs of the CPU oracle with
every sum in the reference's own association (the Hillis-Steele scans of
gpu/add_batch.mojo:79-160, which tests/test_oracle.py checks the oracle
against by running those lane loops literally), for the seeded inputs of
tests/golden/gen.py:

  tile_<i>   single P-path tiles (gpu/add_batch.mojo:45-222) with integral,
             fractional, equal decayed and prior-plus-new weights and ties:
             bucket ids, centroid means and weights;
  decay_<i>  single digests through the batch path (tdigest.mojo:236-315) with
             a count-clock decay (the single-digest decayed stream, scaled
             down): centroids, state, quantile and cdf answers;
  gtime      grouped keys with a time clock and fractional prior weights (the
             serving shape): per-key centroids and quantiles;
  gk3        grouped K3 keys without decay (the grouped ingest shape).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import gen  # noqa: E402
from oracle import pyoracle as o  # noqa: E402


def _digest_out(out, t, ds, xs=None):
    out[t + "_counts"] = np.array([len(d) for d in ds], np.int64)
    out[t + "_m"] = np.concatenate([d.centroids()[0] for d in ds])
    out[t + "_cw"] = np.concatenate([d.centroids()[1] for d in ds])
    out[t + "_state"] = np.array([[d.state()[k] for k in ("log_scale", "clock", "stored_total", "min", "max")]
                                  for d in ds])
    out[t + "_q"] = np.array([[d.quantile(float(q)) if len(d) else np.nan for q in gen.QS] for d in ds])
    if xs is not None:
        out[t + "_cdf"] = np.array([[d.cdf(float(x)) for x in xs] for d in ds])


def main():
    out = {}
    with o.sums_mode(o.SUMS_REFERENCE), o.math_mode(o.MATH_SHARED):
        for i, (scale, comp, kind, x, w) in enumerate(gen.tile_cases()):
            m, cw, ids = o.tile_compress(scale, comp, x, w)
            out[f"tile_{i}_ids"], out[f"tile_{i}_m"], out[f"tile_{i}_cw"] = ids, m, cw
        for c, (scale, comp, lam, nb, bsz) in enumerate(gen.DECAY_DIGESTS):
            d = o.Digest(scale, comp, lam)
            vals = gen.decay_digest_batches(c)
            for v in vals:
                d.add_batch_p(v)
            xs = np.quantile(np.concatenate(vals), np.linspace(0.001, 0.999, 9))
            out[f"decay_{c}_x"] = xs
            _digest_out(out, f"decay_{c}", [d], xs)
        scale, comp, lam, nk = gen.GROUPED_TIME
        ds = [o.Digest(scale, comp, lam) for _ in range(nk)]
        for keys, vals, t in gen.grouped_time_batches():
            o.grouped_add_batch(ds, keys, vals, mode=1, timestamp=t)
        _digest_out(out, "gtime", ds)
        scale, comp, lam, nk = gen.GROUPED_K3
        ds = [o.Digest(scale, comp, lam) for _ in range(nk)]
        for keys, vals in gen.grouped_k3_batches():
            o.grouped_add_batch(ds, keys, vals)
        _digest_out(out, "gk3", ds)
    path = os.path.join(HERE, "reference_order.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
