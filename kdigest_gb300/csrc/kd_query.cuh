// kd_query.cuh — quantile and cdf of one digest (TDigest.quantile / cdf,
// tdigest.mojo:485-587; the GPU query kernels, gpu/query.mojo:45-231), shared by
// the resident-store queries and the stateless entry points.
//
// The reference walks the half-weight midpoints left to right, carrying
// wsf = w0 / 2, wsf += (w[i] + w[i+1]) / 2.  P[i] holds that running value at
// step i (computed once per digest with the same additions), so a query finds
// its interval by binary search and interpolates with the walk's own operands:
// the answers are bit-identical to the walk.
#pragma once

#include "kd_math.h"

struct KdQueryDigest {
  const double* m;
  const double* w;
  const double* P;   // walk prefix: P[0] = w0 / 2, P[i+1] = P[i] + (w[i] + w[i+1]) / 2
  int nc;            // centroids (>= 1)
  double n;          // total weight the walk normalises by
  double mn, mx;     // observed range
  bool scaled;       // singleton test on w * dfac (decay) instead of w
  double dfac;
  double single;     // a tail centroid is a singleton when its (effective) weight <= this
};

__device__ __forceinline__ bool kd_q_singleton(const KdQueryDigest& d, double w) {
  return (d.scaled ? KD_MUL(w, d.dfac) : w) <= d.single;
}

// q in [0, 1] is the caller's check where it applies.
__device__ __forceinline__ double kd_quantile_one(const KdQueryDigest& d, double q) {
  const double* m = d.m;
  const double* w = d.w;
  const int nc = d.nc;
  if (nc == 1) return m[0];
  if (q <= 0.0) return d.mn;
  if (q >= 1.0) return d.mx;
  const double n = d.n;
  const double target = KD_MUL(q, n);
  const double w0 = w[0];
  const double first_half = KD_MUL(w0, 0.5);
  const double wl = w[nc - 1], ml = m[nc - 1];
  const double last_half = KD_MUL(wl, 0.5);
  if (target < first_half) {
    if (kd_q_singleton(d, w0)) return d.mn;
    return KD_ADD(d.mn, KD_MUL(KD_SUB(m[0], d.mn), KD_DIV(target, first_half)));
  }
  if (target > KD_SUB(n, last_half)) {
    if (kd_q_singleton(d, wl)) return d.mx;
    const double frac = KD_DIV(KD_SUB(target, KD_SUB(n, last_half)), last_half);
    return KD_ADD(ml, KD_MUL(KD_SUB(d.mx, ml), frac));
  }
  const double* P = d.P;
  int lo = 1, hi = nc;  // first p in [1, nc-1] with P[p] >= target
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (P[mid] >= target) hi = mid;
    else lo = mid + 1;
  }
  if (lo >= nc) return ml;
  const int k = lo - 1;
  const double dw = KD_MUL(KD_ADD(w[k], w[k + 1]), 0.5);
  const double frac = KD_DIV(KD_SUB(target, P[k]), dw);
  return KD_ADD(m[k], KD_MUL(KD_SUB(m[k + 1], m[k]), frac));
}

__device__ __forceinline__ double kd_cdf_one(const KdQueryDigest& d, double x) {
  const double* m = d.m;
  const double* w = d.w;
  const int nc = d.nc;
  if (x < d.mn) return 0.0;
  if (x > d.mx) return 1.0;
  if (nc == 1) return x < m[0] ? 0.0 : (x > m[0] ? 1.0 : 0.5);
  const double n = d.n;
  if (x < m[0]) {
    if (d.mn == m[0]) return 0.0;
    const double frac = KD_DIV(KD_SUB(x, d.mn), KD_SUB(m[0], d.mn));
    return KD_DIV(KD_MUL(KD_MUL(w[0], 0.5), frac), n);
  }
  if (x > m[nc - 1]) {
    const double ml = m[nc - 1], wl = w[nc - 1];
    if (d.mx == ml) return 1.0;
    const double frac = KD_DIV(KD_SUB(x, ml), KD_SUB(d.mx, ml));
    const double hl = KD_MUL(wl, 0.5);
    return KD_DIV(KD_ADD(KD_SUB(n, hl), KD_MUL(hl, frac)), n);
  }
  const double* P = d.P;
  int lo = 1, hi = nc;  // first p in [1, nc-1] with x <= m[p]
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (x <= m[mid]) hi = mid;
    else lo = mid + 1;
  }
  if (lo >= nc) return 1.0;
  const int k = lo - 1;
  const double dw = KD_MUL(KD_ADD(w[k], w[k + 1]), 0.5);
  if (m[k + 1] == m[k]) return KD_DIV(KD_ADD(P[k], KD_MUL(dw, 0.5)), n);
  const double frac = KD_DIV(KD_SUB(x, m[k]), KD_SUB(m[k + 1], m[k]));
  return KD_DIV(KD_ADD(P[k], KD_MUL(dw, frac)), n);
}
