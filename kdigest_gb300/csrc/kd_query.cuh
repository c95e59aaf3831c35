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

#include "kd_fp64i.cuh"
#include "kd_math.h"

struct KdQueryDigest {
  const double* m;
  const double* w;
  const double* P;   // walk prefix: P[0] = w0 / 2, P[i+1] = P[i] + (w[i] + w[i+1]) / 2
  int nc;            // centroids (>= 1)
  double n;          // total weight the walk normalises by
  const double* mn;  // observed range (read only by the paths that use it)
  const double* mx;
  const double* dfac;  // non-null: singleton test on w * *dfac (decay) instead of w
  double single;     // a tail centroid is a singleton when its (effective) weight <= this
};

// The arithmetic below is the walk's own, operation for operation; its
// comparisons, halvings and divisions run on the integer pipes (kd_fp64i.cuh),
// which give the same bits as the FP64 instructions.

__device__ __forceinline__ bool kd_isnan_bits(double x) {
  return (kd_dbits(x) << 1) > 0xffe0000000000000ull;
}

__device__ __forceinline__ bool kd_q_singleton(const KdQueryDigest& d, double w) {
  return kd_okey(d.dfac ? KD_MUL(w, *d.dfac) : w) <= kd_okey(d.single);
}

// q in [0, 1] is the caller's check where it applies.
__device__ __forceinline__ double kd_quantile_one(const KdQueryDigest& d, double q) {
  const double* m = d.m;
  const double* w = d.w;
  const int nc = d.nc;
  if (nc == 1) return m[0];
  if (kd_isnan_bits(q)) return m[nc - 1];  // no comparison holds: the search runs off the end
  const long long kq = kd_okey(q);
  if (kq <= 0) return *d.mn;                                 // q <= 0
  if (kq >= (long long)0x3ff0000000000000ull) return *d.mx;  // q >= 1
  const double n = d.n;
  const double target = KD_MUL(q, n);
  const long long kt = kd_okey(target);
  const double w0 = w[0];
  const double first_half = kd_half(w0);
  const double wl = w[nc - 1];
  const double last_half = kd_half(wl);
  if (kt < kd_okey(first_half)) {
    if (kd_q_singleton(d, w0)) return *d.mn;
    return KD_ADD(*d.mn, KD_MUL(KD_SUB(m[0], *d.mn), kd_div(target, first_half)));
  }
  const double upper = KD_SUB(n, last_half);
  if (kt > kd_okey(upper)) {
    if (kd_q_singleton(d, wl)) return *d.mx;
    const double ml = m[nc - 1];
    const double frac = kd_div(KD_SUB(target, upper), last_half);
    return KD_ADD(ml, KD_MUL(KD_SUB(*d.mx, ml), frac));
  }
  const double* P = d.P;
  int lo = 1, hi = nc;  // first p in [1, nc-1] with P[p] >= target
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (kd_okey(P[mid]) >= kt) hi = mid;
    else lo = mid + 1;
  }
  if (lo >= nc) return m[nc - 1];
  const int k = lo - 1;
  const double dw = kd_half(KD_ADD(w[k], w[k + 1]));
  const double frac = kd_div(KD_SUB(target, P[k]), dw);
  return KD_ADD(m[k], KD_MUL(KD_SUB(m[k + 1], m[k]), frac));
}

__device__ __forceinline__ double kd_cdf_one(const KdQueryDigest& d, double x) {
  const double* m = d.m;
  const double* w = d.w;
  const int nc = d.nc;
  if (kd_isnan_bits(x)) return nc == 1 ? 0.5 : 1.0;  // no comparison holds
  const long long kx = kd_okey(x);
  const double mn = *d.mn, mx = *d.mx;
  const long long kmn = kd_okey(mn);
  if (kx < kmn) return 0.0;
  if (kx > kd_okey(mx)) return 1.0;
  const long long km0 = kd_okey(m[0]);
  if (nc == 1) return kx < km0 ? 0.0 : (kx > km0 ? 1.0 : 0.5);
  const double n = d.n;
  if (kx < km0) {
    if (kmn == km0) return 0.0;
    const double frac = kd_div(KD_SUB(x, mn), KD_SUB(m[0], mn));
    return kd_div(KD_MUL(kd_half(w[0]), frac), n);
  }
  const double ml = m[nc - 1];
  const long long kml = kd_okey(ml);
  if (kx > kml) {
    if (kd_okey(mx) == kml) return 1.0;
    const double frac = kd_div(KD_SUB(x, ml), KD_SUB(mx, ml));
    const double hl = kd_half(w[nc - 1]);
    return kd_div(KD_ADD(KD_SUB(n, hl), KD_MUL(hl, frac)), n);
  }
  const double* P = d.P;
  int lo = 1, hi = nc;  // first p in [1, nc-1] with x <= m[p]
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (kx <= kd_okey(m[mid])) hi = mid;
    else lo = mid + 1;
  }
  if (lo >= nc) return 1.0;
  const int k = lo - 1;
  const double dw = kd_half(KD_ADD(w[k], w[k + 1]));
  const double mk = m[k], mk1 = m[k + 1];
  if (kd_okey(mk1) == kd_okey(mk)) return kd_div(KD_ADD(P[k], kd_half(dw)), n);
  const double frac = kd_div(KD_SUB(x, mk), KD_SUB(mk1, mk));
  return kd_div(KD_ADD(P[k], KD_MUL(dw, frac)), n);
}
