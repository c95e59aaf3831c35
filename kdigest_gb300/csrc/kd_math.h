/*
 * kd_math.h — FP64 scale-function arithmetic shared bit-for-bit by host and device.
 *
 * The P-path bucket id of every element is floor(k(cum / total)), so a one-ulp
 * difference in k between two implementations can move an element across a
 * bucket edge.  Every function here is therefore written with only IEEE
 * correctly-rounded primitives (+, -, *, /, fma, sqrt) in a fixed evaluation
 * order, so that gcc on the host and nvcc on sm_103a produce identical bits.
 * Host code including this header must be compiled with -ffp-contract=off;
 * device code uses the explicit _rn intrinsics below, which are never fused.
 *
 * Methods (textbook, coefficients derived from the series themselves):
 *   log : x = 2^e * m, m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(s), s = (m-1)/(m+1),
 *         atanh series s + s^3/3 + ... + s^23/23 (Abramowitz & Stegun 4.5.64);
 *         e*ln2 added with a Cody-Waite split of ln2 (hi part has 40 bits).
 *   exp : x = k ln2 + r, |r| <= ln2/2 (same Cody-Waite split), e^r by its Taylor
 *         series to r^13/13!, then scaled by 2^k through the exponent field.
 *   asin: |x| <= 1/2 by the Maclaurin series of asin to x^49 (A&S 4.4.40);
 *         |x| > 1/2 through asin x = pi/2 - 2 asin(sqrt((1-x)/2)).
 * All constants are the double nearest to the exact rational / real value.
 *
 * Scale functions restate src/kdigest/scale.mojo:32-200 (normalizer/k for K0..K3,
 * _clamp_q with eps = 1e-15 for Float64).
 */
#ifndef KD_MATH_H
#define KD_MATH_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define KD_HD __host__ __device__ __forceinline__
#else
#define KD_HD static inline
#include <math.h>
#endif

#if defined(__CUDA_ARCH__)
#define KD_ADD(a, b) __dadd_rn((a), (b))
#define KD_SUB(a, b) __dsub_rn((a), (b))
#define KD_MUL(a, b) __dmul_rn((a), (b))
#define KD_DIV(a, b) __ddiv_rn((a), (b))
#define KD_FMA(a, b, c) __fma_rn((a), (b), (c))
#define KD_SQRT(a) __dsqrt_rn(a)
#define KD_FLOOR(a) floor(a)
#else
#define KD_ADD(a, b) ((a) + (b))
#define KD_SUB(a, b) ((a) - (b))
#define KD_MUL(a, b) ((a) * (b))
#define KD_DIV(a, b) ((a) / (b))
#define KD_FMA(a, b, c) fma((a), (b), (c))
#define KD_SQRT(a) sqrt(a)
#define KD_FLOOR(a) floor(a)
#endif

/* Scale function ids (runtime enum; the reference makes them a type parameter). */
#define KD_SCALE_K0 0
#define KD_SCALE_K1 1
#define KD_SCALE_K2 2
#define KD_SCALE_K3 3

/* Largest tile of the small-tile kernel (one warp per tile, one 32-lane
 * chunk per 32 elements); larger tiles run on a block of warps. */
#define KD_SERIAL_TILE_MAX 128

/* Clamp distance from the q = 0 / 1 singularities (scale.mojo:32-47, Float64). */
#define KD_Q_EPS 1e-15

KD_HD uint64_t kd_bits(double x) {
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
}
KD_HD double kd_from_bits(uint64_t u) {
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
}
KD_HD int kd_isnan(double x) { return x != x; }
KD_HD int kd_isfinite(double x) { return ((kd_bits(x) >> 52) & 0x7ff) != 0x7ff; }

/* 2^k as a double for k in [-1022, 1023]. */
KD_HD double kd_pow2i(int k) { return kd_from_bits((uint64_t)(k + 1023) << 52); }

KD_HD double kd_log(double x) {
  if (kd_isnan(x)) return x;
  if (x < 0.0) return kd_from_bits(0x7ff8000000000000ULL); /* NaN */
  if (x == 0.0) return kd_from_bits(0xfff0000000000000ULL); /* -inf */
  if (!kd_isfinite(x)) return x;                            /* +inf */
  uint64_t b = kd_bits(x);
  int e = (int)((b >> 52) & 0x7ff);
  if (e == 0) { /* subnormal: scale into the normal range (exact) */
    x = KD_MUL(x, 18014398509481984.0); /* 2^54 */
    b = kd_bits(x);
    e = (int)((b >> 52) & 0x7ff) - 54;
  }
  e -= 1023;
  double m = kd_from_bits((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL); /* [1,2) */
  if (m > 0x1.6a09e667f3bcdp+0) { /* > sqrt(2): halve (exact) */
    m = KD_MUL(m, 0.5);
    e += 1;
  }
  double f = KD_SUB(m, 1.0); /* exact (Sterbenz) */
  double s = KD_DIV(f, KD_ADD(2.0, f));
  double z = KD_MUL(s, s);
  double p = 0x1.642c8590b2164p-5; /* 1/23 */
  p = KD_FMA(p, z, 0x1.8618618618618p-5);  /* 1/21 */
  p = KD_FMA(p, z, 0x1.af286bca1af28p-5);  /* 1/19 */
  p = KD_FMA(p, z, 0x1.e1e1e1e1e1e1ep-5);  /* 1/17 */
  p = KD_FMA(p, z, 0x1.1111111111111p-4);  /* 1/15 */
  p = KD_FMA(p, z, 0x1.3b13b13b13b14p-4);  /* 1/13 */
  p = KD_FMA(p, z, 0x1.745d1745d1746p-4);  /* 1/11 */
  p = KD_FMA(p, z, 0x1.c71c71c71c71cp-4);  /* 1/9 */
  p = KD_FMA(p, z, 0x1.2492492492492p-3);  /* 1/7 */
  p = KD_FMA(p, z, 0x1.999999999999ap-3);  /* 1/5 */
  p = KD_FMA(p, z, 0x1.5555555555555p-2);  /* 1/3 */
  double r = KD_MUL(p, z);                 /* s^2/3 + s^4/5 + ... */
  double t = KD_FMA(s, r, s);              /* atanh(s) */
  double lnm = KD_MUL(t, 2.0);             /* exact */
  double ed = (double)e;
  return KD_ADD(KD_MUL(ed, 0x1.62e42fefa4000p-1), KD_FMA(ed, -0x1.8432a1b0e2634p-43, lnm));
}

KD_HD double kd_exp(double x) {
  if (kd_isnan(x)) return x;
  if (x > 709.782712893384) return kd_from_bits(0x7ff0000000000000ULL);
  if (x < -745.2) return 0.0;
  double kf = KD_FLOOR(KD_ADD(KD_MUL(x, 0x1.71547652b82fep+0), 0.5));
  int k = (int)kf;
  double r = KD_FMA(kf, 0x1.8432a1b0e2634p-43, KD_SUB(x, KD_MUL(kf, 0x1.62e42fefa4000p-1)));
  double p = 0x1.6124613a86d09p-33; /* 1/13! */
  p = KD_FMA(p, r, 0x1.1eed8eff8d898p-29); /* 1/12! */
  p = KD_FMA(p, r, 0x1.ae64567f544e4p-26); /* 1/11! */
  p = KD_FMA(p, r, 0x1.27e4fb7789f5cp-22); /* 1/10! */
  p = KD_FMA(p, r, 0x1.71de3a556c734p-19); /* 1/9! */
  p = KD_FMA(p, r, 0x1.a01a01a01a01ap-16); /* 1/8! */
  p = KD_FMA(p, r, 0x1.a01a01a01a01ap-13); /* 1/7! */
  p = KD_FMA(p, r, 0x1.6c16c16c16c17p-10); /* 1/6! */
  p = KD_FMA(p, r, 0x1.1111111111111p-7);  /* 1/5! */
  p = KD_FMA(p, r, 0x1.5555555555555p-5);  /* 1/4! */
  p = KD_FMA(p, r, 0x1.5555555555555p-3);  /* 1/3! */
  p = KD_FMA(p, r, 0.5);
  p = KD_FMA(p, r, 1.0);
  p = KD_FMA(p, r, 1.0);
  if (k > 1023) return KD_MUL(KD_MUL(p, kd_pow2i(1023)), kd_pow2i(k - 1023));
  if (k < -1022) return KD_MUL(KD_MUL(p, kd_pow2i(-1022)), kd_pow2i(k + 1022 < -1022 ? -1022 : k + 1022));
  return KD_MUL(p, kd_pow2i(k));
}

/* asin on [0, 1/2] by its Maclaurin series. */
KD_HD double kd_asin_series(double y) {
  double z = KD_MUL(y, y);
  double p = 0x1.3275586c5f2f0p-9;
  p = KD_FMA(p, z, 0x1.464c0950f7d47p-9);
  p = KD_FMA(p, z, 0x1.5c5f56efaaaabp-9);
  p = KD_FMA(p, z, 0x1.750de64d7d05fp-9);
  p = KD_FMA(p, z, 0x1.90cb77f60c7cep-9);
  p = KD_FMA(p, z, 0x1.b026f57b13b14p-9);
  p = KD_FMA(p, z, 0x1.d3d2a8e0dd67dp-9);
  p = KD_FMA(p, z, 0x1.fcaf8fb6db6dbp-9);
  p = KD_FMA(p, z, 0x1.15ee9d45d1746p-8);
  p = KD_FMA(p, z, 0x1.31683bdef7bdfp-8);
  p = KD_FMA(p, z, 0x1.51ba308d3dcb1p-8);
  p = KD_FMA(p, z, 0x1.782dda12f684cp-8);
  p = KD_FMA(p, z, 0x1.a6863d70a3d71p-8);
  p = KD_FMA(p, z, 0x1.df3bd37a6f4dfp-8);
  p = KD_FMA(p, z, 0x1.12ef3cf3cf3cfp-7);
  p = KD_FMA(p, z, 0x1.3fde50d79435ep-7);
  p = KD_FMA(p, z, 0x1.7a87878787878p-7);
  p = KD_FMA(p, z, 0x1.c99999999999ap-7);
  p = KD_FMA(p, z, 0x1.1c4ec4ec4ec4fp-6);
  p = KD_FMA(p, z, 0x1.6e8ba2e8ba2e9p-6);
  p = KD_FMA(p, z, 0x1.f1c71c71c71c7p-6);
  p = KD_FMA(p, z, 0x1.6db6db6db6db7p-5);
  p = KD_FMA(p, z, 0x1.3333333333333p-4);
  p = KD_FMA(p, z, 0x1.5555555555555p-3);
  return KD_FMA(KD_MUL(y, z), p, y);
}

/* asin(x); NaN outside [-1, 1], as the C library's asin (which the reference's
 * std.math asin is): rounding can put a prefix sum an ulp above its tile
 * total, and K1 (which does not clamp q, scale.mojo:114-118) then evaluates
 * asin slightly above 1.  The NaN reaches the int32 floor, which maps it to 0
 * (kd_floor_i32), or fails the S-path's k-size test as in the reference. */
KD_HD double kd_asin(double x) {
  if (kd_isnan(x)) return x;
  double ax = x < 0.0 ? -x : x;
  if (ax > 1.0) return kd_from_bits(0x7ff8000000000000ULL);
  double r;
  if (ax <= 0.5) {
    r = kd_asin_series(ax);
  } else {
    double t = KD_MUL(KD_SUB(1.0, ax), 0.5); /* exact */
    double s = KD_SQRT(t);
    r = KD_SUB(0x1.921fb54442d18p+0, KD_SUB(KD_MUL(2.0, kd_asin_series(s)), 0x1.1a62633145c07p-54));
  }
  return x < 0.0 ? -r : r;
}

/* floor(x) converted to int32 with saturation; NaN maps to 0.  This pins the
 * reference's Int32(floor(k)) (add_batch.mojo:110) for every double input:
 * the conversion of an out-of-range or NaN value is left undefined by the
 * language, and these are the results of the conversion instruction of the
 * reference's own platform (arm64 / Metal: saturating, NaN -> 0). */
KD_HD int32_t kd_floor_i32(double x) {
  if (kd_isnan(x)) return 0;
  if (x >= 2147483647.0) return 2147483647;
  if (x <= -2147483648.0) return (-2147483647 - 1);
  return (int32_t)KD_FLOOR(x);
}

KD_HD double kd_clamp_q(double q) {
  if (q < KD_Q_EPS) return KD_Q_EPS;
  if (q > KD_SUB(1.0, KD_Q_EPS)) return KD_SUB(1.0, KD_Q_EPS);
  return q;
}

/* normalizer(compression, n) — scale.mojo:86-89, 109-112, 139-143, 171-175. */
KD_HD double kd_normalizer(int scale, double compression, double n) {
  switch (scale) {
    case KD_SCALE_K0: return KD_DIV(compression, 2.0);
    case KD_SCALE_K1: return KD_DIV(compression, 0x1.921fb54442d18p+2); /* 2*pi */
    case KD_SCALE_K2:
      return KD_DIV(compression, KD_ADD(KD_MUL(4.0, kd_log(KD_DIV(n, compression))), 24.0));
    default:
      return KD_DIV(compression, KD_ADD(KD_MUL(4.0, kd_log(KD_DIV(n, compression))), 21.0));
  }
}

/* k(q, normalizer) — scale.mojo:91-94, 114-118, 145-150, 177-184. */
KD_HD double kd_k(int scale, double q, double nrm) {
  switch (scale) {
    case KD_SCALE_K0: return KD_MUL(nrm, q);
    case KD_SCALE_K1: return KD_MUL(nrm, kd_asin(KD_SUB(KD_MUL(2.0, q), 1.0)));
    case KD_SCALE_K2: {
      double qc = kd_clamp_q(q);
      return KD_MUL(nrm, kd_log(KD_DIV(qc, KD_SUB(1.0, qc))));
    }
    default: {
      double qc = kd_clamp_q(q);
      if (qc <= 0.5) return KD_MUL(nrm, kd_log(KD_MUL(2.0, qc)));
      return KD_MUL(-nrm, kd_log(KD_MUL(2.0, KD_SUB(1.0, qc))));
    }
  }
}

/* Bucket id of an element whose inclusive cumulative weight is cum in a tile of
 * total weight tot: floor(k(cum / tot)) (add_batch.mojo:102-112). */
KD_HD int32_t kd_bucket(int scale, double cum, double tot, double nrm) {
  return kd_floor_i32(kd_k(scale, KD_DIV(cum, tot), nrm));
}

/* Order-preserving map from a finite double to uint64 (-0.0 is canonicalised to
 * +0.0 first, so equal values map to equal keys exactly as `==` ties them). */
KD_HD uint64_t kd_order_key(double v) {
  uint64_t u = kd_bits(v);
  if (u == 0x8000000000000000ULL) u = 0;
  return (u & 0x8000000000000000ULL) ? ~u : (u | 0x8000000000000000ULL);
}
KD_HD double kd_from_order_key(uint64_t k) {
  uint64_t u = (k & 0x8000000000000000ULL) ? (k & 0x7fffffffffffffffULL) : ~k;
  return kd_from_bits(u);
}

#endif /* KD_MATH_H */
