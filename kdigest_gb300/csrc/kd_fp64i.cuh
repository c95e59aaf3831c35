// kd_fp64i.cuh — IEEE binary64 results computed on the integer pipes.
//
// GB300 executes FP64 arithmetic at 2 lanes per clock per SM, against 64 lanes
// per clock for 32-bit integer instructions.  The quantile and cdf kernels
// spend most of their FP64 work on comparisons, halvings and two divisions per
// query, which have cheap exact integer forms; this header provides them.
// Every function returns exactly the bits of the IEEE round-to-nearest-even
// operation it stands for.  Operands outside a function's fast path (zeros
// where noted, subnormals, infinities, NaN, results that would leave the
// normal range) are passed to the hardware operation, so the functions are
// total.
#pragma once

#include <stdint.h>

#include "kd_math.h"

__device__ __forceinline__ uint64_t kd_dbits(double x) { return (uint64_t)__double_as_longlong(x); }
__device__ __forceinline__ double kd_bitsd(uint64_t u) { return __longlong_as_double((long long)u); }

// Order key of a non-NaN double: a < b exactly when kd_okey(a) < kd_okey(b),
// and -0.0 and +0.0 share the key 0 (they compare equal).  Negative values
// map to minus their magnitude bits.
__device__ __forceinline__ long long kd_okey(double x) {
  const uint64_t u = kd_dbits(x);
  return (long long)((u >> 63) ? 0x8000000000000000ull - u : u);
}

// x * 0.5, exact: the exponent field drops by one while the result stays
// normal (a biased exponent of 2 or more, below the infinity/NaN code).
__device__ __forceinline__ double kd_half(double x) {
  const uint64_t u = kd_dbits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7ffu;
  return (e > 1u && e < 0x7ffu) ? kd_bitsd(u - (1ull << 52)) : KD_MUL(x, 0.5);
}

// Signed high word of the 128-bit product of unsigned u and signed s.
__device__ __forceinline__ long long kd_mulhi_us(uint64_t u, long long s) {
  const uint64_t hi = __umul64hi(u, (uint64_t)s);
  return (long long)(s < 0 ? hi - u : hi);
}

// a / b rounded to nearest even.
//
// Method: both significands as 53-bit integers A, B (A doubled when A < B so
// the quotient lies in [1, 2)).  A fixed-point reciprocal R ~ 2^115 / B starts
// from the FP32 reciprocal of B's top 24 bits (relative error below 2^-22) and
// takes two Newton-Raphson steps, R <- R + R (2^115 - B R) / 2^115, each
// squaring the error (2^-44, then below the 2^-61 of the truncations).  The
// quotient estimate Q = floor(A R / 2^62) is then within one unit of
// T = floor(A 2^53 / B); the exact remainder A 2^53 - Q B (below 2^56 in
// magnitude, so its low 64 bits are exact) corrects Q to T.  T has 54 bits:
// the top 53 are the significand, the last is the round bit, and the
// remainder is the sticky bit of round-to-nearest-even (Newton-Raphson
// division with a remainder-based final rounding, as in Muller et al.,
// Handbook of Floating-Point Arithmetic, 2nd ed., ch. 4).
__device__ __forceinline__ double kd_div(double a, double b) {
  const uint64_t ua = kd_dbits(a), ub = kd_dbits(b);
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
  const uint64_t sign = (ua ^ ub) & 0x8000000000000000ull;
  if (eb - 1u >= 0x7feu) return KD_DIV(a, b);         // b zero, subnormal, infinite or NaN
  if ((ua << 1) == 0) return kd_bitsd(sign);          // +-0 / normal
  if (ea - 1u >= 0x7feu) return KD_DIV(a, b);         // a subnormal, infinite or NaN
  const uint64_t frac = (1ull << 52) - 1ull;
  uint64_t A = (ua & frac) | (1ull << 52);
  const uint64_t B = (ub & frac) | (1ull << 52);
  int e = (int)ea - (int)eb + 1023;  // biased exponent of A / B in [1, 2)
  if (A < B) {
    A <<= 1;
    --e;
  }
  if (e < 1 || e > 2045) return KD_DIV(a, b);  // subnormal or (after a carry) infinite result
  // seed: 2^86 / v for v = B's top 24 bits, from the FP32 reciprocal of v
  // (built from and read back through the bit fields: no conversion
  // instructions); relative error below 2^-22
  const uint32_t v = (uint32_t)(B >> 29);  // [2^23, 2^24)
  float rb;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rb) : "f"(__uint_as_float((150u << 23) | (v & 0x7fffffu))));
  const uint32_t rbits = __float_as_uint(rb);  // rb in (2^-24, 2^-23]: biased exponent 103 or 104
  uint64_t R = (uint64_t)((rbits & 0x7fffffu) | 0x800000u) << ((rbits >> 23) - 64u);
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    // E = 2^115 - B R as (hi, lo); |E| <= 2^93 (first step), < 2^72 (second)
    const uint64_t plo = B * R, phi = __umul64hi(B, R);
    const uint64_t elo = 0ull - plo;
    const long long ehi = (long long)((1ull << 51) - phi - (plo != 0ull ? 1ull : 0ull));
    // R += R E / 2^115, with E scaled to 53 bits first
    const int sh = it == 0 ? 40 : 17;
    const long long es = (long long)(((uint64_t)ehi << (64 - sh)) | (elo >> sh));
    const long long hi = kd_mulhi_us(R, es);  // (R es) >> 64
    R += (uint64_t)(hi >> (115 - 64 - sh));
  }
  // Q = floor(A R / 2^62), then the exact remainder against A 2^53
  uint64_t Q = (__umul64hi(A, R) << 2) | ((A * R) >> 62);
  long long rem = (long long)((A << 53) - Q * B);
  const long long Bs = (long long)B;
  if (rem < 0) {
    --Q;
    rem += Bs;
  }
  if (rem < 0) {
    --Q;
    rem += Bs;
  }
  if (rem >= Bs) {
    ++Q;
    rem -= Bs;
  }
  if (rem >= Bs) {
    ++Q;
    rem -= Bs;
  }
  uint64_t m = Q >> 1;  // [2^52, 2^53)
  if ((Q & 1ull) && (rem != 0 || (m & 1ull))) ++m;
  if (m == (1ull << 53)) {
    m = 1ull << 52;
    ++e;
  }
  return kd_bitsd(sign | ((uint64_t)e << 52) | (m & frac));
}
