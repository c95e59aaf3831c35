// kd_internal.cuh — shared device-side building blocks of the GB300 t-digest engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kd_math.h"

// P-path semantic tile (gpu/primitives.mojo:40 BLOCK_CAP): every pass compresses
// consecutive 1024-element tiles of the sorted input as independent digests.
#define KD_TILE 1024
// Padded shared-memory stride of a lane chunk: E | 1 keeps 64-bit accesses of
// the 32 lanes on distinct banks for every chunk length E.
#define KD_SMEM_SLOTS 1056  // 32 lanes x 33

#define KD_WARPS_PER_BLOCK 1

// Status codes shared with the C-ABI (include/kdigest_gb300.h).
#define KD_OK 0
#define KD_EINVAL 1
#define KD_EEMPTY 2
#define KD_ERANGE 3
#define KD_ECONVERGE 4
#define KD_ENOMEM 5
#define KD_ECUDA 6
#define KD_ETIMEOUT 7

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ double shfl_up_d(double v, int o) { return __shfl_up_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shfl_down_d(double v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shfl_d(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// Device error word: the first failing condition wins (lowest code is not
// preferred; the first writer is kept).  A batch that sets it is not committed.
struct KdErr {
  int code;          // KD_* status
  int pad;
  long long index;   // first offending element / key, or -1
};

__device__ __forceinline__ void kd_set_error(KdErr* e, int code, long long index) {
  if (atomicCAS(&e->code, 0, code) == 0) e->index = index;
}

// ---------------------------------------------------------------------------
// FP32 filter for the bucket id.
//
// floor(k64) is needed where k64 = kd_k(scale, cum/tot, nrm64) is evaluated in
// FP64 with the shared kd_math.h functions.  The filter evaluates k in FP32
// together with a rigorous bound B on |k32 - k64| (worst-case errors of the
// FP32 conversions, of q = cum * rcp(total) (<= 3 ulp with the truncations),
// of asinf/sqrtf (<= 2 ulp), of the __logf intrinsic (<= 2^-21.41 absolute on
// [0.5, 2], <= 3 ulp elsewhere, documented by CUDA) and of the FP64 reference
// itself, with margins of 5x or more on every term).  When
// floor(k32 - B) == floor(k32 + B) the id is exact; otherwise, and outside the
// domain where the bound holds (q or 1-q below 2^-40, non-finite values), the
// caller evaluates the FP64 path.  The filter never changes a result: it only
// decides which evaluation is needed.
// ---------------------------------------------------------------------------
// Truncating double -> float conversion with integer operations only (the
// FP64 pipe, which also executes F2F conversions, is the bottleneck of the tile
// compress).  Relative error < 2^-23; tiny magnitudes flush to 0 and huge ones
// saturate to inf, both of which send the element to the exact path.
__device__ __forceinline__ float kd_d2f_trunc(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e < -126) return __int_as_float((int)sign);
  if (e > 127) return __int_as_float((int)(sign | 0x7f800000u));
  const unsigned m = (unsigned)((b >> 29) & 0x7fffffu);
  return __int_as_float((int)(sign | ((unsigned)(e + 127) << 23) | m));
}
// Truncating non-negative int64 -> float (integer operations only).
__device__ __forceinline__ float kd_i2f_trunc(long long v) {
  if (v <= 0) return 0.f;
  const int lz = __clzll(v);
  const int e = 63 - lz;  // v in [2^e, 2^(e+1))
  const unsigned long long norm = (unsigned long long)v << lz;  // top bit at 63
  const unsigned m = (unsigned)((norm >> 40) & 0x7fffffu);
  return __int_as_float((int)(((unsigned)(e + 127) << 23) | m));
}

struct KFilterTile {
  float nrm;      // FP32 normaliser
  float nrm_rel;  // bound on its relative error (already includes safety)
  float t32;      // tile total in FP32 (truncated)
  float inv32;    // its reciprocal (round to nearest): q = cum * inv32
  int ok;         // 0 -> the tile must use the exact path for every element
};

__device__ __forceinline__ KFilterTile kfilter_tile(int scale, double compression, float t32) {
  KFilterTile f;
  float c32 = kd_d2f_trunc(compression);
  f.t32 = t32;
  f.inv32 = __frcp_rn(t32);
  f.ok = isfinite(t32) && t32 > 0.f && c32 > 0.f && isfinite(c32);
  const float u = 5.9604645e-08f;  // 2^-24
  if (scale == KD_SCALE_K0) {
    f.nrm = c32 * 0.5f;
    f.nrm_rel = 4.f * u;
  } else if (scale == KD_SCALE_K1) {
    f.nrm = c32 / 6.2831855f;
    f.nrm_rel = 6.f * u;
  } else {
    float lt = logf(t32 / c32);
    float den = 4.f * lt + (scale == KD_SCALE_K2 ? 24.f : 21.f);
    f.nrm = c32 / den;
    // |d den| <= 4 |d log| + rounding; |d log| <= 6u + 2u |lt|
    float dden = 4.f * (6.f * u + 2.f * u * fabsf(lt)) + 4.f * u * (fabsf(4.f * lt) + 24.f);
    f.nrm_rel = dden / fabsf(den) + 6.f * u;
    if (!(fabsf(den) > 1e-3f)) f.ok = 0;
  }
  f.nrm_rel *= 8.f;
  if (!isfinite(f.nrm) || f.nrm == 0.f) f.ok = 0;
  return f;
}

// Returns 1 and writes the exact id when the FP32 evaluation is unambiguous.
//   q ~ cum / tot and r ~ (tot - cum) / tot, each within 6 ulp (float), with r
//   formed from the exact difference whenever q > 1/4; rem_zero: cum == tot.
// The last element of a tile has cum == tot exactly (q64 = 1): for K2/K3 the
// reference clamps q to 1 - 1e-15 there, so k = nrm * C with a constant C
// (ln(qc/(1-qc)) = 34.5395759923... for K2, -ln(2(1-qc)) = 33.8464288117... for
// K3, qc = fl(1 - 1e-15)); the filter resolves that element without FP64 work.
__device__ __forceinline__ int kfilter_id(int scale, const KFilterTile& ft, float q, float r,
                                          bool rem_zero, int32_t* id_out) {
  if (!ft.ok) return 0;
  const float u = 5.9604645e-08f;
  if (!(q >= 9.094947e-13f)) return 0;  // 2^-40: clamp region / tiny q
  float k, b;
  if (scale == KD_SCALE_K0) {
    k = ft.nrm * q;
    b = fabsf(k) * (ft.nrm_rel + 64.f * u);
  } else if (rem_zero && scale != KD_SCALE_K1) {
    k = ft.nrm * (scale == KD_SCALE_K2 ? 34.539576f : 33.846428f);
    b = fabsf(k) * (ft.nrm_rel + 64.f * u);
  } else if (!(r >= 9.094947e-13f) && !(rem_zero && scale == KD_SCALE_K1)) {
    return 0;
  } else if (scale == KD_SCALE_K1) {
    float a;
    if (q < 0.25f) {
      a = 2.f * asinf(sqrtf(q)) - 1.5707964f;
    } else if (q > 0.75f) {
      a = 1.5707964f - 2.f * asinf(sqrtf(r));
    } else {
      a = asinf(2.f * q - 1.f);
    }
    k = ft.nrm * a;
    b = fabsf(ft.nrm) * (64.f * u) + fabsf(k) * (ft.nrm_rel + 64.f * u);
  } else if (scale == KD_SCALE_K2) {
    float lq = __logf(q), l1 = __logf(r);
    float g = lq - l1;
    k = ft.nrm * g;
    // 2^-50 / r: the FP64 reference forms 1 - q64, whose absolute error
    // 2^-53 is relative error 2^-53 / r in ln(1 - q).
    b = fabsf(ft.nrm) * (64.f * u + 32.f * u * (fabsf(lq) + fabsf(l1)) + 8.881784e-16f / r) +
        fabsf(k) * (ft.nrm_rel + 64.f * u);
  } else {
    float g;
    if (q <= 0.5f) g = __logf(2.f * q);
    else g = -__logf(2.f * r);
    k = ft.nrm * g;
    b = fabsf(ft.nrm) * (64.f * u + 32.f * u * fabsf(g) + 8.881784e-16f / r) +
        fabsf(k) * (ft.nrm_rel + 64.f * u);
  }
  if (!isfinite(k) || !isfinite(b) || fabsf(k) > 1.0e7f) return 0;
  float lo = floorf(k - b), hi = floorf(k + b);
  if (lo != hi) return 0;
  *id_out = (int32_t)lo;
  return 1;
}
