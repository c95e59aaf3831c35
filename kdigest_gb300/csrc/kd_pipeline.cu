// kd_pipeline.cu — the GB300 P-path: batched ingest, hierarchical tile compress,
// commit, quantile/cdf queries and batched merges over resident per-key digests.
//
// One ingest (grouped add_batch, grouped.mojo:60-162 with gpu/grouped.mojo:415-643
// semantics per key) runs entirely on the device:
//   prep     validate (key range, finite values) and map values to order keys
//   sort     stable LSD radix sort by (key, value)            (gpu/sort.mojo):
//            the key and the top value bits packed into 64 bits, the low
//            value bits restored and their runs repaired by unpack / repair
//   touched  compact the keys present in the batch
//   prepare  per key: clock / decay / renormalise / min-max   (tdigest.mojo:236-296)
//   level 0  per 1024 tile of (prior centroids ++ new samples): merge-path load
//            fused with the tile compress                     (add_batch.mojo:45-222)
//   level L  re-tile the survivors of keys that exceeded one tile (:481-566)
//   commit   per key: stored total, prune, query prefix, flip the live slot
//            (tdigest.mojo:298-315, 441-458)
// Nothing is written to the live state of any key unless every stage succeeded.
#include <cuda_runtime.h>

#include <algorithm>
#include <unordered_map>
#include <atomic>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <vector>

#include "kd_engine.h"
#include "kd_internal.cuh"
#include "kd_query.cuh"
#include "kd_scan.cuh"
#include "kd_sort.cuh"

#define KD_ERANGE_SCRATCH KD_ERANGE_SCRATCH_INTERNAL  // scratch too small (index = needed)
#define KD_EMORE_LEVELS 101    // internal: keys still above one tile after the levels run
#define KD_ERESORT 102         // internal: the packed sort left an inversion; sort in full
#define KD_PACK_VALUE_BITS 40  // value bits the packed sort orders at least

__device__ __forceinline__ size_t slot_base(long long K, int buf, long long key) {
  return ((size_t)buf * (size_t)K + (size_t)key) * KD_TILE;
}

__device__ __forceinline__ void kd_err_set(KdErrHost* e, int code, long long index) {
  KdErr* ee = reinterpret_cast<KdErr*>(e);
  if (atomicCAS(&ee->code, 0, code) == 0) ee->index = index;
}
__device__ __forceinline__ int kd_err_get(const KdErrHost* e) {
  return *reinterpret_cast<const volatile int*>(&e->code);
}

__device__ __forceinline__ double canon(double v) { return v == 0.0 ? 0.0 : v; }

// ---------------------------------------------------------------------------
// Tile compress in the reference's association order
// ---------------------------------------------------------------------------
// The reference compresses a sorted tile of n <= 1024 pairs on 1024 lanes
// (gpu/add_batch.mojo:45-222, gpu/grouped.mojo:128-276) and its sums have that
// kernel's Hillis-Steele association:
//   - cum[i]: the inclusive scan with offsets 1, 2, 4, ... (cum[i] += cum[i-off]);
//   - the tile total: the scan's lane 1023, i.e. the balanced pairwise tree over
//     [0, 2^ceil(log2 n)) (the lanes past n add exact zeros);
//   - a segment's (sum w, sum w*x) at its end element e: the segmented scan,
//     which is the right-aligned pairwise tree over [head, e] (level-1 pairs
//     (e, e-1), (e-2, e-3), ...; a node without partner carried up).
// The kernels compute exactly these values: the prefix by the scan itself
// (integral weights: any exact order), the total from the window sums the
// scan passes through, and the segment sums by an up-sweep of that tree,
// e - head additions per segment.
//
// Shared-memory staging of one tile.  CAP is the largest tile it holds:
// KD_SERIAL_TILE_MAX (the small-tile kernel, a warp per tile) or KD_TILE (a
// block per tile).  Element p of the tile lives at slot (p / E) * SE + p % E,
// E = ceil(n / 32), SE = E | 1: the block loader writes 32 contiguous ranges
// at once, and the odd stride keeps them on distinct banks.  With CAP =
// KD_SERIAL_TILE_MAX the tile is one chunk (slot p = p).
template <int CAP>
struct WarpTileT {
  static constexpr int SLOTS = CAP == KD_TILE ? KD_SMEM_SLOTS : CAP + 1;
  double x[SLOTS];
  double w[SLOTS];  // weights; after the segment pass: sum(w * x) at each segment end
  // inclusive prefix of w (double, or int64 bits in the integral path); after
  // the segment pass: the weight sum of each segment at its end element
  double L[SLOTS];
  double P[32];                  // scratch: head ballots per round of 32 (unsigned)
  // hf/ef hold a list of up to CAP tile positions (unsigned short) while they
  // are free: the elements left to the FP64 bucket path, the segment end of
  // every position during the segment pass, then the segments whose mean
  // needs a division.
  unsigned char hf[SLOTS];
  unsigned char ef[SLOTS];
  // headpos/endpos also hold the bucket id (int) of every element until the
  // head pass, which writes headpos[k] only after id k has been read.
  alignas(8) unsigned short headpos[CAP];  // tile position of the first element of segment s
  unsigned short endpos[CAP];    // tile position of the last element of segment s

  __device__ unsigned short* poslist() { return reinterpret_cast<unsigned short*>(hf); }
  __device__ int* ids() { return reinterpret_cast<int*>(headpos); }
  __device__ unsigned* hbw() { return reinterpret_cast<unsigned*>(P); }
};
typedef WarpTileT<KD_TILE> WarpTile;
typedef WarpTileT<KD_SERIAL_TILE_MAX> WarpTileSmall;
static_assert(offsetof(WarpTile, ef) == offsetof(WarpTile, hf) + WarpTile::SLOTS &&
                  2 * WarpTile::SLOTS >= 2 * KD_TILE,
              "position list overlays hf/ef");
static_assert(offsetof(WarpTileSmall, ef) == offsetof(WarpTileSmall, hf) + WarpTileSmall::SLOTS &&
                  2 * WarpTileSmall::SLOTS >= 2 * KD_SERIAL_TILE_MAX,
              "position list overlays hf/ef");
// The small-tile loader stages up to KD_SERIAL_TILE_MAX order keys in L and
// as many in the contiguous P .. endpos block.
static_assert(sizeof(((WarpTileSmall*)0)->L) >= 8 * KD_SERIAL_TILE_MAX &&
                  sizeof(WarpTileSmall) - offsetof(WarpTileSmall, P) >= 8 * KD_SERIAL_TILE_MAX,
              "small-tile merge staging");
static_assert(offsetof(WarpTile, endpos) == offsetof(WarpTile, headpos) + 2 * KD_TILE &&
                  offsetof(WarpTileSmall, endpos) ==
                      offsetof(WarpTileSmall, headpos) + 2 * KD_SERIAL_TILE_MAX,
              "bucket ids overlay headpos/endpos");

// Integral weight in [1, 2^42): a tile of such weights has every partial sum
// exact in FP64 (total < 2^52), so int64 arithmetic in any order reproduces
// the reference's FP64 sums bit for bit.
__device__ __forceinline__ bool kd_is_small_int(double w) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(w);
  if (b >> 63) return false;
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e < 0 || e > 41) return false;
  return (b & ((1ull << (52 - e)) - 1ull)) == 0;
}
__device__ __forceinline__ long long kd_small_int(double w) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(w);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  return (long long)(((b & 0xfffffffffffffull) | (1ull << 52)) >> (52 - e));
}

template <bool kInt>
struct TileAcc;
template <>
struct TileAcc<false> {
  typedef double T;
  __device__ static T from_w(double w) { return w; }
  __device__ static T add(T a, T b) { return KD_ADD(a, b); }
  __device__ static T sub(T a, T b) { return KD_SUB(a, b); }
  __device__ static T shfl_up(T v, int o) { return __shfl_up_sync(0xffffffffu, v, o); }
  __device__ static T shfl(T v, int l) { return __shfl_sync(0xffffffffu, v, l); }
  __device__ static double to_d(T v) { return v; }
  __device__ static float to_f(T v) { return kd_d2f_trunc(v); }
  // exact comparisons (positive finite operands): a == b, and 2a == b (doubling is exact)
  __device__ static bool eq(T a, T b) { return __double_as_longlong(a) == __double_as_longlong(b); }
  __device__ static bool is_half(T a, T b) { return __double_as_longlong(KD_ADD(a, a)) == __double_as_longlong(b); }
  __device__ static double store(T v) { return v; }
  __device__ static T load(double v) { return v; }
};
template <>
struct TileAcc<true> {
  typedef long long T;
  __device__ static T from_w(double w) { return kd_small_int(w); }
  __device__ static T add(T a, T b) { return a + b; }
  __device__ static T sub(T a, T b) { return a - b; }
  __device__ static T shfl_up(T v, int o) { return __shfl_up_sync(0xffffffffu, v, o); }
  __device__ static T shfl(T v, int l) { return __shfl_sync(0xffffffffu, v, l); }
  __device__ static double to_d(T v) { return (double)v; }
  __device__ static float to_f(T v) { return kd_i2f_trunc(v); }
  __device__ static bool eq(T a, T b) { return a == b; }
  __device__ static bool is_half(T a, T b) { return a + a == b; }
  __device__ static double store(T v) { return __longlong_as_double(v); }
  __device__ static T load(double v) { return __double_as_longlong(v); }
};

__device__ __forceinline__ int tile_slot(int p, int E, int SE, unsigned inv) {
  const int c = (int)(((unsigned)p * inv) >> 16);  // exact p / E for p < 1024, E <= 1024
  return c * SE + (p - c * E);
}
// Chunk length of a tile: the whole tile up to KD_SERIAL_TILE_MAX elements,
// else ceil(n / 32).
__device__ __forceinline__ int tile_chunk(int n) {
  return n <= KD_SERIAL_TILE_MAX ? n : (n + 31) >> 5;
}
__device__ __forceinline__ unsigned tile_inv(int E) {
  return (65536u + (unsigned)E - 1u) / (unsigned)E;
}
struct SlotMap {
  int E, SE;
  unsigned inv;
  __device__ explicit SlotMap(int n) : E(tile_chunk(n)), SE(tile_chunk(n) | 1), inv(tile_inv(tile_chunk(n))) {}
  __device__ int operator()(int p) const { return tile_slot(p, E, SE, inv); }
};
struct FlatMap {
  __device__ int operator()(int p) const { return p; }
};

// The tile total in the reference's association from one window sum per set
// bit of n: bit k of n is the aligned block [s, s + 2^k), s = n with bits <= k
// cleared, and the balanced tree over [0, 2^ceil(log2 n)) is
// block(top bit) + (... + (block(next) + block(lowest bit))).
struct TotalAcc {
  double v = 0.0;
  bool have = false;
  __device__ void push(double b) {
    v = have ? KD_ADD(b, v) : b;
    have = true;
  }
};
__device__ __forceinline__ int block_end(int n, int k) {  // last position of bit k's block
  return (n & ~((2 << k) - 1)) + (1 << k) - 1;
}

// 2^b * w, exact (w positive and finite; integer exponent arithmetic while the
// result stays normal, which keeps the FP64 pipe free).
__device__ __forceinline__ double kd_scale2(double w, int b) {
  const long long bits = __double_as_longlong(w);
  const int e = (int)((bits >> 52) & 0x7ff);
  if (e >= 1 && e + b <= 2046) return __longlong_as_double(bits + ((long long)b << 52));
  return KD_MUL(w, kd_pow2i(b));
}
// Tiles whose weights are all equal (a batch's new samples at one decay
// factor): every window sum of the reference's scan is a power-of-two multiple
// of w, exact, so the scan value at j is w, plus 2^b * w for each set bit b of j
// in increasing order (P(j) = 2^m w + P(j - 2^m), m the top bit of j).  The
// same value is a segment's sum of j + 1 equal weights.
__device__ __forceinline__ double hs_uniform(double w, int j) {
  double acc = w;
  while (j) {
    acc = KD_ADD(kd_scale2(w, __ffs(j) - 1), acc);
    j &= j - 1;
  }
  return acc;
}
// The same value for j = 32 a + l from lo = hs_uniform(w, l): the bits of l
// come first in the fold, so only the set bits of a (>= 5) remain, the same
// for every lane of a round of 32.
__device__ __forceinline__ double hs_uniform_hi(double w, double lo, int a) {
  double acc = lo;
  while (a) {
    acc = KD_ADD(kd_scale2(w, __ffs(a) + 4), acc);
    a &= a - 1;
  }
  return acc;
}
__device__ __forceinline__ double hs_uniform_total(double w, int n) {
  TotalAcc tot;
  for (int k = 0; (n >> k) != 0; ++k)
    if ((n >> k) & 1) tot.push(kd_scale2(w, k));
  return tot.v;
}

// Segment end of position p from the head ballots of its rounds of 32: the
// position before the next head (or n - 1).  nz has bit r set when round r
// holds a head.
__device__ __forceinline__ int seg_end(const unsigned* hb, unsigned nz, int p, int n) {
  const int r = p >> 5, l = p & 31;
  const unsigned above = hb[r] & ~((2u << l) - 1u);
  if (above) return (r << 5) + __ffs(above) - 2;
  const unsigned rr = r >= 31 ? 0u : nz & ~((2u << r) - 1u);
  if (!rr) return n - 1;
  const int r2 = __ffs(rr) - 1;
  return (r2 << 5) + __ffs(hb[r2]) - 2;
}

// In-place Hillis-Steele scan of v[slot(0 .. n)) by one warp: rounds of
// offsets 1, 2, 4, ... < n; each round sweeps the 32-element blocks from the
// top, so that every read sees the value of the previous round.  Returns the
// tile total (TotalAcc over the window sums the rounds pass through).
template <class Slot>
__device__ double hs_scan_warp(double* v, int n, Slot slot) {
  const int lane = threadIdx.x & 31;
  TotalAcc tot;
  if (n & 1) tot.push(v[slot(n - 1)]);
  int k = 1;
  for (int d = 1; d < n; d <<= 1, ++k) {
    for (int r0 = (n - 1) & ~31; r0 >= 0; r0 -= 32) {
      const int p = r0 + lane;
      const bool act = p < n && p >= d;
      double a = 0.0, b = 0.0;
      if (act) {
        a = v[slot(p)];
        b = v[slot(p - d)];
      }
      __syncwarp();
      if (act) v[slot(p)] = KD_ADD(a, b);
      __syncwarp();
    }
    if ((n >> k) & 1) tot.push(v[slot(block_end(n, k))]);  // window of 2^k complete
  }
  return tot.v;
}

// Compresses the n <= KD_SERIAL_TILE_MAX staged elements of `t` (slot p = p)
// with one warp.  Writes the centroids to om/ow[0..) and returns their number.
template <bool kInt>
__device__ int warp_compress(WarpTileSmall& t, int n, int scale, double compression,
                             int force_exact, int32_t id_last, double* __restrict__ om,
                             double* __restrict__ ow) {
  typedef TileAcc<kInt> A;
  typedef typename A::T T;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;

  // 1-2. Inclusive prefix of the weights in L and the tile total.
  T tot;
  bool uniform = false;  // non-integral tile with all weights equal
  if (kInt) {  // exact int64 sums: a warp scan, 32 elements per round
    T carry = 0;
    for (int r0 = 0; r0 < n; r0 += 32) {
      const int p = r0 + lane;
      T v = p < n ? A::from_w(t.w[p]) : (T)0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const T u = A::shfl_up(v, o);
        if (lane >= o) v = A::add(v, u);
      }
      v = A::add(v, carry);
      if (p < n) t.L[p] = A::store(v);
      carry = A::shfl(v, 31);
    }
    tot = carry;
  } else {
    const double w0 = t.w[0];
    bool same = true;
    for (int p = lane; p < n; p += 32) same = same && __double_as_longlong(t.w[p]) == __double_as_longlong(w0);
    uniform = __all_sync(0xffffffffu, same);
    if (uniform) {
      const double lo = hs_uniform(w0, lane);
      for (int p = lane; p < n; p += 32) t.L[p] = hs_uniform_hi(w0, lo, p >> 5);
      tot = A::load(hs_uniform_total(w0, n));
    } else {
      for (int p = lane; p < n; p += 32) t.L[p] = t.w[p];
      __syncwarp();
      tot = A::load(hs_scan_warp(t.L, n, FlatMap()));
    }
  }
  double totd = A::to_d(tot);
  if (!(totd > 0.0)) {  // add_batch.mojo:98-100 (only reachable with non-integral weights)
    totd = 1.0;
    tot = (T)1;
  }
  __syncwarp();
  const KFilterTile ft = kfilter_tile(scale, compression, kInt ? A::to_f(tot) : kd_d2f_trunc(totd));

  // 3a. Bucket ids of all elements in independent rounds.  Exact shortcuts
  //     first: q == 1/2 gives k == 0 exactly for K1..K3 (asin(0), log(1)), and
  //     an element with cum == total of a K0/K1 tile (q == 1) has the launch
  //     constant id_last.  Then the FP32 filter; positions it cannot resolve
  //     go to a list for the FP64 path.
  int* const ids = t.ids();
  unsigned short* const plist = t.poslist();
  int nneed = 0;
  for (int r0 = 0; r0 < n; r0 += 32) {
    const int p = r0 + lane;
    bool need = false;
    if (p < n) {
      const T cum = A::load(t.L[p]);
      int32_t id = 0;
      bool ok = false;
      if (!force_exact) {
        const bool rz = A::eq(cum, tot);
        if (scale != KD_SCALE_K0 && A::is_half(cum, tot)) {
          ok = true;  // q == 1/2: id 0
        } else if (rz && scale <= KD_SCALE_K1) {
          id = id_last;
          ok = true;
        } else {
          const float q = A::to_f(cum) * ft.inv32;
          const float r = q > 0.25f ? A::to_f(A::sub(tot, cum)) * ft.inv32 : 1.f - q;
          ok = kfilter_id(scale, ft, q, r, rz, &id);
        }
      }
      ids[p] = id;
      need = !ok;
    }
    const unsigned nb = __ballot_sync(0xffffffffu, need);
    if (need) plist[nneed + __popc(nb & lt_mask)] = (unsigned short)p;
    nneed += __popc(nb);
  }
  __syncwarp();
  // 3b. The FP64 path for the listed positions, 32 at a time.
  if (nneed > 0) {
    const double nrm64 = kd_normalizer(scale, compression, totd);
    for (int k = lane; k < nneed; k += 32) {
      const int p = plist[k];
      ids[p] = kd_bucket(scale, A::to_d(A::load(t.L[p])), totd, nrm64);
    }
  }
  __syncwarp();
  // 3c. Heads (an id change or the first element), compacted by ballot, and
  //     the head ballot of every round.  Writing headpos[k] (k <= p) only
  //     clobbers ids of elements already read.
  unsigned* const hb = t.hbw();
  int32_t carry_id = 0;
  int nheads = 0;
  unsigned nz = 0;
  for (int r0 = 0; r0 < n; r0 += 32) {
    const int p = r0 + lane;
    const bool act = p < n;
    const int32_t id = act ? ids[p] : 0;
    int32_t prev = __shfl_up_sync(0xffffffffu, id, 1);
    if (lane == 0) prev = carry_id;
    const bool head = act && (p == 0 || id != prev);
    const unsigned hbits = __ballot_sync(0xffffffffu, head);
    carry_id = __shfl_sync(0xffffffffu, id, 31);
    __syncwarp();
    if (head) t.headpos[nheads + __popc(hbits & lt_mask)] = (unsigned short)p;
    if (lane == 0) hb[r0 >> 5] = hbits;
    if (hbits) nz |= 1u << (r0 >> 5);
    nheads += __popc(hbits);
  }
  __syncwarp();
  const int total_out = nheads;

  // 4. Segment sums, parked at each segment's end element (L: weight, w:
  //    weight * value).  sum(w): with integral weights every order is exact
  //    (int64, summed below); other weights take the up-sweep of each
  //    segment's right-aligned tree, the reference's association: in round r
  //    a position at distance u = e - p from its segment end, u a multiple of
  //    2^(r+1), adds the node 2^r below it when that lies in the same segment
  //    (nodes read in a round are never written in it).  sum(w * x): serial,
  //    one lane per segment; the reference's tree differs from it by rounding
  //    only, which reaches no bucket id (means are not summed into any prefix).
  if (!kInt && uniform) {
    const double w0 = t.w[0];
    for (int sI = lane; sI < total_out; sI += 32) {
      const int e = sI + 1 < total_out ? (int)t.headpos[sI + 1] - 1 : n - 1;
      t.L[e] = hs_uniform(w0, e - (int)t.headpos[sI]);
    }
  } else if (!kInt) {
    unsigned short* const send = t.poslist();  // segment end of every position
    for (int p = lane; p < n; p += 32) {
      send[p] = (unsigned short)seg_end(hb, nz, p, n);
      t.L[p] = t.w[p];
    }
    int ml = 1;
    for (int sI = lane; sI < total_out; sI += 32) {
      const int e = sI + 1 < total_out ? (int)t.headpos[sI + 1] - 1 : n - 1;
      ml = max(ml, e - (int)t.headpos[sI] + 1);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ml = max(ml, __shfl_xor_sync(0xffffffffu, ml, o));
    __syncwarp();
    for (int r = 0; (1 << r) < ml; ++r) {
      const int step = 1 << r;
      const unsigned mask = (2u << r) - 1u;
      for (int p = lane; p < n; p += 32) {
        const int e = send[p];
        if (((unsigned)(e - p) & mask) == 0 && p >= step && send[p - step] == e)
          t.L[p] = KD_ADD(t.L[p], t.L[p - step]);
      }
      __syncwarp();
    }
  }
  for (int sI = lane; sI < total_out; sI += 32) {
    const int h = t.headpos[sI];
    const int e = sI + 1 < total_out ? (int)t.headpos[sI + 1] - 1 : n - 1;
    t.endpos[sI] = (unsigned short)e;
    if (h == e) {  // a single element: its weight; its mean is its value
      if (kInt) t.L[e] = A::store(A::from_w(t.w[e]));
      continue;
    }
    T aw = A::from_w(t.w[h]);
    double awx = KD_MUL(t.w[h], t.x[h]);
    for (int i = h + 1; i <= e; ++i) {
      const double wi = t.w[i];
      if (kInt) aw = A::add(aw, A::from_w(wi));
      awx = KD_ADD(awx, KD_MUL(wi, t.x[i]));
    }
    if (kInt) t.L[e] = A::store(aw);
    t.w[e] = awx;
  }
  __syncwarp();

  // 5. Centroids: mean = sum(wx) / sum(w) clamped to the segment's [first,
  //    last] value (add_batch.mojo:205-218).  A segment whose first and last
  //    values are equal needs no division (the clamp yields that value); the
  //    others are listed and divided 32 at a time with every lane busy.
  unsigned short* const dlist = t.poslist();
  int ndiv = 0;
  for (int s0 = 0; s0 < total_out; s0 += 32) {
    const int sI = s0 + lane;
    bool div = false;
    if (sI < total_out) {
      const int e = t.endpos[sI];
      const int h = t.headpos[sI];
      const double sw = A::to_d(A::load(t.L[e]));
      const double lo_v = t.x[h], hi_v = t.x[e];
      ow[sI] = sw;
      if (__double_as_longlong(lo_v) == __double_as_longlong(hi_v)) {
        om[sI] = lo_v;
      } else if (!(__double_as_longlong(sw) > 0)) {  // zero weight: 0, clamped
        const uint64_t k0 = kd_order_key(0.0);
        om[sI] = k0 < kd_order_key(lo_v) ? lo_v : (k0 > kd_order_key(hi_v) ? hi_v : 0.0);
      } else {
        div = true;
      }
    }
    const unsigned db = __ballot_sync(0xffffffffu, div);
    __syncwarp();  // every lane read its position before the list overwrites them
    if (div) dlist[ndiv + __popc(db & lt_mask)] = (unsigned short)sI;
    ndiv += __popc(db);
  }
  __syncwarp();
  for (int k = lane; k < ndiv; k += 32) {
    const int sI = dlist[k];
    const int e = t.endpos[sI];
    const int h = t.headpos[sI];
    const double sw = A::to_d(A::load(t.L[e]));
    const double lo_v = t.x[h], hi_v = t.x[e];
    double mean = KD_DIV(t.w[e], sw);
    const uint64_t km = kd_order_key(mean);
    if (km < kd_order_key(lo_v)) mean = lo_v;
    else if (km > kd_order_key(hi_v)) mean = hi_v;
    om[sI] = mean;
  }
  __syncwarp();
  return total_out;
}

// ---------------------------------------------------------------------------
// Block-cooperative compress of one tile above the small-tile cap: the same
// values as warp_compress, every stage spread over the block's W warps (the
// tile in the chunk slot layout).  Stores of many keys use blocks of
// KD_TILE_WARPS warps (many tiles per SM: more, smaller blocks); stores of at
// most one key per SM use KD_TILE_WARPS_WIDE, since their upper levels hold a
// few tiles each and wait for one tile's latency.
// ---------------------------------------------------------------------------
#define KD_TILE_WARPS 4
#define KD_TILE_WARPS_WIDE 8
// Chunks of the large-tile sum(w * x): the association the oracle restates
// (128 chunks of ceil(n / 128) elements, carried across groups of 32), held
// by threads 0..127 whatever the block size; the other threads hold none.
#define KD_WX_CHUNKS 128
static_assert(KD_TILE_WARPS * 32 >= KD_WX_CHUNKS && KD_TILE_WARPS_WIDE >= KD_TILE_WARPS,
              "a thread per sum(w * x) chunk");
template <int W>
struct BlockScr {
  double totb;          // tile total (int64 bits in the integral path)
  double totd;
  KFilterTile ft;
  int nneed, ndiv, nout, stop, maxlen;
  unsigned nz;          // rounds of 32 that hold a head
  long long wsum[W];
  double cwx[W];  // per warp: segmented sum(w * x) carried out of its last chunk
  double cw[W];   // the same for sum(w) (int64 bits, integral path)
  int cf[W];      // whether the warp's chunks hold a head
  int rc[32];           // heads per round of 32 elements (then their offsets)
  unsigned hb[32];      // head ballot per round
};

template <bool kInt, int W>
__device__ int block_compress(WarpTile& t, BlockScr<W>& bs, int n, int scale, double compression,
                              int force_exact, int32_t id_last, double* __restrict__ om,
                              double* __restrict__ ow) {
  typedef TileAcc<kInt> A;
  typedef typename A::T T;
  constexpr int NT = W * 32;
  constexpr int PER = KD_TILE / NT;  // positions per thread
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const SlotMap slot(n);
  const unsigned lt_mask = (1u << lane) - 1u;
  const int rounds = (n + 31) >> 5;
  bool uniform = false;  // non-integral tile with all weights equal

  // 1-2. Inclusive prefix of the weights in L and the tile total.
  if (kInt) {
    // exact int64 sums: each warp scans a contiguous range of rounds, then
    // adds the totals of the warps before it
    const int per = (rounds + W - 1) / W;
    const int rb = warp * per, re = min(rounds, rb + per);
    T carry = 0;
    for (int r = rb; r < re; ++r) {
      const int p = r * 32 + lane;
      T v = p < n ? A::from_w(t.w[slot(p)]) : (T)0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const T u = A::shfl_up(v, o);
        if (lane >= o) v = A::add(v, u);
      }
      v = A::add(v, carry);
      if (p < n) t.L[slot(p)] = A::store(v);
      carry = A::shfl(v, 31);
    }
    if (lane == 0) bs.wsum[warp] = (long long)carry;
    __syncthreads();
    T off = 0, all = 0;
#pragma unroll
    for (int w2 = 0; w2 < W; ++w2) {
      const T s2 = (T)bs.wsum[w2];
      if (w2 < warp) off = A::add(off, s2);
      all = A::add(all, s2);
    }
    if (off != 0)
      for (int r = rb; r < re; ++r) {
        const int p = r * 32 + lane;
        if (p < n) t.L[slot(p)] = A::store(A::add(A::load(t.L[slot(p)]), off));
      }
    if (tid == 0) bs.totb = A::store(all);
  } else {
    const double w0 = t.w[slot(0)];
    bool same = true;
    for (int p = tid; p < n; p += NT) same = same && __double_as_longlong(t.w[slot(p)]) == __double_as_longlong(w0);
    uniform = __syncthreads_and(same);
  }
  if (!kInt && uniform) {
    const double w0 = t.w[slot(0)];
    const double lo = hs_uniform(w0, lane);  // p & 31 == lane for p = tid + k * NT
    for (int p = tid; p < n; p += NT) t.L[slot(p)] = hs_uniform_hi(w0, lo, p >> 5);
    if (tid == 0) bs.totb = hs_uniform_total(w0, n);
  } else if (!kInt) {
    // the Hillis-Steele rounds, staged through registers: all reads of a
    // round complete before its writes
    for (int p = tid; p < n; p += NT) t.L[slot(p)] = t.w[slot(p)];
    TotalAcc tot;
    if (tid == 0 && (n & 1)) tot.push(t.w[slot(n - 1)]);
    __syncthreads();
    int k = 1;
    for (int d = 1; d < n; d <<= 1, ++k) {
      double nv[PER];
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const int p = tid + i * NT;
        nv[i] = (p < n && p >= d) ? KD_ADD(t.L[slot(p)], t.L[slot(p - d)]) : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const int p = tid + i * NT;
        if (p < n && p >= d) t.L[slot(p)] = nv[i];
      }
      __syncthreads();
      if (tid == 0 && ((n >> k) & 1)) tot.push(t.L[slot(block_end(n, k))]);
    }
    if (tid == 0) bs.totb = tot.v;
  }
  if (tid == 0) {
    T tot = A::load(bs.totb);
    double totd = A::to_d(tot);
    if (!(totd > 0.0)) {  // add_batch.mojo:98-100
      totd = 1.0;
      tot = (T)1;
    }
    bs.totb = A::store(tot);
    bs.totd = totd;
    bs.ft = kfilter_tile(scale, compression, kInt ? A::to_f(tot) : kd_d2f_trunc(totd));
    bs.nneed = 0;
    bs.ndiv = 0;
  }
  __syncthreads();
  const T tot = A::load(bs.totb);
  const double totd = bs.totd;
  const KFilterTile ft = bs.ft;

  // 3a. Bucket ids; warp w takes rounds w, w + W, ...
  int* const ids = t.ids();
  unsigned short* const plist = t.poslist();
  for (int r0 = warp * 32; r0 < n; r0 += NT) {
    const int p = r0 + lane;
    bool need = false;
    if (p < n) {
      const T cum = A::load(t.L[slot(p)]);
      int32_t id = 0;
      bool ok = false;
      if (!force_exact) {
        const bool rz = A::eq(cum, tot);
        if (scale != KD_SCALE_K0 && A::is_half(cum, tot)) {
          ok = true;
        } else if (rz && scale <= KD_SCALE_K1) {
          id = id_last;
          ok = true;
        } else {
          const float q = A::to_f(cum) * ft.inv32;
          const float r = q > 0.25f ? A::to_f(A::sub(tot, cum)) * ft.inv32 : 1.f - q;
          ok = kfilter_id(scale, ft, q, r, rz, &id);
        }
      }
      ids[p] = id;
      need = !ok;
    }
    const unsigned nb = __ballot_sync(0xffffffffu, need);
    if (nb) {
      int base = 0;
      if (lane == 0) base = atomicAdd(&bs.nneed, __popc(nb));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (need) plist[base + __popc(nb & lt_mask)] = (unsigned short)p;
    }
  }
  __syncthreads();
  // 3b. The FP64 path for the listed positions.
  const int nneed = bs.nneed;
  if (nneed > 0) {
    const double nrm64 = kd_normalizer(scale, compression, totd);
    for (int k = tid; k < nneed; k += NT) {
      const int p = plist[k];
      ids[p] = kd_bucket(scale, A::to_d(A::load(t.L[slot(p)])), totd, nrm64);
    }
  }
  __syncthreads();
  // 3c. Heads: flags per round, offsets by a scan over the rounds, then the
  //     positions (the ids are all read before any position is written).
  for (int r = warp; r < rounds; r += W) {
    const int p = r * 32 + lane;
    const bool act = p < n;
    const int32_t id = act ? ids[p] : 0;
    const int32_t prev = (act && p > 0) ? ids[p - 1] : 0;
    const unsigned hbits = __ballot_sync(0xffffffffu, act && (p == 0 || id != prev));
    if (lane == 0) {
      bs.hb[r] = hbits;
      bs.rc[r] = __popc(hbits);
    }
  }
  __syncthreads();
  if (warp == 0) {
    const int v = lane < rounds ? bs.rc[lane] : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    bs.rc[lane] = incl - v;
    const unsigned nz = __ballot_sync(0xffffffffu, lane < rounds && bs.hb[lane] != 0u);
    if (lane == 31) bs.nout = incl;
    if (lane == 0) {
      bs.nz = nz;
      bs.maxlen = 1;
    }
  }
  __syncthreads();
  for (int r = warp; r < rounds; r += W) {
    const unsigned hbits = bs.hb[r];
    if ((hbits >> lane) & 1u) t.headpos[bs.rc[r] + __popc(hbits & lt_mask)] = (unsigned short)(r * 32 + lane);
  }
  __syncthreads();
  const int total_out = bs.nout;

  // 4. Segment sums, parked at each segment's end element, with the
  //    association of warp_compress: sum(w) exact (integral weights) or by the
  //    up-sweep of the reference's tree, block-wide; sum(w * x) serial per
  //    chunk of ceil(n / 128) elements (one per thread), carried across each
  //    warp's chunks by a segmented Kogge-Stone scan and across the warps in
  //    order (one chunk, n <= KD_SERIAL_TILE_MAX: serial per segment).
  if (!kInt && uniform) {
    const double w0 = t.w[slot(0)];
    for (int sI = tid; sI < total_out; sI += NT) {
      const int e = sI + 1 < total_out ? (int)t.headpos[sI + 1] - 1 : n - 1;
      t.L[slot(e)] = hs_uniform(w0, e - (int)t.headpos[sI]);
    }
  } else if (!kInt) {
    unsigned short* const send = t.poslist();
    const unsigned nz = bs.nz;
    for (int p = tid; p < n; p += NT) {
      send[p] = (unsigned short)seg_end(bs.hb, nz, p, n);
      t.L[slot(p)] = t.w[slot(p)];
    }
    int ml = 1;
    for (int sI = tid; sI < total_out; sI += NT) {
      const int e = sI + 1 < total_out ? (int)t.headpos[sI + 1] - 1 : n - 1;
      ml = max(ml, e - (int)t.headpos[sI] + 1);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ml = max(ml, __shfl_xor_sync(0xffffffffu, ml, o));
    if (lane == 0 && ml > 1) atomicMax(&bs.maxlen, ml);
    __syncthreads();
    const int maxlen = bs.maxlen;
    for (int r = 0; (1 << r) < maxlen; ++r) {
      const int step = 1 << r;
      const unsigned mask = (2u << r) - 1u;
      for (int p = tid; p < n; p += NT) {
        const int e = send[p];
        if (((unsigned)(e - p) & mask) == 0 && p >= step && send[p - step] == e) {
          const int sp = slot(p);
          t.L[sp] = KD_ADD(t.L[sp], t.L[slot(p - step)]);
        }
      }
      __syncthreads();
    }
  }
  if (n <= KD_SERIAL_TILE_MAX) {
    for (int sI = tid; sI < total_out; sI += NT) {  // one chunk: serial, thread per segment
      const int h = t.headpos[sI];
      const int e = sI + 1 < total_out ? (int)t.headpos[sI + 1] - 1 : n - 1;
      t.endpos[sI] = (unsigned short)e;
      if (h == e) {
        if (kInt) t.L[e] = A::store(A::from_w(t.w[e]));
        continue;
      }
      T aw = A::from_w(t.w[h]);
      double awx = KD_MUL(t.w[h], t.x[h]);
      for (int i = h + 1; i <= e; ++i) {
        const double wi = t.w[i];
        if (kInt) aw = A::add(aw, A::from_w(wi));
        awx = KD_ADD(awx, KD_MUL(wi, t.x[i]));
      }
      if (kInt) t.L[e] = A::store(aw);
      t.w[e] = awx;
    }
  } else {
    for (int q = tid; q < n; q += NT) {
      const int sl = slot(q);
      t.hf[sl] = 0;
      t.ef[sl] = 0;
    }
    __syncthreads();
    for (int sI = tid; sI < total_out; sI += NT) {
      const int h = t.headpos[sI];
      t.hf[slot(h)] = 1;
      const int e = sI + 1 < total_out ? (int)t.headpos[sI + 1] - 1 : n - 1;
      t.ef[slot(e)] = 1;
      t.endpos[sI] = (unsigned short)e;
    }
    __syncthreads();
    {  // one chunk per thread: serial pieces, a segmented carry across each
       // warp's 32 chunks, then across the warps in order
      const int E4 = (n + KD_WX_CHUNKS - 1) / KD_WX_CHUNKS;
      const int lo = tid * E4;
      const int cnt = max(0, min(E4, n - lo));  // none for tid >= KD_WX_CHUNKS
      T aw = 0;
      double awx = 0.0;
      bool head_seen = false;
      bool pend = false;
      T pend_w = 0;
      double pend_wx = 0.0;
      int pend_se = 0;
      for (int j = 0; j < cnt; ++j) {
        const int sp = slot(lo + j);
        const double wi = t.w[sp], xi = t.x[sp];
        const double wx = KD_MUL(wi, xi);
        const bool hd = t.hf[sp];
        if (hd || j == 0) {
          if (kInt) aw = A::from_w(wi);
          awx = wx;
        } else {
          if (kInt) aw = A::add(aw, A::from_w(wi));
          awx = KD_ADD(awx, wx);
        }
        if (hd) head_seen = true;
        if (t.ef[sp]) {
          if (head_seen) {
            if (kInt) t.L[sp] = A::store(aw);
            t.w[sp] = awx;
          } else {
            pend = true;
            pend_w = aw;
            pend_wx = awx;
            pend_se = sp;
          }
        }
      }
      T Vw = aw;
      double Vwx = awx;
      int F = head_seen ? 1 : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const T tw = A::shfl_up(Vw, o);
        const double twx = shfl_up_d(Vwx, o);
        const int tf = __shfl_up_sync(0xffffffffu, F, o);
        if (lane >= o) {
          if (!F) {
            if (kInt) Vw = A::add(Vw, tw);
            Vwx = KD_ADD(Vwx, twx);
          }
          F |= tf;
        }
      }
      if (lane == 31) {
        bs.cwx[warp] = Vwx;
        bs.cw[warp] = A::store(Vw);
        bs.cf[warp] = F;
      }
      __syncthreads();
      // the final value of the previous warp's last chunk
      double cwx_prev = 0.0;
      T cw_prev = 0;
      if (warp > 0) {
        cwx_prev = bs.cwx[0];
        cw_prev = A::load(bs.cw[0]);
        for (int g = 1; g < warp; ++g) {
          if (bs.cf[g]) {
            cwx_prev = bs.cwx[g];
            cw_prev = A::load(bs.cw[g]);
          } else {
            cwx_prev = KD_ADD(bs.cwx[g], cwx_prev);
            if (kInt) cw_prev = A::add(A::load(bs.cw[g]), cw_prev);
          }
        }
        if (!F) {
          Vwx = KD_ADD(Vwx, cwx_prev);
          if (kInt) Vw = A::add(Vw, cw_prev);
        }
      }
      double cwx = shfl_up_d(Vwx, 1);
      T cw = A::shfl_up(Vw, 1);
      if (lane == 0) {
        cwx = cwx_prev;
        cw = cw_prev;
      }
      if (pend) {
        if (kInt) t.L[pend_se] = A::store(A::add(cw, pend_w));
        t.w[pend_se] = KD_ADD(cwx, pend_wx);
      }
    }
  }
  __syncthreads();

  // 5. Centroids; the means that need a division are listed and divided with
  //    every thread busy.
  unsigned short* const dlist = t.poslist();
  for (int s0 = warp * 32; s0 < total_out; s0 += NT) {
    const int sI = s0 + lane;
    bool div = false;
    if (sI < total_out) {
      const int e = t.endpos[sI];
      const int h = t.headpos[sI];
      const int se = slot(e), sh = slot(h);
      const double sw = A::to_d(A::load(t.L[se]));
      const double lo_v = t.x[sh], hi_v = t.x[se];
      ow[sI] = sw;
      if (__double_as_longlong(lo_v) == __double_as_longlong(hi_v)) {
        om[sI] = lo_v;
      } else if (!(__double_as_longlong(sw) > 0)) {  // zero weight: 0, clamped
        const uint64_t k0 = kd_order_key(0.0);
        om[sI] = k0 < kd_order_key(lo_v) ? lo_v : (k0 > kd_order_key(hi_v) ? hi_v : 0.0);
      } else {
        div = true;
      }
    }
    const unsigned db = __ballot_sync(0xffffffffu, div);
    if (db) {
      int base = 0;
      if (lane == 0) base = atomicAdd(&bs.ndiv, __popc(db));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (div) dlist[base + __popc(db & lt_mask)] = (unsigned short)sI;
    }
  }
  __syncthreads();
  const int ndiv = bs.ndiv;
  for (int k = tid; k < ndiv; k += NT) {
    const int sI = dlist[k];
    const int e = t.endpos[sI];
    const int h = t.headpos[sI];
    const int se = slot(e), sh = slot(h);
    const double sw = A::to_d(A::load(t.L[se]));
    const double lo_v = t.x[sh], hi_v = t.x[se];
    double mean = KD_DIV(t.w[se], sw);
    const uint64_t km = kd_order_key(mean);
    if (km < kd_order_key(lo_v)) mean = lo_v;
    else if (km > kd_order_key(hi_v)) mean = hi_v;
    om[sI] = mean;
  }
  __syncthreads();  // the tile staging is reused by the block's next tile
  return total_out;
}

// ---------------------------------------------------------------------------
// Stage kernels
// ---------------------------------------------------------------------------
// Sort keys.  Full form: k64 = order key of the value, kout = digest key (the
// sort then runs 8 value passes and ceil(kb / 8) key passes).  Packed form:
// k64 = digest key in the top kb bits above the top 64 - kb bits of the order
// key, kout = the order key's low kb bits.  The sort orders the key and at
// least KD_PACK_VALUE_BITS value bits; samples of one key that agree in the
// sorted bits keep their input order, and k_unpack / k_repair restore the full
// form and the exact order among them.
__global__ void k_prep(long long n, const KdCallArgs* __restrict__ call, long long K, int kb,
                       uint64_t* __restrict__ k64, uint32_t* __restrict__ kout,
                       uint32_t* __restrict__ idx, KdErrHost* err,
                       unsigned long long* __restrict__ kepoch) {
  if (kepoch && blockIdx.x == 0 && threadIdx.x == 0) *kepoch += 1;  // this step's stamp
  const uint32_t* __restrict__ keys = call->keys;
  const double* __restrict__ vals = call->vals;
  const double* __restrict__ wts = call->wts;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const uint32_t key = keys ? keys[i] : 0u;
    const double v = vals[i];
    bool bad = (long long)key >= K || !kd_isfinite(v);
    if (wts && call->carry == 0) {  // carried weights come from the store itself
      const double w = wts[i];
      bad = bad || !(w > 0.0) || !kd_isfinite(w);
    }
    if (bad) {
      atomicMin((unsigned long long*)&err->index, (unsigned long long)i);
      atomicCAS(&err->code, 0, KD_EINVAL);
    }
    const uint64_t ok = kd_order_key(v);
    if (kb > 0) {
      k64[i] = ((uint64_t)key << (64 - kb)) | (ok >> kb);
      kout[i] = (uint32_t)(ok & ((1ull << kb) - 1ull));
    } else {
      k64[i] = ok;
      kout[i] = key;
    }
    if (idx) idx[i] = (uint32_t)i;
  }
}

struct TouchedSrc {
  const uint32_t* key;
  __device__ int4 operator()(long long i) const {
    return make_int4((i == 0 || key[i] != key[i - 1]) ? 1 : 0, 0, 0, 0);
  }
};
struct TouchedDst {
  const uint32_t* key;
  uint32_t* tkey;
  int* tstart;
  uint32_t* tmap;
  long long cap;
  long long K;
  __device__ void operator()(long long i, int4 excl, int4 v) const {
    if (v.x && excl.x < cap) {
      const uint32_t k = key[i];
      tkey[excl.x] = k;
      tstart[excl.x] = (int)i;
      if ((long long)k < K) tmap[k] = (uint32_t)excl.x;
    }
  }
};

// Key-level form of the same list, used when the batch has at least as many
// samples as the store has keys: k_unpack stamped every key that starts a
// run of the sorted batch, so the touched keys are the stamped ones, listed in
// key order - which is the order of their runs.
struct KeyTouchedSrc {
  const unsigned long long* kstamp;
  const unsigned long long* kepoch;
  __device__ int4 operator()(long long k) const {
    return make_int4(kstamp[k] == *kepoch ? 1 : 0, 0, 0, 0);
  }
};
struct KeyTouchedDst {
  const int* kfirst;
  uint32_t* tkey;
  int* tstart;
  uint32_t* tmap;
  long long cap;
  __device__ void operator()(long long k, int4 excl, int4 v) const {
    if (v.x && excl.x < cap) {
      tkey[excl.x] = (uint32_t)k;
      tstart[excl.x] = kfirst[k];
      tmap[k] = (uint32_t)excl.x;
    }
  }
};

struct PrepareArgs {
  KdStoreDev s;
  long long n;
  const uint64_t* k64;
  const uint32_t* tkey;
  const int* tstart;
  const int4* totals;
  int mode;
  const KdCallArgs* call;  // timestamp and merge inputs
  int* tm;
  int* tprior;
  unsigned char* tbuf;
  double* tsf;
  double* tpscale;
  double* st_clock;
  double* st_ls;
  double* st_min;
  double* st_max;
  KdErrHost* err;
};

// _gpu_batch_prepare per touched key (tdigest.mojo:236-296), _advance_clock
// (:324-332), _renormalize (:359-371), _scale_factor (:352-357).
// After the packed sort (digest key and the top value bits, sorted on all but
// the lowest `shift` bits): the sort keys back to (order key, digest key),
// from the sort's last buffers into the free ones, one element per thread.
// Samples of one key that agree in the sorted bits form a run in input order;
// an element smaller than its left neighbour inside such a run is recorded in
// the repair list (fix[0] = count, fix[1..cap]).  Runs of equal values record
// nothing.  A full list sends the step to the full sort.  With kstamp set, the
// first element of every key's run stamps the key with the step's epoch and
// records its position in kfirst.
__global__ void k_unpack(long long n, int kb, int shift, const uint64_t* __restrict__ sk,
                         const uint32_t* __restrict__ skey, const uint32_t* __restrict__ sidx,
                         uint64_t* __restrict__ dk, uint32_t* __restrict__ dkey,
                         uint32_t* __restrict__ didx, int* __restrict__ fix, int cap_fix,
                         KdErrHost* err, long long K, int* __restrict__ kfirst,
                         unsigned long long* __restrict__ kstamp,
                         const unsigned long long* __restrict__ kepoch) {
  const unsigned long long epoch = kstamp ? *kepoch : 0ull;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const uint64_t p = sk[i];
    const uint64_t ok = (p << kb) | (uint64_t)skey[i];
    const uint32_t key = kb > 0 ? (uint32_t)(p >> (64 - kb)) : 0u;
    dk[i] = ok;
    dkey[i] = key;
    if (didx) didx[i] = sidx[i];
    const uint64_t pp = i > 0 ? sk[i - 1] : 0ull;
    if (kstamp && (long long)key < K && (i == 0 || (kb > 0 && (uint32_t)(pp >> (64 - kb)) != key))) {
      kfirst[key] = (int)i;
      kstamp[key] = epoch;
    }
    if (i > 0) {
      if ((pp >> shift) == (p >> shift) && ((pp << kb) | (uint64_t)skey[i - 1]) > ok) {
        const int slot = atomicAdd(&fix[0], 1);
        if (slot < cap_fix) fix[1 + slot] = (int)i;
        else kd_err_set(err, KD_ERESORT, i);
      }
    }
  }
}

// Repairs the runs that hold a recorded inversion: the run's first inversion
// owns it (runs are disjoint, so every run has one writer), finds its ends and
// sorts it by order key, stably, carrying the input indices.  Runs longer
// than KD_PACK_RUN_MAX with an inversion (adversarial data) send the step to
// the full sort.  Source arrays are read-only; only owners write.
#define KD_PACK_RUN_MAX 64
__global__ void k_repair(long long n, int kb, int shift, const uint64_t* __restrict__ sk,
                         const uint32_t* __restrict__ skey, uint64_t* __restrict__ dk,
                         uint32_t* __restrict__ didx, const int* __restrict__ fix, int cap_fix,
                         KdErrHost* err) {
  const int nf = min(fix[0], cap_fix);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += gridDim.x * blockDim.x) {
    const long long i = fix[1 + t];
    const uint64_t top = sk[i] >> shift;
    long long s = i;
    while (s > 0 && i - s < KD_PACK_RUN_MAX && (sk[s - 1] >> shift) == top) --s;
    if (s > 0 && (sk[s - 1] >> shift) == top) {
      kd_err_set(err, KD_ERESORT, i);
      continue;
    }
    bool owner = true;  // no inversion before i in the run
    for (long long a = s + 1; a < i && owner; ++a)
      owner = !(((sk[a - 1] << kb) | (uint64_t)skey[a - 1]) > ((sk[a] << kb) | (uint64_t)skey[a]));
    if (!owner) continue;
    long long e = i + 1;
    while (e < n && e - s <= KD_PACK_RUN_MAX && (sk[e] >> shift) == top) ++e;
    if (e - s > KD_PACK_RUN_MAX) {
      kd_err_set(err, KD_ERESORT, i);
      continue;
    }
    for (long long a = s + 1; a < e; ++a) {  // stable insertion sort by order key
      const uint64_t v = dk[a];
      const uint32_t iv = didx ? didx[a] : 0u;
      long long b = a;
      while (b > s && dk[b - 1] > v) {
        dk[b] = dk[b - 1];
        if (didx) didx[b] = didx[b - 1];
        --b;
      }
      dk[b] = v;
      if (didx) didx[b] = iv;
    }
  }
}

__global__ void k_prepare(PrepareArgs a) {
  const int U = a.totals[0].x;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= U) return;
  if (kd_err_get(a.err)) {  // a failed step: the planner below sees empty keys
    a.tm[j] = 0;
    a.tprior[j] = 0;
    return;
  }
  const uint32_t key = a.tkey[j];
  const int start = a.tstart[j];
  const int end = j + 1 < U ? a.tstart[j + 1] : (int)a.n;
  const int nn = end - start;
  const KdStoreDev& s = a.s;
  const int live = s.cur[key];
  int prior = s.count[key];
  double total = s.total[key], ls = s.log_scale[key], clock = s.clock[key];
  double mn = s.min_v[key], mx = s.max_v[key];
  double pscale = 1.0;
  double sf = 1.0;
  const long long carry = a.call->carry;
  // A carried batch (one-key store): its centroids and buffered samples lead
  // the input; only the rest are the batch's samples.
  const int nb = nn - (int)carry;
  const double vmin = kd_from_order_key(carry ? a.call->carry_mm[0] : a.k64[start]);
  const double vmax = kd_from_order_key(carry ? a.call->carry_mm[1] : a.k64[end - 1]);
  if (carry) prior = 0;
  if (a.mode == KD_MODE_REPLACE || a.mode == KD_MODE_MERGE) {
    prior = 0;
    ls = 0.0;
    if (a.mode == KD_MODE_MERGE) {
      mn = a.call->merge_min[key];
      mx = a.call->merge_max[key];
      clock = a.call->merge_clock[key];
    } else {
      mn = vmin;
      mx = vmax;
      clock = (double)nn;
    }
  } else {
    const bool decay = s.lambda > 0.0;
    double new_clock = clock;
    bool advance = false;
    if (a.mode == KD_MODE_COUNT) {
      new_clock = KD_ADD(clock, (double)nb);
      advance = true;
    } else if (a.call->timestamp > clock) {
      new_clock = a.call->timestamp;
      advance = true;
    }
    if (advance) {
      if (decay && new_clock > clock) {
        ls = KD_ADD(ls, KD_MUL(s.lambda, KD_SUB(new_clock, clock)));
        if (ls > 400.0) {
          pscale = kd_exp(-ls);
          total = KD_MUL(total, pscale);
          ls = 0.0;
        }
      }
      clock = new_clock;
    }
    sf = decay ? kd_exp(ls) : 1.0;
    const double added = KD_MUL((double)nb, sf);
    total = KD_ADD(total, added);
    if (total == added && prior == 0) {
      mn = vmin;
      mx = vmax;
    } else {
      if (vmin < mn) mn = vmin;
      if (vmax > mx) mx = vmax;
    }
  }
  a.tm[j] = prior + nn;
  a.tprior[j] = prior;
  a.tbuf[j] = (unsigned char)(live ^ 1);
  a.tsf[j] = sf;
  a.tpscale[j] = pscale;
  a.st_clock[j] = clock;
  a.st_ls[j] = ls;
  a.st_min[j] = mn;
  a.st_max[j] = mx;
}

// Tiles of a key with m input elements: floor(m/1024) full tiles plus a partial
// tile of r = m mod 1024 elements; only that partial tile can be small.  A
// small tile (r <= cap, cap <= KD_SERIAL_TILE_MAX) goes to the small-tile
// kernel, every other tile to the large-tile kernel.  The split only chooses
// the kernel: both compute a tile in the same canonical order, so cap is a
// tuning parameter that never changes a result.
struct TileSplit {
  int small, large;
};
__device__ __forceinline__ TileSplit tile_split(int m, int cap) {
  const int full = m / KD_TILE, r = m - full * KD_TILE;
  TileSplit t;
  t.small = (r > 0 && r <= cap) ? 1 : 0;
  t.large = full + (r > cap ? 1 : 0);
  return t;
}
__device__ __forceinline__ void write_work(const KdLevelDev& lv, int a, int m, int s_off, int l_off,
                                           long long cap_work, int cap) {
  const int full = m / KD_TILE, r = m - full * KD_TILE;
  int nl = full;
  if (r > cap) ++nl;
  for (int lt = 0; lt < nl; ++lt)
    if (l_off + lt < cap_work) lv.work_l[l_off + lt] = make_int2(a, lt);
  if (r > 0 && r <= cap && s_off < cap_work) lv.work_s[s_off] = make_int2(a, full);
}

// Level-0 plan over the touched keys: small / large tiles, multi-tile keys and
// the dense offset of every key's merged input.
struct Plan0Src {
  const int4* totals;
  const int* tm;
  int small_cap;
  __device__ int4 operator()(long long j) const {
    if (j >= totals[0].x) return make_int4(0, 0, 0, 0);
    const int m = tm[j];
    const TileSplit t = tile_split(m, small_cap);
    return make_int4(t.small, t.large, m > KD_TILE ? 1 : 0, m);
  }
};
struct Plan0Dst {
  const int4* totals;
  const int* tm;
  KdLevelDev cur;
  KdLevelDev nxt;
  long long cap_work;
  long long cap_keys;
  int small_cap;
  __device__ void operator()(long long j, int4 excl, int4 v) const {
    if (j >= totals[0].x) return;
    cur.j[j] = (int)j;
    cur.m[j] = v.w;
    cur.base[j] = excl.w;
    write_work(cur, (int)j, v.w, excl.x, excl.y, cap_work, small_cap);
    if (v.z && excl.z < cap_keys) {
      nxt.j[excl.z] = (int)j;
      nxt.src_tiles[excl.z] = v.x + v.y;
      nxt.mprev[excl.z] = v.w;
    }
  }
};

struct InterArgs {
  const int* A;  // multi-tile keys of level 0
  KdLevelDev cur;
  KdLevelDev nxt;
  int* I;
  long long cap_inter;
  int* needs;
  KdErrHost* err;
};

// Intermediate-tile offsets of the level-0 keys that exceed one tile (one block).
__global__ void __launch_bounds__(1024) k_inter0(InterArgs p) {
  __shared__ int4 sw[32];
  const int A = *p.A;
  const int per = (A + blockDim.x - 1) / blockDim.x;
  const int a0 = min(A, (int)threadIdx.x * per), a1 = min(A, a0 + per);
  int sum = 0;
  for (int a = a0; a < a1; ++a) sum += p.nxt.src_tiles[a];
  int4 tot;
  const int4 incl = block_scan_incl(make_int4(sum, 0, 0, 0), sw, &tot);
  int run = incl.x - sum;
  for (int a = a0; a < a1; ++a) {
    p.nxt.src_base[a] = run;
    p.cur.inter_off[p.nxt.j[a]] = run;
    run += p.nxt.src_tiles[a];
  }
  if (threadIdx.x == 0) {
    *p.I = tot.x;
    if (tot.x > p.cap_inter) {
      atomicMax(&p.needs[2], tot.x);
      kd_err_set(p.err, KD_ERANGE_SCRATCH, tot.x);
    }
  }
}

struct TileArgs {
  KdStoreDev s;
  const int* Tl;
  const int* Ts;
  const int* I;
  KdLevelDev lv;
  const double* dx;
  const double* dw;
  const uint32_t* tkey;
  const unsigned char* tbuf;
  int* st_count;
  double* scr_m;
  double* scr_w;
  int* tcount;
  long long cap_work;
  long long cap_inter;
  int* needs;
  int force_exact;
  int id_last;  // bucket id at q == 1 for K0/K1 (a launch constant)
  KdErrHost* err;
  // Level 0 reads no dense input: each tile is merged on the fly from the
  // key's prior centroids (live slot) and its sorted new samples.
  int level0;
  const uint64_t* k64;    // sorted order keys of the new samples
  const uint32_t* sidx;   // their input positions (per-sample weights), or null
  const KdCallArgs* call;
  const int* tstart;
  const int* tprior;
  const double* tsf;
  const double* tpscale;
  const int4* totals;
  long long n;
};

// Elements [d0 + q0, d0 + q1) of the merged input of touched key j: its prior
// centroids (weights rescaled by the renormalisation factor) and its new
// samples (their own weight, or the key's decay weight), ordered by value with
// priors first on equal values (gpu/sort.mojo:38-41).  A merge-path binary
// search finds where the range starts, then the range is merged in order;
// put(q, value, weight) receives every element.
// Weight of the sample at input position i: its own weight, or the key's decay
// weight sf.  In a carried batch the leading `carry` inputs are the digest's
// centroids and buffered samples, whose stored weights take the
// renormalisation factor like any prior centroid (tdigest.mojo:359-371); the
// batch's own samples take sf.
__device__ __forceinline__ double sample_weight(const double* wts, uint32_t i, long long carry,
                                                double sf, double pscale) {
  if (!wts) return sf;
  if (!carry) return wts[i];
  if ((long long)i >= carry) return sf;
  return pscale != 1.0 ? KD_MUL(wts[i], pscale) : wts[i];
}

template <class Put>
__device__ __forceinline__ void merge_load(const TileArgs& a, int j, int d0, int q0, int q1, Put put) {
  if (q0 >= q1) return;
  const int U = a.totals[0].x;
  const int np = a.tprior[j];
  const int s0 = a.tstart[j];
  const int nn = (j + 1 < U ? a.tstart[j + 1] : (int)a.n) - s0;
  const uint32_t key = a.tkey[j];
  const int live = a.tbuf[j] ^ 1;
  const double* pm = a.s.slot_m + slot_base(a.s.K, live, key);
  const double* pw = a.s.slot_w + slot_base(a.s.K, live, key);
  const double pscale = a.tpscale[j];
  const bool rescale = pscale != 1.0;
  const double sf = a.tsf[j];
  const uint64_t* nk = a.k64 + s0;
  const double* wts = a.call->wts;
  const uint32_t* sidx = a.sidx ? a.sidx + s0 : nullptr;
  const int d = d0 + q0;
  int lo = max(0, d - nn), hi = min(d, np);
  while (lo < hi) {  // priors among the first d merged elements
    const int mid = (lo + hi) >> 1;
    if (kd_order_key(pm[mid]) <= nk[d - mid - 1]) lo = mid + 1;
    else hi = mid;
  }
  int ia = lo, ib = d - lo;
  for (int q = q0; q < q1; ++q) {
    const bool take_prior = ia < np && (ib >= nn || kd_order_key(pm[ia]) <= nk[ib]);
    if (take_prior) {
      put(q, kd_from_order_key(kd_order_key(pm[ia])), rescale ? KD_MUL(pw[ia], pscale) : pw[ia]);
      ++ia;
    } else {
      put(q, kd_from_order_key(nk[ib]), sample_weight(wts, sidx[ib], a.call->carry, sf, pscale));
      ++ib;
    }
  }
}

__device__ __forceinline__ bool tiles_fit(const TileArgs& a, int T) {
  const int I = *a.I;
  if (T > a.cap_work || I > a.cap_inter) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      atomicMax(&a.needs[0], T);
      atomicMax(&a.needs[2], I);
      kd_err_set(a.err, KD_ERANGE_SCRATCH, T);
    }
    return false;
  }
  return true;
}

// Output location of tile (ai, lt): the key's back slot when its input fits one
// tile, else the tile's intermediate slot.
struct TileOut {
  double* m;
  double* w;
  int* count;
};
__device__ __forceinline__ TileOut tile_out(const TileArgs& a, int ai, int lt, int j, int m) {
  TileOut o;
  if (m <= KD_TILE) {
    const uint32_t key = a.tkey[j];
    const int backb = a.tbuf[j];
    o.m = a.s.slot_m + slot_base(a.s.K, backb, key);
    o.w = a.s.slot_w + slot_base(a.s.K, backb, key);
    o.count = a.st_count + j;
  } else {
    const int it = a.lv.inter_off[ai] + lt;
    o.m = a.scr_m + (size_t)it * KD_TILE;
    o.w = a.scr_w + (size_t)it * KD_TILE;
    o.count = a.tcount + it;
  }
  return o;
}

// One warp per tile of the small work list (tiles of at most
// KD_SERIAL_TILE_MAX elements, 4 warps per block): coalesced load, then the
// warp tile compress.  The large work list has its own kernel (k_tiles_blk).
template <int CAP>
__global__ void __launch_bounds__(32 * (CAP == KD_TILE ? 1 : 4)) k_tiles(TileArgs a) {
  static_assert(CAP == KD_SERIAL_TILE_MAX, "the warp tile compress serves small tiles only");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int WPB = CAP == KD_TILE ? 1 : 4;
  WarpTileT<CAP>& t = reinterpret_cast<WarpTileT<CAP>*>(smem_raw)[threadIdx.x >> 5];
  if (kd_err_get(a.err)) return;
  const int T = CAP == KD_TILE ? *a.Tl : *a.Ts;
  if (!tiles_fit(a, T)) return;
  const int2* work = CAP == KD_TILE ? a.lv.work_l : a.lv.work_s;
  const int lane = threadIdx.x & 31;
  const KdStoreDev& s = a.s;
  for (int w = blockIdx.x * WPB + (threadIdx.x >> 5); w < T; w += gridDim.x * WPB) {
    const int2 wk = work[w];
    const int ai = wk.x, lt = wk.y;
    const int j = a.lv.j[ai];
    const int m = a.lv.m[ai];
    const long long src = (long long)a.lv.base[ai] + (long long)lt * KD_TILE;
    const int n = min(KD_TILE, m - lt * KD_TILE);
    const int E = tile_chunk(n), SE = E | 1;
    const unsigned inv = tile_inv(E);
    bool integral = true;
    if (a.level0 && CAP <= KD_SERIAL_TILE_MAX && m <= CAP) {
      // The key's whole merged input is this tile: stage both sorted lists'
      // order keys in shared memory (one round of loads each), then place
      // every element by a shared-memory search (a new sample after the
      // priors <= it, a prior after the new samples < it).
      const int U = a.totals[0].x;
      const int np = a.tprior[j];
      const int s0 = a.tstart[j];
      const int nn = (j + 1 < U ? a.tstart[j + 1] : (int)a.n) - s0;
      const uint32_t key = a.tkey[j];
      const int live = a.tbuf[j] ^ 1;
      const double* pm = s.slot_m + slot_base(s.K, live, key);
      const double* pw = s.slot_w + slot_base(s.K, live, key);
      uint64_t* pk = reinterpret_cast<uint64_t*>(t.L);     // prior order keys
      uint64_t* nk = reinterpret_cast<uint64_t*>(t.P);     // new order keys (P .. endpos)
      for (int i = lane; i < np; i += 32) pk[i] = kd_order_key(pm[i]);
      for (int i = lane; i < nn; i += 32) nk[i] = a.k64[s0 + i];
      __syncwarp();
      const double pscale = a.tpscale[j];
      const double sf = a.tsf[j];
      const double* wts = a.call->wts;
      for (int i = lane; i < np; i += 32) {
        const uint64_t v = pk[i];
        int lo = 0, hi = nn;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (nk[mid] < v) lo = mid + 1;
          else hi = mid;
        }
        const double wv = pscale != 1.0 ? KD_MUL(pw[i], pscale) : pw[i];
        const int slot = tile_slot(i + lo, E, SE, inv);
        t.x[slot] = kd_from_order_key(v);
        t.w[slot] = wv;
        integral = integral && kd_is_small_int(wv);
      }
      for (int i = lane; i < nn; i += 32) {
        const uint64_t v = nk[i];
        int lo = 0, hi = np;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (pk[mid] <= v) lo = mid + 1;
          else hi = mid;
        }
        const double wv = sample_weight(wts, a.sidx ? a.sidx[s0 + i] : 0u, a.call->carry, sf, pscale);
        const int slot = tile_slot(i + lo, E, SE, inv);
        t.x[slot] = kd_from_order_key(v);
        t.w[slot] = wv;
        integral = integral && kd_is_small_int(wv);
      }
      __syncwarp();
    } else if (a.level0) {
      const int per = (n + 31) >> 5;
      merge_load(a, j, lt * KD_TILE, min(n, lane * per), min(n, lane * per + per),
                 [&](int q, double xv, double wv) {
                   const int slot = tile_slot(q, E, SE, inv);
                   t.x[slot] = xv;
                   t.w[slot] = wv;
                   integral = integral && kd_is_small_int(wv);
                 });
    } else {
      for (int p = lane; p < n; p += 32) {
        const int slot = tile_slot(p, E, SE, inv);
        const double wv = a.dw[src + p];
        t.x[slot] = a.dx[src + p];
        t.w[slot] = wv;
        integral = integral && kd_is_small_int(wv);
      }
    }
    integral = __all_sync(0xffffffffu, integral);
    __syncwarp();
    const TileOut o = tile_out(a, ai, lt, j, m);
    const int c = integral
                      ? warp_compress<true>(t, n, s.scale, s.compression, a.force_exact,
                                                 a.id_last, o.m, o.w)
                      : warp_compress<false>(t, n, s.scale, s.compression, a.force_exact,
                                                  a.id_last, o.m, o.w);
    if (lane == 0) *o.count = c;
  }
}

// One block of KD_TILE_WARPS warps per tile above the small-tile cap (the large
// work list): coalesced load into the slot layout, then block_compress.
template <int W>
__global__ void __launch_bounds__(W * 32) k_tiles_blk(TileArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpTile& t = *reinterpret_cast<WarpTile*>(smem_raw);
  __shared__ BlockScr<W> bs;
  if (threadIdx.x == 0) bs.stop = kd_err_get(a.err);  // one read, so the block exits as one
  __syncthreads();
  if (bs.stop) return;
  const int T = *a.Tl;
  if (!tiles_fit(a, T)) return;
  const KdStoreDev& s = a.s;
  for (int wi = blockIdx.x; wi < T; wi += gridDim.x) {
    const int2 wk = a.lv.work_l[wi];
    const int ai = wk.x, lt = wk.y;
    const int j = a.lv.j[ai];
    const int m = a.lv.m[ai];
    const long long src = (long long)a.lv.base[ai] + (long long)lt * KD_TILE;
    const int n = min(KD_TILE, m - lt * KD_TILE);
    const int E = tile_chunk(n), SE = E | 1;
    const unsigned inv = tile_inv(E);
    bool integral = true;
    if (a.level0) {
      const int per = (n + blockDim.x - 1) / blockDim.x;
      const int q0 = min(n, (int)threadIdx.x * per);
      merge_load(a, j, lt * KD_TILE, q0, min(n, q0 + per), [&](int q, double xv, double wv) {
        const int slot = tile_slot(q, E, SE, inv);
        t.x[slot] = xv;
        t.w[slot] = wv;
        integral = integral && kd_is_small_int(wv);
      });
    } else {
      for (int p = threadIdx.x; p < n; p += blockDim.x) {
        const int slot = tile_slot(p, E, SE, inv);
        const double wv = a.dw[src + p];
        t.x[slot] = a.dx[src + p];
        t.w[slot] = wv;
        integral = integral && kd_is_small_int(wv);
      }
    }
    integral = __syncthreads_and(integral);
    const TileOut o = tile_out(a, ai, lt, j, m);
    const int c = integral
                      ? block_compress<true, W>(t, bs, n, s.scale, s.compression, a.force_exact,
                                             a.id_last, o.m, o.w)
                      : block_compress<false, W>(t, bs, n, s.scale, s.compression, a.force_exact,
                                              a.id_last, o.m, o.w);
    if (threadIdx.x == 0) *o.count = c;
  }
}

struct PlanArgs {
  const int* A;
  const int* Iprev;  // intermediate tiles written by the previous level
  KdLevelDev cur;
  KdLevelDev nxt;
  const int* tcount;
  int* gpre;  // dense offset of every previous-level intermediate tile
  const uint32_t* tkey;
  long long cap_work;
  long long cap_inter;
  long long cap_keys;
  long long cap_merged;
  int small_cap;
  int* needs;
  KdErrHost* err;
};

// Levels >= 1 (one block).  The previous level's survivors are laid out densely
// in intermediate-tile order, so one scan of the tile counts gives every active
// key its dense base and size (the reference's _scan_counts_kernel,
// add_batch.mojo:407-452); then each key's new tiling and work lists, and the
// keys still above one tile move on to the next level.
__global__ void __launch_bounds__(1024) k_plan(PlanArgs p) {
  __shared__ int4 sw[32];
  const int A = *p.A;
  if (A == 0 || kd_err_get(p.err)) {
    if (threadIdx.x == 0) {
      *p.cur.Tl = 0;
      *p.cur.Ts = 0;
      *p.cur.I = 0;
      *p.cur.M = 0;
      *p.nxt.A = 0;
    }
    return;
  }
  // 1. exclusive scan of the previous level's tile counts -> gpre
  const int I = *p.Iprev;
  {
    const int per = (I + blockDim.x - 1) / blockDim.x;
    const int s0 = min(I, (int)threadIdx.x * per), s1 = min(I, s0 + per);
    int sum = 0;
    for (int s = s0; s < s1; ++s) sum += p.tcount[s];
    int4 tot;
    int4 incl = block_scan_incl(make_int4(sum, 0, 0, 0), sw, &tot);
    int run = incl.x - sum;
    for (int s = s0; s < s1; ++s) {
      p.gpre[s] = run;
      run += p.tcount[s];
    }
    if (threadIdx.x == 0) p.gpre[I] = tot.x;
    __syncthreads();
  }
  // 2. per active key: dense base / size, tiling
  const int per = (A + blockDim.x - 1) / blockDim.x;
  const int a0 = min(A, (int)threadIdx.x * per), a1 = min(A, a0 + per);
  int4 acc = make_int4(0, 0, 0, 0);
  int acc_inter = 0;
  for (int a = a0; a < a1; ++a) {
    const int sb = p.cur.src_base[a], se = sb + p.cur.src_tiles[a];
    const int base = p.gpre[sb];
    const int m = p.gpre[se] - base;
    p.cur.base[a] = base;
    p.cur.m[a] = m;
    if (m >= p.cur.mprev[a]) kd_err_set(p.err, KD_ECONVERGE, (long long)p.tkey[p.cur.j[a]]);
    const TileSplit t = tile_split(m, p.small_cap);
    const bool fin = m <= KD_TILE;
    acc = i4add(acc, make_int4(t.small, t.large, fin ? 0 : 1, m));
    acc_inter += fin ? 0 : t.small + t.large;
  }
  int4 tot, tot2;
  const int4 incl = block_scan_incl(acc, sw, &tot);
  const int4 incl2 = block_scan_incl(make_int4(acc_inter, 0, 0, 0), sw, &tot2);
  int4 run = make_int4(incl.x - acc.x, incl.y - acc.y, incl.z - acc.z, incl.w - acc.w);
  int run_inter = incl2.x - acc_inter;
  for (int a = a0; a < a1; ++a) {
    const int m = p.cur.m[a];
    const TileSplit t = tile_split(m, p.small_cap);
    const bool fin = m <= KD_TILE;
    p.cur.inter_off[a] = run_inter;
    write_work(p.cur, a, m, run.x, run.y, p.cap_work, p.small_cap);
    if (!fin && run.z < p.cap_keys) {
      p.nxt.j[run.z] = p.cur.j[a];
      p.nxt.src_base[run.z] = run_inter;
      p.nxt.src_tiles[run.z] = t.small + t.large;
      p.nxt.mprev[run.z] = m;
    }
    run = i4add(run, make_int4(t.small, t.large, fin ? 0 : 1, m));
    run_inter += fin ? 0 : t.small + t.large;
  }
  if (threadIdx.x == 0) {
    *p.cur.Ts = tot.x;
    *p.cur.Tl = tot.y;
    *p.cur.I = tot2.x;
    *p.cur.M = tot.w;
    *p.nxt.A = tot.z;
    if (tot.x > p.cap_work || tot.y > p.cap_work || tot2.x > p.cap_inter || tot.w > p.cap_merged) {
      atomicMax(&p.needs[0], max(tot.x, tot.y));
      atomicMax(&p.needs[1], tot.w);
      atomicMax(&p.needs[2], tot2.x);
      kd_err_set(p.err, KD_ERANGE_SCRATCH, tot.y);
    }
  }
}

struct CompactArgs {
  const int* Iprev;
  const int* tcount;
  const int* gpre;
  const double* scr_m;
  const double* scr_w;
  double* dx;
  double* dw;
  KdErrHost* err;
};

// Packs the previous level's survivors densely, one warp per intermediate tile
// (the gather of _gather_tiles_kernel, add_batch.mojo:455-478).
__global__ void k_compact(CompactArgs c) {
  if (kd_err_get(c.err)) return;
  const int I = *c.Iprev;
  const int lane = threadIdx.x & 31;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < I;
       s += (gridDim.x * blockDim.x) >> 5) {
    const int cnt = c.tcount[s];
    const long long d = c.gpre[s];
    const size_t so = (size_t)s * KD_TILE;
    for (int r = lane; r < cnt; r += 32) {
      c.dx[d + r] = c.scr_m[so + r];
      c.dw[d + r] = c.scr_w[so + r];
    }
  }
}

struct CommitArgs {
  KdStoreDev s;
  const int4* totals;
  const uint32_t* tkey;
  const unsigned char* tbuf;
  const int* st_count;
  const double* st_clock;
  const double* st_ls;
  const double* st_min;
  const double* st_max;
  const int* remaining;  // active keys left after the last level
  KdErrHost* err;
  // Batch chain of a pipelined multi-batch ingest (null otherwise): set by the
  // first batch that fails; no later batch of the chain commits.
  int* chain;
};

// _gpu_batch_finish (tdigest.mojo:298-315) + _prune (:441-458) per key, the
// quantile-walk prefix (:526-536), then publication of the new slot.
__device__ __forceinline__ void commit_header(const KdStoreDev& s, const CommitArgs& a, long long j,
                                              uint32_t key, int b, int cnt, double total) {
  const double ls = a.st_ls[j];
  s.count[key] = cnt;
  s.total[key] = total;
  s.log_scale[key] = ls;
  s.clock[key] = a.st_clock[j];
  s.min_v[key] = a.st_min[j];
  s.max_v[key] = a.st_max[j];
  s.dfac[key] = s.lambda > 0.0 ? kd_exp(-ls) : 1.0;
  if (s.bcount) s.bcount[key] = 0;  // a carried batch consumed the buffer
  s.cur[key] = (unsigned char)b;
}

// The serial form: stored total, prune (decay only), walk prefix; returns the
// count after the prune.
__device__ int commit_serial(const KdStoreDev& s, uint32_t key, int b, int cnt, double ls,
                             double* total_out) {
  double* m = s.slot_m + slot_base(s.K, b, key);
  double* w = s.slot_w + slot_base(s.K, b, key);
  double total = 0.0;
  for (int i = 0; i < cnt; ++i) total = KD_ADD(total, w[i]);
  if (s.lambda > 0.0) {
    const double floor_w = KD_MUL(1e-6, kd_exp(ls));
    int k = 0;
    double removed = 0.0;
    for (int i = 0; i < cnt; ++i) {
      const double wi = w[i];
      if (wi >= floor_w) {
        m[k] = m[i];
        w[k] = wi;
        ++k;
      } else {
        removed = KD_ADD(removed, wi);
      }
    }
    if (removed > 0.0) {
      total = KD_SUB(total, removed);
      cnt = k;
    }
  }
  double* P = s.prefix + (size_t)key * KD_TILE;
  if (cnt > 0) {
    double run = KD_MUL(w[0], 0.5);
    P[0] = run;
    for (int i = 0; i + 1 < cnt; ++i) {
      run = KD_ADD(run, KD_MUL(KD_ADD(w[i], w[i + 1]), 0.5));
      P[i + 1] = run;
    }
  }
  *total_out = total;
  return cnt;
}

// With decay: one lane per key, so that the serial FP64 sums keep every lane
// of a warp busy.
__global__ void __launch_bounds__(128) k_commit(CommitArgs a) {
  const int U = a.totals[0].x;
  const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j == 0) {
    if (*a.remaining > 0) kd_err_set(a.err, KD_EMORE_LEVELS, *a.remaining);
    if (a.chain && (kd_err_get(a.err) || *a.remaining > 0)) *a.chain = 1;
  }
  if (j >= U) return;
  if (kd_err_get(a.err) || *a.remaining > 0 || (a.chain && *a.chain)) return;
  const uint32_t key = a.tkey[j];
  const int b = a.tbuf[j];
  double total = 0.0;
  const int cnt = commit_serial(a.s, key, b, a.st_count[j], a.st_ls[j], &total);
  commit_header(a.s, a, j, key, b, cnt, total);
}

// Without decay (no prune): one warp per key.  When all of a key's weights are
// integral (every unit-weight ingest), its stored total and walk prefix are
// exact in integers: prefix[i] = sum(w[0..i)) + w[i] / 2 with total < 1024 *
// 2^42, so every partial sum and half-sum the serial form computes is exact
// and a warp scan over the centroids gives the same bits.  Other keys take
// the serial form on lane 0.
__global__ void __launch_bounds__(256) k_commit_warp(CommitArgs a) {
  const int U = a.totals[0].x;
  const int lane = threadIdx.x & 31;
  const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  if (warp0 == 0 && lane == 0) {
    if (*a.remaining > 0) kd_err_set(a.err, KD_EMORE_LEVELS, *a.remaining);
    if (a.chain && (kd_err_get(a.err) || *a.remaining > 0)) *a.chain = 1;
  }
  int stop = 0;
  if (lane == 0) stop = (kd_err_get(a.err) || *a.remaining > 0 || (a.chain && *a.chain)) ? 1 : 0;
  if (__shfl_sync(0xffffffffu, stop, 0)) return;  // warp-uniform
  const KdStoreDev& s = a.s;
  for (long long j = warp0; j < U; j += nwarps) {
    const uint32_t key = a.tkey[j];
    const int b = a.tbuf[j];
    int cnt = a.st_count[j];
    const double* w = s.slot_w + slot_base(s.K, b, key);
    bool integral = true;
    for (int i = lane; i < cnt; i += 32) integral = integral && kd_is_small_int(w[i]);
    double total = 0.0;
    if (__all_sync(0xffffffffu, integral)) {
      double* P = s.prefix + (size_t)key * KD_TILE;
      long long carry = 0;
      for (int i0 = 0; i0 < cnt; i0 += 32) {
        const int i = i0 + lane;
        const long long wi = i < cnt ? kd_small_int(w[i]) : 0;
        long long incl = wi;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const long long t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        if (i < cnt) P[i] = KD_MUL((double)(2 * (carry + incl - wi) + wi), 0.5);
        carry += __shfl_sync(0xffffffffu, incl, 31);
      }
      total = (double)carry;
    } else if (lane == 0) {
      cnt = commit_serial(s, key, b, cnt, a.st_ls[j], &total);
    }
    if (lane == 0) commit_header(s, a, j, key, b, cnt, total);
  }
}

// ---------------------------------------------------------------------------
// Queries: TDigest.quantile / cdf (tdigest.mojo:485-587) with binary searches
// over the committed prefix (bit-identical to the reference's serial walk).
// ---------------------------------------------------------------------------
// One (key, q | x) query against a resident digest; NaN and the error word on
// failure (key out of range, q outside [0, 1], empty digest).
__device__ __forceinline__ double store_query(const KdStoreDev& s, uint32_t key, double q, bool is_cdf,
                                              KdErrHost* err, long long i) {
  const double nan = kd_from_bits(0x7ff8000000000000ULL);
  if ((long long)key >= s.K || (!is_cdf && !(q >= 0.0 && q <= 1.0))) {
    kd_err_set(err, KD_EINVAL, i);
    return nan;
  }
  const int nc = s.count[key];
  if (nc == 0) {
    kd_err_set(err, KD_EEMPTY, i);
    return nan;
  }
  const int b = s.cur[key];
  KdQueryDigest d;
  d.m = s.slot_m + slot_base(s.K, b, key);
  d.w = s.slot_w + slot_base(s.K, b, key);
  d.P = s.prefix + (size_t)key * KD_TILE;
  d.nc = nc;
  d.n = s.total[key];
  d.mn = s.min_v + key;
  d.mx = s.max_v + key;
  d.dfac = s.lambda > 0.0 ? s.dfac + key : nullptr;
  d.single = 1.0 + 1e-9;  // tdigest.mojo:481-483 (effective weight)
  return is_cdf ? kd_cdf_one(d, q) : kd_quantile_one(d, q);
}

__global__ void k_query(KdStoreDev s, const uint32_t* __restrict__ keys, const double* __restrict__ qx,
                        long long nq, double* __restrict__ out, int is_cdf, KdErrHost* err) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nq;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = store_query(s, keys ? keys[i] : 0u, qx[i], is_cdf != 0, err, i);
}

// Quantile and cdf queries of one call in one launch: indices [0, nq) are the
// quantiles, [nq, nq + nc) the cdfs.
__global__ void k_query2(KdStoreDev s, const uint32_t* __restrict__ qk, const double* __restrict__ qs,
                         long long nq, double* __restrict__ qout, const uint32_t* __restrict__ ck,
                         const double* __restrict__ xs, long long nc, double* __restrict__ cout,
                         KdErrHost* err) {
  const long long tot = nq + nc;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot;
       i += (long long)gridDim.x * blockDim.x) {
    if (i < nq) {
      qout[i] = store_query(s, qk ? qk[i] : 0u, qs[i], false, err, i);
    } else {
      const long long j = i - nq;
      cout[j] = store_query(s, ck ? ck[j] : 0u, xs[j], true, err, i);
    }
  }
}

// ---------------------------------------------------------------------------
// Batched merge (config: many parts -> one group digest, gpu_merge_digests
// semantics through merge_into's rebasing, query.mojo:348-369 and
// tdigest.mojo:589-623).
// ---------------------------------------------------------------------------
__global__ void k_merge_counts(KdStoreDev src, const uint32_t* parts, long long nparts, int* pcount) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < nparts;
       p += (long long)gridDim.x * blockDim.x) {
    const uint32_t k = parts[p];
    const double eff = src.lambda > 0.0 ? KD_MUL(src.total[k], src.dfac[k]) : src.total[k];
    pcount[p] = eff == 0.0 ? 0 : src.count[k];
  }
}
struct PartSrc {
  const int* pc;
  __device__ int4 operator()(long long i) const { return make_int4(pc[i], 0, 0, 0); }
};
struct PartDst {
  int* poff;
  int4* total;
  __device__ void operator()(long long i, int4 excl, int4) const { poff[i] = excl.x; }
};
__global__ void k_merge_gather(KdStoreDev src, const uint32_t* parts, const long long* goff,
                               long long ngroups, long long nparts, const int* pcount,
                               const int* poff, uint32_t* okey, double* oval, double* owt) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < nparts;
       p += (long long)gridDim.x * blockDim.x) {
    long long lo = 0, hi = ngroups - 1;  // group g with goff[g] <= p < goff[g+1]
    while (lo < hi) {
      long long mid = (lo + hi + 1) >> 1;
      if (goff[mid] <= p) lo = mid;
      else hi = mid - 1;
    }
    const uint32_t k = parts[p];
    const int c = pcount[p];
    const int b = src.cur[k];
    const double* m = src.slot_m + slot_base(src.K, b, k);
    const double* w = src.slot_w + slot_base(src.K, b, k);
    const double f = src.lambda > 0.0 ? kd_exp(-src.log_scale[k]) : 1.0;
    const bool rescale = src.lambda > 0.0;
    const long long o = poff[p];
    for (int i = 0; i < c; ++i) {
      okey[o + i] = (uint32_t)lo;
      oval[o + i] = m[i];
      owt[o + i] = rescale ? KD_MUL(w[i], f) : w[i];
    }
  }
}
__global__ void k_merge_headers(KdStoreDev src, const uint32_t* parts, const long long* goff,
                                long long ngroups, const int* pcount, double* gmin, double* gmax,
                                double* gclock) {
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups;
       g += (long long)gridDim.x * blockDim.x) {
    bool seen = false;
    double mn = 0.0, mx = 0.0, clock = 0.0;
    for (long long p = goff[g]; p < goff[g + 1]; ++p) {
      if (pcount[p] == 0) continue;
      const uint32_t k = parts[p];
      const double a = src.min_v[k], b = src.max_v[k], c = src.clock[k];
      if (!seen) {
        mn = a;
        mx = b;
        seen = true;
      } else {
        mn = mn < a ? mn : a;
        mx = mx > b ? mx : b;
      }
      clock = clock > c ? clock : c;
    }
    gmin[g] = mn;
    gmax[g] = mx;
    gclock[g] = clock;
  }
}

// ---------------------------------------------------------------------------
// Host orchestration
// ---------------------------------------------------------------------------
void kd_set_msg(KdSession* s, const char* msg) {
  snprintf(s->last_error, sizeof s->last_error, "%s", msg);
}

int kd_cuda_fail(KdSession* s, cudaError_t e, const char* what) {
  snprintf(s->last_error, sizeof s->last_error, "%s: %s", what, cudaGetErrorString(e));
  return KD_ECUDA;
}

#define KD_CK(call)                                                   \
  do {                                                                \
    cudaError_t e_ = (call);                                          \
    if (e_ != cudaSuccess) return kd_cuda_fail(s, e_, #call);         \
  } while (0)

static int key_bits_for(long long K) {
  int b = 0;
  while (b < 32 && (1LL << b) < K) ++b;
  return b;
}

static const char* err_text(int code) {
  switch (code) {
    case KD_EINVAL: return "invalid input (key out of range, non-finite value or non-positive weight)";
    case KD_EEMPTY: return "query of an empty digest";
    case KD_ECONVERGE: return "P-path hierarchy did not converge (a pass could not shrink a key's centroids)";
    case KD_ETIMEOUT: return "a bounded device wait gave up (sort look-back); nothing was committed";
    default: return "error";
  }
}


static size_t tile_smem() { return sizeof(WarpTile); }
static size_t tile_smem_small() { return sizeof(WarpTileSmall) * 4; }

int kd_pipeline_prepare_device(KdSession* s) {
  // Function attributes are per device: remember which devices are set up.
  // Setting them twice (two threads racing here) is harmless.
  static std::atomic<bool> done[64];
  std::atomic<bool>* flag = (s->device >= 0 && s->device < 64) ? &done[s->device] : nullptr;
  if (flag && flag->load(std::memory_order_acquire)) return KD_OK;
  KD_CK(cudaFuncSetAttribute(k_tiles_blk<KD_TILE_WARPS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tile_smem()));
  KD_CK(cudaFuncSetAttribute(k_tiles_blk<KD_TILE_WARPS_WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tile_smem()));
  KD_CK(cudaFuncSetAttribute(kd_rs_onesweep<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kd_rs_smem(true)));
  KD_CK(cudaFuncSetAttribute(kd_rs_onesweep<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kd_rs_smem(false)));
  KD_CK(cudaFuncSetAttribute(k_tiles<KD_SERIAL_TILE_MAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tile_smem_small()));
  if (flag) flag->store(true, std::memory_order_release);
  return KD_OK;
}

// Host view of an enqueued ingest step: where the hierarchy stands after its
// levels (pointers into the workspace) and how many kernels it launched.
struct KdStepView {
  const int* curA = nullptr;
  const int* Iprev = nullptr;
  long long launches = 0;
  cudaError_t err = cudaSuccess;  // first failed runtime call while enqueueing
  void note(cudaError_t e) {
    if (err == cudaSuccess) err = e;
  }
};

// Stage events.  Inside a capture they must be external records, which become
// event-record nodes of the graph (a plain record would only mark a capture
// dependency and never complete).
static void stage_mark(KdSession* s, int i) {
  if (!s->stats.enabled) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s->stream, &cs);
  if (cs == cudaStreamCaptureStatusActive)
    cudaEventRecordWithFlags(s->stats.ev[i], s->stream, cudaEventRecordExternal);
  else
    cudaEventRecord(s->stats.ev[i], s->stream);
}

static KdSortBufs sort_bufs(const KdSession* s, KdWorkspace& w) {
  KdSortBufs b{{w.k64[0], w.k64[1]}, {w.key[0], w.key[1]}, {w.idx[0], w.idx[1]}, w.ghist,
               w.rs_state, w.rs_ticket, w.rs_epoch_base, &w.rs_epochs_used, w.cap_rs_tiles,
               &reinterpret_cast<KdErr*>(w.err)->code};
  if (s->wait_test > 0) {
    b.spin_limit = s->wait_test;
    b.stall_first = 1;
  }
  return b;
}

static void enqueue_tiles(KdSession* s, KdWorkspace& w, const KdStoreDev& sd, const KdLevelDev& lv,
                          const double* dx, const double* dw, int id_last, KdStepView& v,
                          const TileArgs* level0 = nullptr, long long tiles_bound = -1) {
  cudaStream_t str = s->stream;
  // Wide blocks for stores of at most one key per SM (their levels above 0
  // hold few tiles, each waiting for one tile's latency), narrow ones else.
  const bool wide = sd.K <= (long long)s->num_sms;
  const int nt_large = (wide ? KD_TILE_WARPS_WIDE : KD_TILE_WARPS) * 32;
  // The large-tile grid: the tuned blocks per SM, or one block per tile when
  // the host's bound on the tiles fits the kernel's residency (a single
  // digest's batch: its tiles then run in one wave instead of two).
  int& resident = s->large_resident[wide ? 1 : 0];
  if (resident == 0) {
    int r = 0;
    const cudaError_t e =
        wide ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_tiles_blk<KD_TILE_WARPS_WIDE>, nt_large,
                                                             tile_smem())
             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_tiles_blk<KD_TILE_WARPS>, nt_large,
                                                             tile_smem());
    if (e != cudaSuccess) r = 0;
    cudaGetLastError();
    resident = std::max(r, 1);
  }
  long long grid_large = (long long)s->num_sms * s->large_bps;
  if (tiles_bound > grid_large && tiles_bound <= (long long)s->num_sms * resident)
    grid_large = tiles_bound;
  TileArgs ta{sd, lv.Tl, lv.Ts, lv.I, lv, dx, dw, w.tkey, w.tbuf, w.st_count, w.scr_m,
              w.scr_w, w.tcount, w.cap_work, w.cap_inter, w.needs, s->force_exact, id_last,
              w.err};
  if (level0) {  // merge inputs of level 0
    ta.level0 = 1;
    ta.k64 = level0->k64;
    ta.sidx = level0->sidx;
    ta.call = level0->call;
    ta.tstart = level0->tstart;
    ta.tprior = level0->tprior;
    ta.tsf = level0->tsf;
    ta.tpscale = level0->tpscale;
    ta.totals = level0->totals;
    ta.n = level0->n;
  }
  auto launch_large = [&]() {
    if (wide)
      k_tiles_blk<KD_TILE_WARPS_WIDE><<<(int)grid_large, nt_large, tile_smem(), str>>>(ta);
    else
      k_tiles_blk<KD_TILE_WARPS><<<(int)grid_large, nt_large, tile_smem(), str>>>(ta);
  };
  if (s->concurrent_tiles && s->side) {
    // fork: the small-tile kernel on the side stream, joined back before the
    // next launch on the session stream (inside a capture: a graph branch)
    v.note(cudaEventRecord(s->fork_ev, str));
    v.note(cudaStreamWaitEvent(s->side, s->fork_ev, 0));
    k_tiles<KD_SERIAL_TILE_MAX><<<s->num_sms * s->small_bps, 128, tile_smem_small(), s->side>>>(ta);
    v.note(cudaEventRecord(s->join_ev, s->side));
    launch_large();
    v.note(cudaStreamWaitEvent(str, s->join_ev, 0));
  } else {
    launch_large();
    k_tiles<KD_SERIAL_TILE_MAX><<<s->num_sms * s->small_bps, 128, tile_smem_small(), str>>>(ta);
  }
  v.launches += 2;
}

// Hierarchy levels from+1 .. to (each: plan, compaction of the previous level's
// outputs into a dense input, tiles).
static void enqueue_levels(KdSession* s, KdWorkspace& w, const KdStoreDev& sd, int from, int to,
                           int id_last, KdStepView& v) {
  cudaStream_t str = s->stream;
  for (int L = from + 1; L <= to; ++L) {
    KdLevelDev cur = w.lv[L & 1];
    KdLevelDev nxt = w.lv[(L + 1) & 1];
    cur.A = const_cast<int*>(v.curA);
    PlanArgs pa{v.curA, v.Iprev, cur, nxt, w.tcount, w.doff, w.tkey, w.cap_work, w.cap_inter,
                w.cap_keys, w.cap_merged, s->small_cap, w.needs, w.err};
    k_plan<<<1, 1024, 0, str>>>(pa);
    CompactArgs ca{v.Iprev, w.tcount, w.doff, w.scr_m, w.scr_w, w.dx[L & 1], w.dw[L & 1], w.err};
    k_compact<<<s->num_sms * 4, 256, 0, str>>>(ca);
    v.launches += 2;
    enqueue_tiles(s, w, sd, cur, w.dx[L & 1], w.dw[L & 1], id_last, v);
    v.curA = nxt.A;
    v.Iprev = cur.I;
  }
}

// How a step's commit reports inside a pipelined multi-batch ingest: the batch
// chain flag, and no readback into the workspace's host slots (the caller
// copies each batch's status into a slot of its own).
struct KdTailOut {
  int* chain = nullptr;
  bool no_readback = false;
};

// Commit (prune, prefix, slot flip) and the status readback.
static void enqueue_tail(KdSession* s, KdWorkspace& w, const KdStoreDev& sd, long long keys_max,
                         KdStepView& v, const KdTailOut* out = nullptr) {
  cudaStream_t str = s->stream;
  stage_mark(s, 5);
  CommitArgs ca{sd, w.totals, w.tkey, w.tbuf, w.st_count, w.st_clock, w.st_ls, w.st_min,
                w.st_max, v.curA, w.err, out ? out->chain : nullptr};
  if (sd.lambda > 0.0)
    k_commit<<<(int)((keys_max + 127) / 128), 128, 0, str>>>(ca);
  else
    k_commit_warp<<<(int)std::min<long long>((keys_max + 7) / 8, (long long)s->num_sms * 16), 256, 0,
                    str>>>(ca);
  v.launches += 1;
  stage_mark(s, 6);
  v.note(cudaGetLastError());
  if (out && out->no_readback) return;
  v.note(cudaMemcpyAsync(w.h_err, w.err, sizeof(KdErrHost), cudaMemcpyDeviceToHost, str));
  v.note(cudaMemcpyAsync(w.h_scalars, w.needs, sizeof(int) * 4, cudaMemcpyDeviceToHost, str));
}

// One whole ingest step as device work only (so it can be captured): the
// per-call block, prep, sort, planning, level 0, `levels` hierarchy levels,
// commit and readback.  `part` selects the front (bit 0: per-call block, prep,
// sort, unpack and repair, which read only the batch) and the back (bit 1:
// everything from the touched-key scan on, which reads and writes the store),
// so that a pipelined multi-batch ingest can sort one batch while the previous
// one compresses.  The back finds the sorted batch where the front left it.
#define KD_PART_FRONT 1
#define KD_PART_BACK 2
static KdStepView enqueue_step(KdSession* s, KdStore* st, KdWorkspace& w, long long n, int mode,
                               bool with_idx, int levels, int id_last, bool full_sort,
                               int part = KD_PART_FRONT | KD_PART_BACK,
                               const KdTailOut* out = nullptr) {
  cudaStream_t str = s->stream;
  const KdStoreDev sd = st->d;
  const long long keys_max = std::min<long long>(n, sd.K);
  const int key_bits = key_bits_for(sd.K);
  KdStepView v;
  // Packed form: the sort covers the key bits and at least KD_PACK_VALUE_BITS
  // value bits; lower digits are left to the repair (runs of near-equal values).
  const int first_digit = full_sort ? 0 : std::max(0, (64 - key_bits - KD_PACK_VALUE_BITS) / 8);
  const int sort_bits = full_sort ? key_bits : 0;  // packed keys need no key passes
  // Touched keys from the key-level stamps when the batch has at least as
  // many samples as the store has keys (a scan over K instead of over n).
  const bool key_level = !full_sort && w.kstamp && sd.K <= n && sd.K <= w.cap_tmap;
  int r = kd_radix_sort_result(n, sort_bits, first_digit) ^ (full_sort ? 0 : 1);
  if (part & KD_PART_FRONT) {
    v.note(cudaMemcpyAsync(w.d_call, w.h_call, sizeof(KdCallArgs), cudaMemcpyHostToDevice, str));
    v.note(cudaMemsetAsync(w.totals, 0, sizeof(int4) * 8, str));
    v.note(cudaMemsetAsync(w.needs, 0, sizeof(int) * 4, str));
    v.note(cudaMemsetAsync(w.fix, 0, sizeof(int), str));  // repair-list count
    stage_mark(s, 0);
    {
      int grid = (int)std::min<long long>((n + 255) / 256, (long long)s->num_sms * 16);
      k_prep<<<grid, 256, 0, str>>>(n, w.d_call, sd.K, full_sort ? 0 : key_bits, w.k64[0], w.key[0],
                                    with_idx ? w.idx[0] : nullptr, w.err, w.kepoch);
      v.launches += 1;
    }
    stage_mark(s, 1);
    KdSortBufs sb = sort_bufs(s, w);
    int rs = kd_radix_sort(sb, n, sort_bits, with_idx, s->num_sms, str, first_digit);
    v.launches += kd_radix_sort_launches(n, sort_bits, first_digit);
    if (!full_sort) {  // also for n == 1: the key is still packed
      const int r0 = rs;
      const int grid = (int)std::min<long long>((n + 255) / 256, (long long)s->num_sms * 16);
      const int shift = 8 * first_digit;
      k_unpack<<<grid, 256, 0, str>>>(n, key_bits, shift, w.k64[r0], w.key[r0],
                                      with_idx ? w.idx[r0] : nullptr, w.k64[r0 ^ 1], w.key[r0 ^ 1],
                                      with_idx ? w.idx[r0 ^ 1] : nullptr, w.fix, (int)w.cap_fix, w.err,
                                      sd.K, key_level ? w.kfirst : nullptr,
                                      key_level ? w.kstamp : nullptr, w.kepoch);
      k_repair<<<s->num_sms, 256, 0, str>>>(n, key_bits, shift, w.k64[r0], w.key[r0], w.k64[r0 ^ 1],
                                            with_idx ? w.idx[r0 ^ 1] : nullptr, w.fix, (int)w.cap_fix,
                                            w.err);
      v.launches += 2;
      rs ^= 1;
    }
    if (rs != r) v.note(cudaErrorInvalidValue);  // the back would read the wrong buffers
    stage_mark(s, 2);
  }
  if (!(part & KD_PART_BACK)) return v;
  const uint64_t* k64 = w.k64[r];
  const uint32_t* skey = w.key[r];
  const uint32_t* sidx = with_idx ? w.idx[r] : nullptr;
  // scans with one entry per key: one item per thread when the partials fit
  const bool key_items1 = kd_scan_partials_needed(std::max<long long>(sd.K, keys_max), 1) <= w.cap_partials;
  int scan_launches = 0;
  if (key_level && key_items1)
    scan_launches += kd_scan<1>(KeyTouchedSrc{w.kstamp, w.kepoch},
               KeyTouchedDst{w.kfirst, w.tkey, w.tstart, w.tmap, w.cap_keys}, sd.K, w.partials,
               &w.totals[0], str);
  else if (key_level)
    scan_launches += kd_scan(KeyTouchedSrc{w.kstamp, w.kepoch},
                             KeyTouchedDst{w.kfirst, w.tkey, w.tstart, w.tmap, w.cap_keys}, sd.K,
                             w.partials, &w.totals[0], str);
  else
    scan_launches += kd_scan(TouchedSrc{skey}, TouchedDst{skey, w.tkey, w.tstart, w.tmap, w.cap_keys, sd.K}, n,
            w.partials, &w.totals[0], str);
  {
    PrepareArgs pa{sd, n, k64, w.tkey, w.tstart, w.totals, mode, w.d_call, w.tm, w.tprior,
                   w.tbuf, w.tsf, w.tpscale, w.st_clock, w.st_ls, w.st_min, w.st_max, w.err};
    k_prepare<<<(int)((keys_max + 255) / 256), 256, 0, str>>>(pa);
  }
  // Level-0 arrays live in lv[0]; its scalars in totals[1] = (Ts, Tl, A1, M0)
  // and totals[2].x = I0.
  KdLevelDev l0 = w.lv[0];
  l0.Ts = (int*)&w.totals[1] + 0;
  l0.Tl = (int*)&w.totals[1] + 1;
  l0.M = (int*)&w.totals[1] + 3;
  l0.I = (int*)&w.totals[2] + 0;
  int* a1 = (int*)&w.totals[1] + 2;
  if (key_items1)
    scan_launches += kd_scan<1>(Plan0Src{w.totals, w.tm, s->small_cap},
               Plan0Dst{w.totals, w.tm, l0, w.lv[1], w.cap_work, w.cap_keys, s->small_cap}, keys_max,
               w.partials, &w.totals[1], str);
  else
    scan_launches += kd_scan(Plan0Src{w.totals, w.tm, s->small_cap},
            Plan0Dst{w.totals, w.tm, l0, w.lv[1], w.cap_work, w.cap_keys, s->small_cap}, keys_max,
            w.partials, &w.totals[1], str);
  {
    InterArgs ia{a1, l0, w.lv[1], l0.I, w.cap_inter, w.needs, w.err};
    k_inter0<<<1, 1024, 0, str>>>(ia);
  }
  v.launches += scan_launches + 2;
  stage_mark(s, 3);
  TileArgs m0{};
  m0.k64 = k64;
  m0.sidx = sidx;
  m0.call = w.d_call;
  m0.tstart = w.tstart;
  m0.tprior = w.tprior;
  m0.tsf = w.tsf;
  m0.tpscale = w.tpscale;
  m0.totals = w.totals;
  m0.n = n;
  // level-0 tiles: each key's priors fill at most one tile, its samples n_k / 1024 + 1 more
  enqueue_tiles(s, w, sd, l0, nullptr, nullptr, id_last, v, &m0, n / KD_TILE + 2 * keys_max + 1);
  stage_mark(s, 4);
  v.curA = a1;
  v.Iprev = l0.I;
  enqueue_levels(s, w, sd, 0, levels, id_last, v);
  enqueue_tail(s, w, sd, keys_max, v, out);
  return v;
}

// What a captured step depends on besides the per-call block.
static KdGraphKey step_key(const KdSession* s, const KdStoreDev& sd, const KdWorkspace& w,
                           long long n, bool with_idx, int mode, int L) {
  KdGraphKey key;
  key.n = n;
  key.key_bits = key_bits_for(sd.K);
  key.with_idx = with_idx;
  key.mode = mode;
  key.levels = L;
  key.force_exact = s->force_exact;
  key.timing = s->stats.enabled;
  key.scale = sd.scale;
  key.compression = sd.compression;
  key.generation = w.generation;
  key.tuning = s->small_cap | (s->large_bps << 8) | (s->small_bps << 16) | (s->concurrent_tiles << 24) |
               ((s->wait_test != 0) << 25);
  return key;
}

int kd_pipeline_attempt(KdSession* s, KdStore* st, KdWorkspace& w, const uint32_t* d_keys,
                        const double* d_vals, const double* d_wts, long long n, int mode,
                        double timestamp, const double* d_merge_min, const double* d_merge_max,
                        const double* d_merge_clock, long long carry,
                        const unsigned long long* d_carry_mm) {
  cudaStream_t str = s->stream;
  const KdStoreDev sd = st->d;
  const long long keys_max = std::min<long long>(n, sd.K);
  const bool with_idx = d_wts != nullptr;
  // K0/K1 normalisers do not depend on the tile total, so the id of q == 1
  // is one constant per launch (host FP64, same arithmetic as the device).
  const int id_last = sd.scale <= KD_SCALE_K1
                          ? (int)kd_bucket(sd.scale, 1.0, 1.0, kd_normalizer(sd.scale, sd.compression, 1.0))
                          : 0;
  // The per-call block; the status index starts at +inf so that the first
  // offending sample wins the atomicMin.
  KdCallArgs& c = *w.h_call;
  c.keys = d_keys;
  c.vals = d_vals;
  c.wts = d_wts;
  c.merge_min = d_merge_min;
  c.merge_max = d_merge_max;
  c.merge_clock = d_merge_clock;
  c.timestamp = timestamp;
  c.carry = carry;
  c.carry_mm = d_carry_mm;
  c.err = KdErrHost{0, 0, 0x7fffffffffffffffLL};
  KdSortBufs sb = sort_bufs(s, w);
  kd_rs_epoch_reserve(sb, str);
  int L = std::max(1, std::min(st->levels_hint, s->max_levels));

  const KdGraphKey key = step_key(s, sd, w, n, with_idx, mode, L);
  KdStepView v;
  bool ran = false;
  if (s->use_graphs && w.generation != 0) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(str, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
      KdGraphEntry* g = nullptr;
      for (KdGraphEntry& e : st->graphs)
        if (e.exec && e.key == key) g = &e;
      if (!g && key == st->last_eager) {
        // The same step shape twice in a row: capture it once, replay it after.
        KdGraphEntry& slot = st->graphs[st->graph_next];
        st->graph_next = (st->graph_next + 1) % KD_GRAPH_CACHE;
        if (slot.exec) cudaGraphExecDestroy(slot.exec);
        slot = KdGraphEntry();
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(str, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
          const KdStepView cv = enqueue_step(s, st, w, n, mode, with_idx, L, id_last, false);
          const bool ended = cudaStreamEndCapture(str, &graph) == cudaSuccess;
          if (ended && graph && cv.err == cudaSuccess) {
            cudaGraphExec_t ex = nullptr;
            if (cudaGraphInstantiate(&ex, graph, 0) == cudaSuccess) {
              slot.key = key;
              slot.exec = ex;
              slot.curA = cv.curA;
              slot.Iprev = cv.Iprev;
              slot.launches = cv.launches;
              g = &slot;
            }
          }
          if (graph) cudaGraphDestroy(graph);
        }
        cudaGetLastError();  // a capture that failed leaves the eager path below
      }
      if (g) {
        KD_CK(cudaGraphLaunch(g->exec, str));
        v.curA = g->curA;
        v.Iprev = g->Iprev;
        v.launches = g->launches;
        ran = true;
      }
    }
  }
  if (!ran) {
    v = enqueue_step(s, st, w, n, mode, with_idx, L, id_last, false);
    st->last_eager = key;
    KD_CK(v.err);
  }
  KD_CK(cudaGetLastError());
  KD_CK(cudaStreamSynchronize(str));
  if (w.h_err->code == KD_ERESORT) {
    // Two samples of one key agreed in the packed bits and came out of order:
    // nothing was committed; run the step again with the full sort.
    c.err = KdErrHost{0, 0, 0x7fffffffffffffffLL};
    kd_rs_epoch_reserve(sb, str);
    v = enqueue_step(s, st, w, n, mode, with_idx, L, id_last, true);
    KD_CK(v.err);
    KD_CK(cudaStreamSynchronize(str));
  }
  // Keys still above one tile after the planned levels: run more levels from
  // where the step stopped, then commit again.
  while (w.h_err->code == KD_EMORE_LEVELS && L < s->max_levels) {
    *w.h_err = KdErrHost{0, 0, 0x7fffffffffffffffLL};
    KD_CK(cudaMemcpyAsync(w.err, w.h_err, sizeof(KdErrHost), cudaMemcpyHostToDevice, str));
    const int goal = std::min(s->max_levels, L + 2);
    enqueue_levels(s, w, sd, L, goal, id_last, v);
    L = goal;
    enqueue_tail(s, w, sd, keys_max, v);
    KD_CK(v.err);
    KD_CK(cudaStreamSynchronize(str));
  }
  if (w.h_err->code == KD_EMORE_LEVELS) w.h_err->code = KD_ECONVERGE;
  if (w.h_err->code == 0) st->levels_hint = std::max(1, L);
  KdStageStats& T = s->stats;
  T.launches += v.launches;
  T.ingests += 1;
  if (T.enabled) {
    for (int i = 0; i < KD_NSTAGES; ++i) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, T.ev[i], T.ev[i + 1]) == cudaSuccess) T.ms[i] += ms;
      else cudaGetLastError();  // timing is best effort; never fail the next call
    }
  }
  const KdErrHost e = *w.h_err;
  if (e.code == 0) return KD_OK;
  if (e.code == KD_ERANGE_SCRATCH) return KD_ERANGE_SCRATCH;
  char buf[256];
  snprintf(buf, sizeof buf, "%s (at index %lld)", err_text(e.code), e.index);
  kd_set_msg(s, buf);
  return e.code;
}

int kd_pipeline_ingest(KdSession* s, KdStore* st, const uint32_t* d_keys, const double* d_vals,
                       const double* d_wts, long long n, int mode, double timestamp,
                       const double* d_merge_min, const double* d_merge_max,
                       const double* d_merge_clock, long long carry,
                       const unsigned long long* d_carry_mm) {
  if (n <= 0) return KD_OK;
  if (n > (1LL << 31) - 1) {
    kd_set_msg(s, "batch too large (limit 2^31 - 1 samples per call)");
    return KD_ERANGE;
  }
  int rc = kd_pipeline_prepare_device(s);
  if (rc) return rc;
  long long ncap = kd_ws_batch_cap(n, s->ws.err ? s->ws.cap_n : 0);
  long long keys_max = std::min<long long>(ncap, st->d.K);
  long long want_inter = std::max<long long>(64, 2 * (ncap / KD_TILE) + 64);
  long long want_work = 2 * keys_max + ncap / KD_TILE + 64;
  long long want_merged = 2 * ncap + 64 * keys_max + 1024;
  for (int attempt = 0; attempt < 4; ++attempt) {
    KdWorkspace& w0 = s->ws;
    rc = kd_ws_reserve(s, ncap, keys_max, std::max(want_inter, w0.cap_inter),
                       std::max(want_work, w0.cap_work), std::max(want_merged, w0.cap_merged), st->d.K);
    if (rc == KD_ENOMEM && ncap > n) {  // no room for the doubled capacity: the batch's own
      ncap = n;
      keys_max = std::min<long long>(n, st->d.K);
      want_inter = std::max<long long>(64, 2 * (n / KD_TILE) + 64);
      want_work = 2 * keys_max + n / KD_TILE + 64;
      want_merged = 2 * n + 64 * keys_max + 1024;
      rc = kd_ws_reserve(s, ncap, keys_max, std::max(want_inter, w0.cap_inter),
                         std::max(want_work, w0.cap_work), std::max(want_merged, w0.cap_merged), st->d.K);
    }
    if (rc) return rc;
    rc = kd_pipeline_attempt(s, st, s->ws, d_keys, d_vals, d_wts, n, mode, timestamp, d_merge_min,
                             d_merge_max, d_merge_clock, carry, d_carry_mm);
    if (rc != KD_ERANGE_SCRATCH) return rc;
    const int* need = s->ws.h_scalars;
    want_work = std::max<long long>(want_work, (long long)need[0] + need[0] / 4 + 64);
    want_merged = std::max<long long>(want_merged, (long long)need[1] + need[1] / 4 + 1024);
    want_inter = std::max<long long>(want_inter, (long long)need[2] + need[2] / 4 + 64);
  }
  kd_set_msg(s, "ingest scratch could not be sized");
  return KD_ENOMEM;
}

// Pipelined multi-batch ingest.  Batch i uses workspace i mod 3.  Its front
// (per-call block, prep, sort, unpack, repair: reads only the batch) runs on one
// of two `ahead` streams (alternating, so that consecutive fronts may overlap)
// once the back of batch i - 3 has released that workspace; its
// back (touched keys, prepare, levels, commit: reads and writes the store) runs
// on the session stream after the back of batch i - 1 and its own front.  So
// the sort of one batch overlaps the compress of the previous one, and the
// store sees the batches in order, exactly as from one call each.  The commit
// of a batch that fails (or must be retried) sets the chain flag, and no later
// batch commits; the host then retries from that batch one call at a time
// (full sort, more levels, larger scratch) or reports its error.
static int pipe_fail(KdSession* s, cudaError_t e) { return kd_cuda_fail(s, e, "pipelined ingest"); }

int kd_pipeline_ingest_many(KdSession* s, KdStore* st, long long nb, const uint32_t* const* d_keys,
                            const double* const* d_vals, const long long* ns, int mode,
                            const double* timestamps, long long* done, bool host_inputs,
                            const KdBatchHook* hook) {
  *done = 0;
  if (nb <= 0) return KD_OK;
  auto before = [&](long long i, cudaStream_t str) {
    if (hook && hook->before) hook->before(hook->ctx, i, str);
  };
  long long nmax = 0;
  for (long long i = 0; i < nb; ++i) {
    if (ns[i] > (1LL << 31) - 1) {
      kd_set_msg(s, "batch too large (limit 2^31 - 1 samples per call)");
      *done = i;
      return KD_ERANGE;
    }
    nmax = std::max(nmax, ns[i]);
  }
  if (nmax == 0) {
    for (long long i = 0; i < nb; ++i) before(i, s->stream);
    *done = nb;
    return KD_OK;
  }
  int rc = kd_pipeline_prepare_device(s);
  if (rc) return rc;
  const KdStoreDev sd = st->d;
  if (!s->ahead) {
    if (cudaStreamCreateWithFlags(&s->ahead, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->ahead2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking) != cudaSuccess)
      return pipe_fail(s, cudaGetLastError());
    for (cudaEvent_t& e : s->pipe_ev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return pipe_fail(s, cudaGetLastError());
  }
  // Staging of host inputs: keys (16-byte aligned) then values, per workspace.
  const size_t key_bytes = ((size_t)nmax * 4 + 15) / 16 * 16;
  if (host_inputs && s->stage_bytes < key_bytes + (size_t)nmax * 8) {
    const size_t need = key_bytes + (size_t)nmax * 8;
    for (void*& p : s->d_stage) {
      if (p) cudaFree(p);
      p = nullptr;
    }
    s->mem_used -= std::min(s->mem_used, s->stage_bytes * KD_PIPE_WS);
    s->stage_bytes = 0;
    if (s->mem_budget && s->mem_used + need * KD_PIPE_WS > s->mem_budget) {
      kd_set_msg(s, "device-memory budget exceeded by the multi-batch staging buffers");
      return KD_ENOMEM;
    }
    for (void*& p : s->d_stage)
      if (cudaMalloc(&p, need) != cudaSuccess) {
        cudaGetLastError();
        for (void*& q : s->d_stage) {
          if (q) cudaFree(q);
          q = nullptr;
        }
        kd_set_msg(s, "multi-batch staging buffers could not be allocated");
        return KD_ENOMEM;
      }
    s->stage_bytes = need;
    s->mem_used += need * KD_PIPE_WS;
  }
  if (s->cap_many < nb) {
    if (s->h_many) cudaFreeHost(s->h_many);
    s->h_many = nullptr;
    s->cap_many = 0;
    const long long cap = std::max<long long>(nb, 64);
    if (cudaHostAlloc((void**)&s->h_many, sizeof(KdErrHost) * cap, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      kd_set_msg(s, "pinned status slots for a multi-batch ingest could not be allocated");
      return KD_ENOMEM;
    }
    s->cap_many = cap;
  }
  const int id_last = sd.scale <= KD_SCALE_K1
                          ? (int)kd_bucket(sd.scale, 1.0, 1.0, kd_normalizer(sd.scale, sd.compression, 1.0))
                          : 0;
  cudaStream_t M = s->stream, A = s->ahead;
  cudaEvent_t ev_start = s->pipe_ev[0];
  cudaEvent_t* ev_front = &s->pipe_ev[1];
  cudaEvent_t* ev_free = &s->pipe_ev[1 + KD_PIPE_WS];
  cudaEvent_t* ev_copied = &s->pipe_ev[1 + 2 * KD_PIPE_WS];
  cudaEvent_t* ev_staged = &s->pipe_ev[1 + 3 * KD_PIPE_WS];
  cudaStream_t C = s->copy;
  // Batch t's inputs as the kernels read them: in place, or copied on `str`
  // into staging buffer q (after `after`, when given).
  auto stage = [&](long long t, int q, cudaStream_t str, cudaEvent_t after, KdStepView& v,
                   const uint32_t** kout, const double** vout) {
    *kout = d_keys ? d_keys[t] : nullptr;
    *vout = d_vals[t];
    if (!host_inputs) return;
    if (after) v.note(cudaStreamWaitEvent(str, after, 0));
    char* base_p = (char*)s->d_stage[q];
    if (*kout) {
      v.note(cudaMemcpyAsync(base_p, *kout, (size_t)ns[t] * 4, cudaMemcpyHostToDevice, str));
      *kout = (const uint32_t*)base_p;
    }
    v.note(cudaMemcpyAsync(base_p + key_bytes, *vout, (size_t)ns[t] * 8, cudaMemcpyHostToDevice, str));
    *vout = (const double*)(base_p + key_bytes);
  };
  // One batch alone through the one-call path (which owns the retries).
  auto single = [&](long long t) -> int {
    KdStepView v;
    const uint32_t* kk = nullptr;
    const double* vv = nullptr;
    stage(t, 0, M, nullptr, v, &kk, &vv);
    if (v.err != cudaSuccess) return pipe_fail(s, v.err);
    return kd_pipeline_ingest(s, st, kk, vv, nullptr, ns[t], mode, timestamps ? timestamps[t] : 0.0,
                              nullptr, nullptr, nullptr);
  };
  // again[i]: batch i's size recurs in this call (or the batch before it,
  // possibly the last batch of the previous call, had the same size)
  std::vector<char> again((size_t)nb, 0);
  {
    std::unordered_map<long long, long long> last;
    for (long long i = nb - 1; i >= 0; --i) {
      const long long prev = i > 0 ? ns[i - 1] : st->pipe_last_n;
      again[(size_t)i] = (last.count(ns[i]) || prev == ns[i]) ? 1 : 0;
      last[ns[i]] = i;
    }
  }
  st->pipe_last_n = ns[nb - 1];
  KdWorkspace* ws[KD_PIPE_WS];
  ws[0] = &s->ws;
  for (int q = 1; q < KD_PIPE_WS; ++q) ws[q] = &s->ws_more[q - 1];
  long long base = 0;  // batches before it are committed
  while (base < nb) {
    // Every workspace sized as the one-call path sizes its own (from one batch
    // capacity for the largest batch), and at least as large as any already
    // is (a retry on the one-call path may have grown the first); all get the
    // same request, so they grow together.
    long long capn = 0;
    for (KdWorkspace* wp : ws) capn = std::max(capn, wp->err ? wp->cap_n : 0LL);
    bool exact = false;  // sized for the largest batch itself (no room for the doubled capacity)
    long long ncap = 0, kcap = 0, ci = 0, cw = 0, cm = 0;
    auto size_for = [&](long long nc) {
      ncap = nc;
      kcap = std::min<long long>(ncap, sd.K);
      ci = std::max(64LL, 2 * (ncap / KD_TILE) + 64);
      cw = 2 * kcap + ncap / KD_TILE + 64;
      cm = 2 * ncap + 64 * kcap + 1024;
      for (KdWorkspace* wp : ws) {
        ci = std::max(ci, wp->cap_inter);
        cw = std::max(cw, wp->cap_work);
        cm = std::max(cm, wp->cap_merged);
      }
    };
    size_for(kd_ws_batch_cap(nmax, capn));
    bool room = true;
    for (long long i = base; i < std::min(nb, base + KD_PIPE_WS); ++i) {  // the workspaces in use
      KdWorkspace* wp = ws[i % KD_PIPE_WS];
      rc = kd_ws_reserve(s, ncap, kcap, ci, cw, cm, sd.K, wp);
      if (rc == KD_ENOMEM && !exact && ncap > nmax) {
        exact = true;
        size_for(nmax);
        rc = kd_ws_reserve(s, ncap, kcap, ci, cw, cm, sd.K, wp);
      }
      if (rc == KD_ENOMEM && wp != &s->ws) {
        room = false;  // no memory for the extra workspaces: one call per batch
        break;
      }
      if (rc) {
        *done = base;
        return rc;
      }
    }
    if (!room) {
      for (long long t = base; t < nb; ++t) {
        before(t, M);
        const int r = ns[t] > 0 ? single(t) : KD_OK;
        if (r) {
          *done = t;
          return r;
        }
      }
      *done = nb;
      return KD_OK;
    }
    int* chain = s->ws.chain;
    const int L = std::max(1, std::min(st->levels_hint, s->max_levels));
    // One part of a batch's step on stream `str`: replayed from the store's
    // graph for this workspace and part when its shape was captured, else
    // captured now (eager if capture fails).
    auto run_part = [&](int part, int q, KdWorkspace& w, long long n, cudaStream_t str,
                        const KdTailOut* out, KdStepView& v, bool capture) {
      const KdGraphKey key = step_key(s, sd, w, n, false, mode, L);
      KdGraphEntry& g = st->pipe_graphs[q][part == KD_PART_FRONT ? 0 : 1];
      const bool chain_ok = part == KD_PART_FRONT || st->pipe_chain[q] == chain;
      s->stream = str;
      if (!(g.exec && g.key == key && chain_ok) && s->use_graphs && capture) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = KdGraphEntry();
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(str, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
          const KdStepView cv = enqueue_step(s, st, w, n, mode, false, L, id_last, false, part, out);
          const bool ended = cudaStreamEndCapture(str, &graph) == cudaSuccess;
          cudaGraphExec_t ex = nullptr;
          if (ended && graph && cv.err == cudaSuccess &&
              cudaGraphInstantiate(&ex, graph, 0) == cudaSuccess) {
            g.key = key;
            g.exec = ex;
            g.launches = cv.launches;
            if (part != KD_PART_FRONT) st->pipe_chain[q] = chain;
          }
          if (graph) cudaGraphDestroy(graph);
        }
        cudaGetLastError();  // a capture that failed runs eagerly below
      }
      if (g.exec && g.key == key && chain_ok) {
        v.note(cudaGraphLaunch(g.exec, str));
        v.launches += g.launches;
      } else {
        const KdStepView e = enqueue_step(s, st, w, n, mode, false, L, id_last, false, part, out);
        v.note(e.err);
        v.launches += e.launches;
      }
      s->stream = M;
    };
    const int stats_on = s->stats.enabled;
    s->stats.enabled = 0;  // stage events belong to one stream
    KdStepView v;
    v.note(cudaMemsetAsync(chain, 0, sizeof(int), M));
    v.note(cudaEventRecord(ev_start, M));  // the ahead stream starts after all earlier work
    v.note(cudaStreamWaitEvent(A, ev_start, 0));
    v.note(cudaStreamWaitEvent(s->ahead2, ev_start, 0));
    for (long long i = base; i < nb; ++i) {
      s->h_many[i] = KdErrHost{0, 0, 0};
      if (ns[i] == 0) {  // an empty batch changes nothing
        before(i, M);
        continue;
      }
      const int k = (int)(i % KD_PIPE_WS);
      KdWorkspace& w = *ws[k];
      // consecutive fronts on two streams, so that they may overlap each other too
      cudaStream_t A = (s->front_streams > 1 && (i & 1)) ? s->ahead2 : s->ahead;
      if (i >= base + KD_PIPE_WS) v.note(cudaEventSynchronize(ev_copied[k]));  // its last user read this block
      const uint32_t* kk = nullptr;
      const double* vv = nullptr;
      // the staging buffer is free once the front of its last batch has run
      stage(i, k, C, i >= base + KD_PIPE_WS ? ev_front[k] : nullptr, v, &kk, &vv);
      if (host_inputs) {
        v.note(cudaEventRecord(ev_staged[k], C));
        v.note(cudaStreamWaitEvent(A, ev_staged[k], 0));
      }
      KdCallArgs& c = *w.h_call;
      c = KdCallArgs();
      c.keys = kk;
      c.vals = vv;
      c.timestamp = timestamps ? timestamps[i] : 0.0;
      c.err = KdErrHost{0, 0, 0x7fffffffffffffffLL};
      if (i >= base + KD_PIPE_WS) v.note(cudaStreamWaitEvent(A, ev_free[k], 0));
      KdSortBufs sb = sort_bufs(s, w);
      kd_rs_epoch_reserve(sb, A);
      // capture only a batch size that comes again in this call (a new
      // size for every batch would pay a capture per batch)
      const bool capture = again[i];
      run_part(KD_PART_FRONT, k, w, ns[i], A, nullptr, v, capture);
      v.note(cudaEventRecord(ev_copied[k], A));
      v.note(cudaEventRecord(ev_front[k], A));
      before(i, M);  // after batch i - 1's back, beside batch i's front
      v.note(cudaStreamWaitEvent(M, ev_front[k], 0));
      KdTailOut out{chain, true};
      run_part(KD_PART_BACK, k, w, ns[i], M, &out, v, capture);
      v.note(cudaMemcpyAsync(&s->h_many[i], w.err, sizeof(KdErrHost), cudaMemcpyDeviceToHost, M));
      v.note(cudaEventRecord(ev_free[k], M));
    }
    s->stats.enabled = stats_on;
    v.note(cudaStreamSynchronize(M));
    if (v.err != cudaSuccess) {
      *done = base;
      return pipe_fail(s, v.err);
    }
    s->stats.launches += v.launches;
    long long bad = nb;
    for (long long i = base; i < nb && bad == nb; ++i)
      if (s->h_many[i].code != 0) bad = i;
    s->stats.ingests += bad - base;
    if (bad == nb) break;
    const KdErrHost e = s->h_many[bad];
    if (e.code == KD_ERESORT || e.code == KD_EMORE_LEVELS || e.code == KD_ERANGE_SCRATCH) {
      // Nothing from this batch on was committed: run it alone (the one-call
      // path owns these retries: full sort, more levels, larger scratch), then
      // pipeline the rest.
      const int r = single(bad);
      if (r) {
        *done = bad;
        return r;
      }
      base = bad + 1;
      continue;
    }
    char buf[256];
    snprintf(buf, sizeof buf, "%s (batch %lld, at index %lld)", err_text(e.code), bad, e.index);
    kd_set_msg(s, buf);
    *done = bad;
    return e.code;
  }
  *done = nb;
  return KD_OK;
}

int kd_pipeline_quantile(KdSession* s, KdStore* st, const uint32_t* d_keys, const double* d_q,
                         long long nq, double* d_out, int is_cdf) {
  if (nq <= 0) return KD_OK;
  int rc = s->ws.err ? KD_OK : kd_ws_reserve(s, 1, 1, 64, 64, 64, 1);
  if (rc) return rc;
  KdWorkspace& w = s->ws;
  cudaStream_t str = s->stream;
  KdErrHost init{0, 0, -1};
  *w.h_err = init;
  KD_CK(cudaMemcpyAsync(w.err, w.h_err, sizeof(KdErrHost), cudaMemcpyHostToDevice, str));
  int grid = (int)std::min<long long>((nq + 255) / 256, (long long)s->num_sms * 32);
  k_query<<<grid, 256, 0, str>>>(st->d, d_keys, d_q, nq, d_out, is_cdf, w.err);
  KD_CK(cudaGetLastError());
  KD_CK(cudaMemcpyAsync(w.h_err, w.err, sizeof(KdErrHost), cudaMemcpyDeviceToHost, str));
  KD_CK(cudaStreamSynchronize(str));
  if (w.h_err->code) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s (query %lld)", err_text(w.h_err->code), w.h_err->index);
    kd_set_msg(s, buf);
    return w.h_err->code;
  }
  return KD_OK;
}

int kd_pipeline_query2(KdSession* s, KdStore* st, const uint32_t* qk, const double* qs, long long nq,
                       double* qout, const uint32_t* ck, const double* xs, long long nc, double* cout) {
  if (nq + nc <= 0) return KD_OK;
  int rc = s->ws.err ? KD_OK : kd_ws_reserve(s, 1, 1, 64, 64, 64, 1);
  if (rc) return rc;
  KdWorkspace& w = s->ws;
  cudaStream_t str = s->stream;
  *w.h_err = KdErrHost{0, 0, -1};
  const int grid = (int)std::min<long long>((nq + nc + 255) / 256, (long long)s->num_sms * 32);
  // the status reset, the one kernel, the status read-back
  auto enqueue = [&]() {
    cudaMemcpyAsync(w.err, w.h_err, sizeof(KdErrHost), cudaMemcpyHostToDevice, str);
    k_query2<<<grid, 256, 0, str>>>(st->d, qk, qs, nq, qout, ck, xs, nc, cout, w.err);
    cudaMemcpyAsync(w.h_err, w.err, sizeof(KdErrHost), cudaMemcpyDeviceToHost, str);
  };
  KdQueryArgs args;
  const void* ps[6] = {qk, qs, qout, ck, xs, cout};
  for (int i = 0; i < 6; ++i) args.p[i] = ps[i];
  args.nq = nq;
  args.nc = nc;
  bool ran = false;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (s->use_graphs && cudaStreamIsCapturing(str, &cs) == cudaSuccess &&
      cs == cudaStreamCaptureStatusNone) {
    if (!(st->q_graph && st->q_graph_args == args) && args == st->q_last) {
      if (st->q_graph) cudaGraphExecDestroy(st->q_graph);
      st->q_graph = nullptr;
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(str, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        enqueue();
        if (cudaStreamEndCapture(str, &g) == cudaSuccess && g) {
          cudaGraphExec_t ex = nullptr;
          if (cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) {
            st->q_graph = ex;
            st->q_graph_args = args;
          }
        }
        if (g) cudaGraphDestroy(g);
      }
      cudaGetLastError();  // a failed capture leaves the eager path below
    }
    if (st->q_graph && st->q_graph_args == args) {
      KD_CK(cudaGraphLaunch(st->q_graph, str));
      ran = true;
    }
  }
  if (!ran) enqueue();
  st->q_last = args;
  KD_CK(cudaGetLastError());
  KD_CK(cudaStreamSynchronize(str));
  if (w.h_err->code) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s (query %lld)", err_text(w.h_err->code), w.h_err->index);
    kd_set_msg(s, buf);
    return w.h_err->code;
  }
  return KD_OK;
}

int kd_pipeline_query2_enqueue(KdSession* s, KdStore* st, const uint32_t* qk, const double* qs,
                               long long nq, double* qout, const uint32_t* ck, const double* xs,
                               long long nc, double* cout, KdErrHost* err, cudaStream_t str) {
  if (nq + nc <= 0) return KD_OK;
  const int grid = (int)std::min<long long>((nq + nc + 255) / 256, (long long)s->num_sms * 32);
  k_query2<<<grid, 256, 0, str>>>(st->d, qk, qs, nq, qout, ck, xs, nc, cout, err);
  return cudaGetLastError() == cudaSuccess ? KD_OK : KD_ECUDA;
}

int kd_pipeline_merge(KdSession* s, KdStore* dst, KdStore* src, const long long* h_goff,
                      const uint32_t* h_parts, long long ngroups) {
  if (ngroups <= 0) return KD_OK;
  if (ngroups > dst->d.K) {
    kd_set_msg(s, "more groups than keys in the destination store");
    return KD_EINVAL;
  }
  const long long nparts = h_goff[ngroups];
  for (long long p = 0; p < nparts; ++p)
    if ((long long)h_parts[p] >= src->d.K) {
      kd_set_msg(s, "part key out of range of the source store");
      return KD_EINVAL;
    }
  cudaStream_t str = s->stream;
  // Small device arrays for the plan (freed at the end of the call).
  long long* d_goff = nullptr;
  uint32_t* d_parts = nullptr;
  int *d_pc = nullptr, *d_poff = nullptr;
  double *gmin = nullptr, *gmax = nullptr, *gclock = nullptr;
  int4* part_partials = nullptr;
  int4* d_tot = nullptr;
  int rc = KD_OK;
  uint32_t* okey = nullptr;
  double *oval = nullptr, *owt = nullptr;
  int total_elems = 0;
  auto cleanup = [&]() {
    cudaFree(d_goff); cudaFree(d_parts); cudaFree(d_pc); cudaFree(d_poff);
    cudaFree(gmin); cudaFree(gmax); cudaFree(gclock); cudaFree(part_partials); cudaFree(d_tot);
    cudaFree(okey); cudaFree(oval); cudaFree(owt);
  };
#define KD_CKM(call)                                   \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) {                           \
      rc = kd_cuda_fail(s, e_, #call);                 \
      cleanup();                                       \
      return rc;                                       \
    }                                                  \
  } while (0)
  KD_CKM(cudaMalloc(&d_goff, sizeof(long long) * (ngroups + 1)));
  KD_CKM(cudaMalloc(&d_parts, sizeof(uint32_t) * std::max<long long>(1, nparts)));
  KD_CKM(cudaMalloc(&d_pc, sizeof(int) * std::max<long long>(1, nparts)));
  KD_CKM(cudaMalloc(&d_poff, sizeof(int) * std::max<long long>(1, nparts)));
  KD_CKM(cudaMalloc(&gmin, sizeof(double) * dst->d.K));
  KD_CKM(cudaMalloc(&gmax, sizeof(double) * dst->d.K));
  KD_CKM(cudaMalloc(&gclock, sizeof(double) * dst->d.K));
  KD_CKM(cudaMalloc(&part_partials, sizeof(int4) * kd_scan_partials_needed(std::max<long long>(1, nparts))));
  KD_CKM(cudaMalloc(&d_tot, sizeof(int4)));
  KD_CKM(cudaMemcpyAsync(d_goff, h_goff, sizeof(long long) * (ngroups + 1), cudaMemcpyHostToDevice, str));
  if (nparts > 0)
    KD_CKM(cudaMemcpyAsync(d_parts, h_parts, sizeof(uint32_t) * nparts, cudaMemcpyHostToDevice, str));
  const int grid = s->num_sms * 8;
  k_merge_counts<<<grid, 256, 0, str>>>(src->d, d_parts, nparts, d_pc);
  kd_scan(PartSrc{d_pc}, PartDst{d_poff, d_tot}, nparts, part_partials, d_tot, str);
  k_merge_headers<<<grid, 256, 0, str>>>(src->d, d_parts, d_goff, ngroups, d_pc, gmin, gmax, gclock);
  int4 h_tot{0, 0, 0, 0};
  KD_CKM(cudaMemcpyAsync(&h_tot, d_tot, sizeof(int4), cudaMemcpyDeviceToHost, str));
  KD_CKM(cudaStreamSynchronize(str));
  total_elems = h_tot.x;
  if (total_elems > 0) {
    KD_CKM(cudaMalloc(&okey, sizeof(uint32_t) * total_elems));
    KD_CKM(cudaMalloc(&oval, sizeof(double) * total_elems));
    KD_CKM(cudaMalloc(&owt, sizeof(double) * total_elems));
    k_merge_gather<<<grid, 256, 0, str>>>(src->d, d_parts, d_goff, ngroups, nparts, d_pc, d_poff,
                                          okey, oval, owt);
    rc = kd_pipeline_ingest(s, dst, okey, oval, owt, total_elems, KD_MODE_MERGE, 0.0, gmin, gmax,
                            gclock);
  }
  cleanup();
#undef KD_CKM
  return rc;
}
