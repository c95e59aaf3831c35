// kd_sort.cuh — stable LSD radix sort of (order key u64, digest key u32[, index u32]).
//
// Restates the ordering of gpu/sort.mojo (stable sort by mean, ties by original
// index, _before at :38-41) for many digests at once: the composite key is
// (digest key, order-preserving u64 of the FP64 value).  LSD passes over 8-bit
// digits are stable, so elements with equal (key, value) keep their input order,
// which is exactly the reference's index tie-break.
//
// Each pass: per-block digit histograms (warp-private shared counters), one
// device-wide exclusive scan of the digit-major histogram, then a stable
// scatter in which every warp ranks its 32-element rounds with __match_any_sync.
#pragma once

#include "kd_scan.cuh"

#define KD_RS_THREADS 256
#define KD_RS_WARPS (KD_RS_THREADS / 32)
#define KD_RS_PER_WARP 512
#define KD_RS_ROUNDS (KD_RS_PER_WARP / 32)
#define KD_RS_TILE (KD_RS_WARPS * KD_RS_PER_WARP)

__device__ __forceinline__ unsigned rs_digit(const uint64_t* k64, const uint32_t* key, long long i,
                                             int shift, int from_key) {
  return from_key ? ((key[i] >> shift) & 255u) : (unsigned)((k64[i] >> shift) & 255ull);
}

static __global__ void __launch_bounds__(KD_RS_THREADS) kd_rs_hist(const uint64_t* __restrict__ k64,
                                                           const uint32_t* __restrict__ key,
                                                           long long n, int shift, int from_key,
                                                           int* __restrict__ hist, int nb) {
  __shared__ unsigned cnt[KD_RS_WARPS][256];
  for (int t = threadIdx.x; t < KD_RS_WARPS * 256; t += KD_RS_THREADS) (&cnt[0][0])[t] = 0;
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  const long long base = (long long)blockIdx.x * KD_RS_TILE;
#pragma unroll 4
  for (int r = 0; r < KD_RS_TILE / KD_RS_THREADS; ++r) {
    long long i = base + (long long)r * KD_RS_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&cnt[warp][rs_digit(k64, key, i, shift, from_key)], 1u);
  }
  __syncthreads();
  if (threadIdx.x < 256) {
    unsigned s = 0;
#pragma unroll
    for (int w = 0; w < KD_RS_WARPS; ++w) s += cnt[w][threadIdx.x];
    hist[(long long)threadIdx.x * nb + blockIdx.x] = (int)s;
  }
}

template <bool kIdx>
__global__ void __launch_bounds__(KD_RS_THREADS) kd_rs_scatter(
    const uint64_t* __restrict__ kin, const uint32_t* __restrict__ keyin,
    const uint32_t* __restrict__ idxin, uint64_t* __restrict__ kout, uint32_t* __restrict__ keyout,
    uint32_t* __restrict__ idxout, long long n, int shift, int from_key,
    const int* __restrict__ offs, int nb) {
  __shared__ unsigned wcnt[KD_RS_WARPS][256];
  for (int t = threadIdx.x; t < KD_RS_WARPS * 256; t += KD_RS_THREADS) (&wcnt[0][0])[t] = 0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long base = (long long)blockIdx.x * KD_RS_TILE + (long long)warp * KD_RS_PER_WARP;
  const unsigned lt_mask = (1u << lane) - 1u;
  unsigned rank[KD_RS_ROUNDS];
#pragma unroll
  for (int r = 0; r < KD_RS_ROUNDS; ++r) {
    long long i = base + r * 32 + lane;
    bool valid = i < n;
    unsigned d = valid ? rs_digit(kin, keyin, i, shift, from_key) : 256u;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    unsigned before = peers & lt_mask;
    unsigned c = valid ? wcnt[warp][d] : 0u;
    __syncwarp();
    if (valid && before == 0) wcnt[warp][d] = c + __popc(peers);
    __syncwarp();
    rank[r] = c + __popc(before);
  }
  __syncthreads();
  if (threadIdx.x < 256) {
    unsigned s = 0;
#pragma unroll
    for (int w = 0; w < KD_RS_WARPS; ++w) {
      unsigned v = wcnt[w][threadIdx.x];
      wcnt[w][threadIdx.x] = s;
      s += v;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < KD_RS_ROUNDS; ++r) {
    long long i = base + r * 32 + lane;
    if (i < n) {
      uint64_t kv = kin[i];
      uint32_t kk = keyin[i];
      unsigned d = from_key ? ((kk >> shift) & 255u) : (unsigned)((kv >> shift) & 255ull);
      long long pos = (long long)offs[(long long)d * nb + blockIdx.x] + wcnt[warp][d] + rank[r];
      kout[pos] = kv;
      keyout[pos] = kk;
      if (kIdx) idxout[pos] = idxin[i];
    }
  }
}

struct KdHistSrc {
  const int* h;
  __device__ int4 operator()(long long i) const { return make_int4(h[i], 0, 0, 0); }
};
struct KdHistDst {
  int* h;
  __device__ void operator()(long long i, int4 excl, int4) const { h[i] = excl.x; }
};

struct KdSortBufs {
  uint64_t* k64[2];
  uint32_t* key[2];
  uint32_t* idx[2];  // may be null
  int* hist;         // 256 * nb
  int4* partials;    // scan partials for 256 * nb entries
};

static inline int kd_rs_blocks(long long n) { return (int)((n + KD_RS_TILE - 1) / KD_RS_TILE); }
static inline long long kd_rs_hist_entries(long long n) { return 256LL * kd_rs_blocks(n); }

// Sorts by (key, k64); returns the index (0/1) of the buffer set holding the result.
static inline int kd_radix_sort(KdSortBufs& b, long long n, int key_bits, bool with_idx,
                                cudaStream_t st) {
  int src = 0;
  if (n <= 1) return src;
  const int nb = kd_rs_blocks(n);
  const long long entries = 256LL * nb;
  auto pass = [&](int shift, int from_key) {
    const int dst = src ^ 1;
    kd_rs_hist<<<nb, KD_RS_THREADS, 0, st>>>(b.k64[src], b.key[src], n, shift, from_key, b.hist, nb);
    kd_scan(KdHistSrc{b.hist}, KdHistDst{b.hist}, entries, b.partials, (int4*)nullptr, st);
    if (with_idx)
      kd_rs_scatter<true><<<nb, KD_RS_THREADS, 0, st>>>(b.k64[src], b.key[src], b.idx[src],
                                                        b.k64[dst], b.key[dst], b.idx[dst], n,
                                                        shift, from_key, b.hist, nb);
    else
      kd_rs_scatter<false><<<nb, KD_RS_THREADS, 0, st>>>(b.k64[src], b.key[src], nullptr,
                                                         b.k64[dst], b.key[dst], nullptr, n, shift,
                                                         from_key, b.hist, nb);
    src = dst;
  };
  for (int shift = 0; shift < 64; shift += 8) pass(shift, 0);
  for (int shift = 0; shift < key_bits; shift += 8) pass(shift, 1);
  return src;
}
