// kd_scan.cuh — device-wide exclusive scan of int4 tuples (reduce, scan partials,
// apply).  The element source and sink are functors so that flags, counts and
// compactions are produced and consumed in the same passes that compute them,
// without materialising an input array.
//
//   Src: __device__ int4 operator()(long long i) const   (i < n_max; return 0s past the live end)
//   Dst: __device__ void operator()(long long i, int4 excl, int4 val) const
//   total (optional) receives the sum of all tuples.
#pragma once

#include <cuda_runtime.h>

#define KD_SCAN_THREADS 512
#define KD_SCAN_ITEMS 8
#define KD_SCAN_TILE (KD_SCAN_THREADS * KD_SCAN_ITEMS)

__device__ __forceinline__ int4 i4add(int4 a, int4 b) {
  return make_int4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ int4 i4shfl_up(int4 v, int o) {
  v.x = __shfl_up_sync(0xffffffffu, v.x, o);
  v.y = __shfl_up_sync(0xffffffffu, v.y, o);
  v.z = __shfl_up_sync(0xffffffffu, v.z, o);
  v.w = __shfl_up_sync(0xffffffffu, v.w, o);
  return v;
}

// Block-wide inclusive scan of one int4 per thread; returns the inclusive value
// and writes the block total to *total.
__device__ __forceinline__ int4 block_scan_incl(int4 v, int4* smem_warp, int4* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    int4 t = i4shfl_up(v, o);
    if (lane >= o) v = i4add(v, t);
  }
  if (lane == 31) smem_warp[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int4 w = lane < nwarps ? smem_warp[lane] : make_int4(0, 0, 0, 0);
    for (int o = 1; o < 32; o <<= 1) {
      int4 t = i4shfl_up(w, o);
      if (lane >= o) w = i4add(w, t);
    }
    if (lane < nwarps) smem_warp[lane] = w;
  }
  __syncthreads();
  if (warp > 0) v = i4add(v, smem_warp[warp - 1]);
  *total = smem_warp[nwarps - 1];
  __syncthreads();
  return v;
}

template <class Src, int ITEMS = KD_SCAN_ITEMS>
__global__ void __launch_bounds__(KD_SCAN_THREADS) kd_scan_reduce(Src src, long long n, int4* partials) {
  __shared__ int4 sw[32];
  long long base = (long long)blockIdx.x * (KD_SCAN_THREADS * ITEMS) + (long long)threadIdx.x * ITEMS;
  int4 acc = make_int4(0, 0, 0, 0);
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    long long i = base + k;
    if (i < n) acc = i4add(acc, src(i));
  }
  int4 tot;
  block_scan_incl(acc, sw, &tot);
  if (threadIdx.x == 0) partials[blockIdx.x] = tot;
}

// One block: exclusive scan of the partials in place; total -> *total.
static __global__ void __launch_bounds__(1024) kd_scan_partials(int4* partials, int nb, int4* total) {
  __shared__ int4 sw[32];
  const int per = (nb + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per;
  int4 acc = make_int4(0, 0, 0, 0);
  for (int i = lo; i < lo + per && i < nb; ++i) acc = i4add(acc, partials[i]);
  int4 tot;
  int4 incl = block_scan_incl(acc, sw, &tot);
  int4 run = make_int4(incl.x - acc.x, incl.y - acc.y, incl.z - acc.z, incl.w - acc.w);
  for (int i = lo; i < lo + per && i < nb; ++i) {
    int4 v = partials[i];
    partials[i] = run;
    run = i4add(run, v);
  }
  if (threadIdx.x == 0 && total) *total = tot;
}

template <class Src, class Dst, int ITEMS = KD_SCAN_ITEMS>
__global__ void __launch_bounds__(KD_SCAN_THREADS) kd_scan_apply(Src src, Dst dst, long long n,
                                                                 const int4* partials) {
  __shared__ int4 sw[32];
  long long base = (long long)blockIdx.x * (KD_SCAN_THREADS * ITEMS) + (long long)threadIdx.x * ITEMS;
  int4 vals[ITEMS];
  int4 acc = make_int4(0, 0, 0, 0);
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    long long i = base + k;
    vals[k] = i < n ? src(i) : make_int4(0, 0, 0, 0);
    acc = i4add(acc, vals[k]);
  }
  int4 tot;
  int4 incl = block_scan_incl(acc, sw, &tot);
  int4 run = i4add(partials[blockIdx.x],
                   make_int4(incl.x - acc.x, incl.y - acc.y, incl.z - acc.z, incl.w - acc.w));
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    long long i = base + k;
    if (i < n) dst(i, run, vals[k]);
    run = i4add(run, vals[k]);
  }
}

// A scan that fits one block (n <= KD_SCAN_THREADS * ITEMS) in one launch: the
// same values as reduce / partials / apply (the block's exclusive prefix is the
// global one), the total written before any element is handed to dst.
template <class Src, class Dst, int ITEMS = KD_SCAN_ITEMS>
__global__ void __launch_bounds__(KD_SCAN_THREADS) kd_scan_single(Src src, Dst dst, long long n,
                                                                  int4* total) {
  __shared__ int4 sw[32];
  const long long base = (long long)threadIdx.x * ITEMS;
  int4 vals[ITEMS];
  int4 acc = make_int4(0, 0, 0, 0);
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const long long i = base + k;
    vals[k] = i < n ? src(i) : make_int4(0, 0, 0, 0);
    acc = i4add(acc, vals[k]);
  }
  int4 tot;
  const int4 incl = block_scan_incl(acc, sw, &tot);
  if (threadIdx.x == 0 && total) *total = tot;
  __syncthreads();
  int4 run = make_int4(incl.x - acc.x, incl.y - acc.y, incl.z - acc.z, incl.w - acc.w);
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const long long i = base + k;
    if (i < n) dst(i, run, vals[k]);
    run = i4add(run, vals[k]);
  }
}

// Host launcher; returns the kernels it launched.  `partials` must hold
// ceil(n_max / (KD_SCAN_THREADS * ITEMS)) int4s.  Fewer items per thread give
// more blocks: for short scans (one entry per key) that spreads them over the
// GPU instead of a few blocks.  A scan of one block is one launch.
template <int ITEMS = KD_SCAN_ITEMS, class Src, class Dst>
static inline int kd_scan(Src src, Dst dst, long long n_max, int4* partials, int4* total,
                          cudaStream_t st) {
  if (n_max <= 0) {
    if (total) cudaMemsetAsync(total, 0, sizeof(int4), st);
    return 0;
  }
  constexpr long long tile = (long long)KD_SCAN_THREADS * ITEMS;
  int nb = (int)((n_max + tile - 1) / tile);
  if (nb == 1) {
    kd_scan_single<Src, Dst, ITEMS><<<1, KD_SCAN_THREADS, 0, st>>>(src, dst, n_max, total);
    return 1;
  }
  kd_scan_reduce<Src, ITEMS><<<nb, KD_SCAN_THREADS, 0, st>>>(src, n_max, partials);
  kd_scan_partials<<<1, 1024, 0, st>>>(partials, nb, total);
  kd_scan_apply<Src, Dst, ITEMS><<<nb, KD_SCAN_THREADS, 0, st>>>(src, dst, n_max, partials);
  return 3;
}

static inline long long kd_scan_partials_needed(long long n_max, int items = KD_SCAN_ITEMS) {
  const long long tile = (long long)KD_SCAN_THREADS * items;
  return (n_max + tile - 1) / tile + 1;
}
