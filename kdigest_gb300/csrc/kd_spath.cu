// kd_spath.cu — the single-sample path of a one-key store on the device:
// TDigest.add / add_at and the sequential merge pass they trigger
// (src/kdigest/tdigest.mojo:153-175, 324-458), merge() before reads, and the
// sequential merge_into (:589-623).
//
// The reference runs batches below its GPU crossover through this path
// (tdigest.mojo:177-221), so a one-key store reproduces it exactly: samples
// wait in a buffer of 5 * int(compression) entries, and a full buffer runs the
// merge pass — a stable sort of centroids ++ buffer by mean, then a greedy
// left-to-right sweep that grows a cluster while k(q_right) - k(q_left) <= 1
// or the candidate's mean equals the cluster's running mean.
//
// One CTA runs a whole call; its state lives in shared memory (or in a global
// scratch block when the buffer is too large for it).  The sweep is sequential
// in the reference, and parallel here without changing a bit:
//   * with integral weights every q the sweep forms is an exact prefix sum over
//     the stored total, so k is evaluated for every position in parallel;
//   * one warp follows the chain of cluster starts, 32 candidates per step;
//   * one thread per cluster replays its running mean and weight in order;
//   * with non-integral weights (decay) the chain is first speculated from
//     plain prefix sums, then every decision is re-checked with the exact sums
//     of the chain; a mismatch (or a candidate whose coalescing rests on an
//     exact mean tie) sends the pass to a one-thread replay of the reference
//     loop.
// Every FP64 operation is the reference's, in its order, through the
// correctly rounded intrinsics of kd_math.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>

#include "../../include/kdigest_gb300.h"
#include "kd_engine.h"
#include "kd_internal.cuh"
#include "kd_math.h"

namespace {

constexpr int SP_T = 1024;  // threads of the one CTA
constexpr double SP_RENORM = 400.0;    // tdigest.mojo:43
constexpr int SP_RCP_N = 1 << 16;      // reciprocal table entries
constexpr int SP_RUNS = 64;            // exponent runs per buffer fill
constexpr double SP_PRUNE_EPS = 1e-6;  // tdigest.mojo:47

enum { SP_ADD = 0, SP_FLUSH = 1, SP_MERGE_INTO = 2 };

struct SpStatus {
  int code;
  int noop;
  long long index;  // first rejected sample (KD_EINVAL)
  int count;
  int bcount;
};

struct SpArgs {
  KdStoreDev s;      // the digest (key 0)
  KdStoreDev o;      // merge_into: the other digest (key 0), already flushed
  const double* vals;
  const double* wts;  // per-sample weights, or null (1.0)
  const double* ts;   // per-sample timestamps (add_at), or null (add)
  long long n;
  int op;
  int bmax;  // buffer capacity inside the call: max(buf_cap, KD_TILE)
  int wpb;   // power of two >= bmax (width of the buffer sort)
  unsigned char* scratch;  // global working memory, or null (dynamic shared memory)
  const double* rcp;       // 1 / d for d < SP_RCP_N (d = 0 unused)
  SpStatus* out;
};

struct SpMem {
  double *cm, *cw;  // centroids [KD_TILE]
  double *bm, *bw;  // buffer [bmax]
  unsigned long long* okey;  // buffer sort keys [wpb]
  unsigned* sidx;            // buffer sort positions [wpb]
  double *sm, *sw;  // merged work [KD_TILE + bmax]
  double* kk;       // k at every prefix [KD_TILE + bmax + 1]
  double* rw;       // running cluster weight before each element, or its weight ratio [W + 1]
  long long* pi;    // exact integer prefix of the work weights [W + 1]
  int* cst;         // cluster starts [KD_TILE + 1]
  int* cid;         // cluster (or cluster start) of each element [KD_TILE + bmax]
  int* nb;          // next cluster start after each possible start [KD_TILE + bmax]
  double* sls;      // log-scale of each sample of a segment [bmax]
  double *wsf, *kl;  // weight before each cluster and its k [KD_TILE + 1]
  unsigned long long* pk;  // buffers sorted ahead of their merge [SP_T]
  unsigned* px;
  int *rk, *rn;      // runs of the exponent: first sample, length [SP_RUNS]
  double *rx, *rr;   // value before the run, step
};

__host__ __device__ inline size_t sp_align(size_t b) { return (b + 255) & ~(size_t)255; }

__host__ __device__ inline size_t sp_layout(int bmax, int wpb, unsigned char* base, SpMem* m) {
  const size_t W = (size_t)KD_TILE + bmax;
  size_t off = 0;
  auto take = [&](size_t bytes) -> unsigned char* {
    unsigned char* p = base ? base + off : nullptr;
    off += sp_align(bytes);
    return p;
  };
  SpMem t;
  t.cm = (double*)take(8 * KD_TILE);
  t.cw = (double*)take(8 * KD_TILE);
  t.bm = (double*)take(8 * (size_t)bmax);
  t.bw = (double*)take(8 * (size_t)bmax);
  t.okey = (unsigned long long*)take(8 * (size_t)wpb);
  t.sidx = (unsigned*)take(4 * (size_t)wpb);
  t.sm = (double*)take(8 * W);
  t.sw = (double*)take(8 * W);
  t.kk = (double*)take(8 * (W + 1));
  t.rw = (double*)take(8 * (W + 1));
  t.pi = (long long*)take(8 * (W + 1));
  t.cst = (int*)take(4 * (KD_TILE + 1));
  t.cid = (int*)take(4 * W);
  t.nb = (int*)take(4 * W);
  t.sls = (double*)take(8 * (size_t)bmax);
  t.wsf = (double*)take(8 * (KD_TILE + 1));
  t.kl = (double*)take(8 * (KD_TILE + 1));
  t.pk = (unsigned long long*)take(8 * 1024);
  t.px = (unsigned*)take(4 * 1024);
  t.rk = (int*)take(4 * SP_RUNS);
  t.rn = (int*)take(4 * SP_RUNS);
  t.rx = (double*)take(8 * SP_RUNS);
  t.rr = (double*)take(8 * SP_RUNS);
  if (m) *m = t;
  return off;
}

// Scalars of the call, shared by the CTA.
struct SpSh {
  double st, ls, clock, mn, mx;
  double factor, nrm, renorm_clock;
  long long first_bad;
  double k0, k1;  // FP64 k at q = 0 and q = 1 (filtered sweeps)
  double f0, f1;  // the same with normaliser 1: k(q, nrm) = nrm * k(q, 1) at these q
  double nrm01;   // the K0 / K1 normaliser (it does not depend on the total)
  double inv_st;  // 1 / stored total, for approximate q (filters and speculation only)
  double floor_w; // prune floor 1e-6 * e^{log_scale} of the current merge
  double tot_u;   // ulp of the stored total's binade
  long long tot_base;  // the stored total in units of tot_u
  int C, B, err, nc, mismatch, unsorted, exact, cut, renorm, pre_adv, integral, fast, filt;
  int longreach;  // a cluster start whose reach passed 64 candidates
  int mm_first;   // first candidate whose speculated decision the exact test overturned
  int bfail;      // a bucket of the buffer merge was too large
  int nruns;      // runs of the exponent in the current buffer fill
  long long wsum[32];  // per-warp partial sums of block scans and reductions
};

__device__ __forceinline__ double sp_k(int scale, double q, double nrm) { return kd_k(scale, q, nrm); }

// k at q = p / st in FP32 (integral p, st <= 1e14, 0 <= p <= st), in forms
// without cancellation: q and 1 - q both come from exact integers, asin near
// +-1 goes through asin(1 - 2s) = pi/2 - 2 asin(sqrt(s)).  Against the FP64
// k of the same q the error is below 2e-5 * nrm for every scale (FP32
// rounding of p, st and 1 - q, and the documented few-ulp accuracy of asinf,
// logf and sqrtf); the sweep treats differences within nrm * 2^-12 of the
// limit as undecided and settles them in FP64.
__device__ __forceinline__ float sp_k32(int scale, long long p, double st, float nrmf, float k0f,
                                        float k1f) {
  if (p == 0) return k0f;
  const double rest = st - (double)p;  // exact: integers below 2^47
  if (rest == 0.0) return k1f;
  const float a = (float)p, c = (float)rest, b = (float)st;
  switch (scale) {
    case KD_SCALE_K0:
      return nrmf * (a / b);
    case KD_SCALE_K1: {
      const bool lo = a <= c;
      const float t = 1.57079637f - 2.0f * asinf(sqrtf((lo ? a : c) / b));
      return nrmf * (lo ? -t : t);
    }
    case KD_SCALE_K2:
      return nrmf * logf(a / c);
    default:
      return a <= c ? nrmf * logf(2.0f * a / b) : -nrmf * logf(2.0f * c / b);
  }
}

// k at an FP64 q in FP32, with q and 1 - q each rounded once (1 - q is exact
// in FP64 for q >= 1/2).  The same error bound as sp_k32 holds.  Near 0 and 1,
// where the FP64 k clamps, it returns NaN unless `clamp` asks for the end values.
__device__ __forceinline__ float sp_k32q(int scale, double q, float nrmf, float k0f, float k1f,
                                         bool clamp) {
  if (!(q > 1e-14)) return clamp ? k0f : __int_as_float(0x7fc00000);
  if (!(q < 1.0 - 1e-14)) return clamp ? k1f : __int_as_float(0x7fc00000);
  const float a = (float)q, c = (float)(1.0 - q);
  switch (scale) {
    case KD_SCALE_K0:
      return nrmf * a;
    case KD_SCALE_K1: {
      const bool lo = a <= c;
      const float t = 1.57079637f - 2.0f * asinf(sqrtf(lo ? a : c));
      return nrmf * (lo ? -t : t);
    }
    case KD_SCALE_K2:
      return nrmf * logf(a / c);
    default:
      return a <= c ? nrmf * logf(2.0f * a) : -nrmf * logf(2.0f * c);
  }
}

// The k-size test of the merge pass for candidate j of the cluster that starts
// at s0: k(q(j + 1)) - k(q(s0)) <= 1 with FP64 k at exact prefix positions.
// Filtered: the FP32 difference decides unless it is within tau of 1; then (and
// only then) the FP64 values are evaluated.  ks64 caches the start's FP64 k.
struct SpFit {
  int scale;
  bool filt;
  bool spec;  // non-integral weights: FP32 k of approximate sums, a speculation only
  float tau;
  double st, nrm;
  const float* k32;
  const double* kk;
  const long long* pi;
  __device__ double k64(int i) const {
    return filt ? sp_k(scale, KD_DIV((double)pi[i], st), nrm) : kk[i];
  }
  __device__ bool fits(int s0, int j, double& ks64) const {
    if (spec) return k32[j + 1] - k32[s0] <= 1.0f;
    if (!filt) return KD_SUB(kk[j + 1], kk[s0]) <= 1.0;
    const float d = k32[j + 1] - k32[s0];
    if (d <= 1.0f - tau) return true;
    if (d > 1.0f + tau) return false;
    if (ks64 != ks64) ks64 = k64(s0);
    return KD_SUB(k64(j + 1), ks64) <= 1.0;
  }
};

// Block-wide exclusive prefix of v[0..n) into out[0..n] (out[n] = total), in
// any association order: used only where the sums are exact (integers below
// 2^53) or a speculation that is re-checked exactly.
__device__ void sp_prefix(const double* v, double* out, int n, double* tmp_warp) {
  // per-thread chunk sums, then a serial scan of the 1024 chunk sums by warp 0
  const int per = (n + SP_T - 1) / SP_T;
  const int b = threadIdx.x * per, e = min(n, b + per);
  double sum = 0.0;
  for (int i = b; i < e; ++i) sum = KD_ADD(sum, v[i]);
  tmp_warp[threadIdx.x] = sum;
  __syncthreads();
  if (threadIdx.x < 32) {
    // warp scan over 1024 values: each lane owns 32 consecutive chunks
    double* mine = tmp_warp + threadIdx.x * 32;
    double acc = 0.0;
    for (int i = 0; i < 32; ++i) acc = KD_ADD(acc, mine[i]);
    double incl = acc;
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)threadIdx.x >= o) incl = KD_ADD(incl, y);
    }
    double run = __shfl_up_sync(0xffffffffu, incl, 1);
    if (threadIdx.x == 0) run = 0.0;
    for (int i = 0; i < 32; ++i) {  // chunk sums -> exclusive chunk offsets, in place
      const double v = mine[i];
      mine[i] = run;
      run = KD_ADD(run, v);
    }
  }
  __syncthreads();
  double run = tmp_warp[threadIdx.x];
  for (int i = b; i < e; ++i) {
    out[i] = run;
    run = KD_ADD(run, v[i]);
  }
  if (e == n && b < e) out[n] = run;
  if (n == 0 && threadIdx.x == 0) out[0] = 0.0;
  __syncthreads();
}

// w as an integer when it is one in [1, 2^53] (integer ops only).
__device__ __forceinline__ bool sp_int53(double w, long long* out) {
  const unsigned long long b = kd_bits(w);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if ((b >> 63) || e < 0 || e > 52) return false;
  const unsigned long long mant = (b & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
  const int sh = 52 - e;
  if (sh > 0 && (mant & ((1ull << sh) - 1ull))) return false;
  *out = (long long)(mant >> sh);
  return true;
}

// Block-wide sum of one int64 per thread (every thread gets the total).
__device__ long long sp_isum(long long v, SpSh& sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh.wsum[threadIdx.x >> 5] = v;
  __syncthreads();
  long long t = 0;
  for (int w = 0; w < SP_T / 32; ++w) t += sh.wsum[w];
  __syncthreads();
  return t;
}

// Block-wide exclusive scan of one int64 per thread; *total gets the sum.
__device__ long long sp_iscan(long long v, SpSh& sh, long long* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh.wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    long long t = sh.wsum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    sh.wsum[lane] = t;
  }
  __syncthreads();
  const long long excl = x - v + (w > 0 ? sh.wsum[w - 1] : 0);
  *total = sh.wsum[SP_T / 32 - 1];
  __syncthreads();
  return excl;
}

// Integer exclusive prefix out[0..n] of integral weights v[0..n) (exact).
__device__ void sp_iprefix(const double* v, long long* out, int n, SpSh& sh) {
  const int per = (n + SP_T - 1) / SP_T;
  const int b = threadIdx.x * per, e = min(n, b + per);
  long long sum = 0;
  for (int i = b; i < e; ++i) {
    long long x = 0;
    sp_int53(v[i], &x);
    sum += x;
  }
  long long total;
  long long run = sp_iscan(sum, sh, &total);
  for (int i = b; i < e; ++i) {
    out[i] = run;
    long long x = 0;
    sp_int53(v[i], &x);
    run += x;
  }
  if (threadIdx.x == 0) out[n] = total;
  __syncthreads();
}

// Stable ascending sort of the buffer (bm[0..B)) by value: bitonic over
// (order key, position), so equal values (and -0.0 / +0.0) keep their order.
// Up to one element per thread the keys stay in registers: strides below 32
// exchange through warp shuffles, larger ones through shared memory.
// Sorts blocks of P consecutive threads' (key, idx) pairs, each block on its
// own (P a power of two, threads [0, nthr) hold elements, nthr a multiple of P
// or P itself): 32-element runs in registers (bitonic over warp shuffles), then
// runs merged pairwise.  Keys are distinct (value key, then position; the
// padding has positions of its own), so an element's place in a merged run is
// its place in its own run plus the number of partner-run elements before it.
// The sorted blocks land in okey / sidx [0, nthr).
__device__ __forceinline__ void sp_sort_regs(unsigned long long key, unsigned idx, int P, int nthr,
                                             unsigned long long* okey, unsigned* sidx) {
  const int i = threadIdx.x;
  const int R = P < 32 ? P : 32;
  const bool warp_on = (i & ~31) < nthr;
  if (warp_on) {
    const int lane = i & 31;  // every run ends ascending
    for (int k = 2; k <= R; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, j);
        const unsigned oi = __shfl_xor_sync(0xffffffffu, idx, j);
        const bool up = (lane & k) == 0;
        const bool lower = (lane & j) == 0;
        const bool other_less = ok < key || (ok == key && oi < idx);
        if ((lower == up) == other_less) {
          key = ok;
          idx = oi;
        }
      }
    }
  }
  if (i < nthr) {
    okey[i] = key;
    sidx[i] = idx;
  }
  __syncthreads();
  int at = i;  // where this thread's element sits
  for (int run = 32; run < P; run <<= 1) {
    int pos = 0;
    if (i < nthr) {
      const int base = (at / run) * run;
      const int other = base ^ run;
      int lo = 0, hi = run;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const unsigned long long ok = okey[other + mid];
        if (ok < key || (ok == key && sidx[other + mid] < idx)) lo = mid + 1;
        else hi = mid;
      }
      pos = (base < other ? base : other) + (at - base) + lo;
    }
    __syncthreads();
    if (i < nthr) {
      okey[pos] = key;
      sidx[pos] = idx;
      at = pos;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ void sp_sort_buffer(const SpMem& m, int B) {
  int P = 1;
  while (P < B) P <<= 1;
  if (P > SP_T) {
    for (int i = threadIdx.x; i < P; i += SP_T) {
      m.okey[i] = i < B ? kd_order_key(m.bm[i]) : ~0ull;
      m.sidx[i] = i < B ? (unsigned)i : 0xffffffffu;
    }
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = threadIdx.x; i < P; i += SP_T) {
          const int ixj = i ^ j;
          if (ixj > i) {
            const unsigned long long a = m.okey[i], b = m.okey[ixj];
            const unsigned ia = m.sidx[i], ib = m.sidx[ixj];
            const bool gt = a > b || (a == b && ia > ib);
            if (gt == ((i & k) == 0)) {
              m.okey[i] = b;
              m.okey[ixj] = a;
              m.sidx[i] = ib;
              m.sidx[ixj] = ia;
            }
          }
        }
        __syncthreads();
      }
    }
    return;
  }
  const int i = threadIdx.x;
  unsigned long long key = ~0ull;
  unsigned idx = 0x80000000u | (unsigned)i;
  if (i < B) {
    key = kd_order_key(m.bm[i]);
    idx = (unsigned)i;
  }
  sp_sort_regs(key, idx, P, P < 32 ? 32 : P, m.okey, m.sidx);
}

// The merge pass (tdigest.mojo:391-439, _prune :441-458) over C centroids and
// B buffered samples in shared state.  Leaves the new centroids in cm/cw.
// Places centroids ++ buffer in their stable sorted order without sorting the
// buffer: a buffered value's bucket is the number of centroids at or below it
// (centroids sort first on equal values), its place is its bucket plus the
// number of buffered values before it, and those are the values of earlier
// buckets plus its rank inside its own bucket, counted directly.  Needs sorted
// centroids; returns false (and places nothing) when a bucket holds more than
// 64 values, where counting would cost more than sorting.
__device__ bool sp_bucket_merge(const SpMem& m, SpSh& sh, int C, int B) {
  int* off = m.nb;     // [C + 1]: bucket sizes, then their offsets (free until the reach)
  int* fill = m.cid;   // [C + 1]
  int* bk = reinterpret_cast<int*>(m.kk);  // bucket of each buffered value (free until k)
  unsigned long long* tk = m.okey;         // buffered keys grouped by bucket
  unsigned* ti = m.sidx;
  for (int k = threadIdx.x; k <= C; k += SP_T) {
    off[k] = 0;
    fill[k] = 0;
  }
  if (threadIdx.x == 0) sh.bfail = 0;
  __syncthreads();
  for (int b = threadIdx.x; b < B; b += SP_T) {
    const unsigned long long key = kd_order_key(m.bm[b]);
    int lo = 0, hi = C;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (kd_order_key(m.cm[mid]) <= key) lo = mid + 1;
      else hi = mid;
    }
    bk[b] = lo;
    atomicAdd(&off[lo], 1);
  }
  __syncthreads();
  const int c = threadIdx.x < C ? off[threadIdx.x] : 0;  // C <= 1024 = SP_T
  if (c > 64 || (threadIdx.x == 0 && off[C] > 64)) sh.bfail = 1;  // off[C]: the last bucket
  long long total;
  const long long excl = sp_iscan(c, sh, &total);  // synchronises
  if (threadIdx.x < C) off[threadIdx.x] = (int)excl;
  if (threadIdx.x == 0) off[C] = (int)total;
  __syncthreads();
  if (sh.bfail) return false;
  for (int b = threadIdx.x; b < B; b += SP_T) {
    const int k = bk[b];
    const int slot = off[k] + atomicAdd(&fill[k], 1);
    tk[slot] = kd_order_key(m.bm[b]);
    ti[slot] = (unsigned)b;
  }
  __syncthreads();
  for (int b = threadIdx.x; b < B; b += SP_T) {
    const int k = bk[b];
    const unsigned long long key = kd_order_key(m.bm[b]);
    const int lo = off[k], hi = k < C ? off[k + 1] : B;
    int within = 0;
    for (int t = lo; t < hi; ++t) {
      const unsigned long long ok = tk[t];
      within += (ok < key || (ok == key && ti[t] < (unsigned)b)) ? 1 : 0;
    }
    const int pos = k + lo + within;
    m.sm[pos] = m.bm[b];
    m.sw[pos] = m.bw[b];
  }
  for (int i = threadIdx.x; i < C; i += SP_T) {
    const int pos = i + off[i + 1];
    m.sm[pos] = m.cm[i];
    m.sw[pos] = m.cw[i];
  }
  __syncthreads();
  return true;
}

// pk / px: the buffer's sorted order when it was sorted ahead (else null).
__device__ __noinline__ void sp_merge(const SpArgs& a, const SpMem& m, SpSh& sh,
                                      const unsigned long long* pk, const unsigned* px) {
  const int B = sh.B, C = sh.C;
  if (B == 0) return;
  const int scale = a.s.scale;
  const bool decay = a.s.lambda > 0.0;
  // 1. work = centroids ++ buffer, stably sorted by mean
  if (threadIdx.x == 0) sh.unsorted = 0;
  __syncthreads();
  for (int i = threadIdx.x; i + 1 < C; i += SP_T)
    if (m.cm[i] > m.cm[i + 1]) sh.unsorted = 1;
  __syncthreads();
  if (sh.unsorted && threadIdx.x == 0) {  // stable insertion sort (tdigest.mojo:64-77)
    for (int i = 1; i < C; ++i) {
      const double km = m.cm[i], kw = m.cw[i];
      int j = i - 1;
      while (j >= 0 && m.cm[j] > km) {
        m.cm[j + 1] = m.cm[j];
        m.cw[j + 1] = m.cw[j];
        --j;
      }
      m.cm[j + 1] = km;
      m.cw[j + 1] = kw;
    }
  }
  __syncthreads();
  const bool placed = !pk && C > 0 && C <= SP_T && sp_bucket_merge(m, sh, C, B);
  if (!placed && !pk) {
    sp_sort_buffer(m, B);
    pk = m.okey;
    px = m.sidx;
  }
  for (int i = threadIdx.x; !placed && i < C; i += SP_T) {  // centroids precede equal values
    const unsigned long long v = kd_order_key(m.cm[i]);
    int lo = 0, hi = B;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (pk[mid] < v) lo = mid + 1;
      else hi = mid;
    }
    m.sm[i + lo] = m.cm[i];
    m.sw[i + lo] = m.cw[i];
  }
  for (int j = threadIdx.x; !placed && j < B; j += SP_T) {
    const unsigned long long v = pk[j];
    int lo = 0, hi = C;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (kd_order_key(m.cm[mid]) <= v) lo = mid + 1;
      else hi = mid;
    }
    const unsigned si = px[j];
    if (si >= (unsigned)B) {  // a sort that lost an element: fail, never read past the buffer
      sh.err = KD_ECUDA;
      continue;
    }
    m.sm[j + lo] = m.bm[si];
    m.sw[j + lo] = m.bw[si];
  }
  __syncthreads();
  if (sh.err) return;
  const int W = C + B;
  // 2. totals: k limits use the effective total, q positions the stored one
  if (threadIdx.x == 32 && decay) sh.floor_w = KD_MUL(SP_PRUNE_EPS, kd_exp(sh.ls));
  if (threadIdx.x == 0) {
    if (scale <= KD_SCALE_K1) {
      sh.nrm = sh.nrm01;
    } else {
      const double eff = decay ? KD_MUL(sh.st, kd_exp(-sh.ls)) : sh.st;
      sh.nrm = kd_normalizer(scale, a.s.compression, eff);
    }
    sh.B = 0;
    sh.exact = 1;
    sh.mismatch = 0;
    sh.mm_first = 0x7fffffff;
    sh.longreach = 0;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < W; i += SP_T) {
    long long x;
    if (!sp_int53(m.sw[i], &x)) sh.exact = 0;
  }
  __syncthreads();
  const double st = sh.st, nrm = sh.nrm;
  // 3. k at every prefix.  Integral weights: the prefix is exact in integers,
  //    so every q the sweep forms is known up front.  Otherwise a speculation.
  const bool exact_w = sh.exact != 0;
  if (exact_w) {
    sp_iprefix(m.sw, m.pi, W, sh);
    if (threadIdx.x == 0 && m.pi[W] > (1LL << 53)) sh.exact = 0;
    __syncthreads();
  }
  const bool exact = sh.exact != 0;
  if (threadIdx.x == 0) {
    sh.filt = exact && (double)m.pi[W] <= st && st >= 1.0 && st <= 1e14;
    // nrm * k(q, 1) rounds exactly as k(q, nrm) at q = 0 and 1
    sh.k0 = KD_MUL(nrm, sh.f0);
    sh.k1 = KD_MUL(nrm, sh.f1);
    sh.inv_st = KD_DIV(1.0, st);
  }
  __syncthreads();
  SpFit fit;
  fit.scale = scale;
  fit.filt = sh.filt != 0;
  fit.spec = !exact;
  // FP32 error bound: 3.3e-6 * nrm (K0, K1) and 1.8e-5 * nrm (K2, K3) on a
  // difference; the undecided band is several times wider
  fit.tau = (float)KD_MUL(nrm, scale <= KD_SCALE_K1 ? 0x1p-15 : 0x1p-13);
  fit.st = st;
  fit.nrm = nrm;
  fit.k32 = reinterpret_cast<const float*>(m.kk);
  fit.kk = m.kk;
  fit.pi = m.pi;
  if (fit.filt) {
    float* k32 = reinterpret_cast<float*>(m.kk);
    const float nrmf = (float)nrm, k0f = (float)sh.k0, k1f = (float)sh.k1;
    for (int i = threadIdx.x; i <= W; i += SP_T) k32[i] = sp_k32(scale, m.pi[i], st, nrmf, k0f, k1f);
  } else if (exact) {
    for (int i = threadIdx.x; i <= W; i += SP_T)
      m.kk[i] = sp_k(scale, KD_DIV((double)m.pi[i], st), nrm);
  } else {
    sp_prefix(m.sw, m.rw, W, m.wsf);
    float* k32 = reinterpret_cast<float*>(m.kk);
    const float nrmf = (float)nrm, k0f = (float)sh.k0, k1f = (float)sh.k1;
    const double inv_st = sh.inv_st;
    for (int i = threadIdx.x; i <= W; i += SP_T)
      k32[i] = sp_k32q(scale, KD_MUL(m.rw[i], inv_st), nrmf, k0f, k1f, true);
  }
  __syncthreads();
  // 4. for every element as a cluster start, where that cluster would end:
  //    candidates coalesce while the k span fits or their mean equals the start's
  //    (then all between are equal, and so is the running mean)
  const double* sm = m.sm;
  const double* sw = m.sw;
  // With FP32 k non-decreasing along the prefix (checked), the sure fits of a
  // start form a prefix of its candidates, found by binary search; the
  // candidates after it are tested one by one (exactly where undecided).
  if (threadIdx.x == 0) sh.unsorted = 0;  // here: FP32 k not monotone
  __syncthreads();
  if (fit.filt || fit.spec)
    for (int i = threadIdx.x; i < W; i += SP_T)
      if (fit.k32[i + 1] < fit.k32[i]) sh.unsorted = 1;
  __syncthreads();
  const bool mono = (fit.filt || fit.spec) && !sh.unsorted;
  const float sure = fit.spec ? 1.0f : 1.0f - fit.tau;
  for (int s0 = threadIdx.x; s0 < W; s0 += SP_T) {
    double ks64 = __longlong_as_double(0x7ff8000000000000LL);  // not yet evaluated
    const unsigned long long ms = kd_order_key(sm[s0]);
    int j = s0 + 1, steps = 0;
    while (j < W && steps < 64 && kd_order_key(sm[j]) == ms) {  // equal means coalesce
      ++j;
      ++steps;
    }
    if (steps < 64 && mono) {
      const float k0 = fit.k32[s0];
      int lo = j, hi = W;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (fit.k32[mid + 1] - k0 <= sure) lo = mid + 1;
        else hi = mid;
      }
      j = lo;
      steps = 0;
    }
    while (j < W && steps < 64) {
      if (!(kd_order_key(sm[j]) == ms || fit.fits(s0, j, ks64))) break;
      ++j;
      ++steps;
    }
    m.nb[s0] = (j < W && steps >= 64) ? -1 : j;
    if (j < W && steps >= 64) sh.longreach = 1;
  }
  __syncthreads();
  // 5. the chain of cluster starts from element 0.  With every reach known, the
  //    chain comes from jump tables J_k(s) = next^(2^k)(s): each lane of warp 0
  //    takes one of 32 consecutive hops at once.  J_0 is the reach array, J_1 to
  //    J_4 (16-bit) live in the k array, which the chain no longer needs.
  const bool jumps = !sh.longreach && W + 1 <= 65535;
  if (jumps) {
    unsigned short* J = reinterpret_cast<unsigned short*>(m.kk);
    const int stride = W + 1;
    for (int k = 1; k <= 4; ++k) {
      for (int x = threadIdx.x; x <= W; x += SP_T) {
        int y;
        if (k == 1) {
          const int a1 = x < W ? m.nb[x] : W;
          y = a1 < W ? m.nb[a1] : W;
        } else {
          const unsigned short* P = J + (size_t)(k - 2) * stride;
          y = P[P[x]];
        }
        J[(size_t)(k - 1) * stride + x] = (unsigned short)y;
      }
      __syncthreads();
    }
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      int base = 0, nc = 0;
      bool overflow = false;
      while (base < W) {
        int x = base;  // next^lane(base)
        if (lane & 1) x = x < W ? m.nb[x] : W;
        for (int k = 1; k <= 4; ++k)
          if ((lane >> k) & 1) x = J[(size_t)(k - 1) * stride + x];
        const unsigned valid = __ballot_sync(0xffffffffu, x < W);
        const int cnt = __popc(valid);  // the chain increases, so the valid lanes lead
        if (nc + cnt > KD_TILE) {
          overflow = true;
          break;
        }
        if (x < W) m.cst[nc + lane] = x;
        nc += cnt;
        const int last = __shfl_sync(0xffffffffu, x, 31);
        base = last < W ? m.nb[last] : W;
      }
      if (lane == 0) {
        m.cst[overflow ? KD_TILE : nc] = W;
        sh.nc = overflow ? -1 : nc;
      }
    }
  }
  // otherwise one lane hops along the reaches; a cluster longer than the
  // precomputed reach is scanned 32 candidates at a time
  if (!jumps && threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const int* const nbp = m.nb;
    int* const cstp = m.cst;
    int s0 = 0, nc = 0;
    bool overflow = false;
    while (s0 < W) {
      // the common case: hop along precomputed reaches (one lane is enough)
      if (lane == 0) {
        while (s0 < W && nc < KD_TILE) {
          const int b = nbp[s0];
          if (b < 0) break;
          cstp[nc++] = s0;
          s0 = b;
        }
      }
      s0 = __shfl_sync(0xffffffffu, s0, 0);
      nc = __shfl_sync(0xffffffffu, nc, 0);
      if (s0 >= W) break;
      if (nc >= KD_TILE) {
        overflow = true;
        break;
      }
      if (lane == 0) cstp[nc] = s0;
      ++nc;
      int b = nbp[s0];
      if (b < 0) {
        double ks64 = __longlong_as_double(0x7ff8000000000000LL);
        const unsigned long long ms = kd_order_key(sm[s0]);
        b = W;
        for (int j0 = s0 + 65; j0 < W; j0 += 32) {
          const int j = j0 + lane;
          bool split = false;
          if (j < W) split = !(kd_order_key(sm[j]) == ms || fit.fits(s0, j, ks64));
          const unsigned bal = __ballot_sync(0xffffffffu, split);
          if (bal) {
            b = j0 + __ffs(bal) - 1;
            break;
          }
        }
      }
      s0 = b;
    }
    if (lane == 0) {
      m.cst[overflow ? KD_TILE : nc] = W;
      sh.nc = overflow ? -1 : nc;
    }
  }
  __syncthreads();
  int nc = sh.nc;
  if (nc < 0) {
    if (threadIdx.x == 0) sh.err = KD_ERANGE;
    __syncthreads();
    return;
  }
  // 6. each cluster's running mean and weight, in order (Centroid.add_sample,
  //    centroid.mojo:25-36)
  if (exact) {
    // the running weight before element j is pi[j] - pi[start]: every ratio
    // w / (cur_w + w) is known up front; only the mean stays a chain
    for (int j = threadIdx.x; j < W; j += SP_T) {
      int lo = 0, hi = nc;  // the last cluster start <= j
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (m.cst[mid] <= j) lo = mid;
        else hi = mid;
      }
      const int s0 = m.cst[lo];
      if (j > s0) {
        const long long d = m.pi[j + 1] - m.pi[s0];
        m.rw[j] = (kd_bits(sw[j]) == 0x3ff0000000000000ULL && d < SP_RCP_N)
                      ? a.rcp[d]  // 1 / d, computed once by the same division
                      : KD_DIV(sw[j], (double)d);
      }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nc; t += SP_T) {
      const int s0 = m.cst[t], e = m.cst[t + 1];
      double cur_m = sm[s0];
#pragma unroll 4
      for (int j = s0 + 1; j < e; ++j) cur_m = KD_ADD(cur_m, KD_MUL(KD_SUB(sm[j], cur_m), m.rw[j]));
      if (e < W && sm[e] == cur_m) sh.mismatch = 1;  // the reference coalesces an exact mean tie
      m.cm[t] = cur_m;
      m.cw[t] = (double)(m.pi[e] - m.pi[s0]);
    }
    __syncthreads();
  } else {
    // running weights first (a serial chain of additions per cluster), then
    // every ratio w / (cur_w + w) in parallel, then the mean chains
    for (int t = threadIdx.x; t < nc; t += SP_T) {
      const int s0 = m.cst[t], e = m.cst[t + 1];
      double cur_w = sw[s0];
      m.cid[s0] = t;
      for (int j = s0 + 1; j < e; ++j) {
        m.rw[j] = cur_w;
        cur_w = KD_ADD(cur_w, sw[j]);
        m.cid[j] = t;
      }
      if (e < W) m.rw[e] = cur_w;
      m.cw[t] = cur_w;
    }
    __syncthreads();
    double* ratio = m.kk;  // the k array is free once the chain is known
    for (int j = threadIdx.x; j < W; j += SP_T)
      if (m.cst[m.cid[j]] != j) ratio[j] = KD_DIV(sw[j], KD_ADD(m.rw[j], sw[j]));
    __syncthreads();
    for (int t = threadIdx.x; t < nc; t += SP_T) {
      const int s0 = m.cst[t], e = m.cst[t + 1];
      double cur_m = sm[s0];
#pragma unroll 4
      for (int j = s0 + 1; j < e; ++j) cur_m = KD_ADD(cur_m, KD_MUL(KD_SUB(sm[j], cur_m), ratio[j]));
      if (e < W && sm[e] == cur_m) {  // the reference coalesces an exact mean tie
        sh.mismatch = 1;
        atomicMin(&sh.mm_first, e);
      }
      m.cm[t] = cur_m;
    }
    __syncthreads();
  }
  // 7. non-integral weights: re-check every decision with the chain's exact sums
  //    (also after a mean tie in step 6, so that mm_first is the first
  //    overturned decision of all)
  if (!exact) {
    if (threadIdx.x == 0) {
      double acc = 0.0;
      for (int t = 0; t < nc; ++t) {
        m.wsf[t] = acc;
        acc = KD_ADD(acc, m.cw[t]);
      }
    }
    __syncthreads();
    // the exact test k(q_right) - k(q_left) <= 1 through the FP32 filter; the
    // FP64 k only where the FP32 difference cannot decide
    // (the filter's q may be off by an ulp or two of FP64: far inside its band,
    // so it multiplies by 1/st; the undecided cases divide exactly)
    const float nrmf = (float)nrm, k0f = (float)sh.k0, k1f = (float)sh.k1;
    const double inv_st = sh.inv_st;
    float* kl32 = reinterpret_cast<float*>(m.kl);
    for (int t = threadIdx.x; t < nc; t += SP_T)
      kl32[t] = sp_k32q(scale, KD_MUL(m.wsf[t], inv_st), nrmf, k0f, k1f, false);
    __syncthreads();
    for (int j = 1 + threadIdx.x; j < W; j += SP_T) {
      const int t = m.cid[j];
      const bool start = m.cst[t] == j;
      const int tt = start ? t - 1 : t;
      const double num = KD_ADD(KD_ADD(m.wsf[tt], m.rw[j]), sw[j]);
      const float d = sp_k32q(scale, KD_MUL(num, inv_st), nrmf, k0f, k1f, false) - kl32[tt];
      bool fits;
      if (d <= 1.0f - fit.tau) {
        fits = true;
      } else if (d > 1.0f + fit.tau) {
        fits = false;
      } else {  // undecided (or an end of the scale): FP64
        fits = KD_SUB(sp_k(scale, KD_DIV(num, st), nrm), sp_k(scale, KD_DIV(m.wsf[tt], st), nrm)) <=
               1.0;
      }
      if (start ? fits : (!fits && !(sm[j] == sm[m.cst[tt]]))) {
        sh.mismatch = 1;
        atomicMin(&sh.mm_first, j);
      }
    }
    __syncthreads();
  }
  // 8. mismatch: the reference loop, one thread.  With non-integral weights it
  //    resumes at the first overturned candidate j0: every decision before j0
  //    is the reference's, so the clusters before the one holding j0 - 1 are
  //    final, and that cluster's state is rebuilt with the reference's own
  //    operations (weights before it summed in order, its running mean from
  //    the ratios step 6 left in kk, its running weight from rw).
  if (sh.mismatch) {
    if (threadIdx.x == 0) {
      double wsf = 0.0, cur_m = sm[0], cur_w = sw[0];
      int k = 0, i0 = 1;
      const int j0 = sh.mm_first;
      if (!exact && j0 > 0 && j0 < W) {
        const int t = m.cid[j0];
        const int tt = m.cst[t] == j0 ? t - 1 : t;  // the cluster holding j0 - 1
        for (int u = 0; u < tt; ++u) wsf = KD_ADD(wsf, m.cw[u]);
        const int s0 = m.cst[tt];
        const double* ratio = m.kk;
        cur_m = sm[s0];
        for (int j = s0 + 1; j < j0; ++j) cur_m = KD_ADD(cur_m, KD_MUL(KD_SUB(sm[j], cur_m), ratio[j]));
        cur_w = m.rw[j0];
        k = tt;
        i0 = j0;
      }
      double kq = sp_k(scale, KD_DIV(wsf, st), nrm);
      bool overflow = false;
      for (int i = i0; i < W; ++i) {
        const double qr = KD_DIV(KD_ADD(KD_ADD(wsf, cur_w), sw[i]), st);
        const double span = KD_SUB(sp_k(scale, qr, nrm), kq);
        if (sm[i] == cur_m || span <= 1.0) {
          const double nw = KD_ADD(cur_w, sw[i]);
          cur_m = KD_ADD(cur_m, KD_MUL(KD_SUB(sm[i], cur_m), KD_DIV(sw[i], nw)));
          cur_w = nw;
        } else {
          if (k >= KD_TILE - 1) {
            overflow = true;
            break;
          }
          m.cm[k] = cur_m;
          m.cw[k] = cur_w;
          ++k;
          wsf = KD_ADD(wsf, cur_w);
          kq = sp_k(scale, KD_DIV(wsf, st), nrm);
          cur_m = sm[i];
          cur_w = sw[i];
        }
      }
      m.cm[k] = cur_m;
      m.cw[k] = cur_w;
      sh.nc = k + 1;
      if (overflow) sh.err = KD_ERANGE;
    }
    __syncthreads();
    nc = sh.nc;
  }
  // 9. prune decayed mass (tdigest.mojo:441-458): a parallel test first; the
  //    serial removal (its sum is in centroid order) only when something goes
  if (threadIdx.x == 0) sh.bfail = 0;  // here: some centroid falls below the floor
  __syncthreads();
  if (decay)
    for (int i = threadIdx.x; i < nc; i += SP_T)
      if (!(m.cw[i] >= sh.floor_w)) sh.bfail = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = nc;
    if (decay && sh.bfail) {
      const double floor_w = sh.floor_w;
      int k = 0;
      double removed = 0.0;
      for (int i = 0; i < c; ++i) {
        const double wi = m.cw[i];
        if (wi >= floor_w) {
          m.cm[k] = m.cm[i];
          m.cw[k] = wi;
          ++k;
        } else {
          removed = KD_ADD(removed, wi);
        }
      }
      if (removed > 0.0) {
        sh.st = KD_SUB(sh.st, removed);
        c = k;
      }
    }
    sh.C = c;
  }
  __syncthreads();
}

// Renormalise (tdigest.mojo:359-371): every stored weight and the total by
// e^{-log_scale}; the exponent restarts at 0.
__device__ void sp_renormalize(const SpMem& m, SpSh& sh) {
  if (threadIdx.x == 0) sh.factor = kd_exp(-sh.ls);
  __syncthreads();
  const double f = sh.factor;
  for (int i = threadIdx.x; i < sh.C; i += SP_T) m.cw[i] = KD_MUL(m.cw[i], f);
  for (int i = threadIdx.x; i < sh.B; i += SP_T) m.bw[i] = KD_MUL(m.bw[i], f);
  __syncthreads();
  if (threadIdx.x == 0) {
    sh.st = KD_MUL(sh.st, f);
    sh.ls = 0.0;
  }
  __syncthreads();
}

// Reduction that keeps the first occurrence among equal values (the reference
// updates its running min / max only on a strict improvement).
struct SpPick {
  unsigned long long key;  // order key (equal values compare equal)
  long long seq;
  double v;
};
__device__ __forceinline__ SpPick sp_pick_min(SpPick a, SpPick b) {
  if (b.key < a.key || (b.key == a.key && b.seq < a.seq)) return b;
  return a;
}
__device__ __forceinline__ SpPick sp_pick_max(SpPick a, SpPick b) {
  if (b.key > a.key || (b.key == a.key && b.seq < a.seq)) return b;
  return a;
}
__device__ SpPick sp_shfl(SpPick p, int o) {
  SpPick q;
  q.key = __shfl_down_sync(0xffffffffu, p.key, o);
  q.seq = __shfl_down_sync(0xffffffffu, p.seq, o);
  q.v = __shfl_down_sync(0xffffffffu, p.v, o);
  return q;
}

__device__ void sp_reduce_minmax(SpPick& mn, SpPick& mx, SpPick* red) {
  for (int o = 16; o > 0; o >>= 1) {
    mn = sp_pick_min(mn, sp_shfl(mn, o));
    mx = sp_pick_max(mx, sp_shfl(mx, o));
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    red[w] = mn;
    red[32 + w] = mx;
  }
  __syncthreads();
  if (w == 0) {
    mn = red[lane];
    mx = red[32 + lane];
    for (int o = 16; o > 0; o >>= 1) {
      mn = sp_pick_min(mn, sp_shfl(mn, o));
      mx = sp_pick_max(mx, sp_shfl(mx, o));
    }
    if (lane == 0) {
      red[0] = mn;
      red[32] = mx;
    }
  }
  __syncthreads();
  mn = red[0];
  mx = red[32];
  __syncthreads();
}

// The add loop over samples [0, n_eff) (tdigest.mojo:153-175, 334-350): each
// sample advances the clock, is buffered with its decay-scaled weight, and a
// full buffer runs the merge pass.
// st += w_0 + w_1 + ... (bw[B0 .. B0 + cut)), added in order.  Inside the
// binade [2^E, 2^(E+1)) of st every sum st + w rounds to st + round(w / u) * u
// with u = 2^(E-52), the same rounding for every st, unless w / u lies exactly
// half-way between integers.  So while st stays below 2^(E+1) - 2u the serial
// sum is st plus the integer prefix of round(w / u), in units of u: one block
// scan.  A step that would leave the binade, a tie, and what follows them are
// added one at a time.
__device__ void sp_add_total(const SpMem& m, SpSh& sh, int B0, int cut) {
  if (threadIdx.x == 0) {
    const double st = sh.st;
    const unsigned long long b = kd_bits(st);
    const int ex = (int)((b >> 52) & 0x7ff);
    sh.fast = st > 0.0 && ex > 53 && ex < 2000;  // normal, positive, u a normal power of two
    if (sh.fast) {
      sh.tot_u = kd_pow2i(ex - 1075);                        // u
      sh.tot_base = (long long)KD_MUL(st, kd_pow2i(1075 - ex)); // st / u, in [2^52, 2^53)
    }
  }
  __syncthreads();
  const double* const bw = m.bw + B0;
  long long* const nk = m.pi;  // free outside merges
  int first_bad = cut;
  if (sh.fast) {
    const double inv_u = kd_pow2i(1075 - (int)((kd_bits(sh.st) >> 52) & 0x7ff));
    const int per = (cut + SP_T - 1) / SP_T;
    const int k0 = threadIdx.x * per, k1 = min(cut, k0 + per);
    long long sum = 0;
    int bad = cut;
    for (int k = k0; k < k1; ++k) {
      const double t = KD_MUL(bw[k], inv_u);  // exact: a power-of-two scale
      long long n = 0;
      if (!(t < 1099511627776.0)) {           // 2^40: far beyond the binade anyway
        if (bad == cut) bad = k;
        n = 1LL << 40;
      } else {
        const double f = floor(t);
        const double fr = KD_SUB(t, f);  // exact
        if (fr == 0.5 && bad == cut) bad = k;  // a tie: rounding depends on st
        n = (long long)f + (fr > 0.5 ? 1 : 0);
      }
      nk[k] = n;
      sum += n;
    }
    if (bad < cut) atomicMin(&sh.cut, bad);  // sh.cut is free here: reused as "first bad"
    long long total;
    long long run = sp_iscan(sum, sh, &total);
    const long long limit = (1LL << 53) - 2 - sh.tot_base;
    for (int k = k0; k < k1; ++k) {
      run += nk[k];
      if (run > limit) {
        atomicMin(&sh.cut, k);
        break;
      }
      nk[k] = run;  // inclusive prefix
    }
    __syncthreads();
    first_bad = sh.cut;
  }
  if (threadIdx.x == 0) {
    double st = sh.st;
    int k = 0;
    if (sh.fast && first_bad > 0) {  // exact: st + prefix * u stays below 2^(E+1) - u
      st = KD_MUL((double)(sh.tot_base + nk[first_bad - 1]), sh.tot_u);
      k = first_bad;
    }
    for (; k < cut; ++k) st = KD_ADD(st, bw[k]);
    sh.st = st;
  }
  __syncthreads();
}

__device__ __noinline__ void sp_add_decay(const SpArgs& a, const SpMem& m, SpSh& sh, long long n_eff,
                             SpPick* red) {
  const bool decay = true;
  const double lambda = a.s.lambda;
  const int L = a.s.buf_cap;
  long long i = 0;
  while (i < n_eff && !sh.err) {
    const long long room = (long long)(L - sh.B);
    const int seg = (int)(n_eff - i < room ? n_eff - i : room);
    const int B0 = sh.B;
    // clock, decay exponent and renormalisation, in sample order (one thread)
    if (threadIdx.x == 0) {
      int cut = 0;
      sh.renorm = 0;
      sh.nruns = 0;
      double clock = sh.clock, ls = sh.ls;
      if (!a.ts && clock == floor(clock) && fabs(clock) < 4.0e15) {
        // Count clock: every step is exactly clock + 1, so the exponent step
        // lambda * (new - old) is exactly lambda.  Only the exponent's own
        // chain of additions stays serial.
        // The threshold test compares bit patterns (the exponent is never
        // negative), so only the additions wait on each other.
        const unsigned long long renorm_bits = kd_bits(SP_RENORM);
        double* const sls = m.sls;
        int adv = 0, k = 0;
        if (sh.pre_adv && seg > 0) {
          sls[0] = ls;
          k = 1;
        }
        // Inside one binade [2^e, 2^(e+1)) of the exponent, and unless lambda
        // sits exactly half-way between two multiples of its ulp u, every step
        // rounds x + lambda to x + r with the same r: the values form runs
        // x + r, x + 2r, ... that other threads fill in.  Crossings, ties and
        // the renormalisation threshold are stepped one at a time.
        int nr = 0;
        while (k < seg && nr < SP_RUNS) {
          const double y = KD_ADD(ls, lambda);
          if (kd_bits(y) > renorm_bits) break;  // the per-sample loop below handles it
          const unsigned long long bx = kd_bits(ls);
          const int ex = (int)((bx >> 52) & 0x7ff);
          int n = 1;
          double r = KD_SUB(y, ls);
          if (ls > 0.0 && ex > 53 && ex < 2000) {
            const double top = KD_SUB(kd_pow2i(ex - 1022), kd_pow2i(ex - 1075));  // 2^(e+1) - u
            const double t = KD_MUL(lambda, kd_pow2i(1075 - ex));  // lambda / u, exact
            const bool tie = KD_SUB(t, floor(t)) == 0.5;
            if (!tie && y <= top) {
              const double D = KD_SUB(top, ls);  // exact: multiples of u
              if (r == 0.0) {
                n = seg - k;  // below half an ulp: the exponent no longer moves
              } else {
                // largest m with x + m r + lambda < top, and x + (m + 1) r <= 400
                double mf = floor(KD_DIV(KD_SUB(D, lambda), r));
                const double mr = floor(KD_DIV(KD_SUB(SP_RENORM, ls), r)) - 1.0;
                if (mr < mf) mf = mr;
                long long mm = mf > 1e9 ? 1000000000LL : (long long)mf;
                while (mm > 0 && !(lambda < KD_SUB(D, KD_MUL((double)mm, r)))) --mm;
                while (mm > 0 && KD_ADD(ls, KD_MUL((double)(mm + 1), r)) > SP_RENORM) --mm;
                if (mm < 0) mm = 0;
                n = (int)((long long)(seg - k) < mm + 1 ? (long long)(seg - k) : mm + 1);
              }
            }
          }
          m.rk[nr] = k;
          m.rn[nr] = n;
          m.rx[nr] = ls;
          m.rr[nr] = r;
          ++nr;
          ls = KD_ADD(ls, KD_MUL((double)n, r));
          k += n;
          adv += n;
        }
        sh.nruns = nr;
        for (; k < seg; ++k) {
          const double nl = KD_ADD(ls, lambda);
          if (kd_bits(nl) > renorm_bits) {
            ls = nl;
            sh.renorm = 1;
            sh.renorm_clock = KD_ADD(clock, (double)(adv + 1));
            break;
          }
          ls = nl;
          ++adv;
          sls[k] = ls;
        }
        cut = k;
        clock = KD_ADD(clock, (double)adv);
      } else {
        for (int k = 0; k < seg; ++k) {
          const long long j = i + k;
          bool advance;
          double nc = clock;
          if (sh.pre_adv && k == 0) {
            advance = false;  // this sample's clock step ran before the renormalisation
          } else if (a.ts) {
            advance = a.ts[j] > clock;
            nc = a.ts[j];
          } else {
            advance = true;
            nc = KD_ADD(clock, 1.0);
          }
          if (advance) {
            if (nc > clock) {
              ls = KD_ADD(ls, KD_MUL(lambda, KD_SUB(nc, clock)));
              if (ls > SP_RENORM) {
                sh.renorm = 1;
                sh.renorm_clock = nc;
                break;
              }
            }
            clock = nc;
          }
          m.sls[k] = ls;
          cut = k + 1;
        }
      }
      sh.pre_adv = 0;
      sh.clock = clock;
      sh.ls = ls;
      sh.cut = cut;
    }
    __syncthreads();
    for (int q = 0; q < sh.nruns; ++q) {  // the exponent runs: x + j r, exact
      const int k0 = m.rk[q], n = m.rn[q];
      const double x = m.rx[q], r = m.rr[q];
      for (int j = threadIdx.x; j < n; j += SP_T) m.sls[k0 + j] = KD_ADD(x, KD_MUL((double)(j + 1), r));
    }
    __syncthreads();
    const int cut = sh.cut;
    // buffer the samples with their scaled weights (weight * e^{log_scale})
    for (int k = threadIdx.x; k < cut; k += SP_T) {
      const double w = a.wts ? a.wts[i + k] : 1.0;
      m.bm[B0 + k] = a.vals[i + k];
      m.bw[B0 + k] = decay ? KD_MUL(w, kd_exp(m.sls[k])) : w;  // w * 1.0 == w
    }
    __syncthreads();
    // running min / max (reset by the first sample of an empty digest) and the
    // stored total, in sample order
    if (cut > 0) {
      const bool reset = sh.st == 0.0 && B0 == 0;
      SpPick mn{~0ull, 0x7fffffffffffffffLL, 0.0}, mx{0ull, 0x7fffffffffffffffLL, 0.0};
      if (!reset && threadIdx.x == 0) {
        mn = SpPick{kd_order_key(sh.mn), -1, sh.mn};
        mx = SpPick{kd_order_key(sh.mx), -1, sh.mx};
      }
      for (int k = threadIdx.x; k < cut; k += SP_T) {
        const double v = m.bm[B0 + k];
        const SpPick p{kd_order_key(v), (long long)k, v};
        mn = sp_pick_min(mn, p);
        mx = sp_pick_max(mx, p);
      }
      sp_reduce_minmax(mn, mx, red);
      if (threadIdx.x == 0) {
        sh.mn = mn.v;
        sh.mx = mx.v;
      }
      sp_add_total(m, sh, B0, cut);  // the stored total, as the serial sum gives it
      if (threadIdx.x == 0) sh.B = B0 + cut;
      __syncthreads();
    }
    i += cut;
    if (sh.renorm) {
      // The next sample's clock step took the exponent (now in sh.ls) past the
      // threshold: renormalise, finish that step, then insert the sample.
      sp_renormalize(m, sh);
      if (threadIdx.x == 0) {
        sh.clock = sh.renorm_clock;
        sh.pre_adv = 1;
        sh.renorm = 0;
      }
      __syncthreads();
    }
    if (sh.B >= L) sp_merge(a, m, sh, nullptr, nullptr);
    __syncthreads();
  }
}

// Buffers samples [i, i + cut) of the call (weights w * e^0 == w) and adds them
// to the stored total: exactly in integers when every weight is one and the
// total stays below 2^53, else in sample order.
__device__ void sp_append(const SpArgs& a, const SpMem& m, SpSh& sh, long long i, int cut) {
  const int B0 = sh.B;
  long long part = 0;
  for (int k = threadIdx.x; k < cut; k += SP_T) {
    const double w = a.wts ? a.wts[i + k] : 1.0;
    m.bm[B0 + k] = a.vals[i + k];
    m.bw[B0 + k] = w;
    long long x = 0;
    sp_int53(w, &x);
    part += x;
  }
  const long long sum = sh.integral ? sp_isum(part, sh) : 0;  // synchronises
  if (!sh.integral) __syncthreads();
  if (threadIdx.x == 0) {
    double tot = sh.st;
    const bool exact = sh.integral && tot == floor(tot) && tot >= 0.0 &&
                       tot <= 4503599627370496.0 && sum <= (1LL << 52);
    if (exact) {
      tot = KD_ADD(tot, (double)sum);
    } else {
      for (int k = 0; k < cut; ++k) tot = KD_ADD(tot, m.bw[B0 + k]);
    }
    sh.st = tot;
    sh.B = B0 + cut;
  }
  __syncthreads();
}

// Without decay the exponent never moves and nothing is pruned, so the clock
// and the running min / max have no effect on any merge: they are settled once
// for the whole call (count clock: integral clocks below 2^52 add exactly, so
// clock + n is the sum of n additions of 1; time clock: the latest timestamp,
// the earliest of equal ones; min / max: the first occurrence of the extreme,
// reset by the first sample of an empty digest).  Per buffer fill only the
// samples, the stored total and the merge remain.
__device__ __noinline__ void sp_add_plain(const SpArgs& a, const SpMem& m, SpSh& sh, long long n_eff,
                             SpPick* red) {
  const int L = a.s.buf_cap;
  if (n_eff == 0) return;
  {
    const bool reset = sh.st == 0.0 && sh.B == 0;
    SpPick mn{~0ull, 0x7fffffffffffffffLL, 0.0}, mx{0ull, 0x7fffffffffffffffLL, 0.0};
    if (!reset && threadIdx.x == 0) {
      mn = SpPick{kd_order_key(sh.mn), -1, sh.mn};
      mx = SpPick{kd_order_key(sh.mx), -1, sh.mx};
    }
    for (long long k = threadIdx.x; k < n_eff; k += SP_T) {
      const double v = a.vals[k];
      const SpPick p{kd_order_key(v), k, v};
      mn = sp_pick_min(mn, p);
      mx = sp_pick_max(mx, p);
    }
    sp_reduce_minmax(mn, mx, red);
    if (threadIdx.x == 0) {
      sh.mn = mn.v;
      sh.mx = mx.v;
    }
    if (a.ts) {
      SpPick tm{kd_order_key(sh.clock), -1, sh.clock}, dummy{~0ull, -1, 0.0};
      for (long long k = threadIdx.x; k < n_eff; k += SP_T) {
        const double t = a.ts[k];
        if (t == t) tm = sp_pick_max(tm, SpPick{kd_order_key(t), k, t});
      }
      sp_reduce_minmax(dummy, tm, red);
      if (threadIdx.x == 0 && tm.seq >= 0 && tm.v > sh.clock) sh.clock = tm.v;
    } else if (threadIdx.x == 0) {
      if (sh.clock == floor(sh.clock) && fabs(sh.clock) < 4.0e15 && n_eff < (1LL << 40)) {
        sh.clock = KD_ADD(sh.clock, (double)n_eff);
      } else {
        double c = sh.clock;
        for (long long k = 0; k < n_eff; ++k) c = KD_ADD(c, 1.0);
        sh.clock = c;
      }
    }
    __syncthreads();
  }
  long long i = 0;
  while (i < n_eff && !sh.err) {
    const int B0 = sh.B;
    const long long room = (long long)(L - B0);
    const int cut = (int)(n_eff - i < room ? n_eff - i : room);
    sp_append(a, m, sh, i, cut);
    i += cut;
    if (sh.B >= L) sp_merge(a, m, sh, nullptr, nullptr);
    __syncthreads();
  }
}

__device__ void sp_add(const SpArgs& a, const SpMem& m, SpSh& sh, long long n_eff, SpPick* red) {
  if (a.s.lambda > 0.0) sp_add_decay(a, m, sh, n_eff, red);
  else sp_add_plain(a, m, sh, n_eff, red);
}

// Writes the call's result to the store: new centroids into the back slot,
// the quantile-walk prefix, the header and the buffer; then flips the slot.
__device__ void sp_commit(const SpArgs& a, const SpMem& m, SpSh& sh) {
  const KdStoreDev& s = a.s;
  const int live = s.cur[0];
  const int b = live ^ 1;
  double* dm = s.slot_m + (size_t)b * (size_t)s.K * KD_TILE;
  double* dw = s.slot_w + (size_t)b * (size_t)s.K * KD_TILE;
  const int C = sh.C, B = sh.B;
  for (int i = threadIdx.x; i < C; i += SP_T) {
    dm[i] = m.cm[i];
    dw[i] = m.cw[i];
  }
  for (int i = threadIdx.x; i < B; i += SP_T) {
    s.buf_m[i] = m.bm[i];
    s.buf_w[i] = m.bw[i];
  }
  // The quantile-walk prefix, the same arithmetic as the batch path's commit:
  // P[0] = w0/2, P[i+1] = P[i] + (w_i + w_{i+1})/2.  With integral weights
  // below 2^52 every step is exact, so P[i] = (w_0 + ... + w_{i-1}) + w_i/2.
  if (threadIdx.x == 0) sh.exact = 1;
  __syncthreads();
  long long wi = 0;
  if (threadIdx.x < C && !sp_int53(m.cw[threadIdx.x], &wi)) sh.exact = 0;
  __syncthreads();
  const bool int_p = sh.exact && C <= SP_T;
  if (int_p) {
    long long total;
    const long long excl = sp_iscan(wi, sh, &total);
    if (total <= (1LL << 52) && threadIdx.x < C)
      s.prefix[threadIdx.x] = KD_ADD((double)excl, KD_MUL(m.cw[threadIdx.x], 0.5));
    if (threadIdx.x == 0 && total > (1LL << 52)) sh.exact = 0;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double* P = s.prefix;
    if (C > 0 && !(int_p && sh.exact)) {
      double run = KD_MUL(m.cw[0], 0.5);
      P[0] = run;
      for (int i = 0; i + 1 < C; ++i) {
        run = KD_ADD(run, KD_MUL(KD_ADD(m.cw[i], m.cw[i + 1]), 0.5));
        P[i + 1] = run;
      }
    }
    s.count[0] = C;
    s.total[0] = sh.st;
    s.log_scale[0] = sh.ls;
    s.clock[0] = sh.clock;
    s.min_v[0] = sh.mn;
    s.max_v[0] = sh.mx;
    s.dfac[0] = s.lambda > 0.0 ? kd_exp(-sh.ls) : 1.0;
    s.bcount[0] = B;
    __threadfence();
    s.cur[0] = (unsigned char)b;
    a.out->count = C;
    a.out->bcount = B;
  }
}

// Renormalises the other digest of a merge_into in place (its weights, total
// and exponent; the walk prefix follows the new weights).
__device__ void sp_renorm_other(const SpArgs& a, SpSh& sh, double factor) {
  const KdStoreDev& o = a.o;
  const int live = o.cur[0];
  double* ow = o.slot_w + (size_t)live * (size_t)o.K * KD_TILE;
  const int C = o.count[0];
  for (int i = threadIdx.x; i < C; i += SP_T) ow[i] = KD_MUL(ow[i], factor);
  __syncthreads();
  if (threadIdx.x == 0) {
    double* P = o.prefix;
    if (C > 0) {
      double run = KD_MUL(ow[0], 0.5);
      P[0] = run;
      for (int i = 0; i + 1 < C; ++i) {
        run = KD_ADD(run, KD_MUL(KD_ADD(ow[i], ow[i + 1]), 0.5));
        P[i + 1] = run;
      }
    }
    o.total[0] = KD_MUL(o.total[0], factor);
    o.log_scale[0] = 0.0;
    o.dfac[0] = 1.0;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(SP_T) k_spath(SpArgs a) {
  extern __shared__ __align__(256) unsigned char sp_smem[];
  __shared__ SpSh sh;
  __shared__ SpPick red[64];
  SpMem m;
  sp_layout(a.bmax, a.wpb, a.scratch ? a.scratch : sp_smem, &m);
  const KdStoreDev& s = a.s;
  const int live = s.cur[0];
  if (threadIdx.x == 0) {
    sh.C = s.count[0];
    sh.B = s.bcount[0];
    sh.st = s.total[0];
    sh.ls = s.log_scale[0];
    sh.clock = s.clock[0];
    sh.mn = s.min_v[0];
    sh.mx = s.max_v[0];
    sh.err = 0;
    sh.pre_adv = 0;
    sh.renorm = 0;
    sh.first_bad = a.n;
    sh.integral = 1;
    a.out->noop = 0;
    sh.f0 = sp_k(s.scale, 0.0, 1.0);
  } else if (threadIdx.x == 32) {
    sh.f1 = sp_k(s.scale, 1.0, 1.0);
  } else if (threadIdx.x == 64) {
    sh.nrm01 = s.scale <= KD_SCALE_K1 ? kd_normalizer(s.scale, s.compression, 1.0) : 0.0;
  }
  __syncthreads();
  {
    const double* lm = s.slot_m + (size_t)live * (size_t)s.K * KD_TILE;
    const double* lw = s.slot_w + (size_t)live * (size_t)s.K * KD_TILE;
    for (int i = threadIdx.x; i < sh.C; i += SP_T) {
      m.cm[i] = lm[i];
      m.cw[i] = lw[i];
    }
    for (int i = threadIdx.x; i < sh.B; i += SP_T) {
      m.bm[i] = s.buf_m[i];
      m.bw[i] = s.buf_w[i];
    }
  }
  __syncthreads();
  if (a.op == SP_ADD) {
    // the first invalid sample ends the loop there (the reference raises at it)
    for (long long i = threadIdx.x; i < a.n; i += SP_T) {
      const double v = a.vals[i];
      const double w = a.wts ? a.wts[i] : 1.0;
      const bool bad = !kd_isfinite(v) || !(w > 0.0) || !kd_isfinite(w);
      if (bad) atomicMin((unsigned long long*)&sh.first_bad, (unsigned long long)i);
      long long x;
      if (!sp_int53(w, &x)) sh.integral = 0;
    }
    __syncthreads();
    sp_add(a, m, sh, sh.first_bad, red);
    if (threadIdx.x == 0 && !sh.err && sh.first_bad < a.n) {
      a.out->code = KD_EINVAL;
      a.out->index = sh.first_bad;
    }
  } else if (a.op == SP_FLUSH) {
    sp_merge(a, m, sh, nullptr, nullptr);
  } else {  // SP_MERGE_INTO (tdigest.mojo:589-623)
    const KdStoreDev& o = a.o;
    const double o_st = o.total[0], o_ls = o.log_scale[0];
    const double o_eff = o.lambda > 0.0 ? KD_MUL(o_st, kd_exp(-o_ls)) : o_st;
    if (o_eff == 0.0) {
      if (threadIdx.x == 0) a.out->noop = 1;
      return;
    }
    sp_merge(a, m, sh, nullptr, nullptr);
    if (s.lambda > 0.0) sp_renormalize(m, sh);
    double o_total = o_st;
    if (o.lambda > 0.0) {
      const double f = kd_exp(-o_ls);
      sp_renorm_other(a, sh, f);
      o_total = o.total[0];
    }
    const int oC = o.count[0];
    const int olive = o.cur[0];
    const double* om = o.slot_m + (size_t)olive * (size_t)o.K * KD_TILE;
    const double* ow = o.slot_w + (size_t)olive * (size_t)o.K * KD_TILE;
    for (int i = threadIdx.x; i < oC; i += SP_T) {
      m.bm[i] = om[i];
      m.bw[i] = ow[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const bool was_empty = sh.st == 0.0;
      sh.B = oC;
      sh.st = KD_ADD(sh.st, o_total);
      const double omn = o.min_v[0], omx = o.max_v[0];
      if (was_empty) {
        sh.mn = omn;
        sh.mx = omx;
      } else {
        sh.mn = sh.mn < omn ? sh.mn : omn;
        sh.mx = sh.mx > omx ? sh.mx : omx;
      }
      sh.clock = sh.clock > o.clock[0] ? sh.clock : o.clock[0];
    }
    __syncthreads();
    sp_merge(a, m, sh, nullptr, nullptr);
  }
  __syncthreads();
  if (sh.err) {
    if (threadIdx.x == 0) {
      a.out->code = sh.err;
      a.out->index = -1;
    }
    return;
  }
  sp_commit(a, m, sh);
}

// 1 / d for the unit-weight ratios of the merge pass, made once per device by
// the same correctly rounded division the pass would run.
__device__ double sp_rcp_table[SP_RCP_N];

__global__ void k_rcp_init() {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < SP_RCP_N; d += gridDim.x * blockDim.x)
    sp_rcp_table[d] = d == 0 ? 0.0 : KD_DIV(1.0, (double)d);
}

int sp_fail(KdSession* s, int code, const char* msg) {
  kd_set_msg(s, msg);
  return code;
}

// Buffer storage of a one-key store, made on first use of the path.
int sp_ensure(KdSession* s, KdStore* st) {
  KdStoreDev& d = st->d;
  if (d.K != 1) return sp_fail(s, KD_EINVAL, "the single-sample path serves one-digest stores");
  if (d.bcount) return KD_OK;
  if (!(d.compression < 1e6)) return sp_fail(s, KD_EINVAL, "compression too large for the single-sample path");
  long long L = (long long)d.compression * 5;  // Int(compression) * _BUFFER_FACTOR
  if (L < 1) L = 1;
  if (L > (1 << 20)) return sp_fail(s, KD_EINVAL, "compression too large for the single-sample path");
  const size_t bytes = 64 + (size_t)L * 16;
  if (s->mem_budget && s->mem_used + bytes > s->mem_budget)
    return sp_fail(s, KD_ENOMEM, "device-memory budget exceeded by the sample buffer");
  int* bc = nullptr;
  double* bm = nullptr;
  double* bw = nullptr;
  if (cudaMalloc(&bc, 64) != cudaSuccess || cudaMalloc(&bm, (size_t)L * 8) != cudaSuccess ||
      cudaMalloc(&bw, (size_t)L * 8) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(bc);
    cudaFree(bm);
    return sp_fail(s, KD_ENOMEM, "sample buffer allocation failed");
  }
  if (cudaMemsetAsync(bc, 0, 64, s->stream) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(bc);
    cudaFree(bm);
    cudaFree(bw);
    return sp_fail(s, KD_ENOMEM, "sample buffer initialisation failed");
  }
  d.bcount = bc;
  d.buf_m = bm;
  d.buf_w = bw;
  d.buf_cap = (int)L;
  s->mem_used += bytes;
  st->bytes += bytes;
  kd_store_drop_graphs(st);  // captured steps hold the store view by value
  return KD_OK;
}

struct SpShape {
  int bmax, wpb;
  size_t bytes;
};
SpShape sp_shape(const KdStoreDev& d) {
  SpShape sh;
  sh.bmax = std::max(d.buf_cap, KD_TILE);
  sh.wpb = 1;
  while (sh.wpb < sh.bmax) sh.wpb <<= 1;
  sh.bytes = sp_layout(sh.bmax, sh.wpb, nullptr, nullptr);
  return sh;
}

constexpr size_t SP_SMEM_MAX = 220 * 1024;  // beyond this the state lives in global scratch

// The call's status block sits behind the buffer count in the same allocation.
SpStatus* sp_status(KdStore* st) {
  return reinterpret_cast<SpStatus*>(reinterpret_cast<char*>(st->d.bcount) + 16);
}

int sp_run(KdSession* s, KdStore* st, int op, const double* d_vals, const double* d_wts,
           const double* d_ts, long long n, KdStore* other, SpStatus* result) {
  KdStoreDev& d = st->d;
  const SpShape shp = sp_shape(d);
  unsigned char* scratch = nullptr;
  size_t smem = shp.bytes;
  if (shp.bytes > SP_SMEM_MAX) {
    if (st->sp_scratch_bytes < shp.bytes) {
      if (st->sp_scratch) cudaFree(st->sp_scratch);
      st->sp_scratch = nullptr;
      st->sp_scratch_bytes = 0;
      if (cudaMalloc(&st->sp_scratch, shp.bytes) != cudaSuccess) {
        cudaGetLastError();
        return sp_fail(s, KD_ENOMEM, "single-sample path scratch allocation failed");
      }
      st->sp_scratch_bytes = shp.bytes;
    }
    scratch = (unsigned char*)st->sp_scratch;
    smem = 0;
  }
  static std::atomic<bool> attr_done[64];
  const int dev = s->device;
  if (smem && dev >= 0 && dev < 64 && !attr_done[dev].load()) {
    cudaError_t e = cudaFuncSetAttribute(k_spath, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)SP_SMEM_MAX);
    if (e != cudaSuccess) return kd_cuda_fail(s, e, "single-sample path attributes");
    attr_done[dev].store(true);
  }
  static std::atomic<bool> rcp_done[64];
  static const double* rcp_ptr[64];
  if (dev < 0 || dev >= 64) return sp_fail(s, KD_EINVAL, "device ordinal out of range");
  if (!rcp_done[dev].load()) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, sp_rcp_table);
    if (e != cudaSuccess) return kd_cuda_fail(s, e, "reciprocal table");
    k_rcp_init<<<64, 256, 0, s->stream>>>();
    e = cudaGetLastError();
    if (e != cudaSuccess) return kd_cuda_fail(s, e, "reciprocal table");
    rcp_ptr[dev] = (const double*)p;
    rcp_done[dev].store(true);
  }
  SpStatus* dstat = sp_status(st);
  SpArgs a;
  a.s = d;
  a.o = other ? other->d : d;
  a.vals = d_vals;
  a.wts = d_wts;
  a.ts = d_ts;
  a.n = n;
  a.op = op;
  a.bmax = shp.bmax;
  a.wpb = shp.wpb;
  a.scratch = scratch;
  a.rcp = rcp_ptr[dev];
  a.out = dstat;
  cudaStream_t str = s->stream;
  cudaError_t e = cudaMemsetAsync(dstat, 0, sizeof(SpStatus), str);
  if (e != cudaSuccess) return kd_cuda_fail(s, e, "single-sample path");
  k_spath<<<1, SP_T, smem, str>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return kd_cuda_fail(s, e, "single-sample path launch");
  SpStatus h{};
  e = cudaMemcpyAsync(&h, dstat, sizeof(SpStatus), cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess) e = cudaStreamSynchronize(str);
  if (e != cudaSuccess) return kd_cuda_fail(s, e, "single-sample path");
  *result = h;
  s->stats.launches += 1;
  return KD_OK;
}

int sp_after(KdSession* s, KdStore* st, const SpStatus& r) {
  if (r.code == KD_ERANGE) {
    return sp_fail(s, KD_ERANGE, "a merge pass produced more than 1024 centroids");
  }
  if (r.code != KD_OK && r.code != KD_EINVAL)
    return sp_fail(s, r.code, "single-sample path: internal consistency check failed");
  if (!r.noop && r.code != KD_ERANGE) {
    st->pending = r.bcount > 0;
    st->carry = true;
  }
  if (r.code == KD_EINVAL) {
    char msg[160];
    snprintf(msg, sizeof msg,
             "sample %lld: value must be finite (got NaN or inf) and weight positive and finite",
             r.index);
    kd_set_msg(s, msg);
    return KD_EINVAL;
  }
  return r.code;
}

__global__ void k_carry_build(KdStoreDev s, const double* __restrict__ vals, long long n, int C,
                              int B, double* __restrict__ ov, double* __restrict__ ow,
                              unsigned long long* mm) {
  const int live = s.cur[0];
  const double* lm = s.slot_m + (size_t)live * (size_t)s.K * KD_TILE;
  const double* lw = s.slot_w + (size_t)live * (size_t)s.K * KD_TILE;
  const long long tot = (long long)C + B + n;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < tot;
       i += (long long)gridDim.x * blockDim.x) {
    double v, w;
    if (i < C) {
      v = lm[i];
      w = lw[i];
    } else if (i < C + B) {
      v = s.buf_m[i - C];
      w = s.buf_w[i - C];
    } else {
      v = vals[i - C - B];
      w = 0.0;  // the batch's samples take the decay weight of the step
      if (kd_isfinite(v)) {
        const unsigned long long k = kd_order_key(v);
        atomicMin(&mm[0], k);
        atomicMax(&mm[1], k);
      }
    }
    ov[i] = v;
    ow[i] = w;
  }
}

}  // namespace

int kd_spath_flush(KdSession* s, KdStore* st) {
  if (!st->pending) return KD_OK;
  cudaSetDevice(s->device);
  SpStatus r{};
  int rc = sp_run(s, st, SP_FLUSH, nullptr, nullptr, nullptr, 0, nullptr, &r);
  if (rc) return rc;
  return sp_after(s, st, r);
}

int kd_spath_carry_ingest(KdSession* s, KdStore* st, const double* d_vals, long long n, int mode,
                          double timestamp) {
  cudaStream_t str = s->stream;
  int hc[2] = {0, 0};
  cudaError_t e = cudaMemcpyAsync(&hc[0], st->d.count, 4, cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess && st->d.bcount)
    e = cudaMemcpyAsync(&hc[1], st->d.bcount, 4, cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess) e = cudaStreamSynchronize(str);
  if (e != cudaSuccess) return kd_cuda_fail(s, e, "carried batch");
  const long long carry = (long long)hc[0] + hc[1];
  if (carry == 0) {
    st->carry = false;
    st->pending = false;
    return kd_pipeline_ingest(s, st, nullptr, d_vals, nullptr, n, mode, timestamp, nullptr,
                              nullptr, nullptr);
  }
  const long long tot = carry + n;
  void* buf = nullptr;
  const size_t bytes = (size_t)tot * 16 + 64;
  if (cudaMalloc(&buf, bytes) != cudaSuccess) {
    cudaGetLastError();
    return sp_fail(s, KD_ENOMEM, "carried batch staging allocation failed");
  }
  unsigned long long* mm = (unsigned long long*)buf;
  double* ov = (double*)((char*)buf + 64);
  double* ow = ov + tot;
  const unsigned long long init[2] = {~0ull, 0ull};
  e = cudaMemcpyAsync(mm, init, 16, cudaMemcpyHostToDevice, str);
  if (e == cudaSuccess) {
    const int grid = (int)std::min<long long>((tot + 255) / 256, (long long)s->num_sms * 8);
    k_carry_build<<<grid, 256, 0, str>>>(st->d, d_vals, n, hc[0], hc[1], ov, ow, mm);
    e = cudaGetLastError();
  }
  int rc = e == cudaSuccess ? KD_OK : kd_cuda_fail(s, e, "carried batch");
  if (rc == KD_OK) {
    rc = kd_pipeline_ingest(s, st, nullptr, ov, ow, tot, mode, timestamp, nullptr, nullptr,
                            nullptr, carry, mm);
    if (rc == KD_OK) {
      st->carry = false;
      st->pending = false;
    }
  }
  cudaStreamSynchronize(str);
  cudaFree(buf);
  return rc;
}

// Frees the buffer and scratch of a store (their bytes are part of st->bytes,
// which the caller gives back to the session).
void kd_spath_free(KdSession*, KdStore* st) {
  KdStoreDev& d = st->d;
  if (d.bcount) {
    cudaFree(d.bcount);
    cudaFree(d.buf_m);
    cudaFree(d.buf_w);
  }
  d.bcount = nullptr;
  d.buf_m = nullptr;
  d.buf_w = nullptr;
  if (st->sp_scratch) cudaFree(st->sp_scratch);
  st->sp_scratch = nullptr;
  st->sp_scratch_bytes = 0;
}

extern "C" {

KD_API int kd_store_add(kd_store* h, const double* values, const double* weights,
                        const double* timestamps, int64_t n, int flags) {
  if (!h) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;
  if (n < 0 || (n > 0 && !values)) return sp_fail(s, KD_EINVAL, "values must be non-null");
  if (n == 0) return KD_OK;
  cudaSetDevice(s->device);
  int rc = sp_ensure(s, st);
  if (rc) return rc;
  const double* dv = values;
  const double* dw = weights;
  const double* dt = timestamps;
  void* tmp = nullptr;
  cudaStream_t str = s->stream;
  if (!(flags & KD_PTR_DEVICE)) {
    const size_t per = 8 * (1 + (weights ? 1 : 0) + (timestamps ? 1 : 0));
    if (cudaMalloc(&tmp, (size_t)n * per) != cudaSuccess) {
      cudaGetLastError();
      return sp_fail(s, KD_ENOMEM, "sample staging allocation failed");
    }
    double* p = (double*)tmp;
    cudaError_t e = cudaMemcpyAsync(p, values, (size_t)n * 8, cudaMemcpyHostToDevice, str);
    dv = p;
    p += n;
    if (weights && e == cudaSuccess) {
      e = cudaMemcpyAsync(p, weights, (size_t)n * 8, cudaMemcpyHostToDevice, str);
      dw = p;
      p += n;
    }
    if (timestamps && e == cudaSuccess) {
      e = cudaMemcpyAsync(p, timestamps, (size_t)n * 8, cudaMemcpyHostToDevice, str);
      dt = p;
    }
    if (e != cudaSuccess) {
      cudaStreamSynchronize(str);
      cudaFree(tmp);
      return kd_cuda_fail(s, e, "sample staging");
    }
  }
  SpStatus r{};
  rc = sp_run(s, st, SP_ADD, dv, dw, dt, n, nullptr, &r);
  if (tmp) cudaFree(tmp);
  if (rc) return rc;
  return sp_after(s, st, r);
}

KD_API int kd_store_flush(kd_store* h) {
  if (!h) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;
  return kd_spath_flush(s, st);
}

KD_API int kd_store_merge_into(kd_store* dst, kd_store* src) {
  if (!dst || !src || dst == src) return KD_EINVAL;
  KdStore* st = &dst->st;
  KdStore* so = &src->st;
  KdSession* s = st->sess;
  if (!s || !so->sess) return KD_EINVAL;
  if (so->sess->device != s->device)
    return sp_fail(s, KD_EINVAL, "merge_into needs both digests on one device");
  if (st->d.K != 1 || so->d.K != 1)
    return sp_fail(s, KD_EINVAL, "merge_into joins two one-digest stores");
  cudaSetDevice(s->device);
  int rc = sp_ensure(s, st);
  if (rc) return rc;
  if (so->sess != s) cudaStreamSynchronize(so->sess->stream);
  rc = kd_spath_flush(so->sess, so);  // other.merge()
  if (rc) return rc;
  SpStatus r{};
  rc = sp_run(s, st, SP_MERGE_INTO, nullptr, nullptr, nullptr, 0, so, &r);
  if (rc) return rc;
  if (!r.noop && so->d.lambda > 0.0) so->carry = true;
  return sp_after(s, st, r);
}

}  // extern "C"
