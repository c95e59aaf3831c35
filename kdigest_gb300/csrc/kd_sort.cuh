// kd_sort.cuh — stable LSD radix sort of (order key u64, digest key u32[, index u32]).
//
// Restates the ordering of gpu/sort.mojo (stable sort by mean, ties by original
// index, _before at :38-41) for many digests at once: the composite key is
// (digest key, order-preserving u64 of the FP64 value).  LSD passes over 8-bit
// digits are stable, so elements with equal (key, value) keep their input order,
// which is exactly the reference's index tie-break.
//
// One histogram pass computes the digit counts of every pass (they do not
// depend on the order of the elements).  Each pass is then one kernel: a block
// takes the next tile through an atomic ticket, ranks its elements stably with
// warp __match_any_sync, publishes its per-digit counts, obtains the counts of
// all preceding tiles by decoupled look-back, stages the tile in shared memory
// in digit order and writes it out in coalesced runs.  Look-back waits are
// bounded: a block that gives up publishes what it has (its scatter stays
// inside [0, n), since a partial prefix is never larger than the true one),
// raises KD_ETIMEOUT, and the batch is not committed.
#pragma once

#include "kd_scan.cuh"

#ifndef KD_RS_THREADS
#define KD_RS_THREADS 256
#endif
#ifndef KD_RS_MIN_BLOCKS
#define KD_RS_MIN_BLOCKS 3
#endif
#define KD_RS_WARPS (KD_RS_THREADS / 32)
// One thread per digit in the per-digit stages (scan, look-back, scatter table).
static_assert(KD_RS_THREADS >= 256 && KD_RS_THREADS % 32 == 0, "a radix block needs a thread per digit");
#ifndef KD_RS_PER_WARP
#define KD_RS_PER_WARP 512
#endif
#define KD_RS_ROUNDS (KD_RS_PER_WARP / 32)
#define KD_RS_TILE (KD_RS_WARPS * KD_RS_PER_WARP)
#define KD_RS_MAXPASS 12
#define KD_RS_SPIN_LIMIT (1 << 22)

// Look-back words: [63:34] epoch, [33:32] status (1 aggregate, 2 inclusive),
// [31:0] count (counts never exceed n < 2^31).  The epoch of pass p of a sort is
// (device epoch base) + p: the histogram kernel advances the base by
// KD_RS_EPOCH_STRIDE per sort, so a replayed CUDA graph gets fresh epochs too,
// and words left by earlier sorts never read as ready.
#define KD_LB_AGG 1ull
#define KD_LB_INC 2ull
#define KD_RS_EPOCH_STRIDE 16u
#define KD_RS_EPOCH_LIMIT ((1u << 30) - 2u * KD_RS_EPOCH_STRIDE)
__device__ __forceinline__ unsigned long long lb_pack(unsigned epoch, unsigned long long st,
                                                      unsigned long long cnt) {
  return ((unsigned long long)epoch << 34) | (st << 32) | cnt;
}

static __global__ void __launch_bounds__(KD_RS_THREADS) kd_rs_hist_all(
    const uint64_t* __restrict__ k64, const uint32_t* __restrict__ key, long long n,
    int key_passes, int first_digit, unsigned* __restrict__ ghist, unsigned* __restrict__ epoch_base) {
  __shared__ unsigned h[KD_RS_MAXPASS][256];
  if (blockIdx.x == 0 && threadIdx.x == 0) *epoch_base += KD_RS_EPOCH_STRIDE;
  for (int t = threadIdx.x; t < KD_RS_MAXPASS * 256; t += KD_RS_THREADS) (&h[0][0])[t] = 0;
  __syncthreads();
  for (long long i = (long long)blockIdx.x * KD_RS_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * KD_RS_THREADS) {
    const uint64_t v = k64[i];
    for (int p = first_digit; p < 8; ++p) atomicAdd(&h[p][(unsigned)(v >> (8 * p)) & 255u], 1u);
    if (key_passes > 0) {  // the packed form carries no key digits: skip the read
      const uint32_t kk = key[i];
      for (int p = 0; p < key_passes; ++p) atomicAdd(&h[8 + p][(kk >> (8 * p)) & 255u], 1u);
    }
  }
  __syncthreads();
  const int used = (8 + key_passes) * 256;
  for (int t = threadIdx.x; t < used; t += KD_RS_THREADS) {
    const unsigned c = (&h[0][0])[t];
    if (c) atomicAdd(&ghist[t], c);
  }
}

struct KdRsPass {
  const uint64_t* kin;
  const uint32_t* keyin;
  const uint32_t* idxin;
  uint64_t* kout;
  uint32_t* keyout;
  uint32_t* idxout;
  long long n;
  int shift;
  int from_key;
  const unsigned* ghist;  // 256 digit counts of this pass
  unsigned long long* state;
  unsigned long long* ticket;
  unsigned long long ticket_base;
  const unsigned* epoch_base;  // device epoch base of this sort
  int pass;                    // epoch = *epoch_base + pass
  int* err_code;  // device status word (KdErr.code)
  long long spin_limit;  // polls of a look-back wait before it gives up
  int stall_first;       // tests only: tile 0 never publishes (its successor's wait runs out)
};

// Predecessor words read per look-back round trip (GB300: 2 to 8 measure
// alike, 16 and above cost more L2 traffic than they save round trips).
#ifndef KD_LB_WINDOW
#define KD_LB_WINDOW 4
#endif
// Pause before polling again when no predecessor word was ready (0: none);
// with the bounded poll count this caps a look-back wait near one second.
#ifndef KD_LB_BACKOFF_NS
#define KD_LB_BACKOFF_NS 256
#endif

template <bool kIdx>
__global__ void __launch_bounds__(KD_RS_THREADS, KD_RS_MIN_BLOCKS) kd_rs_onesweep(KdRsPass a) {
  extern __shared__ __align__(16) unsigned char rs_smem[];
  uint64_t* sk = reinterpret_cast<uint64_t*>(rs_smem);
  uint32_t* skey = reinterpret_cast<uint32_t*>(sk + KD_RS_TILE);
  uint32_t* sidx = skey + KD_RS_TILE;
  __shared__ unsigned wcnt[KD_RS_WARPS][256];
  __shared__ unsigned blk_off[256];
  __shared__ long long gpos[256];
  __shared__ int4 scan_tmp[32];
  __shared__ int bid_s;
  if (threadIdx.x == 0) bid_s = (int)(atomicAdd(a.ticket, 1ull) - a.ticket_base);
  for (int t = threadIdx.x; t < KD_RS_WARPS * 256; t += KD_RS_THREADS) (&wcnt[0][0])[t] = 0;
  __syncthreads();
  const int b = bid_s;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long tile0 = (long long)b * KD_RS_TILE;
  const long long base = tile0 + (long long)warp * KD_RS_PER_WARP;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int shift = a.shift;
  const unsigned epoch = *a.epoch_base + (unsigned)a.pass;
  // 1. stable rank of every element among the warp's elements of its digit;
  //    ranks (< 512) are packed two per register
  unsigned rank2[KD_RS_ROUNDS / 2];
  unsigned char dig[KD_RS_ROUNDS];
  unsigned dv[KD_RS_ROUNDS];
  // all loads of the thread first, so their latency is exposed once
#pragma unroll
  for (int r = 0; r < KD_RS_ROUNDS; ++r) {
    const long long i = base + r * 32 + lane;
    dv[r] = 256u;
    if (i < a.n) dv[r] = a.from_key ? (a.keyin[i] >> shift) & 255u : (unsigned)(a.kin[i] >> shift) & 255u;
  }
#pragma unroll
  for (int r = 0; r < KD_RS_ROUNDS; ++r) {
    const unsigned d = dv[r];
    const bool valid = d < 256u;
    dig[r] = (unsigned char)(d & 255u);
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned before = peers & lt_mask;
    const unsigned c = valid ? wcnt[warp][d] : 0u;
    __syncwarp();
    if (valid && before == 0) wcnt[warp][d] = c + __popc(peers);
    __syncwarp();
    const unsigned rk = c + __popc(before);
    if (r & 1) rank2[r >> 1] |= rk << 16;
    else rank2[r >> 1] = rk;
  }
  __syncthreads();

  // 2. per digit: exclusive prefix over warps, tile count, tile offset
  unsigned cnt_d = 0;
  if (threadIdx.x < 256) {
    unsigned s = 0;
#pragma unroll
    for (int w = 0; w < KD_RS_WARPS; ++w) {
      const unsigned v = wcnt[w][threadIdx.x];
      wcnt[w][threadIdx.x] = s;
      s += v;
    }
    cnt_d = s;
  }
  unsigned gbase = 0;
  {
    int4 tot;
    const unsigned g = threadIdx.x < 256 ? a.ghist[threadIdx.x] : 0u;
    const int4 inc = block_scan_incl(make_int4((int)cnt_d, (int)g, 0, 0), scan_tmp, &tot);
    if (threadIdx.x < 256) {
      const unsigned off = (unsigned)(inc.x - (int)cnt_d);
      blk_off[threadIdx.x] = off;
      gbase = (unsigned)(inc.y - (int)g);
      // the staging position of a warp's digit-d run: tile offset + warp prefix
#pragma unroll
      for (int w = 0; w < KD_RS_WARPS; ++w) wcnt[w][threadIdx.x] += off;
    }
  }
  // 3. decoupled look-back, one thread per digit, KD_LB_WINDOW predecessors per
  //    round trip (independent loads), bounded waits
  if (threadIdx.x < 256) {
    const int d = threadIdx.x;
    volatile unsigned long long* st = a.state;
    unsigned long long excl = 0;
    if (b == 0) {
      if (!a.stall_first) st[d] = lb_pack(epoch, KD_LB_INC, cnt_d);
    } else {
      st[(size_t)b * 256 + d] = lb_pack(epoch, KD_LB_AGG, cnt_d);
      long long hi = b - 1;  // next predecessor to account for
      long long spins = 0;
      bool done = false, timed_out = false;
      while (!done) {
        unsigned long long v[KD_LB_WINDOW];
#pragma unroll
        for (int k = 0; k < KD_LB_WINDOW; ++k)
          v[k] = hi - k >= 0 ? st[(size_t)(hi - k) * 256 + d] : lb_pack(epoch, KD_LB_INC, 0);
        // consume the window from hi downwards up to the first not-ready word
        int k = 0;
        for (; k < KD_LB_WINDOW; ++k) {
          const unsigned long long w = v[k];
          const bool ready = (unsigned)(w >> 34) == epoch && ((w >> 32) & 3ull) != 0ull;
          if (!ready) break;
          excl += w & 0xffffffffull;
          if (((w >> 32) & 3ull) == KD_LB_INC) {
            done = true;
            break;
          }
        }
        if (done) break;
        hi -= k;
        if (k == 0 && ++spins > a.spin_limit) {
          timed_out = true;
          break;
        }
#if KD_LB_BACKOFF_NS > 0
        if (k == 0) __nanosleep(KD_LB_BACKOFF_NS);
#endif
      }
      if (timed_out) atomicCAS(a.err_code, 0, KD_ETIMEOUT);
      st[(size_t)b * 256 + d] = lb_pack(epoch, KD_LB_INC, excl + cnt_d);
    }
    // staged position i of digit d goes to gpos[d] + i
    gpos[d] = (long long)gbase + (long long)excl - (long long)blk_off[d];
  }
  __syncthreads();
  // 4. stage in digit order (the tile is re-read from L1/L2)
#pragma unroll
  for (int r = 0; r < KD_RS_ROUNDS; ++r) {
    const long long i = base + r * 32 + lane;
    if (i < a.n) {
      const unsigned d = dig[r];
      const unsigned rk = (rank2[r >> 1] >> ((r & 1) * 16)) & 0xffffu;
      const unsigned lp = wcnt[warp][d] + rk;
      const uint64_t kvv = a.kin[i];
      const uint32_t kkv = a.keyin[i];
      sk[lp] = kvv;
      skey[lp] = kkv;
      if (kIdx) sidx[lp] = a.idxin[i];
    }
  }
  __syncthreads();
  // 5. coalesced write-out of digit runs
  const int cnt = (int)min((long long)KD_RS_TILE, a.n - tile0);
  for (int i = threadIdx.x; i < cnt; i += KD_RS_THREADS) {
    const uint64_t v = sk[i];
    const uint32_t k2 = skey[i];
    const unsigned d = a.from_key ? (k2 >> shift) & 255u : (unsigned)(v >> shift) & 255u;
    const long long pos = gpos[d] + i;
    a.kout[pos] = v;
    a.keyout[pos] = k2;
    if (kIdx) a.idxout[pos] = sidx[i];
  }
}

struct KdSortBufs {
  uint64_t* k64[2];
  uint32_t* key[2];
  uint32_t* idx[2];               // may be null
  unsigned* ghist;                // KD_RS_MAXPASS * 256
  unsigned long long* state;      // 256 per tile
  unsigned long long* ticket;     // device ticket counter (reset per sort)
  unsigned* epoch_base;           // device epoch base, advanced by every sort
  unsigned long long* epochs_used;  // host: epochs consumed since the last clear
  long long state_tiles;          // tiles the look-back array holds
  int* err_code;
  long long spin_limit = KD_RS_SPIN_LIMIT;
  int stall_first = 0;            // tests only (KdRsPass::stall_first)
};

static inline int kd_rs_blocks(long long n) { return (int)((n + KD_RS_TILE - 1) / KD_RS_TILE); }
static inline size_t kd_rs_smem(bool with_idx) {
  return (size_t)KD_RS_TILE * (8 + 4 + (with_idx ? 4 : 0));
}

// Host bookkeeping, once before every sort is enqueued or replayed: when the
// epoch field would wrap, the look-back words and the base are cleared first.
static inline void kd_rs_epoch_reserve(KdSortBufs& b, cudaStream_t st) {
  if (*b.epochs_used + KD_RS_EPOCH_STRIDE >= KD_RS_EPOCH_LIMIT) {
    cudaMemsetAsync(b.state, 0, sizeof(unsigned long long) * 256 * (size_t)b.state_tiles, st);
    cudaMemsetAsync(b.epoch_base, 0, sizeof(unsigned), st);
    *b.epochs_used = 0;
  }
  *b.epochs_used += KD_RS_EPOCH_STRIDE;
}

// Sorts by (key, k64); returns the index (0/1) of the buffer set holding the
// result.  Enqueues device work only (no host state), so it can be captured.
static inline int kd_radix_sort(KdSortBufs& b, long long n, int key_bits, bool with_idx,
                                int num_sms, cudaStream_t st, int first_digit = 0) {
  int src = 0;
  if (n <= 1) return src;
  const int nb = kd_rs_blocks(n);
  const int key_passes = (key_bits + 7) / 8;
  cudaMemsetAsync(b.ghist, 0, sizeof(unsigned) * KD_RS_MAXPASS * 256, st);
  cudaMemsetAsync(b.ticket, 0, sizeof(unsigned long long), st);
  unsigned long long ticket_base = 0;
  kd_rs_hist_all<<<num_sms * 8, KD_RS_THREADS, 0, st>>>(b.k64[0], b.key[0], n, key_passes,
                                                        first_digit, b.ghist, b.epoch_base);
  auto pass = [&](int shift, int from_key, int pidx) {
    const int dst = src ^ 1;
    KdRsPass a{b.k64[src], b.key[src], b.idx[src], b.k64[dst], b.key[dst], b.idx[dst], n, shift,
               from_key, b.ghist + pidx * 256, b.state, b.ticket, ticket_base, b.epoch_base, pidx,
               b.err_code, b.spin_limit, b.stall_first};
    if (with_idx)
      kd_rs_onesweep<true><<<nb, KD_RS_THREADS, kd_rs_smem(true), st>>>(a);
    else
      kd_rs_onesweep<false><<<nb, KD_RS_THREADS, kd_rs_smem(false), st>>>(a);
    ticket_base += (unsigned long long)nb;
    src = dst;
  };
  for (int p = first_digit; p < 8; ++p) pass(8 * p, 0, p);  // digits below first_digit unsorted
  for (int p = 0; p < key_passes; ++p) pass(8 * p, 1, 8 + p);
  return src;
}

// The buffer set kd_radix_sort leaves its result in (0/1), without sorting.
static inline int kd_radix_sort_result(long long n, int key_bits, int first_digit = 0) {
  if (n <= 1) return 0;
  return ((8 - first_digit) + (key_bits + 7) / 8) & 1;
}

static inline int kd_radix_sort_launches(long long n, int key_bits, int first_digit = 0) {
  return n > 1 ? 1 + (8 - first_digit) + (key_bits + 7) / 8 : 0;
}
