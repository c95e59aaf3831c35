// kd_pipeline.cu — the GB300 P-path: batched ingest, hierarchical tile compress,
// commit, quantile/cdf queries and batched merges over resident per-key digests.
//
// One ingest (grouped add_batch, grouped.mojo:60-162 with gpu/grouped.mojo:415-643
// semantics per key) runs entirely on the device:
//   prep     validate (key range, finite values) and map values to order keys
//   sort     stable LSD radix sort by (key, value)            (gpu/sort.mojo)
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
#include <cstdio>
#include <cstring>
#include <vector>

#include "kd_engine.h"
#include "kd_internal.cuh"
#include "kd_scan.cuh"
#include "kd_sort.cuh"

#define KD_ERANGE_SCRATCH 100  // internal: intermediate scratch too small (index = needed)

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
// Warp tile compress (canonical association order; see oracle/kd_oracle.c)
// ---------------------------------------------------------------------------
struct WarpTile {
  double x[KD_SMEM_SLOTS];
  double w[KD_SMEM_SLOTS];
  double L[KD_SMEM_SLOTS];  // in-chunk inclusive prefix of w
  unsigned char f[KD_SMEM_SLOTS];  // bit0 head, bit1 end
};

__device__ __forceinline__ void emit_centroid(double* om, double* ow, int slot, double sw,
                                              double swx, double lo_v, double hi_v) {
  double mean = sw > 0.0 ? KD_DIV(swx, sw) : 0.0;
  mean = mean < lo_v ? lo_v : mean;
  mean = mean > hi_v ? hi_v : mean;
  om[slot] = mean;
  ow[slot] = sw;
}

// Compresses the n (<= 1024) staged elements of `t`; lane c owns elements
// [c*E, c*E+E) stored at t.*[c*SE + j].  The loader has filled x, w and L.
// Returns the number of centroids written to om/ow[0..).
__device__ int warp_compress(WarpTile& t, int n, int scale, double compression, int force_exact,
                             double* __restrict__ om, double* __restrict__ ow) {
  const int lane = threadIdx.x & 31;
  const int E = (n + 31) >> 5;
  const int SE = E | 1;
  const int lo = lane * E;
  const int cnt = max(0, min(E, n - lo));
  const int sb = lane * SE;

  // Chunk totals -> Kogge-Stone over lanes -> exclusive lane prefix P.
  double S = cnt > 0 ? t.L[sb + cnt - 1] : 0.0;
  double I = S;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    double v = shfl_up_d(I, o);
    if (lane >= o) I = KD_ADD(I, v);
  }
  double P = shfl_up_d(I, 1);
  const int cl = (n - 1) / E;  // lane holding the last element
  double last_cum = 0.0;
  if (cnt > 0) last_cum = lane == 0 ? t.L[sb + cnt - 1] : KD_ADD(P, t.L[sb + cnt - 1]);
  double tot = shfl_d(last_cum, cl);
  if (!(tot > 0.0)) tot = 1.0;
  const KFilterTile ft = kfilter_tile(scale, compression, tot);

  // Bucket ids and head / end flags.
  int32_t prev_id = 0, first_id = 0;
  int nend = 0;
  double nrm64 = 0.0;
  bool have_nrm = false;
  for (int j = 0; j < E; ++j) {
    const bool act = j < cnt;
    double cum = 0.0;
    int32_t id = 0;
    bool ok = true;
    if (act) {
      cum = lane == 0 ? t.L[sb + j] : KD_ADD(P, t.L[sb + j]);
      ok = !force_exact && kfilter_id(scale, ft, cum, tot, &id);
    }
    const bool need = act && !ok;
    if (__any_sync(0xffffffffu, need)) {
      if (!have_nrm) {
        nrm64 = kd_normalizer(scale, compression, tot);
        have_nrm = true;
      }
      if (need) id = kd_bucket(scale, cum, tot, nrm64);
    }
    if (act) {
      unsigned char h = 0;
      if (j > 0 && id != prev_id) {
        h = 1;
        t.f[sb + j - 1] |= 2;
        ++nend;
      }
      t.f[sb + j] = h;
      if (j == 0) first_id = id;
      prev_id = id;
    }
  }
  const int32_t left_last = __shfl_up_sync(0xffffffffu, prev_id, 1);
  const int32_t right_first = __shfl_down_sync(0xffffffffu, first_id, 1);
  if (cnt > 0) {
    if (lane == 0 || first_id != left_last) t.f[sb] |= 1;
    if (lo + cnt == n || right_first != prev_id) {
      t.f[sb + cnt - 1] |= 2;
      ++nend;
    }
  }
  __syncwarp();

  // Output slots: exclusive prefix of segment ends over lanes.
  int incl_e = nend;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(0xffffffffu, incl_e, o);
    if (lane >= o) incl_e += v;
  }
  int slot = incl_e - nend;
  const int total_out = __shfl_sync(0xffffffffu, incl_e, 31);

  // Segment sums: serial pieces inside the chunk.
  double aw = 0.0, awx = 0.0, head_x = 0.0;
  bool head_seen = false;
  int last_head = -1;
  bool pend = false;
  double pend_w = 0.0, pend_wx = 0.0, pend_x = 0.0;
  int pend_slot = 0;
  for (int j = 0; j < cnt; ++j) {
    const unsigned char f = t.f[sb + j];
    const double wi = t.w[sb + j], xi = t.x[sb + j];
    const double wx = KD_MUL(wi, xi);
    if ((f & 1) || j == 0) {
      aw = wi;
      awx = wx;
    } else {
      aw = KD_ADD(aw, wi);
      awx = KD_ADD(awx, wx);
    }
    if (f & 1) {
      head_seen = true;
      head_x = xi;
      last_head = lo + j;
    }
    if (f & 2) {
      if (head_seen) {
        emit_centroid(om, ow, slot, aw, awx, head_x, xi);
      } else {
        pend = true;
        pend_w = aw;
        pend_wx = awx;
        pend_x = xi;
        pend_slot = slot;
      }
      ++slot;
    }
  }
  // Segmented Kogge-Stone of the trailing pieces carries sums across lanes.
  double Vw = aw, Vwx = awx;
  int F = head_seen ? 1 : 0;
  int hp = last_head;  // inclusive max-scan of head positions
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    double tw = shfl_up_d(Vw, o), twx = shfl_up_d(Vwx, o);
    int tf = __shfl_up_sync(0xffffffffu, F, o);
    int th = __shfl_up_sync(0xffffffffu, hp, o);
    if (lane >= o) {
      if (!F) {
        Vw = KD_ADD(Vw, tw);
        Vwx = KD_ADD(Vwx, twx);
      }
      F |= tf;
      hp = max(hp, th);
    }
  }
  const double cw = shfl_up_d(Vw, 1), cwx = shfl_up_d(Vwx, 1);
  const int hprev = __shfl_up_sync(0xffffffffu, hp, 1);
  if (pend) {
    const int hq = max(hprev, 0);
    const int hl = hq / E;
    const double hx = t.x[hl * SE + (hq - hl * E)];
    emit_centroid(om, ow, pend_slot, KD_ADD(cw, pend_w), KD_ADD(cwx, pend_wx), hx, pend_x);
  }
  __syncwarp();
  return total_out;
}

// ---------------------------------------------------------------------------
// Stage kernels
// ---------------------------------------------------------------------------
__global__ void k_prep(long long n, const uint32_t* __restrict__ keys, const double* __restrict__ vals,
                       const double* __restrict__ wts, long long K, uint64_t* __restrict__ k64,
                       uint32_t* __restrict__ kout, uint32_t* __restrict__ idx, KdErrHost* err) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const uint32_t key = keys ? keys[i] : 0u;
    const double v = vals[i];
    bool bad = (long long)key >= K || !kd_isfinite(v);
    if (wts) {
      const double w = wts[i];
      bad = bad || !(w > 0.0) || !kd_isfinite(w);
    }
    if (bad) {
      atomicMin((unsigned long long*)&err->index, (unsigned long long)i);
      atomicCAS(&err->code, 0, KD_EINVAL);
    }
    k64[i] = kd_order_key(v);
    kout[i] = key;
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
  long long cap;
  __device__ void operator()(long long i, int4 excl, int4 v) const {
    if (v.x && excl.x < cap) {
      tkey[excl.x] = key[i];
      tstart[excl.x] = (int)i;
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
  double timestamp;
  const double* merge_min;
  const double* merge_max;
  const double* merge_clock;
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
__global__ void k_prepare(PrepareArgs a) {
  const int U = a.totals[0].x;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= U || kd_err_get(a.err)) return;
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
  const double vmin = kd_from_order_key(a.k64[start]);
  const double vmax = kd_from_order_key(a.k64[end - 1]);
  if (a.mode == KD_MODE_REPLACE || a.mode == KD_MODE_MERGE) {
    prior = 0;
    ls = 0.0;
    if (a.mode == KD_MODE_MERGE) {
      mn = a.merge_min[key];
      mx = a.merge_max[key];
      clock = a.merge_clock[key];
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
      new_clock = KD_ADD(clock, (double)nn);
      advance = true;
    } else if (a.timestamp > clock) {
      new_clock = a.timestamp;
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
    const double added = KD_MUL((double)nn, sf);
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

struct Plan0Src {
  const int4* totals;
  const int* tm;
  __device__ int4 operator()(long long j) const {
    if (j >= totals[0].x) return make_int4(0, 0, 0, 0);
    const int m = tm[j];
    const int tiles = (m + KD_TILE - 1) / KD_TILE;
    const bool fin = tiles <= 1;
    return make_int4(tiles, fin ? 0 : tiles, fin ? 0 : 1, 0);
  }
};
struct Plan0Dst {
  const int4* totals;
  const int* tm;
  int* ttile_off;
  int* tinter_off;
  int* ttiles;
  KdLevelDev nxt;
  __device__ void operator()(long long j, int4 excl, int4 v) const {
    if (j >= totals[0].x) return;
    ttile_off[j] = excl.x;
    tinter_off[j] = excl.y;
    ttiles[j] = v.x;
    if (v.z) {
      nxt.j[excl.z] = (int)j;
      nxt.src_base[excl.z] = excl.y;
      nxt.src_tiles[excl.z] = v.x;
      nxt.mprev[excl.z] = tm[j];
    }
  }
};

struct L0Args {
  KdStoreDev s;
  long long n;
  const uint64_t* k64;
  const uint32_t* idx;
  const double* wts;
  const uint32_t* tkey;
  const int* tstart;
  const int* tm;
  const int* tprior;
  const unsigned char* tbuf;
  const double* tsf;
  const double* tpscale;
  const int* ttile_off;
  const int* ttiles;
  const int* tinter_off;
  const int4* totals;
  double* scr_m;
  double* scr_w;
  int* tcount;
  int* st_count;
  long long cap_inter;
  int force_exact;
  KdErrHost* err;
};

// Level 0: merge-path load of (prior centroids ++ new samples) fused with the
// tile compress.  Priors precede new samples on ties (their indices are lower).
__global__ void __launch_bounds__(32 * KD_WARPS_PER_BLOCK) k_level0(L0Args a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpTile& t = reinterpret_cast<WarpTile*>(smem_raw)[threadIdx.x >> 5];
  if (kd_err_get(a.err)) return;
  const int U = a.totals[0].x;
  const int T0 = a.totals[1].x;
  const int I0 = a.totals[1].y;
  if (I0 > a.cap_inter) {
    if (blockIdx.x == 0 && threadIdx.x == 0) kd_err_set(a.err, KD_ERANGE_SCRATCH, I0);
    return;
  }
  const int lane = threadIdx.x & 31;
  const KdStoreDev& s = a.s;
  for (int w = blockIdx.x * KD_WARPS_PER_BLOCK + (threadIdx.x >> 5); w < T0;
       w += gridDim.x * KD_WARPS_PER_BLOCK) {
    int lo = 0, hi = U - 1;  // last j with ttile_off[j] <= w
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (a.ttile_off[mid] <= w) lo = mid;
      else hi = mid - 1;
    }
    const int j = lo;
    const int lt = w - a.ttile_off[j];
    const int m = a.tm[j];
    const int tstart_m = lt * KD_TILE;
    const int n = min(KD_TILE, m - tstart_m);
    const uint32_t key = a.tkey[j];
    const int np = a.tprior[j];
    const int backb = a.tbuf[j];
    const double* pm = s.slot_m + slot_base(s.K, backb ^ 1, key);
    const double* pw = s.slot_w + slot_base(s.K, backb ^ 1, key);
    const double pscale = a.tpscale[j];
    const bool rescale = pscale != 1.0;
    const int ns = a.tstart[j];
    const int nn = (j + 1 < U ? a.tstart[j + 1] : (int)a.n) - ns;
    const uint64_t* nk = a.k64 + ns;
    const double sf = a.tsf[j];

    // Lane chunk [lo_e, lo_e + cnt) of merged positions.
    const int E = (n + 31) >> 5, SE = E | 1;
    const int lo_e = lane * E;
    const int cnt = max(0, min(E, n - lo_e));
    const int sb = lane * SE;
    if (cnt > 0) {
      const int d0 = tstart_m + lo_e;
      int ilo = max(0, d0 - nn), ihi = min(d0, np);
      while (ilo < ihi) {
        int mid = (ilo + ihi) >> 1;
        if (canon(pm[mid]) <= kd_from_order_key(nk[d0 - mid - 1])) ilo = mid + 1;
        else ihi = mid;
      }
      int i = ilo, jn = d0 - ilo;
      double acc = 0.0;
      for (int c = 0; c < cnt; ++c) {
        double xv, wv;
        bool take_prior = i < np;
        if (take_prior && jn < nn) take_prior = canon(pm[i]) <= kd_from_order_key(nk[jn]);
        if (take_prior) {
          xv = canon(pm[i]);
          wv = rescale ? KD_MUL(pw[i], pscale) : pw[i];
          ++i;
        } else {
          xv = kd_from_order_key(nk[jn]);
          wv = a.wts ? a.wts[a.idx[ns + jn]] : sf;
          ++jn;
        }
        acc = c == 0 ? wv : KD_ADD(acc, wv);
        t.x[sb + c] = xv;
        t.w[sb + c] = wv;
        t.L[sb + c] = acc;
      }
    }
    __syncwarp();
    const bool fin = a.ttiles[j] == 1;
    double* om;
    double* ow;
    if (fin) {
      om = s.slot_m + slot_base(s.K, backb, key);
      ow = s.slot_w + slot_base(s.K, backb, key);
    } else {
      const size_t base = (size_t)(a.tinter_off[j] + lt) * KD_TILE;
      om = a.scr_m + base;
      ow = a.scr_w + base;
    }
    const int c = warp_compress(t, n, s.scale, s.compression, a.force_exact, om, ow);
    if (lane == 0) {
      if (fin) a.st_count[j] = c;
      else a.tcount[a.tinter_off[j] + lt] = c;
    }
  }
}

struct PlanArgs {
  KdLevelDev cur;
  KdLevelDev nxt;
  const int* prev_count;
  int* prev_doff;
  const uint32_t* tkey;
  long long cap_inter;
  long long cap_keys;
  KdErrHost* err;
};

// Levels >= 1: per active key, dense offsets of its previous-level survivors
// (the reference's _scan_counts_kernel, add_batch.mojo:407-452) and the new
// tiling; keys still above one tile move on to the next level.
__global__ void __launch_bounds__(1024) k_plan(PlanArgs p) {
  __shared__ int4 sw[32];
  const int A = *p.cur.A;
  if (A == 0 || kd_err_get(p.err)) {
    if (threadIdx.x == 0) {
      *p.cur.T = 0;
      *p.cur.I = 0;
      *p.nxt.A = 0;
    }
    return;
  }
  const int per = (A + blockDim.x - 1) / blockDim.x;
  const int a0 = min(A, (int)threadIdx.x * per), a1 = min(A, a0 + per);
  int4 acc = make_int4(0, 0, 0, 0);
  for (int a = a0; a < a1; ++a) {
    int run = 0;
    const int sbase = p.cur.src_base[a], sn = p.cur.src_tiles[a];
    for (int s = sbase; s < sbase + sn; ++s) {
      p.prev_doff[s] = run;
      run += p.prev_count[s];
    }
    p.cur.m[a] = run;
    if (run >= p.cur.mprev[a]) kd_err_set(p.err, KD_ECONVERGE, (long long)p.tkey[p.cur.j[a]]);
    const int tiles = (run + KD_TILE - 1) / KD_TILE;
    const bool fin = tiles <= 1;
    acc = i4add(acc, make_int4(tiles, fin ? 0 : tiles, fin ? 0 : 1, 0));
  }
  int4 tot;
  int4 incl = block_scan_incl(acc, sw, &tot);
  int4 run = make_int4(incl.x - acc.x, incl.y - acc.y, incl.z - acc.z, 0);
  for (int a = a0; a < a1; ++a) {
    const int m = p.cur.m[a];
    const int tiles = (m + KD_TILE - 1) / KD_TILE;
    const bool fin = tiles <= 1;
    p.cur.tile_off[a] = run.x;
    p.cur.inter_off[a] = run.y;
    if (!fin) {
      p.nxt.j[run.z] = p.cur.j[a];
      p.nxt.src_base[run.z] = run.y;
      p.nxt.src_tiles[run.z] = tiles;
      p.nxt.mprev[run.z] = m;
    }
    run = i4add(run, make_int4(tiles, fin ? 0 : tiles, fin ? 0 : 1, 0));
  }
  if (threadIdx.x == 0) {
    *p.cur.T = tot.x;
    *p.cur.I = tot.y;
    *p.nxt.A = tot.z;
    if (tot.y > p.cap_inter) kd_err_set(p.err, KD_ERANGE_SCRATCH, tot.y);
  }
}

struct LLArgs {
  KdStoreDev s;
  KdLevelDev cur;
  const uint32_t* tkey;
  const unsigned char* tbuf;
  int* st_count;
  const double* src_m;
  const double* src_w;
  const int* src_count;
  const int* src_doff;
  double* dst_m;
  double* dst_w;
  int* dst_count;
  int force_exact;
  KdErrHost* err;
};

// Levels >= 1: dense load of the previous level's survivors (the gather of
// _gather_tiles_kernel, add_batch.mojo:455-478, fused into the load).
__global__ void __launch_bounds__(32 * KD_WARPS_PER_BLOCK) k_level(LLArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpTile& t = reinterpret_cast<WarpTile*>(smem_raw)[threadIdx.x >> 5];
  if (kd_err_get(a.err)) return;
  const int A = *a.cur.A;
  const int T = *a.cur.T;
  const int lane = threadIdx.x & 31;
  const KdStoreDev& s = a.s;
  for (int w = blockIdx.x * KD_WARPS_PER_BLOCK + (threadIdx.x >> 5); w < T;
       w += gridDim.x * KD_WARPS_PER_BLOCK) {
    int lo = 0, hi = A - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (a.cur.tile_off[mid] <= w) lo = mid;
      else hi = mid - 1;
    }
    const int ai = lo;
    const int lt = w - a.cur.tile_off[ai];
    const int m = a.cur.m[ai];
    const int dstart = lt * KD_TILE;
    const int n = min(KD_TILE, m - dstart);
    const int j = a.cur.j[ai];
    const uint32_t key = a.tkey[j];
    const int sbase = a.cur.src_base[ai], sn = a.cur.src_tiles[ai];
    const int E = (n + 31) >> 5, SE = E | 1;
    const int lo_e = lane * E;
    const int cnt = max(0, min(E, n - lo_e));
    const int sb = lane * SE;
    if (cnt > 0) {
      const int d0 = dstart + lo_e;
      int l2 = sbase, h2 = sbase + sn - 1;  // last source tile with doff <= d0
      while (l2 < h2) {
        int mid = (l2 + h2 + 1) >> 1;
        if (a.src_doff[mid] <= d0) l2 = mid;
        else h2 = mid - 1;
      }
      int sidx = l2;
      int r = d0 - a.src_doff[sidx];
      double acc = 0.0;
      const int send = sbase + sn;
      for (int c = 0; c < cnt; ++c) {
        while (r >= a.src_count[sidx] && sidx + 1 < send) {
          ++sidx;
          r = 0;
        }
        if (r >= a.src_count[sidx]) {  // inconsistent counts: never read past the key's tiles
          kd_err_set(a.err, KD_ECONVERGE, -2);
          break;
        }
        const size_t off = (size_t)sidx * KD_TILE + r;
        const double xv = a.src_m[off], wv = a.src_w[off];
        ++r;
        acc = c == 0 ? wv : KD_ADD(acc, wv);
        t.x[sb + c] = xv;
        t.w[sb + c] = wv;
        t.L[sb + c] = acc;
      }
    }
    __syncwarp();
    const bool fin = m <= KD_TILE;
    double* om;
    double* ow;
    const int backb = a.tbuf[j];
    if (fin) {
      om = s.slot_m + slot_base(s.K, backb, key);
      ow = s.slot_w + slot_base(s.K, backb, key);
    } else {
      const size_t base = (size_t)(a.cur.inter_off[ai] + lt) * KD_TILE;
      om = a.dst_m + base;
      ow = a.dst_w + base;
    }
    const int c = warp_compress(t, n, s.scale, s.compression, a.force_exact, om, ow);
    if (lane == 0) {
      if (fin) a.st_count[j] = c;
      else a.dst_count[a.cur.inter_off[ai] + lt] = c;
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
};

// _gpu_batch_finish (tdigest.mojo:298-315) + _prune (:441-458) per key, the
// quantile-walk prefix (:526-536), then publication of the new slot.
// One lane per key keeps every lane of a warp on useful FP64 work.
__global__ void k_commit(CommitArgs a) {
  const int U = a.totals[0].x;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j == 0 && *a.remaining > 0) kd_err_set(a.err, KD_ECONVERGE, -1);
  if (j >= U) return;
  if (kd_err_get(a.err) || *a.remaining > 0) return;
  const KdStoreDev& s = a.s;
  const uint32_t key = a.tkey[j];
  const int b = a.tbuf[j];
  double* m = s.slot_m + slot_base(s.K, b, key);
  double* w = s.slot_w + slot_base(s.K, b, key);
  int cnt = a.st_count[j];
  double total = 0.0;
  for (int i = 0; i < cnt; ++i) total = KD_ADD(total, w[i]);
  const double ls = a.st_ls[j];
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
  s.count[key] = cnt;
  s.total[key] = total;
  s.log_scale[key] = ls;
  s.clock[key] = a.st_clock[j];
  s.min_v[key] = a.st_min[j];
  s.max_v[key] = a.st_max[j];
  s.dfac[key] = s.lambda > 0.0 ? kd_exp(-ls) : 1.0;
  s.cur[key] = (unsigned char)b;
}

// ---------------------------------------------------------------------------
// Queries: TDigest.quantile / cdf (tdigest.mojo:485-587) with binary searches
// over the committed prefix (bit-identical to the reference's serial walk).
// ---------------------------------------------------------------------------
__global__ void k_query(KdStoreDev s, const uint32_t* __restrict__ keys, const double* __restrict__ qx,
                        long long nq, double* __restrict__ out, int is_cdf, KdErrHost* err) {
  const double nan = kd_from_bits(0x7ff8000000000000ULL);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nq;
       i += (long long)gridDim.x * blockDim.x) {
    const uint32_t key = keys ? keys[i] : 0u;
    const double q = qx[i];
    if ((long long)key >= s.K) {
      kd_err_set(err, KD_EINVAL, i);
      out[i] = nan;
      continue;
    }
    if (!is_cdf && !(q >= 0.0 && q <= 1.0)) {
      kd_err_set(err, KD_EINVAL, i);
      out[i] = nan;
      continue;
    }
    const int nc = s.count[key];
    if (nc == 0) {
      kd_err_set(err, KD_EEMPTY, i);
      out[i] = nan;
      continue;
    }
    const int b = s.cur[key];
    const double* m = s.slot_m + slot_base(s.K, b, key);
    const double* w = s.slot_w + slot_base(s.K, b, key);
    const double* P = s.prefix + (size_t)key * KD_TILE;
    const double n = s.total[key];
    const double mn = s.min_v[key], mx = s.max_v[key];
    const bool decay = s.lambda > 0.0;
    const double dfac = s.dfac[key];
    double r;
    if (!is_cdf) {
      if (nc == 1) {
        r = m[0];
      } else if (q <= 0.0) {
        r = mn;
      } else if (q >= 1.0) {
        r = mx;
      } else {
        const double target = KD_MUL(q, n);
        const double w0 = w[0];
        const double first_half = KD_MUL(w0, 0.5);
        const double wl = w[nc - 1], ml = m[nc - 1];
        const double last_half = KD_MUL(wl, 0.5);
        if (target < first_half) {
          const double eff = decay ? KD_MUL(w0, dfac) : w0;
          r = eff <= 1.0 + 1e-9 ? mn : KD_ADD(mn, KD_MUL(KD_SUB(m[0], mn), KD_DIV(target, first_half)));
        } else if (target > KD_SUB(n, last_half)) {
          const double eff = decay ? KD_MUL(wl, dfac) : wl;
          if (eff <= 1.0 + 1e-9) {
            r = mx;
          } else {
            const double frac = KD_DIV(KD_SUB(target, KD_SUB(n, last_half)), last_half);
            r = KD_ADD(ml, KD_MUL(KD_SUB(mx, ml), frac));
          }
        } else {
          int lo = 1, hi = nc;  // first p in [1, nc-1] with P[p] >= target
          while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (P[mid] >= target) hi = mid;
            else lo = mid + 1;
          }
          if (lo >= nc) {
            r = ml;
          } else {
            const int k = lo - 1;
            const double dw = KD_MUL(KD_ADD(w[k], w[k + 1]), 0.5);
            const double frac = KD_DIV(KD_SUB(target, P[k]), dw);
            r = KD_ADD(m[k], KD_MUL(KD_SUB(m[k + 1], m[k]), frac));
          }
        }
      }
    } else {
      const double x = q;
      if (x < mn) {
        r = 0.0;
      } else if (x > mx) {
        r = 1.0;
      } else if (nc == 1) {
        r = x < m[0] ? 0.0 : (x > m[0] ? 1.0 : 0.5);
      } else if (x < m[0]) {
        if (mn == m[0]) r = 0.0;
        else {
          const double frac = KD_DIV(KD_SUB(x, mn), KD_SUB(m[0], mn));
          r = KD_DIV(KD_MUL(KD_MUL(w[0], 0.5), frac), n);
        }
      } else if (x > m[nc - 1]) {
        const double ml = m[nc - 1], wl = w[nc - 1];
        if (mx == ml) r = 1.0;
        else {
          const double frac = KD_DIV(KD_SUB(x, ml), KD_SUB(mx, ml));
          const double hl = KD_MUL(wl, 0.5);
          r = KD_DIV(KD_ADD(KD_SUB(n, hl), KD_MUL(hl, frac)), n);
        }
      } else {
        int lo = 1, hi = nc;  // first p in [1, nc-1] with x <= m[p]
        while (lo < hi) {
          int mid = (lo + hi) >> 1;
          if (x <= m[mid]) hi = mid;
          else lo = mid + 1;
        }
        if (lo >= nc) {
          r = 1.0;
        } else {
          const int k = lo - 1;
          const double dw = KD_MUL(KD_ADD(w[k], w[k + 1]), 0.5);
          if (m[k + 1] == m[k]) {
            r = KD_DIV(KD_ADD(P[k], KD_MUL(dw, 0.5)), n);
          } else {
            const double frac = KD_DIV(KD_SUB(x, m[k]), KD_SUB(m[k + 1], m[k]));
            r = KD_DIV(KD_ADD(P[k], KD_MUL(dw, frac)), n);
          }
        }
      }
    }
    out[i] = r;
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
int kd_cuda_fail(KdSession* s, cudaError_t e, const char* what) {
  s->last_error = std::string(what) + ": " + cudaGetErrorString(e);
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
    default: return "error";
  }
}

static int level_grid(KdSession* s) { return s->num_sms * 2; }

static size_t tile_smem() { return sizeof(WarpTile) * KD_WARPS_PER_BLOCK; }

static int ensure_attrs(KdSession* s) {
  static bool done = false;
  if (done) return KD_OK;
  KD_CK(cudaFuncSetAttribute(k_level0, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tile_smem()));
  KD_CK(cudaFuncSetAttribute(k_level, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tile_smem()));
  done = true;
  return KD_OK;
}

int kd_pipeline_ingest(KdSession* s, KdStore* st, const uint32_t* d_keys, const double* d_vals,
                       const double* d_wts, long long n, int mode, double timestamp,
                       const double* d_merge_min, const double* d_merge_max,
                       const double* d_merge_clock) {
  if (n <= 0) return KD_OK;
  if (n > (1LL << 31) - 1) {
    s->last_error = "batch too large (limit 2^31 - 1 samples per call)";
    return KD_ERANGE;
  }
  int rc = ensure_attrs(s);
  if (rc) return rc;
  cudaStream_t str = s->stream;
  const KdStoreDev sd = st->d;
  const long long keys_max = std::min<long long>(n, sd.K);
  long long inter = std::max<long long>(64, 2 * (n / KD_TILE) + 64);
  if (s->ws.cap_inter > inter) inter = s->ws.cap_inter;
  for (int attempt = 0; attempt < 4; ++attempt) {
    rc = kd_ws_reserve(s, n, keys_max, inter);
    if (rc) return rc;
    KdWorkspace& w = s->ws;
    {
      // index starts at +inf so that the first offending sample wins the atomicMin
      KdErrHost init{0, 0, 0x7fffffffffffffffLL};
      *w.h_err = init;
      KD_CK(cudaMemcpyAsync(w.err, w.h_err, sizeof(KdErrHost), cudaMemcpyHostToDevice, str));
    }
    KD_CK(cudaMemsetAsync(w.totals, 0, sizeof(int4) * 8, str));
    const bool with_idx = d_wts != nullptr;
    {
      int grid = (int)std::min<long long>((n + 255) / 256, (long long)s->num_sms * 16);
      k_prep<<<grid, 256, 0, str>>>(n, d_keys, d_vals, d_wts, sd.K, w.k64[0], w.key[0],
                                    with_idx ? w.idx[0] : nullptr, w.err);
    }
    KdSortBufs sb{{w.k64[0], w.k64[1]}, {w.key[0], w.key[1]}, {w.idx[0], w.idx[1]}, w.hist, w.partials};
    const int r = kd_radix_sort(sb, n, key_bits_for(sd.K), with_idx, str);
    const uint64_t* k64 = w.k64[r];
    const uint32_t* skey = w.key[r];
    const uint32_t* sidx = with_idx ? w.idx[r] : nullptr;
    kd_scan(TouchedSrc{skey}, TouchedDst{skey, w.tkey, w.tstart, w.cap_keys}, n, w.partials,
            &w.totals[0], str);
    {
      PrepareArgs pa{sd, n, k64, w.tkey, w.tstart, w.totals, mode, timestamp,
                     d_merge_min, d_merge_max, d_merge_clock, w.tm, w.tprior, w.tbuf, w.tsf,
                     w.tpscale, w.st_clock, w.st_ls, w.st_min, w.st_max, w.err};
      k_prepare<<<(int)((keys_max + 255) / 256), 256, 0, str>>>(pa);
    }
    // Level-1 active list is produced directly by the level-0 plan.
    KdLevelDev l1 = w.lv[1];
    l1.A = ((int*)&w.totals[1]) + 2;
    kd_scan(Plan0Src{w.totals, w.tm},
            Plan0Dst{w.totals, w.tm, w.ttile_off, w.tinter_off, w.ttiles, l1}, keys_max,
            w.partials, &w.totals[1], str);
    {
      L0Args la{sd, n, k64, sidx, d_wts, w.tkey, w.tstart, w.tm, w.tprior, w.tbuf, w.tsf,
                w.tpscale, w.ttile_off, w.ttiles, w.tinter_off, w.totals, w.scr_m[0],
                w.scr_w[0], w.tcount[0], w.st_count, w.cap_inter, s->force_exact, w.err};
      k_level0<<<level_grid(s), 32 * KD_WARPS_PER_BLOCK, tile_smem(), str>>>(la);
    }
    int* remaining = l1.A;
    for (int L = 1; L <= s->max_levels; ++L) {
      KdLevelDev cur = w.lv[L & 1];
      KdLevelDev nxt = w.lv[(L + 1) & 1];
      if (L == 1) cur.A = l1.A;
      // the next level's A lives in its own scalar (never aliased to totals)
      PlanArgs pa{cur, nxt, w.tcount[(L - 1) & 1], w.doff[(L - 1) & 1], w.tkey, w.cap_inter,
                  w.cap_keys, w.err};
      k_plan<<<1, 1024, 0, str>>>(pa);
      LLArgs la{sd, cur, w.tkey, w.tbuf, w.st_count, w.scr_m[(L - 1) & 1], w.scr_w[(L - 1) & 1],
                w.tcount[(L - 1) & 1], w.doff[(L - 1) & 1], w.scr_m[L & 1], w.scr_w[L & 1],
                w.tcount[L & 1], s->force_exact, w.err};
      k_level<<<level_grid(s), 32 * KD_WARPS_PER_BLOCK, tile_smem(), str>>>(la);
      remaining = nxt.A;
    }
    {
      CommitArgs ca{sd, w.totals, w.tkey, w.tbuf, w.st_count, w.st_clock, w.st_ls, w.st_min,
                    w.st_max, remaining, w.err};
      k_commit<<<(int)((keys_max + 127) / 128), 128, 0, str>>>(ca);
    }
    KD_CK(cudaGetLastError());
    KD_CK(cudaMemcpyAsync(w.h_err, w.err, sizeof(KdErrHost), cudaMemcpyDeviceToHost, str));
    KD_CK(cudaStreamSynchronize(str));
    const KdErrHost e = *w.h_err;
    if (e.code == 0) return KD_OK;
    if (e.code == KD_ERANGE_SCRATCH) {
      inter = std::max<long long>(inter * 2, e.index + e.index / 2 + 64);
      continue;
    }
    char buf[256];
    snprintf(buf, sizeof buf, "%s (at index %lld)", err_text(e.code), e.index);
    s->last_error = buf;
    return e.code;
  }
  s->last_error = "intermediate scratch could not be sized";
  return KD_ENOMEM;
}

int kd_pipeline_quantile(KdSession* s, KdStore* st, const uint32_t* d_keys, const double* d_q,
                         long long nq, double* d_out, int is_cdf) {
  if (nq <= 0) return KD_OK;
  int rc = kd_ws_reserve(s, 1, 1, 64);
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
    s->last_error = buf;
    return w.h_err->code;
  }
  return KD_OK;
}

int kd_pipeline_merge(KdSession* s, KdStore* dst, KdStore* src, const long long* h_goff,
                      const uint32_t* h_parts, long long ngroups) {
  if (ngroups <= 0) return KD_OK;
  if (ngroups > dst->d.K) {
    s->last_error = "more groups than keys in the destination store";
    return KD_EINVAL;
  }
  const long long nparts = h_goff[ngroups];
  for (long long p = 0; p < nparts; ++p)
    if ((long long)h_parts[p] >= src->d.K) {
      s->last_error = "part key out of range of the source store";
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
