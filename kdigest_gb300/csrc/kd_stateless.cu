// kd_stateless.cu — the reference's GPU entry points over caller-held digests.
//
// The reference's host state keeps every digest on the host (TDigest,
// tdigest.mojo:236-315) and hands the GPU its centroid arrays per call:
//   gpu_grouped_compress_weighted  (gpu/grouped.mojo:415-643)
//   gpu_quantile / gpu_cdf          (gpu/query.mojo:320-342)
//   gpu_merge_digests               (gpu/query.mojo:348-369)
// These entry points take the same inputs as flat CSR arrays and return the
// results the same way, so such a caller can use this library without keeping
// its digests resident.  The compress-type calls run the resident pipeline on
// a session-owned scratch store in replace mode (each key's input compressed on
// its own, with its given weights), then gather the keys' centroids.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/kdigest_gb300.h"
#include "kd_engine.h"
#include "kd_internal.cuh"
#include "kd_query.cuh"

namespace {

int fail(KdSession* s, int code, const char* msg) {
  kd_set_msg(s, msg);
  return code;
}

#define SL_CK(call)                                                   \
  do {                                                                \
    cudaError_t e_ = (call);                                          \
    if (e_ != cudaSuccess) return kd_cuda_fail(s, e_, #call);         \
  } while (0)

// Session working memory of these calls (grown, budget-accounted).
int sl_reserve(KdSession* s, size_t bytes) {
  if (s->sl_bytes >= bytes) return KD_OK;
  if (s->sl_buf) kd_dfree(s, s->sl_buf, s->sl_bytes);
  s->sl_buf = nullptr;
  s->sl_bytes = 0;
  const size_t b = std::max(bytes, (size_t)(1 << 20));
  int rc = kd_dalloc(s, &s->sl_buf, b);
  if (rc) return rc;
  s->sl_bytes = b;
  return KD_OK;
}

struct Carve {
  char* p;
  size_t off = 0;
  template <class T>
  T* take(size_t n) {
    off = (off + 255) & ~(size_t)255;
    T* r = reinterpret_cast<T*>(p + off);
    off += sizeof(T) * n;
    return r;
  }
  template <class T>
  static size_t need(size_t off, size_t n) {
    return ((off + 255) & ~(size_t)255) + sizeof(T) * n;
  }
};

// ---------------------------------------------------------------------------
// gpu_quantile / gpu_cdf over a CSR of digests
// ---------------------------------------------------------------------------
// Per digest: the walk's total (the weights summed in order, <= 0 -> 1,
// gpu/query.mojo:253-257) and its walk prefix.  Digests above one block are
// skipped here; their queries fail (gpu/query.mojo:252-253).
__global__ void k_sl_prep(const int64_t* off, long long nd, const double* w, double* total,
                          double* P) {
  for (long long d = (long long)blockIdx.x * blockDim.x + threadIdx.x; d < nd;
       d += (long long)gridDim.x * blockDim.x) {
    const long long b = off[d], nc = off[d + 1] - b;
    if (nc > KD_TILE) continue;
    double t = 0.0;
    for (long long i = 0; i < nc; ++i) t = KD_ADD(t, w[b + i]);
    total[d] = t > 0.0 ? t : 1.0;
    if (nc > 0) {
      double run = KD_MUL(w[b], 0.5);
      P[b] = run;
      for (long long i = 0; i + 1 < nc; ++i) {
        run = KD_ADD(run, KD_MUL(KD_ADD(w[b + i], w[b + i + 1]), 0.5));
        P[b + i + 1] = run;
      }
    }
  }
}

__global__ void k_sl_query(const int64_t* off, long long nd, const double* m, const double* w,
                           const double* P, const double* total, const double* mn,
                           const double* mx, const uint32_t* ids, const double* qx, long long nq,
                           double* out, int is_cdf, KdErrHost* err) {
  const double nan = kd_from_bits(0x7ff8000000000000ULL);
  KdErr* e = reinterpret_cast<KdErr*>(err);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nq;
       i += (long long)gridDim.x * blockDim.x) {
    const long long d = ids ? (long long)ids[i] : 0;
    if (d >= nd) {
      if (atomicCAS(&e->code, 0, KD_EINVAL) == 0) e->index = i;
      out[i] = nan;
      continue;
    }
    const long long b = off[d], nc = off[d + 1] - b;
    if (nc == 0 || nc > KD_TILE) {  // gpu/query.mojo:248-253
      if (atomicCAS(&e->code, 0, nc == 0 ? KD_EEMPTY : KD_ERANGE) == 0) e->index = i;
      out[i] = nan;
      continue;
    }
    KdQueryDigest q;
    q.m = m + b;
    q.w = w + b;
    q.P = P + b;
    q.nc = (int)nc;
    q.n = total[d];
    q.mn = mn + d;
    q.mx = mx + d;
    q.dfac = nullptr;
    q.single = 1.0 + 1e-6;  // the GPU kernels' test on the raw weight (query.mojo:103,113)
    out[i] = is_cdf ? kd_cdf_one(q, qx[i]) : kd_quantile_one(q, qx[i]);
  }
}

int sl_query(kd_session* h, const int64_t* offsets, int64_t nd, const double* means,
             const double* weights, const double* min_v, const double* max_v, const uint32_t* ids,
             const double* qx, int64_t nq, double* out, int flags, int is_cdf) {
  if (!h) return KD_EINVAL;
  KdSession* s = &h->s;
  if (nd < 0 || nq < 0) return fail(s, KD_EINVAL, "negative sizes");
  if (nq == 0) return KD_OK;
  if (nd == 0 || !offsets || !qx || !out || !min_v || !max_v) return fail(s, KD_EINVAL, "null arrays");
  cudaSetDevice(s->device);
  const bool dev = (flags & KD_PTR_DEVICE) != 0;
  long long ncent = 0;
  if (!dev) {
    if (offsets[0] != 0) return fail(s, KD_EINVAL, "offsets[0] must be 0");
    for (int64_t d = 0; d < nd; ++d)
      if (offsets[d + 1] < offsets[d]) return fail(s, KD_EINVAL, "offsets must be non-decreasing");
    ncent = offsets[nd];
  } else {
    int64_t last = 0;
    SL_CK(cudaMemcpy(&last, offsets + nd, 8, cudaMemcpyDeviceToHost));
    ncent = last;
  }
  if (ncent > 0 && (!means || !weights)) return fail(s, KD_EINVAL, "null centroid arrays");
  int rc = s->ws.err ? KD_OK : kd_ws_reserve(s, 1, 1, 64, 64, 64, 1);
  if (rc) return rc;
  // working memory: prefix and totals; host inputs are staged alongside
  size_t bytes = Carve::need<double>(0, (size_t)ncent + 1);
  bytes = Carve::need<double>(bytes, (size_t)nd);
  if (!dev) {
    bytes = Carve::need<int64_t>(bytes, (size_t)nd + 1);
    bytes = Carve::need<double>(bytes, (size_t)ncent * 2 + 2 * (size_t)nd + 2 * (size_t)nq);
    bytes = Carve::need<uint32_t>(bytes, (size_t)nq);
  }
  rc = sl_reserve(s, bytes);
  if (rc) return rc;
  Carve c{(char*)s->sl_buf};
  double* P = c.take<double>((size_t)ncent + 1);
  double* tot = c.take<double>((size_t)nd);
  cudaStream_t str = s->stream;
  const int64_t* doff = offsets;
  const double *dm = means, *dw = weights, *dmn = min_v, *dmx = max_v, *dq = qx;
  const uint32_t* dids = ids;
  double* dout = out;
  if (!dev) {
    int64_t* o = c.take<int64_t>((size_t)nd + 1);
    double* buf = c.take<double>((size_t)ncent * 2 + 2 * (size_t)nd + 2 * (size_t)nq);
    uint32_t* ib = c.take<uint32_t>((size_t)nq);
    SL_CK(cudaMemcpyAsync(o, offsets, 8 * ((size_t)nd + 1), cudaMemcpyHostToDevice, str));
    double* p = buf;
    if (ncent > 0) {
      SL_CK(cudaMemcpyAsync(p, means, 8 * (size_t)ncent, cudaMemcpyHostToDevice, str));
      SL_CK(cudaMemcpyAsync(p + ncent, weights, 8 * (size_t)ncent, cudaMemcpyHostToDevice, str));
    }
    dm = p;
    dw = p + ncent;
    p += 2 * ncent;
    SL_CK(cudaMemcpyAsync(p, min_v, 8 * (size_t)nd, cudaMemcpyHostToDevice, str));
    SL_CK(cudaMemcpyAsync(p + nd, max_v, 8 * (size_t)nd, cudaMemcpyHostToDevice, str));
    dmn = p;
    dmx = p + nd;
    p += 2 * nd;
    SL_CK(cudaMemcpyAsync(p, qx, 8 * (size_t)nq, cudaMemcpyHostToDevice, str));
    dq = p;
    dout = p + nq;
    if (ids) {
      SL_CK(cudaMemcpyAsync(ib, ids, 4 * (size_t)nq, cudaMemcpyHostToDevice, str));
      dids = ib;
    }
    doff = o;
  }
  KdWorkspace& w = s->ws;
  *w.h_err = KdErrHost{0, 0, -1};
  SL_CK(cudaMemcpyAsync(w.err, w.h_err, sizeof(KdErrHost), cudaMemcpyHostToDevice, str));
  k_sl_prep<<<(int)std::min<long long>((nd + 127) / 128, (long long)s->num_sms * 8), 128, 0, str>>>(
      doff, nd, dw, tot, P);
  k_sl_query<<<(int)std::min<long long>((nq + 255) / 256, (long long)s->num_sms * 32), 256, 0, str>>>(
      doff, nd, dm, dw, P, tot, dmn, dmx, dids, dq, nq, dout, is_cdf, w.err);
  SL_CK(cudaGetLastError());
  SL_CK(cudaMemcpyAsync(w.h_err, w.err, sizeof(KdErrHost), cudaMemcpyDeviceToHost, str));
  if (!dev) SL_CK(cudaMemcpyAsync(out, dout, 8 * (size_t)nq, cudaMemcpyDeviceToHost, str));
  SL_CK(cudaStreamSynchronize(str));
  if (w.h_err->code) {
    char buf[200];
    const int code = w.h_err->code;
    snprintf(buf, sizeof buf, "%s (query or digest %lld)",
             code == KD_EEMPTY ? "cannot query an empty digest"
             : code == KD_ERANGE ? "a digest exceeds one block (1024 centroids); compress it first"
                                 : "digest id out of range",
             w.h_err->index);
    kd_set_msg(s, buf);
    return code;
  }
  return KD_OK;
}

// ---------------------------------------------------------------------------
// Compress-type calls: every key's input through the pipeline in replace mode
// ---------------------------------------------------------------------------
// Copies the centroids of the keys with input (use[k]) to out at offs[k].
__global__ void k_sl_gather(KdStoreDev d, const long long* offs, const unsigned char* use, long long K,
                            double* om, double* ow) {
  const int lane = threadIdx.x & 31;
  for (long long k = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < K;
       k += ((long long)gridDim.x * blockDim.x) >> 5) {
    if (!use[k]) continue;
    const int cnt = d.count[k];
    const size_t base = ((size_t)d.cur[k] * (size_t)d.K + (size_t)k) * KD_TILE;
    const long long o = offs[k];
    for (int i = lane; i < cnt; i += 32) {
      om[o + i] = d.slot_m[base + i];
      ow[o + i] = d.slot_w[base + i];
    }
  }
}

// The scratch store of K keys for the grouped calls (recreated for another K).
int scratch_many(KdSession* s, long long K, int scale, double compression, KdStore** out) {
  KdStore* st = s->scratch_many;
  if (st && st->d.K != K) {
    kd_store_free(st);
    delete st;
    s->scratch_many = st = nullptr;
  }
  if (!st) {
    st = new (std::nothrow) KdStore();
    if (!st) return KD_ENOMEM;
    st->sess = s;
    st->d.K = K;
    int rc = kd_store_alloc(s, st);
    if (rc) {
      delete st;
      return rc;
    }
    s->scratch_many = st;
  }
  st->d.scale = scale;
  st->d.compression = compression;
  st->d.lambda = 0.0;
  *out = st;
  return KD_OK;
}

// Compresses the weighted batch (keys, vals, wts; every key's input in the
// order the reference concatenates it) on the scratch store and returns each
// key's centroids in the output CSR.  has_input[k]: key k had any input.
int compress_keys(KdSession* s, int scale, double compression, long long K,
                  const std::vector<uint32_t>& keys, const std::vector<double>& vals,
                  const std::vector<double>& wts, const std::vector<unsigned char>& has_input,
                  int64_t* out_offsets, double* out_means, double* out_weights, int64_t cap,
                  int64_t* out_n) {
  const long long M = (long long)vals.size();
  KdStore* st = nullptr;
  int rc = scratch_many(s, K, scale, compression, &st);
  if (rc) return rc;
  cudaStream_t str = s->stream;
  size_t bytes = Carve::need<uint32_t>(0, (size_t)M + 1);
  bytes = Carve::need<double>(bytes, 2 * (size_t)M + 2);
  rc = sl_reserve(s, bytes);
  if (rc) return rc;
  {
    Carve c{(char*)s->sl_buf};
    uint32_t* dk = c.take<uint32_t>((size_t)M + 1);
    double* dv = c.take<double>(2 * (size_t)M + 2);
    if (M > 0) {
      SL_CK(cudaMemcpyAsync(dk, keys.data(), 4 * (size_t)M, cudaMemcpyHostToDevice, str));
      SL_CK(cudaMemcpyAsync(dv, vals.data(), 8 * (size_t)M, cudaMemcpyHostToDevice, str));
      SL_CK(cudaMemcpyAsync(dv + M, wts.data(), 8 * (size_t)M, cudaMemcpyHostToDevice, str));
      rc = kd_pipeline_ingest(s, st, dk, dv, dv + M, M, KD_MODE_REPLACE, 0.0, nullptr, nullptr, nullptr);
      if (rc) return rc;
    }
  }
  std::vector<int> cnt((size_t)K, 0);
  SL_CK(cudaMemcpyAsync(cnt.data(), st->d.count, 4 * (size_t)K, cudaMemcpyDeviceToHost, str));
  SL_CK(cudaStreamSynchronize(str));
  std::vector<long long> offs((size_t)K + 1, 0);
  for (long long k = 0; k < K; ++k) offs[k + 1] = offs[k] + (has_input[k] ? cnt[k] : 0);
  for (long long k = 0; k <= K; ++k) out_offsets[k] = offs[k];
  const long long total = offs[K];
  if (out_n) *out_n = total;
  if (cap < total) return fail(s, KD_ERANGE, "output capacity too small (needed size in *out_n)");
  if (total == 0) return KD_OK;
  bytes = Carve::need<long long>(0, (size_t)K + 1);
  bytes = Carve::need<unsigned char>(bytes, (size_t)K);
  bytes = Carve::need<double>(bytes, 2 * (size_t)total);
  rc = sl_reserve(s, bytes);
  if (rc) return rc;
  Carve c{(char*)s->sl_buf};
  long long* doffs = c.take<long long>((size_t)K + 1);
  unsigned char* duse = c.take<unsigned char>((size_t)K);
  double* dom = c.take<double>(2 * (size_t)total);
  SL_CK(cudaMemcpyAsync(doffs, offs.data(), 8 * ((size_t)K + 1), cudaMemcpyHostToDevice, str));
  SL_CK(cudaMemcpyAsync(duse, has_input.data(), (size_t)K, cudaMemcpyHostToDevice, str));
  k_sl_gather<<<(int)std::min<long long>((K + 7) / 8, (long long)s->num_sms * 16), 256, 0, str>>>(
      st->d, doffs, duse, K, dom, dom + total);
  SL_CK(cudaGetLastError());
  SL_CK(cudaMemcpyAsync(out_means, dom, 8 * (size_t)total, cudaMemcpyDeviceToHost, str));
  SL_CK(cudaMemcpyAsync(out_weights, dom + total, 8 * (size_t)total, cudaMemcpyDeviceToHost, str));
  SL_CK(cudaStreamSynchronize(str));
  return KD_OK;
}

bool is_finite_value(double v) { return kd_isfinite(v) != 0; }
bool good_weight(double v) { return v > 0.0 && kd_isfinite(v); }

}  // namespace

extern "C" {

KD_API int kd_quantile(kd_session* s, const int64_t* offsets, int64_t ndigests, const double* means,
                       const double* weights, const double* min_v, const double* max_v,
                       const uint32_t* ids, const double* qs, int64_t nq, double* out, int flags) {
  return sl_query(s, offsets, ndigests, means, weights, min_v, max_v, ids, qs, nq, out, flags, 0);
}

KD_API int kd_cdf(kd_session* s, const int64_t* offsets, int64_t ndigests, const double* means,
                  const double* weights, const double* min_v, const double* max_v,
                  const uint32_t* ids, const double* xs, int64_t nx, double* out, int flags) {
  return sl_query(s, offsets, ndigests, means, weights, min_v, max_v, ids, xs, nx, out, flags, 1);
}

KD_API int kd_grouped_compress(kd_session* h, int scale, double compression, int64_t num_keys,
                               const uint32_t* keys, const double* values, int64_t n,
                               const double* new_weights, const int64_t* prior_offsets,
                               const double* prior_means, const double* prior_weights,
                               int64_t* out_offsets, double* out_means, double* out_weights,
                               int64_t cap, int64_t* out_n, double* out_min, double* out_max) {
  if (!h) return KD_EINVAL;
  KdSession* s = &h->s;
  if (out_n) *out_n = 0;
  if (scale < KD_K0 || scale > KD_K3) return fail(s, KD_EINVAL, "unknown scale function");
  if (!(compression > 0.0) || !kd_isfinite(compression)) return fail(s, KD_EINVAL, "compression must be positive and finite");
  if (num_keys <= 0 || num_keys > 0x7fffffffLL || n < 0) return fail(s, KD_EINVAL, "bad sizes");
  if ((n > 0 && (!keys || !values)) || !out_offsets) return fail(s, KD_EINVAL, "null arrays");
  // validate everything before any work (grouped.mojo:74-97)
  for (int64_t i = 0; i < n; ++i) {
    if ((int64_t)keys[i] >= num_keys) return fail(s, KD_EINVAL, "key out of range [0, num_keys)");
    if (!is_finite_value(values[i])) return fail(s, KD_EINVAL, "value must be finite");
  }
  if (new_weights)
    for (int64_t k = 0; k < num_keys; ++k)
      if (!good_weight(new_weights[k])) return fail(s, KD_EINVAL, "new weights must be positive and finite");
  long long np = 0;
  if (prior_offsets) {
    if (prior_offsets[0] != 0) return fail(s, KD_EINVAL, "prior_offsets[0] must be 0");
    for (int64_t k = 0; k < num_keys; ++k)
      if (prior_offsets[k + 1] < prior_offsets[k]) return fail(s, KD_EINVAL, "prior_offsets must be non-decreasing");
    np = prior_offsets[num_keys];
    if (np > 0 && (!prior_means || !prior_weights)) return fail(s, KD_EINVAL, "null prior arrays");
    for (long long i = 0; i < np; ++i)
      if (!is_finite_value(prior_means[i]) || !good_weight(prior_weights[i]))
        return fail(s, KD_EINVAL, "prior centroids must be finite with positive weights");
  }
  cudaSetDevice(s->device);
  // Per key: its prior centroids first, then its new samples in batch order,
  // each of weight new_weights[k] (gpu/grouped.mojo:489-538).  Priors of all
  // keys lead the batch, so the stable sort by (key, value, position) puts a
  // key's priors before its new samples on equal values.
  const size_t M = (size_t)np + (size_t)n;
  std::vector<uint32_t> bk(M);
  std::vector<double> bv(M), bw(M);
  std::vector<unsigned char> has((size_t)num_keys, 0);
  size_t j = 0;
  for (int64_t k = 0; k < num_keys && prior_offsets; ++k)
    for (long long i = prior_offsets[k]; i < prior_offsets[k + 1]; ++i, ++j) {
      bk[j] = (uint32_t)k;
      bv[j] = prior_means[i];
      bw[j] = prior_weights[i];
      has[(size_t)k] = 1;
    }
  std::vector<double> mn((size_t)num_keys, 0.0), mx((size_t)num_keys, 0.0);
  std::vector<unsigned char> seen((size_t)num_keys, 0);
  for (int64_t i = 0; i < n; ++i, ++j) {
    const uint32_t k = keys[i];
    const double v = values[i];
    bk[j] = k;
    bv[j] = v;
    bw[j] = new_weights ? new_weights[k] : 1.0;
    has[k] = 1;
    if (!seen[k]) {  // the new samples' own range (gpu/grouped.mojo:517-538)
      mn[k] = mx[k] = v;
      seen[k] = 1;
    } else {
      if (v < mn[k]) mn[k] = v;
      if (v > mx[k]) mx[k] = v;
    }
  }
  if (out_min) std::memcpy(out_min, mn.data(), 8 * (size_t)num_keys);
  if (out_max) std::memcpy(out_max, mx.data(), 8 * (size_t)num_keys);
  return compress_keys(s, scale, compression, num_keys, bk, bv, bw, has, out_offsets, out_means,
                       out_weights, cap, out_n);
}

KD_API int kd_merge(kd_session* h, int scale, double compression, const int64_t* part_offsets,
                    int64_t nparts, const double* means, const double* weights,
                    const int64_t* group_offsets, int64_t ngroups, const uint32_t* part_ids,
                    int64_t* out_offsets, double* out_means, double* out_weights, int64_t cap,
                    int64_t* out_n) {
  if (!h) return KD_EINVAL;
  KdSession* s = &h->s;
  if (out_n) *out_n = 0;
  if (scale < KD_K0 || scale > KD_K3) return fail(s, KD_EINVAL, "unknown scale function");
  if (!(compression > 0.0) || !kd_isfinite(compression)) return fail(s, KD_EINVAL, "compression must be positive and finite");
  if (nparts < 0 || ngroups <= 0 || ngroups > 0x7fffffffLL) return fail(s, KD_EINVAL, "bad sizes");
  if (!part_offsets || !group_offsets || !out_offsets) return fail(s, KD_EINVAL, "null arrays");
  if (part_offsets[0] != 0 || group_offsets[0] != 0) return fail(s, KD_EINVAL, "offsets must start at 0");
  for (int64_t p = 0; p < nparts; ++p)
    if (part_offsets[p + 1] < part_offsets[p]) return fail(s, KD_EINVAL, "part_offsets must be non-decreasing");
  for (int64_t g = 0; g < ngroups; ++g)
    if (group_offsets[g + 1] < group_offsets[g]) return fail(s, KD_EINVAL, "group_offsets must be non-decreasing");
  const long long nref = group_offsets[ngroups];
  if (!part_ids && nref > nparts) return fail(s, KD_EINVAL, "groups reference more parts than exist");
  if (part_offsets[nparts] > 0 && (!means || !weights)) return fail(s, KD_EINVAL, "null centroid arrays");
  size_t M = 0;
  for (long long r = 0; r < nref; ++r) {
    const long long p = part_ids ? (long long)part_ids[r] : r;
    if (p >= nparts) return fail(s, KD_EINVAL, "part id out of range");
    M += (size_t)(part_offsets[p + 1] - part_offsets[p]);
  }
  for (long long i = 0; i < part_offsets[nparts]; ++i)
    if (!is_finite_value(means[i]) || !good_weight(weights[i]))
      return fail(s, KD_EINVAL, "centroids must be finite with positive weights");
  cudaSetDevice(s->device);
  // group g: the centroids of its parts concatenated in part order
  // (gpu/query.mojo:360-368), compressed once.
  std::vector<uint32_t> bk(M);
  std::vector<double> bv(M), bw(M);
  std::vector<unsigned char> has((size_t)ngroups, 0);
  size_t j = 0;
  for (int64_t g = 0; g < ngroups; ++g)
    for (long long r = group_offsets[g]; r < group_offsets[g + 1]; ++r) {
      const long long p = part_ids ? (long long)part_ids[r] : r;
      for (long long i = part_offsets[p]; i < part_offsets[p + 1]; ++i, ++j) {
        bk[j] = (uint32_t)g;
        bv[j] = means[i];
        bw[j] = weights[i];
        has[(size_t)g] = 1;
      }
    }
  return compress_keys(s, scale, compression, ngroups, bk, bv, bw, has, out_offsets, out_means,
                       out_weights, cap, out_n);
}

}  // extern "C"

// Integer-pipe FP64 helpers next to the FP64 instructions they stand for.
__global__ void k_fp64i_selftest(int op, const double* __restrict__ a, const double* __restrict__ b,
                                 long long n, double* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double x = a[i], y = b ? b[i] : 0.0;
    double r;
    switch (op) {
      case 0: r = kd_div(x, y); break;
      case 1: r = KD_DIV(x, y); break;
      case 2: r = kd_half(x); break;
      case 3: r = KD_MUL(x, 0.5); break;
      case 4: r = kd_okey(x) < kd_okey(y) ? 1.0 : (kd_okey(x) == kd_okey(y) ? 0.5 : 0.0); break;
      default: r = x < y ? 1.0 : (x == y ? 0.5 : 0.0); break;
    }
    out[i] = r;
  }
}

extern "C" KD_API int kd_selftest_fp64(int op, const double* a, const double* b, int64_t n,
                                       double* out) {
  if (op < 0 || op > 5 || n < 0 || (n > 0 && (!a || !out || (op != 2 && op != 3 && !b))))
    return KD_EINVAL;
  if (n == 0) return KD_OK;
  const int grid = (int)std::min<long long>((n + 255) / 256, 4096);
  k_fp64i_selftest<<<grid, 256>>>(op, a, op == 2 || op == 3 ? nullptr : b, n, out);
  if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return KD_ECUDA;
  return KD_OK;
}
