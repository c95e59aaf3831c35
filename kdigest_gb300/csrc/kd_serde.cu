// kd_serde.cu — batched to_bytes / from_bytes of many keys on the device
// (checkpoint and restore of a resident store).
//
// Every key's record is the reference's wire format (tdigest.mojo:627-698): a
// version byte 1, eight little-endian FP64 header fields (compression, decay
// lambda, log_scale, clock, stored_total, min, max, count) and count (mean,
// weight) pairs.  Records of the listed keys are concatenated; offsets[i] is
// where key i's record starts.  Export writes each record with a warp, one
// byte per lane in turn, so the warp's stores are contiguous whatever the
// record's alignment.  Import validates every record before any key changes,
// then installs them (live slot, header, quantile prefix, decay factor) with the
// same arithmetic as the single-key path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/kdigest_gb300.h"
#include "kd_engine.h"
#include "kd_internal.cuh"
#include "kd_math.h"
#include "kd_scan.cuh"

namespace {

// Key of list entry i: keys[i], or key0 + i for the implicit list 0..K-1.
__device__ __forceinline__ uint32_t list_key(const uint32_t* keys, long long key0, long long i) {
  return keys ? keys[i] : (uint32_t)(key0 + i);
}

// Centroid counts of the listed keys.
__global__ void k_counts(KdStoreDev s, const uint32_t* keys, long long nkeys, int* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nkeys;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = s.count[list_key(keys, 0, i)];
}

__device__ __forceinline__ uint8_t f64_byte(double v, int b) {
  return (uint8_t)((unsigned long long)__double_as_longlong(v) >> (8 * b));
}

__global__ void k_export(KdStoreDev s, const uint32_t* keys, long long key0, long long nkeys,
                         const long long* __restrict__ offsets, uint8_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nkeys;
       i += ((long long)gridDim.x * blockDim.x) >> 5) {
    const uint32_t key = list_key(keys, key0, i);
    const int cnt = s.count[key];
    const size_t slot = ((size_t)s.cur[key] * s.K + key) * KD_TILE;
    const double* m = s.slot_m + slot;
    const double* w = s.slot_w + slot;
    const double hdr[8] = {s.compression, s.lambda, s.log_scale[key], s.clock[key],
                           s.total[key],   s.min_v[key], s.max_v[key], (double)cnt};
    uint8_t* rec = out + offsets[i];
    const long long len = 65 + 16LL * cnt;
    for (long long b = lane; b < len; b += 32) {
      uint8_t v;
      if (b == 0) {
        v = 1;  // serialization version (tdigest.mojo:61)
      } else if (b < 65) {
        v = f64_byte(hdr[(b - 1) >> 3], (int)((b - 1) & 7));
      } else {
        const long long c = (b - 65) >> 4;
        const int f = (int)((b - 65) & 15);
        v = f64_byte(f < 8 ? m[c] : w[c], f & 7);
      }
      rec[b] = v;
    }
  }
}

__device__ __forceinline__ double get_f64_dev(const uint8_t* p) {
  unsigned long long b = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) b |= (unsigned long long)p[i] << (8 * i);
  return __longlong_as_double((long long)b);
}

// Validation of every record (the lowest failing index wins).
__global__ void k_import_check(KdStoreDev s, const uint32_t* keys, long long nkeys,
                               const uint8_t* __restrict__ buf, const long long* __restrict__ offsets,
                               KdErrHost* err) {
  // device-resident records: the same checks as the host-side ones
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nkeys;
       i += (long long)gridDim.x * blockDim.x) {
    const long long off = offsets[i], len = offsets[i + 1] - offsets[i];
    int code = 0;
    if ((long long)list_key(keys, 0, i) >= s.K) {
      code = KD_EINVAL;
    } else if (len <= 0 || buf[off] != 1) {
      code = KD_EINVAL;  // unrecognized serialization version
    } else if (len < 65) {
      code = KD_ERANGE;  // truncated
    } else {
      const double c = get_f64_dev(buf + off + 57);
      if (!(c >= 0.0) || c > (double)KD_TILE || c != floor(c) || 65 + 16 * (long long)c > len)
        code = KD_ERANGE;
    }
    if (code) {
      atomicMin((unsigned long long*)&err->index, (unsigned long long)i);
      atomicCAS(&err->code, 0, code);
    }
  }
}

__global__ void k_import(KdStoreDev s, const uint32_t* keys, long long key0, long long nkeys,
                         const uint8_t* __restrict__ buf, const long long* __restrict__ offsets) {
  const int lane = threadIdx.x & 31;
  for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nkeys;
       i += ((long long)gridDim.x * blockDim.x) >> 5) {
    const uint32_t key = list_key(keys, key0, i);
    const uint8_t* rec = buf + offsets[i];
    const int cnt = (int)get_f64_dev(rec + 57);
    const size_t slot = ((size_t)s.cur[key] * s.K + key) * KD_TILE;
    double* m = s.slot_m + slot;
    double* w = s.slot_w + slot;
    for (int c = lane; c < cnt; c += 32) {
      m[c] = get_f64_dev(rec + 65 + 16 * c);
      w[c] = get_f64_dev(rec + 73 + 16 * c);
    }
    __syncwarp();
    if (lane == 0) {
      s.count[key] = cnt;
      if (s.bcount) s.bcount[key] = 0;  // an installed digest has no buffered samples
      s.log_scale[key] = get_f64_dev(rec + 17);
      s.clock[key] = get_f64_dev(rec + 25);
      s.total[key] = get_f64_dev(rec + 33);
      s.min_v[key] = get_f64_dev(rec + 41);
      s.max_v[key] = get_f64_dev(rec + 49);
      // quantile-walk prefix and decay factor, as for a single key
      double* P = s.prefix + (size_t)key * KD_TILE;
      if (cnt > 0) {
        double run = KD_MUL(w[0], 0.5);
        P[0] = run;
        for (int c = 0; c + 1 < cnt; ++c) {
          run = KD_ADD(run, KD_MUL(KD_ADD(w[c], w[c + 1]), 0.5));
          P[c + 1] = run;
        }
      }
      s.dfac[key] = s.lambda > 0.0 ? kd_exp(-s.log_scale[key]) : 1.0;
    }
  }
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

int ck(KdSession* s, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return KD_OK;
  cudaGetLastError();
  return kd_cuda_fail(s, e, what);
}

constexpr long long kChunkBytes = 256LL << 20;  // bytes staged per round trip

// Consecutive keys [i0, i1) whose records fit one chunk (at least one key).
long long chunk_end(const int64_t* off, long long i0, long long nkeys) {
  long long i1 = i0 + 1;
  while (i1 < nkeys && off[i1 + 1] - off[i0] <= kChunkBytes) ++i1;
  return i1;
}

}  // namespace

#define KD_SCK(call)                      \
  do {                                    \
    const int rc_ = ck(s, (call), #call); \
    if (rc_) return rc_;                  \
  } while (0)

// A one-key store whose digest was installed from records: the centroids may
// come in any order, so the next batch sorts them together with its samples.
static void imported(KdStore* st) {
  if (st->d.K == 1) {
    st->pending = false;
    st->carry = true;
  }
}

extern "C" {

KD_API int kd_store_export(kd_store* h, const uint32_t* keys, int64_t nkeys, uint8_t* buf,
                           int64_t cap, int64_t* offsets, int flags) {
  if (!h || !offsets || nkeys < 0) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  const KdStoreDev& d = st->d;
  if (!keys && nkeys > d.K) {
    kd_set_msg(s, "more keys than the store holds");
    return KD_EINVAL;
  }
  const bool dev = (flags & KD_PTR_DEVICE) != 0;
  if (keys && !dev)
    for (int64_t i = 0; i < nkeys; ++i)
      if ((long long)keys[i] >= d.K) {
        kd_set_msg(s, "key out of range [0, num_keys)");
        return KD_EINVAL;
      }
  cudaSetDevice(s->device);
  cudaStream_t str = s->stream;
  offsets[0] = 0;
  if (nkeys == 0) return KD_OK;
  {
    const int frc = kd_spath_flush(s, st);  // each record is to_bytes, which merges first
    if (frc) return frc;
  }
  DevBuf dkeys, dcnt, doff, dout;
  const uint32_t* kp = keys;
  if (keys && !dev) {
    KD_SCK(cudaMalloc(&dkeys.p, (size_t)nkeys * 4));
    KD_SCK(cudaMemcpyAsync(dkeys.p, keys, (size_t)nkeys * 4, cudaMemcpyHostToDevice, str));
    kp = (const uint32_t*)dkeys.p;
  }
  KD_SCK(cudaMalloc(&dcnt.p, (size_t)nkeys * 4));
  const int grid = (int)std::min<long long>((nkeys + 255) / 256, (long long)s->num_sms * 16);
  k_counts<<<grid, 256, 0, str>>>(d, kp, nkeys, (int*)dcnt.p);
  std::vector<int> cnt((size_t)nkeys);
  KD_SCK(cudaMemcpyAsync(cnt.data(), dcnt.p, (size_t)nkeys * 4, cudaMemcpyDeviceToHost, str));
  KD_SCK(cudaStreamSynchronize(str));
  for (int64_t i = 0; i < nkeys; ++i) offsets[i + 1] = offsets[i] + 65 + 16LL * cnt[i];
  if (!buf) return KD_OK;  // sizes only
  if (cap < offsets[nkeys]) {
    kd_set_msg(s, "byte buffer too small");
    return KD_ERANGE;
  }
  KD_SCK(cudaMalloc(&doff.p, (size_t)(nkeys + 1) * 8));
  if (!dev) KD_SCK(cudaMalloc(&dout.p, (size_t)std::min<long long>(offsets[nkeys], kChunkBytes + 65 + 16 * KD_TILE)));
  std::vector<long long> rel((size_t)nkeys + 1);
  for (long long i0 = 0; i0 < nkeys;) {
    const long long i1 = dev ? nkeys : chunk_end(offsets, i0, nkeys);
    for (long long i = i0; i <= i1; ++i) rel[(size_t)(i - i0)] = offsets[i] - offsets[i0];
    KD_SCK(cudaMemcpyAsync(doff.p, rel.data(), (size_t)(i1 - i0 + 1) * 8, cudaMemcpyHostToDevice, str));
    uint8_t* out = dev ? buf + offsets[i0] : (uint8_t*)dout.p;
    const long long n = i1 - i0;
    const int g = (int)std::min<long long>((n * 32 + 255) / 256, (long long)s->num_sms * 16);
    k_export<<<g, 256, 0, str>>>(d, kp ? kp + i0 : nullptr, i0, n, (const long long*)doff.p, out);
    KD_SCK(cudaGetLastError());
    if (!dev)
      KD_SCK(cudaMemcpyAsync(buf + offsets[i0], out, (size_t)(offsets[i1] - offsets[i0]),
                             cudaMemcpyDeviceToHost, str));
    KD_SCK(cudaStreamSynchronize(str));
    i0 = i1;
  }
  return KD_OK;
}

static double get_f64_host(const uint8_t* p) {
  unsigned long long b = 0;
  for (int i = 0; i < 8; ++i) b |= (unsigned long long)p[i] << (8 * i);
  double v;
  memcpy(&v, &b, 8);
  return v;
}

KD_API int kd_store_import(kd_store* h, const uint32_t* keys, int64_t nkeys, const uint8_t* buf,
                           const int64_t* offsets, int flags) {
  if (!h || nkeys < 0 || (nkeys > 0 && (!buf || !offsets))) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  const KdStoreDev& d = st->d;
  const bool dev = (flags & KD_PTR_DEVICE) != 0;
  if (nkeys == 0) return KD_OK;
  if (!keys && nkeys > d.K) {
    kd_set_msg(s, "more records than the store has keys");
    return KD_EINVAL;
  }
  for (int64_t i = 0; i < nkeys; ++i)
    if (offsets[i + 1] < offsets[i]) {
      kd_set_msg(s, "offsets must be non-decreasing");
      return KD_EINVAL;
    }
  cudaSetDevice(s->device);
  cudaStream_t str = s->stream;
  KD_SCK(cudaStreamSynchronize(str));
  DevBuf dkeys, doff, dbuf, derr;
  if (!dev) {  // validate every record before any key changes
    for (int64_t i = 0; i < nkeys; ++i) {
      const int64_t len = offsets[i + 1] - offsets[i];
      const uint8_t* r = buf + offsets[i];
      char msg[160];
      if (keys && (long long)keys[i] >= d.K) {
        snprintf(msg, sizeof msg, "record %lld: key out of range [0, num_keys)", (long long)i);
        kd_set_msg(s, msg);
        return KD_EINVAL;
      }
      if (len <= 0 || r[0] != 1) {
        snprintf(msg, sizeof msg, "record %lld: unrecognized digest serialization version", (long long)i);
        kd_set_msg(s, msg);
        return KD_EINVAL;
      }
      const double c = len >= 65 ? get_f64_host(r + 57) : -1.0;
      if (len < 65 || !(c >= 0.0) || c > (double)KD_TILE || c != (double)(long long)c ||
          65 + 16 * (long long)c > len) {
        snprintf(msg, sizeof msg, "record %lld: truncated or malformed digest", (long long)i);
        kd_set_msg(s, msg);
        return KD_ERANGE;
      }
    }
  } else {
    KD_SCK(cudaMalloc(&doff.p, (size_t)(nkeys + 1) * 8));
    KD_SCK(cudaMemcpyAsync(doff.p, offsets, (size_t)(nkeys + 1) * 8, cudaMemcpyHostToDevice, str));
    KD_SCK(cudaMalloc(&derr.p, sizeof(KdErrHost)));
    KdErrHost init{0, 0, 0x7fffffffffffffffLL}, got{};
    KD_SCK(cudaMemcpyAsync(derr.p, &init, sizeof init, cudaMemcpyHostToDevice, str));
    const int g = (int)std::min<long long>((nkeys + 255) / 256, (long long)s->num_sms * 16);
    k_import_check<<<g, 256, 0, str>>>(d, keys, nkeys, buf, (const long long*)doff.p, (KdErrHost*)derr.p);
    KD_SCK(cudaMemcpyAsync(&got, derr.p, sizeof got, cudaMemcpyDeviceToHost, str));
    KD_SCK(cudaStreamSynchronize(str));
    if (got.code) {
      char msg[160];
      snprintf(msg, sizeof msg, "record %lld: malformed digest", got.index);
      kd_set_msg(s, msg);
      return got.code;
    }
  }
  // install
  const uint32_t* kp = keys;
  if (keys && !dev) {
    KD_SCK(cudaMalloc(&dkeys.p, (size_t)nkeys * 4));
    KD_SCK(cudaMemcpyAsync(dkeys.p, keys, (size_t)nkeys * 4, cudaMemcpyHostToDevice, str));
    kp = (const uint32_t*)dkeys.p;
  }
  if (dev) {
    const int g = (int)std::min<long long>((nkeys * 32 + 255) / 256, (long long)s->num_sms * 16);
    k_import<<<g, 256, 0, str>>>(d, kp, 0, nkeys, buf, (const long long*)doff.p);
    KD_SCK(cudaGetLastError());
    KD_SCK(cudaStreamSynchronize(str));
    imported(st);
    return KD_OK;
  }
  KD_SCK(cudaMalloc(&doff.p, (size_t)(nkeys + 1) * 8));
  KD_SCK(cudaMalloc(&dbuf.p, (size_t)std::min<long long>(offsets[nkeys] - offsets[0], kChunkBytes + 65 + 16 * KD_TILE)));
  std::vector<long long> rel((size_t)nkeys + 1);
  for (long long i0 = 0; i0 < nkeys;) {
    const long long i1 = chunk_end(offsets, i0, nkeys);
    for (long long i = i0; i <= i1; ++i) rel[(size_t)(i - i0)] = offsets[i] - offsets[i0];
    KD_SCK(cudaMemcpyAsync(doff.p, rel.data(), (size_t)(i1 - i0 + 1) * 8, cudaMemcpyHostToDevice, str));
    KD_SCK(cudaMemcpyAsync(dbuf.p, buf + offsets[i0], (size_t)(offsets[i1] - offsets[i0]),
                           cudaMemcpyHostToDevice, str));
    const long long n = i1 - i0;
    const int g = (int)std::min<long long>((n * 32 + 255) / 256, (long long)s->num_sms * 16);
    k_import<<<g, 256, 0, str>>>(d, kp ? kp + i0 : nullptr, i0, n, (const uint8_t*)dbuf.p,
                                 (const long long*)doff.p);
    KD_SCK(cudaGetLastError());
    KD_SCK(cudaStreamSynchronize(str));
    i0 = i1;
  }
  imported(st);
  return KD_OK;
}

}  // extern "C"
