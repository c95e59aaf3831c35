// kd_keymap.cu — device-resident dictionary from arbitrary 64-bit keys to the
// dense digest ids [0, n) a store is indexed by.
//
// The reference indexes grouped digests by dense int ids (grouped.mojo:63,
// 83-85) and leaves the mapping from application keys to them upstream.  Here
// the mapping runs on the device next to the store: an open-addressing table
// (linear probing, power-of-two size at least twice the capacity) of
// (key, id) slots.  A new key is claimed with a compare-and-swap on its slot;
// the claiming thread takes the next id from a counter and publishes it, and a
// thread that meets a claimed slot whose id is not yet published waits for it
// with a bounded spin.  Ids are dense and stable for the life of the map;
// their order among keys first seen in the same call follows the threads'
// races (a key's digest never depends on it).  One key value is reserved as
// the empty-slot marker.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <new>

#include "../../include/kdigest_gb300.h"
#include "kd_engine.h"
#include "kd_internal.cuh"

#define KD_KEYMAP_EMPTY 0xffffffffffffffffull
#define KD_KEYMAP_NOID 0xffffffffu
#define KD_KEYMAP_SPIN_LIMIT (1 << 20)

struct kd_keymap {
  KdSession* s = nullptr;
  unsigned long long* keys = nullptr;  // [size]
  unsigned* ids = nullptr;             // [size]
  unsigned long long* counter = nullptr;  // next id (counts past capacity when full)
  KdErrHost* err = nullptr;
  long long size = 0;                  // slots (power of two)
  long long capacity = 0;              // ids available
};

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  // SplitMix64 finaliser: every input bit affects every output bit
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

// Returns the id of key k (inserting it when `insert`), KD_KEYMAP_NOID when it
// is absent (lookup) or cannot be stored (the status word says why).
__device__ unsigned probe(unsigned long long* __restrict__ tk, unsigned* __restrict__ ti,
                          unsigned long long* counter, long long size, long long capacity,
                          unsigned long long k, bool insert, KdErrHost* err, long long i,
                          int spin_limit, bool stall) {
  unsigned long long h = mix64(k) & (unsigned long long)(size - 1);
  for (long long step = 0; step < size; ++step, h = (h + 1) & (unsigned long long)(size - 1)) {
    // A plain (L1-cached) read: a stale "empty" only sends the thread to the
    // compare-and-swap, which reads the slot's real value; a slot never
    // changes once it holds a key.  Hot keys then stay in every SM's L1.
    unsigned long long cur = tk[h];
    if (cur == KD_KEYMAP_EMPTY) {
      if (!insert) return KD_KEYMAP_NOID;
      cur = atomicCAS(&tk[h], KD_KEYMAP_EMPTY, k);
      if (cur == KD_KEYMAP_EMPTY) {  // claimed: take an id and publish it
        const unsigned long long id = atomicAdd(counter, 1ull);
        if (id >= (unsigned long long)capacity) {
          if (atomicCAS(&err->code, 0, KD_ENOMEM) == 0) err->index = i;
          atomicExch(&ti[h], KD_KEYMAP_NOID - 1);  // published as "no id"
          return KD_KEYMAP_NOID;
        }
        if (stall) return (unsigned)id;  // tests only: the id is never published
        __threadfence();
        atomicExch(&ti[h], (unsigned)id);
        return (unsigned)id;
      }
    }
    if (cur == k) {  // present: wait (bounded) until its id is published
      const unsigned id0 = ti[h];  // a published id never changes
      if (id0 == KD_KEYMAP_NOID - 1) {
        if (insert && atomicCAS(&err->code, 0, KD_ENOMEM) == 0) err->index = i;
        return KD_KEYMAP_NOID;
      }
      if (id0 != KD_KEYMAP_NOID) return id0;
      for (int spin = 0; spin < spin_limit; ++spin) {
        const unsigned id = *(volatile unsigned*)&ti[h];
        if (id == KD_KEYMAP_NOID - 1) {  // stored when the map was already full
          if (insert && atomicCAS(&err->code, 0, KD_ENOMEM) == 0) err->index = i;
          return KD_KEYMAP_NOID;
        }
        if (id != KD_KEYMAP_NOID) return id;
        if (spin >= 64) __nanosleep(64);  // let the claiming thread run
      }
      if (atomicCAS(&err->code, 0, KD_ETIMEOUT) == 0) err->index = i;
      return KD_KEYMAP_NOID;
    }
  }
  if (insert && atomicCAS(&err->code, 0, KD_ENOMEM) == 0) err->index = i;
  return KD_KEYMAP_NOID;
}

__global__ void k_keymap(unsigned long long* tk, unsigned* ti, unsigned long long* counter,
                         long long size,
                         long long capacity, const unsigned long long* __restrict__ in, long long n,
                         unsigned* __restrict__ out, int insert, KdErrHost* err, int spin_limit,
                         int stall_first) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = in[i];
    if (k == KD_KEYMAP_EMPTY) {  // the reserved marker cannot be a key
      if (atomicCAS(&err->code, 0, KD_EINVAL) == 0) err->index = i;
      out[i] = KD_KEYMAP_NOID;
      continue;
    }
    // tests only: the key of input 0 is claimed without its id being published
    out[i] = probe(tk, ti, counter, size, capacity, k, insert != 0, err, i, spin_limit,
                   stall_first && k == in[0]);
  }
}

int run(kd_keymap* m, const uint64_t* keys, int64_t n, uint32_t* ids, int flags, bool insert) {
  KdSession* s = m->s;
  if (n < 0 || (n > 0 && (!keys || !ids))) return KD_EINVAL;
  if (n == 0) return KD_OK;
  cudaSetDevice(s->device);
  cudaStream_t str = s->stream;
  const bool dev = (flags & KD_PTR_DEVICE) != 0;
  const unsigned long long* dk = (const unsigned long long*)keys;
  unsigned* dout = ids;
  void* tmp = nullptr;
  if (!dev) {
    if (cudaMalloc(&tmp, (size_t)n * 12) != cudaSuccess) {
      cudaGetLastError();
      kd_set_msg(s, "key map staging allocation failed");
      return KD_ENOMEM;
    }
  }
  KdErrHost init{0, 0, -1}, got{};
  cudaError_t e = cudaSuccess;
  if (!dev) e = cudaMemcpyAsync(tmp, keys, (size_t)n * 8, cudaMemcpyHostToDevice, str);
  if (!dev) {
    dk = (const unsigned long long*)tmp;
    dout = (unsigned*)((char*)tmp + (size_t)n * 8);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->err, &init, sizeof init, cudaMemcpyHostToDevice, str);
  if (e == cudaSuccess) {
    const int grid = (int)std::min<long long>((n + 255) / 256, (long long)s->num_sms * 16);
    const int spin_limit = s->wait_test > 0 ? s->wait_test : KD_KEYMAP_SPIN_LIMIT;
    k_keymap<<<grid, 256, 0, str>>>(m->keys, m->ids, m->counter, m->size, m->capacity, dk, n,
                                    dout, insert ? 1 : 0, m->err, spin_limit,
                                    s->wait_test > 0 && insert ? 1 : 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&got, m->err, sizeof got, cudaMemcpyDeviceToHost, str);
  if (e == cudaSuccess && !dev)
    e = cudaMemcpyAsync(ids, dout, (size_t)n * 4, cudaMemcpyDeviceToHost, str);
  const cudaError_t es = cudaStreamSynchronize(str);
  if (e == cudaSuccess) e = es;
  if (tmp) cudaFree(tmp);
  if (e != cudaSuccess) return kd_cuda_fail(s, e, "key map");
  if (got.code) {
    char msg[160];
    snprintf(msg, sizeof msg,
             got.code == KD_ENOMEM ? "key map full (key %lld)"
             : got.code == KD_EINVAL ? "key %lld is the reserved empty-slot marker"
                                     : "key map wait gave up (key %lld)",
             got.index);
    kd_set_msg(s, msg);
    return got.code;
  }
  return KD_OK;
}

}  // namespace

extern "C" {

KD_API int kd_keymap_create(kd_session* h, int64_t capacity, kd_keymap** out) {
  if (!h || !out || capacity <= 0 || capacity > 0x7fffffffLL) return KD_EINVAL;
  *out = nullptr;
  KdSession* s = &h->s;
  cudaSetDevice(s->device);
  long long size = 16;
  while (size < 2 * capacity) size <<= 1;
  kd_keymap* m = new (std::nothrow) kd_keymap();
  if (!m) return KD_ENOMEM;
  m->s = s;
  m->size = size;
  m->capacity = capacity;
  const size_t bytes = (size_t)size * 12 + 64;
  if (s->mem_budget && s->mem_used + bytes > s->mem_budget) {
    delete m;
    kd_set_msg(s, "device-memory budget exceeded by the key map");
    return KD_ENOMEM;
  }
  bool ok = cudaMalloc(&m->keys, (size_t)size * 8) == cudaSuccess &&
            cudaMalloc(&m->ids, (size_t)size * 4) == cudaSuccess &&
            cudaMalloc(&m->counter, 8) == cudaSuccess &&
            cudaMalloc(&m->err, sizeof(KdErrHost)) == cudaSuccess;
  if (ok) {
    ok = cudaMemsetAsync(m->keys, 0xff, (size_t)size * 8, s->stream) == cudaSuccess &&
         cudaMemsetAsync(m->ids, 0xff, (size_t)size * 4, s->stream) == cudaSuccess &&
         cudaMemsetAsync(m->counter, 0, 8, s->stream) == cudaSuccess &&
         cudaStreamSynchronize(s->stream) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    if (m->keys) cudaFree(m->keys);
    if (m->ids) cudaFree(m->ids);
    if (m->counter) cudaFree(m->counter);
    if (m->err) cudaFree(m->err);
    delete m;
    kd_set_msg(s, "key map allocation failed");
    return KD_ENOMEM;
  }
  s->mem_used += bytes;
  s->keymaps.push_back(m);
  *out = m;
  return KD_OK;
}

KD_API int kd_keymap_map(kd_keymap* m, const uint64_t* keys, int64_t n, uint32_t* ids, int flags) {
  if (!m || !m->s) return KD_EINVAL;
  return run(m, keys, n, ids, flags, true);
}

KD_API int kd_keymap_lookup(kd_keymap* m, const uint64_t* keys, int64_t n, uint32_t* ids,
                            int flags) {
  if (!m || !m->s) return KD_EINVAL;
  return run(m, keys, n, ids, flags, false);
}

KD_API int64_t kd_keymap_size(kd_keymap* m) {
  if (!m || !m->s) return -1;
  cudaSetDevice(m->s->device);
  unsigned long long c = 0;
  cudaStreamSynchronize(m->s->stream);
  if (cudaMemcpy(&c, m->counter, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return (int64_t)std::min<unsigned long long>(c, (unsigned long long)m->capacity);
}

KD_API void kd_keymap_destroy(kd_keymap* m) {
  if (!m) return;
  if (m->s) {
    KdSession* s = m->s;
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    s->keymaps.erase(std::remove(s->keymaps.begin(), s->keymaps.end(), m), s->keymaps.end());
    kd_keymap_orphan(m);
  }
  delete m;
}

}  // extern "C"

void kd_keymap_orphan(kd_keymap* m) {
  KdSession* s = m->s;
  if (!s) return;
  s->mem_used -= std::min(s->mem_used, (size_t)m->size * 12 + 64);
  cudaFree(m->keys);
  cudaFree(m->ids);
  cudaFree(m->counter);
  cudaFree(m->err);
  m->keys = nullptr;
  m->ids = nullptr;
  m->counter = nullptr;
  m->err = nullptr;
  m->s = nullptr;
}
