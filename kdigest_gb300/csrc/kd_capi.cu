// kd_capi.cu — C-ABI of the engine: sessions, resident stores, workspaces,
// host<->device staging and the to_bytes/from_bytes wire format.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/kdigest_gb300.h"
#include "kd_engine.h"
#include "kd_internal.cuh"
#include "kd_scan.cuh"
#include "kd_sort.cuh"


#define KD_CK(call)                                           \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return kd_cuda_fail(s, e_, #call); \
  } while (0)

static int fail(KdSession* s, int code, const char* msg) {
  kd_set_msg(s, msg);
  return code;
}

// ---------------------------------------------------------------------------
// Device memory accounting against the session budget
// ---------------------------------------------------------------------------
static int dalloc(KdSession* s, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  if (s->mem_budget && s->mem_used + bytes > s->mem_budget) {
    char buf[200];
    snprintf(buf, sizeof buf, "device-memory budget exceeded (%zu + %zu > %zu bytes)", s->mem_used,
             bytes, s->mem_budget);
    kd_set_msg(s, buf);
    return KD_ENOMEM;
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(s, KD_ENOMEM, "cudaMalloc failed");
  }
  s->mem_used += bytes;
  return KD_OK;
}
static void dfree(KdSession* s, void* p, size_t bytes) {
  if (!p) return;
  cudaFree(p);
  if (bytes == 0) bytes = 16;
  s->mem_used -= std::min(s->mem_used, bytes);
}
int kd_dalloc(KdSession* s, void** p, size_t bytes) { return dalloc(s, p, bytes); }
void kd_dfree(KdSession* s, void* p, size_t bytes) { dfree(s, p, bytes); }

void kd_ws_free(KdWorkspace& w) {
  void* ptrs[] = {w.k64[0], w.k64[1], w.key[0], w.key[1], w.idx[0], w.idx[1], w.ghist,
                  w.rs_state, w.rs_ticket, w.partials,
                  w.tkey, w.tstart, w.tm, w.tprior, w.tbuf, w.tsf, w.tpscale, w.tmap,
                  w.st_clock, w.st_ls, w.st_min, w.st_max, w.st_count, w.lv_storage,
                  w.work[0], w.work[1], w.work[2], w.work[3], w.dx[0], w.dx[1], w.dw[0], w.dw[1], w.scr_m, w.scr_w,
                  w.tcount, w.doff, w.needs, w.totals, w.d_call, w.rs_epoch_base, w.fix,
                  w.kfirst, w.kstamp, w.kepoch, w.chain};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (w.h_call) cudaFreeHost(w.h_call);
  if (w.h_scalars) cudaFreeHost(w.h_scalars);
  if (w.h_stage) cudaFreeHost(w.h_stage);
  // the host-call staging buffer is owned separately (stage_in / session destroy)
  void* d_in = w.d_in;
  size_t d_in_bytes = w.d_in_bytes;
  w = KdWorkspace();
  w.d_in = d_in;
  w.d_in_bytes = d_in_bytes;
}

static size_t ws_bytes(long long n, long long keys, long long inter, long long work,
                       long long merged, long long tmap, long long partials) {
  size_t b = 0;
  b += (size_t)n * (8 + 8 + 4 + 4 + 4 + 4);
  b += (size_t)kd_rs_blocks(n) * 256 * 8 + KD_RS_MAXPASS * 256 * 4 + 8;
  b += (size_t)partials * sizeof(int4);
  b += (size_t)keys * (4 * 4 + 1 + 8 * 6) + (size_t)keys * 8 * 4 * 2;
  b += (size_t)tmap * (4 + 4 + 8) + 8 + 4;
  b += (size_t)work * 8 * 4;
  b += (size_t)merged * 16 * 2;
  b += (size_t)inter * (KD_TILE * 16 + 8);
  b += sizeof(KdCallArgs) + sizeof(unsigned) + sizeof(int) * (KD_FIX_CAP + 1);
  return b;
}

int kd_ws_reserve(KdSession* s, long long n, long long keys, long long inter, long long work,
                  long long merged, long long tmap, KdWorkspace* wp) {
  KdWorkspace& w = wp ? *wp : s->ws;
  if (w.err && n <= w.cap_n && keys <= w.cap_keys && inter <= w.cap_inter && work <= w.cap_work &&
      merged <= w.cap_merged && tmap <= w.cap_tmap)
    return KD_OK;
  const auto t_grow = std::chrono::steady_clock::now();
  struct GrowTimer {  // counts the (re)allocation and its host time, however it ends
    KdSession* s;
    std::chrono::steady_clock::time_point t0;
    ~GrowTimer() {
      ++s->ws_grows;
      s->ws_grow_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
  } grow_timer{s, t_grow};
  long long nn = std::max(n, w.cap_n), kk = std::max(keys, w.cap_keys);
  long long ii = std::max(inter, w.cap_inter), ww = std::max(work, w.cap_work);
  long long mm = std::max(merged, w.cap_merged), tt = std::max(tmap, w.cap_tmap);
  // Callers size every capacity from one doubled batch capacity when a batch
  // outgrows the workspace (kd_ws_batch_cap), so a run of ever larger batches
  // reallocates once per doubling; each reallocation frees the old buffers,
  // which waits for the device.
  if (nn > w.cap_n && w.cap_n > 0) nn = std::max(nn, std::min<long long>(2 * w.cap_n, (1LL << 31) - 1));
  nn = std::max<long long>(nn, 4096);
  kk = std::max<long long>(kk, 64);
  ii = std::max<long long>(ii, 64);
  ww = std::max<long long>(ww, 128);
  mm = std::max<long long>(mm, 8192);
  tt = std::max<long long>(tt, 1);
  size_t old_bytes = w.err ? ws_bytes(w.cap_n, w.cap_keys, w.cap_inter, w.cap_work, w.cap_merged,
                                      w.cap_tmap, w.cap_partials)
                           : 0;
  kd_ws_free(w);
  s->mem_used -= std::min(s->mem_used, old_bytes);
  // room for a one-item-per-thread scan over the keys as well as the default one over the samples
  long long parts = std::max(kd_scan_partials_needed(nn), kd_scan_partials_needed(kk, 1)) + 4;
  size_t need = ws_bytes(nn, kk, ii, ww, mm, tt, parts);
  if (s->mem_budget && s->mem_used + need > s->mem_budget) {
    char buf[200];
    snprintf(buf, sizeof buf, "device-memory budget exceeded by the ingest workspace (%zu bytes)", need);
    kd_set_msg(s, buf);
    return KD_ENOMEM;
  }
  auto A = [&](void** p, size_t bytes) -> bool {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
      cudaGetLastError();
      *p = nullptr;
      return false;
    }
    return true;
  };
  bool ok = true;
  for (int i = 0; i < 2; ++i) {
    ok &= A((void**)&w.k64[i], sizeof(uint64_t) * nn);
    ok &= A((void**)&w.key[i], sizeof(uint32_t) * nn);
    ok &= A((void**)&w.idx[i], sizeof(uint32_t) * nn);
    ok &= A((void**)&w.work[2 * i], sizeof(int2) * ww);
    ok &= A((void**)&w.work[2 * i + 1], sizeof(int2) * ww);
    ok &= A((void**)&w.dx[i], sizeof(double) * mm);
    ok &= A((void**)&w.dw[i], sizeof(double) * mm);
  }
  ok &= A((void**)&w.ghist, sizeof(unsigned) * KD_RS_MAXPASS * 256);
  ok &= A((void**)&w.rs_state, sizeof(unsigned long long) * 256 * (size_t)kd_rs_blocks(nn));
  ok &= A((void**)&w.rs_ticket, sizeof(unsigned long long));
  ok &= A((void**)&w.rs_epoch_base, sizeof(unsigned));
  if (ok) {
    cudaMemset(w.rs_state, 0, sizeof(unsigned long long) * 256 * (size_t)kd_rs_blocks(nn));
    cudaMemset(w.rs_epoch_base, 0, sizeof(unsigned));
    w.cap_rs_tiles = kd_rs_blocks(nn);
    w.rs_epochs_used = 0;
  }
  ok &= A((void**)&w.partials, sizeof(int4) * parts);
  ok &= A((void**)&w.tkey, sizeof(uint32_t) * kk);
  ok &= A((void**)&w.tstart, sizeof(int) * kk);
  ok &= A((void**)&w.tm, sizeof(int) * kk);
  ok &= A((void**)&w.tprior, sizeof(int) * kk);
  ok &= A((void**)&w.tbuf, kk);
  ok &= A((void**)&w.tsf, sizeof(double) * kk);
  ok &= A((void**)&w.tpscale, sizeof(double) * kk);
  ok &= A((void**)&w.tmap, sizeof(uint32_t) * tt);
  ok &= A((void**)&w.kfirst, sizeof(int) * tt);
  ok &= A((void**)&w.kstamp, sizeof(unsigned long long) * tt);
  ok &= A((void**)&w.kepoch, sizeof(unsigned long long));
  ok &= A((void**)&w.chain, sizeof(int));
  if (ok) {  // no key carries a stamp; the first step's epoch is 1
    cudaMemset(w.kstamp, 0, sizeof(unsigned long long) * tt);
    cudaMemset(w.kepoch, 0, sizeof(unsigned long long));
  }
  ok &= A((void**)&w.st_clock, sizeof(double) * kk);
  ok &= A((void**)&w.st_ls, sizeof(double) * kk);
  ok &= A((void**)&w.st_min, sizeof(double) * kk);
  ok &= A((void**)&w.st_max, sizeof(double) * kk);
  ok &= A((void**)&w.st_count, sizeof(int) * kk);
  ok &= A((void**)&w.lv_storage, sizeof(int) * (kk * 8 * 2 + 64));
  ok &= A((void**)&w.scr_m, sizeof(double) * KD_TILE * ii);
  ok &= A((void**)&w.scr_w, sizeof(double) * KD_TILE * ii);
  ok &= A((void**)&w.tcount, sizeof(int) * ii);
  ok &= A((void**)&w.doff, sizeof(int) * (ii + 1));
  ok &= A((void**)&w.needs, sizeof(int) * 4);
  ok &= A((void**)&w.fix, sizeof(int) * (KD_FIX_CAP + 1));
  ok &= A((void**)&w.totals, sizeof(int4) * 8);
  ok &= A((void**)&w.d_call, sizeof(KdCallArgs));
  ok &= cudaHostAlloc((void**)&w.h_call, sizeof(KdCallArgs), cudaHostAllocDefault) == cudaSuccess;
  ok &= cudaHostAlloc((void**)&w.h_scalars, 64 * sizeof(int), cudaHostAllocDefault) == cudaSuccess;
  if (!ok) {
    kd_ws_free(w);
    return fail(s, KD_ENOMEM, "workspace allocation failed");
  }
  w.err = &w.d_call->err;
  w.h_err = &w.h_call->err;
  static std::atomic<unsigned long long> generations{0};
  w.generation = ++generations;  // buffers moved: captured graphs are stale
  int* lvp = w.lv_storage;
  for (int i = 0; i < 2; ++i) {
    KdLevelDev& L = w.lv[i];
    L.j = lvp; lvp += kk;
    L.src_base = lvp; lvp += kk;
    L.src_tiles = lvp; lvp += kk;
    L.mprev = lvp; lvp += kk;
    L.m = lvp; lvp += kk;
    L.base = lvp; lvp += kk;
    L.inter_off = lvp; lvp += kk;
    lvp += kk;  // spare
    L.work_l = w.work[2 * i];
    L.work_s = w.work[2 * i + 1];
  }
  for (int i = 0; i < 2; ++i) {
    w.lv[i].A = lvp++;
    w.lv[i].Tl = lvp++;
    w.lv[i].Ts = lvp++;
    w.lv[i].I = lvp++;
    w.lv[i].M = lvp++;
  }
  w.cap_n = nn;
  w.cap_keys = kk;
  w.cap_inter = ii;
  w.cap_work = ww;
  w.cap_merged = mm;
  w.cap_tmap = tt;
  w.cap_partials = parts;
  w.cap_fix = KD_FIX_CAP;
  s->mem_used += need;
  return KD_OK;
}

// Device staging for host-pointer calls.
static int stage_in(KdSession* s, size_t bytes) {
  KdWorkspace& w = s->ws;
  if (w.d_in_bytes >= bytes) return KD_OK;
  if (w.d_in) dfree(s, w.d_in, w.d_in_bytes);
  w.d_in = nullptr;
  w.d_in_bytes = 0;
  size_t b = std::max(bytes, (size_t)2 * w.d_in_bytes);
  int rc = dalloc(s, &w.d_in, b);
  if (rc) return rc;
  w.d_in_bytes = b;
  return KD_OK;
}

// ---------------------------------------------------------------------------
// Store allocation
// ---------------------------------------------------------------------------
int kd_store_alloc(KdSession* s, KdStore* st) {
  KdStoreDev& d = st->d;
  const size_t K = (size_t)d.K;
  const size_t slots = 2 * K * KD_TILE;
  size_t bytes = slots * 16 + K * KD_TILE * 8 + K * (1 + 4 + 8 * 7);
  if (s->mem_budget && s->mem_used + bytes > s->mem_budget) {
    char buf[200];
    snprintf(buf, sizeof buf, "device-memory budget exceeded by a %lld-key store (%zu bytes)",
             (long long)K, bytes);
    kd_set_msg(s, buf);
    return KD_ENOMEM;
  }
  void* p[12] = {};
  size_t sz[12] = {slots * 8, slots * 8, K * KD_TILE * 8, K, K * 4, K * 8, K * 8, K * 8, K * 8, K * 8, K * 8, 0};
  for (int i = 0; i < 11; ++i) {
    if (cudaMalloc(&p[i], sz[i] ? sz[i] : 16) != cudaSuccess) {
      cudaGetLastError();
      for (int k = 0; k < i; ++k) cudaFree(p[k]);
      return fail(s, KD_ENOMEM, "store allocation failed");
    }
  }
  d.slot_m = (double*)p[0];
  d.slot_w = (double*)p[1];
  d.prefix = (double*)p[2];
  d.cur = (unsigned char*)p[3];
  d.count = (int*)p[4];
  d.total = (double*)p[5];
  d.log_scale = (double*)p[6];
  d.clock = (double*)p[7];
  d.min_v = (double*)p[8];
  d.max_v = (double*)p[9];
  d.dfac = (double*)p[10];
  cudaStream_t str = s->stream;
  cudaMemsetAsync(d.cur, 0, K, str);
  cudaMemsetAsync(d.count, 0, K * 4, str);
  cudaMemsetAsync(d.total, 0, K * 8, str);
  cudaMemsetAsync(d.log_scale, 0, K * 8, str);
  cudaMemsetAsync(d.clock, 0, K * 8, str);
  cudaMemsetAsync(d.min_v, 0, K * 8, str);
  cudaMemsetAsync(d.max_v, 0, K * 8, str);
  // dfac = 1.0 everywhere: fill via a one-off copy of a pattern
  std::vector<double> ones(std::min<size_t>(K, 1 << 20), 1.0);
  for (size_t o = 0; o < K; o += ones.size()) {
    size_t c = std::min(ones.size(), K - o);
    cudaMemcpy(d.dfac + o, ones.data(), c * 8, cudaMemcpyHostToDevice);
  }
  cudaError_t e = cudaStreamSynchronize(str);
  if (e != cudaSuccess) return kd_cuda_fail(s, e, "store init");
  st->bytes = bytes;
  s->mem_used += bytes;
  return KD_OK;
}

void kd_store_drop_graphs(KdStore* st) {
  for (KdGraphEntry& g : st->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = KdGraphEntry();
  }
  for (auto& row : st->pipe_graphs)
    for (KdGraphEntry& g : row) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g = KdGraphEntry();
    }
  st->last_eager = KdGraphKey();
  if (st->q_graph) cudaGraphExecDestroy(st->q_graph);
  st->q_graph = nullptr;
  st->q_graph_args = KdQueryArgs();
  st->q_last = KdQueryArgs();
}

void kd_store_free(KdStore* st) {
  kd_store_drop_graphs(st);
  kd_spath_free(st->sess, st);
  st->pending = false;
  st->carry = false;
  KdStoreDev& d = st->d;
  void* p[] = {d.slot_m, d.slot_w, d.prefix, d.cur, d.count, d.total, d.log_scale, d.clock,
               d.min_v, d.max_v, d.dfac};
  for (void* q : p)
    if (q) cudaFree(q);
  d.slot_m = d.slot_w = d.prefix = nullptr;
  d.cur = nullptr;
  d.count = nullptr;
  d.total = d.log_scale = d.clock = d.min_v = d.max_v = d.dfac = nullptr;
  if (st->sess) st->sess->mem_used -= std::min(st->sess->mem_used, st->bytes);
  st->bytes = 0;
}

// One-key maintenance: quantile prefix and decay factor after a direct write.
__global__ void k_fix_key(KdStoreDev s, uint32_t key) {
  const int b = s.cur[key];
  const double* w = s.slot_w + ((size_t)b * s.K + key) * KD_TILE;
  double* P = s.prefix + (size_t)key * KD_TILE;
  const int cnt = s.count[key];
  if (cnt > 0) {
    double run = KD_MUL(w[0], 0.5);
    P[0] = run;
    for (int i = 0; i + 1 < cnt; ++i) {
      run = KD_ADD(run, KD_MUL(KD_ADD(w[i], w[i + 1]), 0.5));
      P[i + 1] = run;
    }
  }
  s.dfac[key] = s.lambda > 0.0 ? kd_exp(-s.log_scale[key]) : 1.0;
}

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
extern "C" {

KD_API int kd_version(void) { return 10000; }

KD_API const char* kd_status_string(int status) {
  switch (status) {
    case KD_OK: return "ok";
    case KD_EINVAL: return "invalid argument";
    case KD_EEMPTY: return "empty digest";
    case KD_ERANGE: return "out of range";
    case KD_ECONVERGE: return "P-path did not converge";
    case KD_ENOMEM: return "out of device memory / budget";
    case KD_ECUDA: return "CUDA error";
    case KD_ETIMEOUT: return "bounded device wait timed out";
    default: return "unknown status";
  }
}

KD_API int kd_session_create(int device, size_t mem_budget, kd_session** out) {
  if (!out) return KD_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return KD_ECUDA;
  }
  if (device < 0 || device >= ndev) return KD_EINVAL;
  kd_session* h = new (std::nothrow) kd_session();
  if (!h) return KD_ENOMEM;
  KdSession* s = &h->s;
  s->device = device;
  s->mem_budget = mem_budget;
  // The session stream (and its fork for concurrent tile kernels) take the
  // device's highest priority; the sort streams of a pipelined ingest keep the
  // default.  The block scheduler then hands freed SMs to the in-order chain of
  // store updates first, and the next batch's sort fills the rest (pipelined
  // grouped ingest of 2^22-pair batches into 65,536 keys: 0.68 -> 0.64 ms per
  // batch on GB300).
  int prio_least = 0, prio_greatest = 0;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest) != cudaSuccess ||
      cudaStreamCreateWithPriority(&s->stream, cudaStreamNonBlocking, prio_greatest) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return KD_ECUDA;
  }
  if (cudaStreamCreateWithPriority(&s->side, cudaStreamNonBlocking, prio_greatest) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->join_ev, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    if (s->fork_ev) cudaEventDestroy(s->fork_ev);
    if (s->side) cudaStreamDestroy(s->side);
    cudaStreamDestroy(s->stream);
    delete h;
    return KD_ECUDA;
  }
  cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, device);
  *out = h;
  return KD_OK;
}

KD_API void kd_session_destroy(kd_session* h) {
  if (!h) return;
  KdSession* s = &h->s;
  cudaSetDevice(s->device);
  // Servers and stores still alive lose their session: servers stop and drain,
  // stores give back their device memory and become orphans (destroying them
  // later only frees their host object).
  for (kd_server* v : std::vector<kd_server*>(s->servers)) kd_server_orphan(v);
  s->servers.clear();
  cudaStreamSynchronize(s->stream);
  for (kd_keymap* m : s->keymaps) kd_keymap_orphan(m);
  s->keymaps.clear();
  for (KdStore* st : s->stores) {
    kd_store_free(st);
    st->sess = nullptr;
  }
  s->stores.clear();
  if (s->scratch_store) {
    kd_store_free(s->scratch_store);
    delete s->scratch_store;
  }
  if (s->scratch_many) {
    kd_store_free(s->scratch_many);
    delete s->scratch_many;
  }
  if (s->sl_buf) cudaFree(s->sl_buf);
  s->sl_buf = nullptr;
  if (s->ws.d_in) cudaFree(s->ws.d_in);
  s->ws.d_in = nullptr;
  kd_ws_free(s->ws);
  for (KdWorkspace& w : s->ws_more) kd_ws_free(w);
  for (cudaEvent_t e : s->pipe_ev)
    if (e) cudaEventDestroy(e);
  if (s->ahead) cudaStreamDestroy(s->ahead);
  if (s->ahead2) cudaStreamDestroy(s->ahead2);
  if (s->copy) cudaStreamDestroy(s->copy);
  for (void* p : s->d_stage)
    if (p) cudaFree(p);
  if (s->h_many) cudaFreeHost(s->h_many);
  for (int i = 0; i <= KD_NSTAGES; ++i)
    if (s->stats.ev[i]) cudaEventDestroy(s->stats.ev[i]);
  cudaEventDestroy(s->join_ev);
  cudaEventDestroy(s->fork_ev);
  cudaStreamDestroy(s->side);
  cudaStreamDestroy(s->stream);
  delete h;
}

KD_API const char* kd_last_error(kd_session* h) { return h ? h->s.last_error : "null session"; }

KD_API int kd_session_sync(kd_session* h) {
  if (!h) return KD_EINVAL;
  KdSession* s = &h->s;
  KD_CK(cudaStreamSynchronize(s->stream));
  return KD_OK;
}

KD_API void* kd_session_stream(kd_session* h) { return h ? (void*)h->s.stream : nullptr; }

KD_API int kd_session_alloc_stats(kd_session* h, int64_t* grows, double* seconds) {
  if (!h) return KD_EINVAL;
  if (grows) *grows = h->s.ws_grows;
  if (seconds) *seconds = h->s.ws_grow_s;
  return KD_OK;
}

KD_API int kd_session_stats(kd_session* h, double* stage_ms, int cap, int64_t* launches,
                            int64_t* ingests) {
  if (!h) return KD_EINVAL;
  const KdStageStats& t = h->s.stats;
  for (int i = 0; i < cap && i < KD_NSTAGES; ++i) stage_ms[i] = t.ms[i];
  if (launches) *launches = t.launches;
  if (ingests) *ingests = t.ingests;
  return KD_NSTAGES;
}

KD_API void kd_session_reset_stats(kd_session* h) {
  if (!h) return;
  KdStageStats& t = h->s.stats;
  for (int i = 0; i < KD_NSTAGES; ++i) t.ms[i] = 0.0;
  t.launches = 0;
  t.ingests = 0;
}

KD_API int kd_session_set_option(kd_session* h, int option, int value) {
  if (!h) return KD_EINVAL;
  KdSession* s = &h->s;
  if (option == KD_OPT_FORCE_EXACT_K) s->force_exact = value ? 1 : 0;
  else if (option == KD_OPT_STAGE_TIMING) {
    if (value && !s->stats.enabled) {
      for (int i = 0; i <= KD_NSTAGES; ++i)
        if (!s->stats.ev[i]) KD_CK(cudaEventCreate(&s->stats.ev[i]));
    }
    s->stats.enabled = value ? 1 : 0;
  }
  else if (option == KD_OPT_MAX_LEVELS) {
    if (value < 1 || value > 64) return fail(s, KD_EINVAL, "max levels must be in [1, 64]");
    s->max_levels = value;
  } else if (option == KD_OPT_GRAPHS) {
    s->use_graphs = value ? 1 : 0;
  } else if (option == KD_OPT_SMALL_TILE_CAP) {
    if (value < 1 || value > KD_SERIAL_TILE_MAX) return fail(s, KD_EINVAL, "small tile cap must be in [1, 128]");
    s->small_cap = value;
  } else if (option == KD_OPT_LARGE_BLOCKS_PER_SM) {
    if (value < 1 || value > 64) return fail(s, KD_EINVAL, "blocks per SM must be in [1, 64]");
    s->large_bps = value;
  } else if (option == KD_OPT_SMALL_BLOCKS_PER_SM) {
    if (value < 1 || value > 64) return fail(s, KD_EINVAL, "blocks per SM must be in [1, 64]");
    s->small_bps = value;
  } else if (option == KD_OPT_CONCURRENT_TILES) {
    s->concurrent_tiles = value ? 1 : 0;
  } else if (option == KD_OPT_FRONT_STREAMS) {
    if (value < 1 || value > 2) return fail(s, KD_EINVAL, "front streams must be 1 or 2");
    s->front_streams = value;
  } else if (option == KD_OPT_TEST_WAIT) {
    if (value < 0 || value > (1 << 22)) return fail(s, KD_EINVAL, "test wait limit must be in [0, 2^22]");
    s->wait_test = value;
  } else {
    return fail(s, KD_EINVAL, "unknown option");
  }
  return KD_OK;
}

static int valid_scale(int scale) { return scale >= KD_K0 && scale <= KD_K3; }

KD_API int kd_store_create(kd_session* h, int64_t num_keys, int scale, double compression,
                           double decay_lambda, kd_store** out) {
  if (!h || !out) return KD_EINVAL;
  KdSession* s = &h->s;
  *out = nullptr;
  if (num_keys < 1 || num_keys > (1LL << 32)) return fail(s, KD_EINVAL, "num_keys must be in [1, 2^32]");
  if (!valid_scale(scale)) return fail(s, KD_EINVAL, "unknown scale function");
  if (!(compression > 0.0) || !kd_isfinite(compression)) return fail(s, KD_EINVAL, "compression must be positive and finite");
  if (!(decay_lambda >= 0.0) || !kd_isfinite(decay_lambda)) return fail(s, KD_EINVAL, "decay rate must be >= 0 and finite");
  cudaSetDevice(s->device);
  kd_store* st = new (std::nothrow) kd_store();
  if (!st) return KD_ENOMEM;
  st->st.sess = s;
  st->st.d.K = num_keys;
  st->st.d.scale = scale;
  st->st.d.compression = compression;
  st->st.d.lambda = decay_lambda;
  int rc = kd_store_alloc(s, &st->st);
  if (rc) {
    delete st;
    return rc;
  }
  *out = st;
  s->stores.push_back(&st->st);
  return KD_OK;
}

KD_API void kd_store_destroy(kd_store* st) {
  if (!st) return;
  KdSession* s = st->st.sess;
  if (s) {  // an orphan (its session destroyed first) has no device memory left
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    s->stores.erase(std::remove(s->stores.begin(), s->stores.end(), &st->st), s->stores.end());
    kd_store_free(&st->st);
  }
  delete st;
}

// Kernel-addressable view of a host pointer, or null.  Page-locked (pinned)
// host memory is mapped into the device address space: on GB300 the kernels
// read it in place over the coherent host link, so an ingest from pinned
// buffers needs no staging copy (the bytes still cross the link once, inside
// the call).  Pageable memory returns null and is staged.
static const void* mapped_view(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

KD_API int kd_store_ingest(kd_store* h, const uint32_t* keys, const double* values, int64_t n,
                           int clock_mode, double timestamp, int flags) {
  if (!h) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  if (n < 0 || (n > 0 && !values)) return fail(s, KD_EINVAL, "values must be non-null");
  if (clock_mode != KD_CLOCK_COUNT && clock_mode != KD_CLOCK_TIME) return fail(s, KD_EINVAL, "unknown clock mode");
  if (clock_mode == KD_CLOCK_TIME && !kd_isfinite(timestamp)) return fail(s, KD_EINVAL, "timestamp must be finite");
  if (n == 0) return KD_OK;
  cudaSetDevice(s->device);
  const uint32_t* dk = keys;
  const double* dv = values;
  const void* mk = (flags & KD_PTR_DEVICE) || !keys ? nullptr : mapped_view(keys);
  const void* mv = (flags & KD_PTR_DEVICE) ? nullptr : mapped_view(values);
  if (!(flags & KD_PTR_DEVICE) && mv && (!keys || mk)) {  // pinned: read in place
    dk = (const uint32_t*)mk;
    dv = (const double*)mv;
  } else if (!(flags & KD_PTR_DEVICE)) {
    size_t kb = keys ? ((size_t)n * 4 + 15) / 16 * 16 : 0;
    int rc = stage_in(s, kb + (size_t)n * 8);
    if (rc) return rc;
    char* base = (char*)s->ws.d_in;
    if (keys) {
      KD_CK(cudaMemcpyAsync(base, keys, (size_t)n * 4, cudaMemcpyHostToDevice, s->stream));
      dk = (const uint32_t*)base;
    }
    KD_CK(cudaMemcpyAsync(base + kb, values, (size_t)n * 8, cudaMemcpyHostToDevice, s->stream));
    dv = (const double*)(base + kb);
  }
  const int mode = clock_mode == KD_CLOCK_TIME ? KD_MODE_TIME : KD_MODE_COUNT;
  if (st->carry && st->d.K == 1)  // the digest came from the single-sample path
    return kd_spath_carry_ingest(s, st, dv, n, mode, timestamp);
  return kd_pipeline_ingest(s, st, dk, dv, nullptr, n, mode, timestamp, nullptr, nullptr, nullptr);
}

KD_API int kd_store_ingest_many(kd_store* h, int64_t nbatch, const uint32_t* const* keys,
                                const double* const* values, const int64_t* n, int clock_mode,
                                const double* timestamps, int flags, int64_t* batches_done) {
  if (batches_done) *batches_done = 0;
  if (!h) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  if (nbatch < 0 || (nbatch > 0 && (!values || !n))) return fail(s, KD_EINVAL, "null batch arrays");
  if (clock_mode != KD_CLOCK_COUNT && clock_mode != KD_CLOCK_TIME) return fail(s, KD_EINVAL, "unknown clock mode");
  if (clock_mode == KD_CLOCK_TIME && nbatch > 0 && !timestamps) return fail(s, KD_EINVAL, "timestamps must be non-null");
  for (int64_t i = 0; i < nbatch; ++i) {
    if (n[i] < 0 || (n[i] > 0 && !values[i])) return fail(s, KD_EINVAL, "values must be non-null");
    if (clock_mode == KD_CLOCK_TIME && !kd_isfinite(timestamps[i])) return fail(s, KD_EINVAL, "timestamp must be finite");
  }
  if (nbatch == 0) return KD_OK;
  cudaSetDevice(s->device);
  // Device pointers are read in place; host memory (pinned or pageable) is
  // staged batch by batch by the copy engine.  A one-key digest carried from
  // the single-sample path takes one call per batch.
  const bool each = st->carry && st->d.K == 1;
  std::vector<const uint32_t*> dk((size_t)nbatch, nullptr);
  std::vector<const double*> dv((size_t)nbatch, nullptr);
  for (int64_t i = 0; i < nbatch; ++i) {
    dk[i] = keys ? keys[i] : nullptr;
    dv[i] = values[i];
  }
  if (each) {
    for (int64_t i = 0; i < nbatch; ++i) {
      const int rc = kd_store_ingest(h, keys ? keys[i] : nullptr, values[i], n[i], clock_mode,
                                     timestamps ? timestamps[i] : 0.0, flags);
      if (rc) {
        if (batches_done) *batches_done = i;
        return rc;
      }
    }
    if (batches_done) *batches_done = nbatch;
    return KD_OK;
  }
  const int mode = clock_mode == KD_CLOCK_TIME ? KD_MODE_TIME : KD_MODE_COUNT;
  long long done = 0;
  const int rc = kd_pipeline_ingest_many(s, st, nbatch, dk.data(), dv.data(), (const long long*)n, mode,
                                         clock_mode == KD_CLOCK_TIME ? timestamps : nullptr, &done,
                                         !(flags & KD_PTR_DEVICE));
  if (rc == KD_ENOMEM && done == 0) {
    // no room for the pipeline's extra buffers: one call per batch
    for (int64_t i = 0; i < nbatch; ++i) {
      const int r = kd_store_ingest(h, keys ? keys[i] : nullptr, values[i], n[i], clock_mode,
                                    timestamps ? timestamps[i] : 0.0, flags);
      if (r) {
        if (batches_done) *batches_done = i;
        return r;
      }
    }
    if (batches_done) *batches_done = nbatch;
    return KD_OK;
  }
  if (batches_done) *batches_done = done;
  return rc;
}

static int query_common(kd_store* h, const uint32_t* keys, const double* q, int64_t nq,
                        double* out, int flags, int is_cdf) {
  if (!h) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  if (nq < 0 || (nq > 0 && (!q || !out))) return fail(s, KD_EINVAL, "null query arrays");
  if (nq == 0) return KD_OK;
  cudaSetDevice(s->device);
  int frc = kd_spath_flush(s, st);  // quantile / cdf run merge() first (tdigest.mojo:493,542)
  if (frc) return frc;
  if (flags & KD_PTR_DEVICE) return kd_pipeline_quantile(s, st, keys, q, nq, out, is_cdf);
  size_t kb = keys ? ((size_t)nq * 4 + 15) / 16 * 16 : 0;
  int rc = stage_in(s, kb + (size_t)nq * 16);
  if (rc) return rc;
  char* base = (char*)s->ws.d_in;
  const uint32_t* dk = nullptr;
  if (keys) {
    KD_CK(cudaMemcpyAsync(base, keys, (size_t)nq * 4, cudaMemcpyHostToDevice, s->stream));
    dk = (const uint32_t*)base;
  }
  double* dq = (double*)(base + kb);
  double* dout = dq + nq;
  KD_CK(cudaMemcpyAsync(dq, q, (size_t)nq * 8, cudaMemcpyHostToDevice, s->stream));
  int qrc = kd_pipeline_quantile(s, st, dk, dq, nq, dout, is_cdf);
  if (qrc == KD_ECUDA) return qrc;
  KD_CK(cudaMemcpyAsync(out, dout, (size_t)nq * 8, cudaMemcpyDeviceToHost, s->stream));
  KD_CK(cudaStreamSynchronize(s->stream));
  return qrc;
}

KD_API int kd_store_quantile(kd_store* h, const uint32_t* keys, const double* qs, int64_t nq,
                             double* out, int flags) {
  return query_common(h, keys, qs, nq, out, flags, 0);
}
KD_API int kd_store_cdf(kd_store* h, const uint32_t* keys, const double* xs, int64_t nx,
                        double* out, int flags) {
  return query_common(h, keys, xs, nx, out, flags, 1);
}

KD_API int kd_store_query_batch(kd_store* h, const uint32_t* qkeys, const double* qs, int64_t nq,
                                double* qout, const uint32_t* ckeys, const double* xs, int64_t nc,
                                double* cout, int flags) {
  if (!h) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  if (nq < 0 || nc < 0 || (nq > 0 && (!qs || !qout)) || (nc > 0 && (!xs || !cout)))
    return fail(s, KD_EINVAL, "null query arrays");
  if (nq + nc == 0) return KD_OK;
  cudaSetDevice(s->device);
  int frc = kd_spath_flush(s, st);  // quantile / cdf run merge() first (tdigest.mojo:493,542)
  if (frc) return frc;
  if (flags & KD_PTR_DEVICE) return kd_pipeline_query2(s, st, qkeys, qs, nq, qout, ckeys, xs, nc, cout);
  const size_t kq = qkeys ? ((size_t)nq * 4 + 15) / 16 * 16 : 0;
  const size_t kc = ckeys ? ((size_t)nc * 4 + 15) / 16 * 16 : 0;
  int rc = stage_in(s, kq + kc + (size_t)(nq + nc) * 16);
  if (rc) return rc;
  char* base = (char*)s->ws.d_in;
  const uint32_t* dqk = nullptr;
  const uint32_t* dck = nullptr;
  if (qkeys) {
    KD_CK(cudaMemcpyAsync(base, qkeys, (size_t)nq * 4, cudaMemcpyHostToDevice, s->stream));
    dqk = (const uint32_t*)base;
  }
  if (ckeys) {
    KD_CK(cudaMemcpyAsync(base + kq, ckeys, (size_t)nc * 4, cudaMemcpyHostToDevice, s->stream));
    dck = (const uint32_t*)(base + kq);
  }
  double* dq = (double*)(base + kq + kc);
  double* dx = dq + nq;
  double* dqo = dx + nc;
  double* dco = dqo + nq;
  if (nq) KD_CK(cudaMemcpyAsync(dq, qs, (size_t)nq * 8, cudaMemcpyHostToDevice, s->stream));
  if (nc) KD_CK(cudaMemcpyAsync(dx, xs, (size_t)nc * 8, cudaMemcpyHostToDevice, s->stream));
  int qrc = kd_pipeline_query2(s, st, dqk, dq, nq, dqo, dck, dx, nc, dco);
  if (qrc == KD_ECUDA) return qrc;
  if (nq) KD_CK(cudaMemcpyAsync(qout, dqo, (size_t)nq * 8, cudaMemcpyDeviceToHost, s->stream));
  if (nc) KD_CK(cudaMemcpyAsync(cout, dco, (size_t)nc * 8, cudaMemcpyDeviceToHost, s->stream));
  KD_CK(cudaStreamSynchronize(s->stream));
  return qrc;
}

KD_API int kd_store_merge(kd_store* dst, kd_store* src, const int64_t* group_offsets,
                          const uint32_t* parts, int64_t ngroups) {
  if (!dst || !src) return KD_EINVAL;
  KdSession* s = dst->st.sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  if (src->st.sess != s) return fail(s, KD_EINVAL, "stores belong to different sessions");
  if (ngroups < 0 || (ngroups > 0 && (!group_offsets || !parts))) return fail(s, KD_EINVAL, "null group arrays");
  if (ngroups == 0) return KD_OK;
  if (group_offsets[0] != 0) return fail(s, KD_EINVAL, "group_offsets[0] must be 0");
  for (int64_t g = 0; g < ngroups; ++g)
    if (group_offsets[g + 1] < group_offsets[g]) return fail(s, KD_EINVAL, "group_offsets must be non-decreasing");
  cudaSetDevice(s->device);
  int rc = kd_pipeline_merge(s, &dst->st, &src->st, (const long long*)group_offsets, parts, ngroups);
  if (rc == KD_OK) {  // every destination digest was replaced (its buffer cleared)
    dst->st.pending = false;
    dst->st.carry = false;
  }
  return rc;
}

KD_API int kd_store_get_digest(kd_store* h, uint32_t key, double* header8, double* means,
                               double* weights, int64_t cap, int64_t* out_count) {
  if (!h) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  const KdStoreDev& d = st->d;
  if ((long long)key >= d.K) return fail(s, KD_EINVAL, "key out of range [0, num_keys)");
  cudaSetDevice(s->device);
  KD_CK(cudaStreamSynchronize(s->stream));
  unsigned char cur = 0;
  int cnt = 0;
  double ls = 0, clock = 0, total = 0, mn = 0, mx = 0;
  KD_CK(cudaMemcpy(&cur, d.cur + key, 1, cudaMemcpyDeviceToHost));
  KD_CK(cudaMemcpy(&cnt, d.count + key, 4, cudaMemcpyDeviceToHost));
  KD_CK(cudaMemcpy(&ls, d.log_scale + key, 8, cudaMemcpyDeviceToHost));
  KD_CK(cudaMemcpy(&clock, d.clock + key, 8, cudaMemcpyDeviceToHost));
  KD_CK(cudaMemcpy(&total, d.total + key, 8, cudaMemcpyDeviceToHost));
  KD_CK(cudaMemcpy(&mn, d.min_v + key, 8, cudaMemcpyDeviceToHost));
  KD_CK(cudaMemcpy(&mx, d.max_v + key, 8, cudaMemcpyDeviceToHost));
  if (header8) {
    double hdr[8] = {d.compression, d.lambda, ls, clock, total, mn, mx, (double)cnt};
    memcpy(header8, hdr, sizeof hdr);
  }
  if (out_count) *out_count = cnt;
  if (means || weights) {
    if (cap < cnt) return fail(s, KD_ERANGE, "centroid capacity too small");
    size_t off = ((size_t)cur * d.K + key) * KD_TILE;
    if (cnt > 0 && means) KD_CK(cudaMemcpy(means, d.slot_m + off, (size_t)cnt * 8, cudaMemcpyDeviceToHost));
    if (cnt > 0 && weights) KD_CK(cudaMemcpy(weights, d.slot_w + off, (size_t)cnt * 8, cudaMemcpyDeviceToHost));
  }
  return KD_OK;
}

KD_API int kd_store_set_digest(kd_store* h, uint32_t key, const double* header8,
                               const double* means, const double* weights, int64_t count) {
  if (!h || !header8) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  KdStoreDev& d = st->d;
  if ((long long)key >= d.K) return fail(s, KD_EINVAL, "key out of range [0, num_keys)");
  if (count < 0 || count > KD_TILE) return fail(s, KD_ERANGE, "a digest holds at most 1024 centroids");
  if (count > 0 && (!means || !weights)) return fail(s, KD_EINVAL, "null centroid arrays");
  cudaSetDevice(s->device);
  KD_CK(cudaStreamSynchronize(s->stream));
  unsigned char cur = 0;
  KD_CK(cudaMemcpy(&cur, d.cur + key, 1, cudaMemcpyDeviceToHost));
  size_t off = ((size_t)cur * d.K + key) * KD_TILE;
  int cnt = (int)count;
  if (cnt > 0) {
    KD_CK(cudaMemcpy(d.slot_m + off, means, (size_t)cnt * 8, cudaMemcpyHostToDevice));
    KD_CK(cudaMemcpy(d.slot_w + off, weights, (size_t)cnt * 8, cudaMemcpyHostToDevice));
  }
  KD_CK(cudaMemcpy(d.count + key, &cnt, 4, cudaMemcpyHostToDevice));
  KD_CK(cudaMemcpy(d.log_scale + key, &header8[2], 8, cudaMemcpyHostToDevice));
  KD_CK(cudaMemcpy(d.clock + key, &header8[3], 8, cudaMemcpyHostToDevice));
  KD_CK(cudaMemcpy(d.total + key, &header8[4], 8, cudaMemcpyHostToDevice));
  KD_CK(cudaMemcpy(d.min_v + key, &header8[5], 8, cudaMemcpyHostToDevice));
  KD_CK(cudaMemcpy(d.max_v + key, &header8[6], 8, cudaMemcpyHostToDevice));
  k_fix_key<<<1, 1, 0, s->stream>>>(d, key);
  KD_CK(cudaGetLastError());
  if (d.bcount) KD_CK(cudaMemsetAsync(d.bcount + key, 0, 4, s->stream));  // a new digest has no buffer
  KD_CK(cudaStreamSynchronize(s->stream));
  if (d.K == 1) {  // centroids in any order: the next batch sorts them with its samples
    st->pending = false;
    st->carry = true;
  }
  return KD_OK;
}

static void put_f64(uint8_t* p, double v) {
  uint64_t b = kd_bits(v);
  for (int i = 0; i < 8; ++i) p[i] = (uint8_t)(b >> (8 * i));
}
static double get_f64(const uint8_t* p) {
  uint64_t b = 0;
  for (int i = 0; i < 8; ++i) b |= (uint64_t)p[i] << (8 * i);
  return kd_from_bits(b);
}

KD_API int kd_store_to_bytes(kd_store* h, uint32_t key, uint8_t* buf, int64_t cap, int64_t* out_len) {
  if (!h) return KD_EINVAL;
  KdSession* s = h->st.sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  cudaSetDevice(s->device);
  int rc = kd_spath_flush(s, &h->st);  // to_bytes runs merge() first (tdigest.mojo:639)
  if (rc) return rc;
  double hdr[8];
  int64_t cnt = 0;
  rc = kd_store_get_digest(h, key, hdr, nullptr, nullptr, 0, &cnt);
  if (rc) return rc;
  const int64_t need = 1 + 8 * 8 + 16 * cnt;
  if (out_len) *out_len = need;
  if (!buf) return KD_OK;
  if (cap < need) return fail(s, KD_ERANGE, "byte buffer too small");
  std::vector<double> m(std::max<int64_t>(cnt, 1)), w(std::max<int64_t>(cnt, 1));
  rc = kd_store_get_digest(h, key, hdr, m.data(), w.data(), cnt, &cnt);
  if (rc) return rc;
  buf[0] = 1; /* serialization version (tdigest.mojo:61) */
  for (int i = 0; i < 8; ++i) put_f64(buf + 1 + 8 * i, hdr[i]);
  for (int64_t i = 0; i < cnt; ++i) {
    put_f64(buf + 65 + 16 * i, m[i]);
    put_f64(buf + 73 + 16 * i, w[i]);
  }
  return KD_OK;
}

KD_API int kd_store_from_bytes(kd_store* h, uint32_t key, const uint8_t* buf, int64_t len) {
  if (!h) return KD_EINVAL;
  KdSession* s = h->st.sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  if (len <= 0 || !buf || buf[0] != 1) return fail(s, KD_EINVAL, "unrecognized digest serialization version");
  if (len < 65) return fail(s, KD_ERANGE, "truncated digest: not enough bytes for a Float64");
  double hdr[8];
  for (int i = 0; i < 8; ++i) hdr[i] = get_f64(buf + 1 + 8 * i);
  const int64_t cnt = (int64_t)hdr[7];
  if (cnt < 0 || 65 + 16 * cnt > len) return fail(s, KD_ERANGE, "truncated digest: not enough bytes for a Float64");
  if (cnt > KD_TILE) return fail(s, KD_ERANGE, "a digest holds at most 1024 centroids");
  std::vector<double> m(std::max<int64_t>(cnt, 1)), w(std::max<int64_t>(cnt, 1));
  for (int64_t i = 0; i < cnt; ++i) {
    m[i] = get_f64(buf + 65 + 16 * i);
    w[i] = get_f64(buf + 73 + 16 * i);
  }
  return kd_store_set_digest(h, key, hdr, m.data(), w.data(), cnt);
}

KD_API int kd_store_stats(kd_store* h, int64_t* num_keys, int64_t* total_centroids, size_t* device_bytes) {
  if (!h) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  cudaSetDevice(s->device);
  if (num_keys) *num_keys = st->d.K;
  if (device_bytes) *device_bytes = st->bytes;
  if (total_centroids) {
    KD_CK(cudaStreamSynchronize(s->stream));
    std::vector<int> c((size_t)st->d.K);
    KD_CK(cudaMemcpy(c.data(), st->d.count, c.size() * 4, cudaMemcpyDeviceToHost));
    int64_t t = 0;
    for (int v : c) t += v;
    *total_centroids = t;
  }
  return KD_OK;
}

KD_API int kd_store_counts(kd_store* h, int32_t* out, int flags) {
  if (!h || !out) return KD_EINVAL;
  KdStore* st = &h->st;
  KdSession* s = st->sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  cudaSetDevice(s->device);
  KD_CK(cudaMemcpyAsync(out, st->d.count, (size_t)st->d.K * 4,
                        (flags & KD_PTR_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                        s->stream));
  KD_CK(cudaStreamSynchronize(s->stream));
  return KD_OK;
}

KD_API int kd_compress(kd_session* h, int scale, double compression, const double* means,
                       const double* weights, int64_t n, int flags, double* out_means,
                       double* out_weights, int64_t cap, int64_t* out_n) {
  if (!h) return KD_EINVAL;
  KdSession* s = &h->s;
  if (out_n) *out_n = 0;
  if (!valid_scale(scale)) return fail(s, KD_EINVAL, "unknown scale function");
  if (!(compression > 0.0) || !kd_isfinite(compression)) return fail(s, KD_EINVAL, "compression must be positive and finite");
  if (n < 0 || (n > 0 && (!means || !weights))) return fail(s, KD_EINVAL, "null input arrays");
  if (n == 0) return KD_OK;
  cudaSetDevice(s->device);
  if (!s->scratch_store) {
    KdStore* st = new (std::nothrow) KdStore();
    if (!st) return KD_ENOMEM;
    st->sess = s;
    st->d.K = 1;
    int rc = kd_store_alloc(s, st);
    if (rc) {
      delete st;
      return rc;
    }
    s->scratch_store = st;
  }
  KdStore* st = s->scratch_store;
  st->d.scale = scale;
  st->d.compression = compression;
  st->d.lambda = 0.0;
  const double* dm = means;
  const double* dw = weights;
  if (!(flags & KD_PTR_DEVICE)) {
    int rc = stage_in(s, (size_t)n * 16);
    if (rc) return rc;
    double* base = (double*)s->ws.d_in;
    KD_CK(cudaMemcpyAsync(base, means, (size_t)n * 8, cudaMemcpyHostToDevice, s->stream));
    KD_CK(cudaMemcpyAsync(base + n, weights, (size_t)n * 8, cudaMemcpyHostToDevice, s->stream));
    dm = base;
    dw = base + n;
  }
  int rc = kd_pipeline_ingest(s, st, nullptr, dm, dw, n, KD_MODE_REPLACE, 0.0, nullptr, nullptr, nullptr);
  if (rc) return rc;
  unsigned char cur = 0;
  int cnt = 0;
  KD_CK(cudaMemcpy(&cur, st->d.cur, 1, cudaMemcpyDeviceToHost));
  KD_CK(cudaMemcpy(&cnt, st->d.count, 4, cudaMemcpyDeviceToHost));
  if (out_n) *out_n = cnt;
  if (cap < cnt) return fail(s, KD_ERANGE, "output capacity too small");
  const size_t off = (size_t)cur * KD_TILE;
  cudaMemcpyKind kind = (flags & KD_PTR_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (cnt > 0) {
    KD_CK(cudaMemcpyAsync(out_means, st->d.slot_m + off, (size_t)cnt * 8, kind, s->stream));
    KD_CK(cudaMemcpyAsync(out_weights, st->d.slot_w + off, (size_t)cnt * 8, kind, s->stream));
  }
  KD_CK(cudaStreamSynchronize(s->stream));
  return KD_OK;
}

}  // extern "C"
