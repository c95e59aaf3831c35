// kd_noalloc.cu — P-path compress that allocates nothing.
//
// Some callers cannot call cudaMalloc.  A host program that owns every byte of
// device memory through its own pool (a query engine or an ML framework with
// a fixed budget) may leave no room for a library to allocate behind its back,
// and memory taken that way escapes its accounting.  A latency-critical loop
// cannot afford cudaMalloc/cudaFree either, because they can synchronise the
// whole device and stall the caller's other streams.  kd_compress_noalloc serves
// such callers: it runs the same kernels as kd_compress, on working memory
// taken from one fixed array in this library's device image.
//
// The array (kd_noalloc_scratch, KD_NOALLOC_SCRATCH_BYTES) exists on every GPU
// on which the library's device code is loaded, and stays there until the
// process exits.  It bounds a call to KD_NOALLOC_MAX_N input centroids; larger
// calls are rejected with KD_ERANGE.  The caller still provides the input and
// output arrays.
//
// Set-up: the first call on a device (that device current) resolves the
// array's device address with cudaGetSymbolAddress and sets the kernels'
// shared-memory attributes; make that first call before any stream capture.
//
// Sharing: every call on a device uses the same array, and the array keeps the
// last call's contents.  Each call clears what the pipeline needs to start at
// zero and waits for its own GPU work before it returns, so calls made one
// after another are independent.  Calls whose GPU work overlaps (several host
// threads calling at once on one device) race on the array and return wrong
// results.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/kdigest_gb300.h"
#include "kd_engine.h"
#include "kd_internal.cuh"
#include "kd_math.h"
#include "kd_scan.cuh"
#include "kd_sort.cuh"

// In host code this name is only a handle for the runtime's symbol lookup, not a
// device address: the address comes from cudaGetSymbolAddress at set-up.
static __device__ __align__(256) unsigned char kd_noalloc_scratch[KD_NOALLOC_SCRATCH_BYTES];

namespace {

// Fixed capacities of the carved workspace: one key, at most KD_NOALLOC_MAX_N
// input centroids.  A level's dense input never exceeds its predecessor's, so
// the level-0 bounds hold at every level.
constexpr long long kN = KD_NOALLOC_MAX_N;
constexpr long long kTiles = (kN + KD_TILE - 1) / KD_TILE;
constexpr long long kKeys = 32;             // touched-key arrays (one key is used)
constexpr long long kWork = kTiles + 16;    // work tiles per level
constexpr long long kInter = kTiles + 8;    // intermediate tiles per level
constexpr long long kMerged = kN + KD_TILE; // dense elements per level

struct Carver {
  uintptr_t base;
  size_t off = 0;
  template <class T>
  T* take(long long count) {
    off = (off + 255) & ~(size_t)255;
    T* p = reinterpret_cast<T*>(base + off);
    off += sizeof(T) * (size_t)count;
    return p;
  }
};

// Carves the workspace, the 1-key store and the host-input staging area out of
// the array at `base`; returns the bytes used.
size_t carve(uintptr_t base, KdWorkspace& w, KdStoreDev& d, double** stage) {
  Carver c{base};
  *stage = c.take<double>(2 * kN);
  for (int i = 0; i < 2; ++i) {
    w.k64[i] = c.take<uint64_t>(kN);
    w.key[i] = c.take<uint32_t>(kN);
    w.idx[i] = c.take<uint32_t>(kN);
    w.work[2 * i] = c.take<int2>(kWork);
    w.work[2 * i + 1] = c.take<int2>(kWork);
    w.dx[i] = c.take<double>(kMerged);
    w.dw[i] = c.take<double>(kMerged);
  }
  w.ghist = c.take<unsigned>(KD_RS_MAXPASS * 256);
  w.cap_rs_tiles = kd_rs_blocks(kN);
  w.rs_state = c.take<unsigned long long>(256 * w.cap_rs_tiles);
  w.rs_ticket = c.take<unsigned long long>(1);
  w.rs_epoch_base = c.take<unsigned>(1);
  w.cap_partials = kd_scan_partials_needed(kN) + 4;
  w.partials = c.take<int4>(w.cap_partials);
  w.tkey = c.take<uint32_t>(kKeys);
  w.tstart = c.take<int>(kKeys);
  w.tm = c.take<int>(kKeys);
  w.tprior = c.take<int>(kKeys);
  w.tbuf = c.take<unsigned char>(kKeys);
  w.tsf = c.take<double>(kKeys);
  w.tpscale = c.take<double>(kKeys);
  w.tmap = c.take<uint32_t>(1);
  w.st_clock = c.take<double>(kKeys);
  w.st_ls = c.take<double>(kKeys);
  w.st_min = c.take<double>(kKeys);
  w.st_max = c.take<double>(kKeys);
  w.st_count = c.take<int>(kKeys);
  int* lvp = c.take<int>(kKeys * 8 * 2 + 64);
  w.scr_m = c.take<double>(KD_TILE * kInter);
  w.scr_w = c.take<double>(KD_TILE * kInter);
  w.tcount = c.take<int>(kInter);
  w.doff = c.take<int>(kInter + 1);
  w.needs = c.take<int>(4);
  w.cap_fix = kN;  // every element fits the repair list (runs longer than
                   // KD_PACK_RUN_MAX still take the full sort, as on the session path)
  w.fix = c.take<int>(w.cap_fix + 1);
  w.totals = c.take<int4>(8);
  w.d_call = c.take<KdCallArgs>(1);
  w.err = &w.d_call->err;
  // Per level: eight per-key arrays, then five device scalars per level.
  for (int i = 0; i < 2; ++i) {
    KdLevelDev& L = w.lv[i];
    L.j = lvp; lvp += kKeys;
    L.src_base = lvp; lvp += kKeys;
    L.src_tiles = lvp; lvp += kKeys;
    L.mprev = lvp; lvp += kKeys;
    L.m = lvp; lvp += kKeys;
    L.base = lvp; lvp += kKeys;
    L.inter_off = lvp; lvp += kKeys;
    lvp += kKeys;
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
  w.cap_n = kN;
  w.cap_keys = kKeys;
  w.cap_inter = kInter;
  w.cap_work = kWork;
  w.cap_merged = kMerged;
  w.cap_tmap = 1;
  w.rs_epochs_used = 0;
  // The 1-key store: two centroid slots, the quantile prefix and a 64-byte
  // header block (cur, count, total, log_scale, clock, min, max, dfac).
  d.K = 1;
  d.slot_m = c.take<double>(2 * KD_TILE);
  d.slot_w = c.take<double>(2 * KD_TILE);
  d.prefix = c.take<double>(KD_TILE);
  unsigned char* hdr = c.take<unsigned char>(64);
  d.cur = hdr;
  d.count = reinterpret_cast<int*>(hdr + 4);
  d.total = reinterpret_cast<double*>(hdr + 8);
  d.log_scale = reinterpret_cast<double*>(hdr + 16);
  d.clock = reinterpret_cast<double*>(hdr + 24);
  d.min_v = reinterpret_cast<double*>(hdr + 32);
  d.max_v = reinterpret_cast<double*>(hdr + 40);
  d.dfac = reinterpret_cast<double*>(hdr + 48);
  return c.off;
}

struct DeviceSlot {
  std::atomic<bool> ready{false};
  uintptr_t base = 0;
  int num_sms = 0;
};
constexpr int kMaxDevices = 64;
DeviceSlot g_dev[kMaxDevices];
std::mutex g_setup;

int say(char* msg, int cap, int code, const char* text) {
  if (msg && cap > 0) snprintf(msg, (size_t)cap, "%s", text);
  return code;
}

int say_cuda(char* msg, int cap, cudaError_t e, const char* what) {
  if (msg && cap > 0) snprintf(msg, (size_t)cap, "%s: %s", what, cudaGetErrorString(e));
  return KD_ECUDA;
}

// Once per device, with that device current.
int setup_device(int dev, char* msg, int cap) {
  DeviceSlot& slot = g_dev[dev];
  if (slot.ready.load(std::memory_order_acquire)) return KD_OK;
  std::lock_guard<std::mutex> lock(g_setup);
  if (slot.ready.load(std::memory_order_relaxed)) return KD_OK;
  void* ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, kd_noalloc_scratch);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return say_cuda(msg, cap, e, "cudaGetSymbolAddress(kd_noalloc_scratch)");
  }
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return say_cuda(msg, cap, e, "cudaDeviceGetAttribute");
  KdWorkspace w;
  KdStoreDev d{};
  double* stage = nullptr;
  if (carve((uintptr_t)ptr, w, d, &stage) > (size_t)KD_NOALLOC_SCRATCH_BYTES)
    return say(msg, cap, KD_ENOMEM, "no-allocation scratch layout exceeds its fixed array");
  KdSession s;
  s.device = dev;
  int rc = kd_pipeline_prepare_device(&s);
  if (rc) return say(msg, cap, rc, s.last_error);
  slot.base = (uintptr_t)ptr;
  slot.num_sms = sms;
  slot.ready.store(true, std::memory_order_release);
  return KD_OK;
}

}  // namespace

#define KD_NA_CK(call)                                              \
  do {                                                              \
    cudaError_t e_ = (call);                                        \
    if (e_ != cudaSuccess) return say_cuda(msg, msg_cap, e_, #call); \
  } while (0)

extern "C" {

KD_API int kd_compress_noalloc(int scale, double compression, const double* means,
                               const double* weights, int64_t n, int flags, double* out_means,
                               double* out_weights, int64_t cap, int64_t* out_n, void* stream,
                               char* msg, int msg_cap) {
  if (msg && msg_cap > 0) msg[0] = '\0';
  if (out_n) *out_n = 0;
  if (scale < KD_K0 || scale > KD_K3) return say(msg, msg_cap, KD_EINVAL, "unknown scale function");
  if (!(compression > 0.0) || !kd_isfinite(compression))
    return say(msg, msg_cap, KD_EINVAL, "compression must be positive and finite");
  if (n < 0 || (n > 0 && (!means || !weights))) return say(msg, msg_cap, KD_EINVAL, "null input arrays");
  if (n > KD_NOALLOC_MAX_N) {
    char buf[160];
    snprintf(buf, sizeof buf,
             "%lld centroids exceed the no-allocation limit of %d per call (KD_NOALLOC_MAX_N)",
             (long long)n, KD_NOALLOC_MAX_N);
    return say(msg, msg_cap, KD_ERANGE, buf);
  }
  if (n == 0) return KD_OK;
  {
    // Every call synchronises its stream and reads results back through
    // pageable host memory, which a stream capture cannot hold: refuse before
    // touching the stream, so that the caller's capture stays valid.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    KD_NA_CK(cudaStreamIsCapturing((cudaStream_t)stream, &cs));
    if (cs != cudaStreamCaptureStatusNone)
      return say(msg, msg_cap, KD_EINVAL, "kd_compress_noalloc cannot be captured in a CUDA graph");
  }
  int dev = 0;
  KD_NA_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return say(msg, msg_cap, KD_EINVAL, "device ordinal beyond the no-allocation table (64 devices)");
  int rc = setup_device(dev, msg, msg_cap);
  if (rc) return rc;

  KdSession s;  // plain host object on the stack: no device or heap memory
  s.device = dev;
  s.use_graphs = 0;  // instantiating a CUDA graph would allocate
  s.stream = (cudaStream_t)stream;
  s.num_sms = g_dev[dev].num_sms;
  KdStore st;
  st.sess = &s;
  double* stage = nullptr;
  KdWorkspace& w = s.ws;
  carve(g_dev[dev].base, w, st.d, &stage);
  st.d.scale = scale;
  st.d.compression = compression;
  st.d.lambda = 0.0;
  KdCallArgs h_call{};
  int h_scalars[64] = {};
  w.h_call = &h_call;
  w.h_err = &h_call.err;
  w.h_scalars = h_scalars;

  cudaStream_t str = s.stream;
  // What must start at zero: the store header (slot selector, counts) and the
  // sort's look-back words with their epoch base, whose count restarts at zero
  // every call.
  KD_NA_CK(cudaMemsetAsync(st.d.cur, 0, 64, str));
  KD_NA_CK(cudaMemsetAsync(w.rs_state, 0, sizeof(unsigned long long) * 256 * (size_t)w.cap_rs_tiles, str));
  KD_NA_CK(cudaMemsetAsync(w.rs_epoch_base, 0, sizeof(unsigned), str));
  const double* dm = means;
  const double* dw = weights;
  if (!(flags & KD_PTR_DEVICE)) {
    KD_NA_CK(cudaMemcpyAsync(stage, means, (size_t)n * 8, cudaMemcpyHostToDevice, str));
    KD_NA_CK(cudaMemcpyAsync(stage + n, weights, (size_t)n * 8, cudaMemcpyHostToDevice, str));
    dm = stage;
    dw = stage + n;
  }
  rc = kd_pipeline_attempt(&s, &st, w, nullptr, dm, dw, n, KD_MODE_REPLACE, 0.0, nullptr, nullptr,
                           nullptr);
  // Not expected for n <= KD_NOALLOC_MAX_N (no level's input exceeds the
  // previous level's); reported rather than computed wrongly if it happened.
  if (rc == KD_ERANGE_SCRATCH_INTERNAL)
    return say(msg, msg_cap, KD_ENOMEM, "input needs more working memory than the fixed array holds");
  if (rc) return say(msg, msg_cap, rc, s.last_error);
  unsigned char cur = 0;
  int cnt = 0;
  KD_NA_CK(cudaMemcpyAsync(&cur, st.d.cur, 1, cudaMemcpyDeviceToHost, str));
  KD_NA_CK(cudaMemcpyAsync(&cnt, st.d.count, 4, cudaMemcpyDeviceToHost, str));
  KD_NA_CK(cudaStreamSynchronize(str));
  if (out_n) *out_n = cnt;
  if (cap < cnt) return say(msg, msg_cap, KD_ERANGE, "output capacity too small");
  const size_t off = (size_t)cur * KD_TILE;
  const cudaMemcpyKind kind = (flags & KD_PTR_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (cnt > 0) {
    KD_NA_CK(cudaMemcpyAsync(out_means, st.d.slot_m + off, (size_t)cnt * 8, kind, str));
    KD_NA_CK(cudaMemcpyAsync(out_weights, st.d.slot_w + off, (size_t)cnt * 8, kind, str));
  }
  KD_NA_CK(cudaStreamSynchronize(str));
  return KD_OK;
}

}  // extern "C"
