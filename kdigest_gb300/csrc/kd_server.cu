// kd_server.cu — serving loop over a resident store: ingest and query requests
// arrive one by one from client threads and are served by continuous batching.
//
// Semantics (deterministic in the request stream, whatever the load):
//   * requests carry non-decreasing timestamps; request r belongs to window
//     floor(ts / window) of the timestamp axis;
//   * a window's query requests are answered against the store as it was
//     before that window's ingests (so a query sees every ingest of earlier
//     windows and none of later ones);
//   * a window's ingest requests are applied as one grouped batch: their
//     samples concatenated in arrival order, every touched key's clock moving
//     to the window's last ingest timestamp (add_at semantics, time decay).
// A window closes when a request of a later window arrives, when the client
// advances the clock past its end, or on flush — never on a wall-clock timer,
// so the batches, and therefore every result, depend only on the request
// stream.  Requests that arrive while earlier windows are on the GPU are
// admitted into the open window while the session's device memory when the
// server started (store, workspaces) plus the device footprint of the requests
// buffered or in flight (staging, and their share of the ingest workspaces)
// stays within the budget.  The baseline is fixed, so a request that fits
// alone is always admitted once the queue drains.
//
// The worker takes every closed window (up to KD_SRV_GROUP) as one group and
// runs the group through the pipelined multi-batch ingest, one batch per
// window: window i + 1's prep and sort run on a side stream beside window i's
// queries, compress and commit, and each window's queries are enqueued between
// the commits of the windows before and after it.  The next group's
// host->device copy runs on a copy stream while the current group computes.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/kdigest_gb300.h"
#include "kd_engine.h"
#include "kd_math.h"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
  int64_t id = 0;
  int kind = 0;
  double ts = 0.0;
  long long window = 0;
  std::vector<uint32_t> keys;
  std::vector<double> vals;  // values, q or x
  double* out = nullptr;     // caller's output (queries)
  size_t dev_bytes = 0;      // device footprint until completion (staging, workspace share)
  int status = -1;  // -1 while pending
  double t_submit = 0.0, t_done = 0.0;
};

// Pinned host and device buffers of one staged window (two alternate).
struct Buf {
  size_t cap_i = 0, cap_q = 0;
  uint32_t *h_ik = nullptr, *d_ik = nullptr;
  double *h_iv = nullptr, *d_iv = nullptr;
  uint32_t *h_qk = nullptr, *d_qk = nullptr;
  double *h_qv = nullptr, *d_qv = nullptr, *h_qo = nullptr, *d_qo = nullptr;
  cudaEvent_t copied = nullptr;
};

// Windows a worker takes at once (each is one batch of the pipelined ingest).
#define KD_SRV_GROUP 4
// A window with more ingest pairs than this runs alone through the one-call
// ingest: the pipelined ingest sizes every workspace it uses for its largest
// batch, so a large window inside a group would grow all three (gigabytes at a
// million keys, each growth a device-wide synchronisation).
#define KD_SRV_GROUP_BIG (1LL << 18)
// Latencies kept for the percentiles: every one up to this many completions,
// then a uniform sample of this size (reservoir sampling, Algorithm R of
// Vitter, "Random sampling with a reservoir", ACM TOMS 11(1), 1985), so a
// long-running server holds a fixed 8 MB for them.
#define KD_SRV_LAT_CAP ((size_t)1 << 20)

// splitmix64: the reservoir's replacement indices (seeded, so repeatable).
uint64_t srv_rand(uint64_t& x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// One window of a staged group: its requests [r0, r1) of the group's list and
// its place in the group's buffers.
struct Win {
  long long window = 0;
  size_t r0 = 0, r1 = 0;
  long long oi = 0, n_ing = 0;           // ingest pairs at [oi, oi + n_ing)
  long long oq = 0, n_qq = 0, n_qc = 0;  // quantile pairs from oq, then the cdf pairs
  double ts = 0.0;                       // last ingest timestamp of the window
};

struct Staged {
  std::vector<std::shared_ptr<Req>> reqs;  // window by window, arrival order within
  std::vector<Win> wins;
  long long n_ing = 0, n_q = 0;
  int buf = 0;
};

void free_buf(Buf& b) {
  void* dv[] = {b.d_ik, b.d_iv, b.d_qk, b.d_qv, b.d_qo};
  for (void* p : dv)
    if (p) cudaFree(p);
  void* hv[] = {b.h_ik, b.h_iv, b.h_qk, b.h_qv, b.h_qo};
  for (void* p : hv)
    if (p) cudaFreeHost(p);
  if (b.copied) cudaEventDestroy(b.copied);
  b = Buf();
}

// Device bytes of a buffer set: ingest keys and values, query keys, values
// and results.
size_t buf_dev_bytes(const Buf& b) { return b.cap_i * 12 + b.cap_q * 20; }

// Device footprint of one request while it is buffered and served: its
// staging, and for ingest pairs the share of the ingest workspace they need
// (sort buffers, dense level inputs: about 100 bytes per sample).
size_t req_dev_bytes(int kind, long long n) {
  return (size_t)n * (kind == KD_REQ_INGEST ? 12 + 100 : 20) + 64;
}

bool grow_buf(Buf& b, size_t ni, size_t nq) {
  if (!b.copied && cudaEventCreateWithFlags(&b.copied, cudaEventDisableTiming) != cudaSuccess) return false;
  bool ok = true;
  if (ni > b.cap_i) {
    size_t c = std::max(ni, 2 * b.cap_i);
    if (b.d_ik) cudaFree(b.d_ik);
    if (b.d_iv) cudaFree(b.d_iv);
    if (b.h_ik) cudaFreeHost(b.h_ik);
    if (b.h_iv) cudaFreeHost(b.h_iv);
    b.d_ik = nullptr, b.d_iv = nullptr, b.h_ik = nullptr, b.h_iv = nullptr;
    ok = ok && cudaMalloc(&b.d_ik, c * 4) == cudaSuccess && cudaMalloc(&b.d_iv, c * 8) == cudaSuccess &&
         cudaHostAlloc((void**)&b.h_ik, c * 4, cudaHostAllocDefault) == cudaSuccess &&
         cudaHostAlloc((void**)&b.h_iv, c * 8, cudaHostAllocDefault) == cudaSuccess;
    b.cap_i = ok ? c : 0;
  }
  if (ok && nq > b.cap_q) {
    size_t c = std::max(nq, 2 * b.cap_q);
    void* dv[] = {b.d_qk, b.d_qv, b.d_qo};
    for (void* p : dv)
      if (p) cudaFree(p);
    void* hv[] = {b.h_qk, b.h_qv, b.h_qo};
    for (void* p : hv)
      if (p) cudaFreeHost(p);
    ok = cudaMalloc(&b.d_qk, c * 4) == cudaSuccess && cudaMalloc(&b.d_qv, c * 8) == cudaSuccess &&
         cudaMalloc(&b.d_qo, c * 8) == cudaSuccess &&
         cudaHostAlloc((void**)&b.h_qk, c * 4, cudaHostAllocDefault) == cudaSuccess &&
         cudaHostAlloc((void**)&b.h_qv, c * 8, cudaHostAllocDefault) == cudaSuccess &&
         cudaHostAlloc((void**)&b.h_qo, c * 8, cudaHostAllocDefault) == cudaSuccess;
    b.cap_q = ok ? c : 0;
  }
  if (!ok) cudaGetLastError();
  return ok;
}

}  // namespace

struct kd_server {
  KdStore* st = nullptr;
  KdSession* s = nullptr;
  double window_s = 0.001;
  size_t budget = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::shared_ptr<Req>> pending;  // arrival order (= timestamp order)
  std::unordered_map<int64_t, std::shared_ptr<Req>> live;  // submitted, not yet waited for
  int64_t next_id = 1;
  double last_ts = -std::numeric_limits<double>::infinity();
  double clock_ts = -std::numeric_limits<double>::infinity();
  long long newest_window = std::numeric_limits<long long>::min();
  bool flushing = false, stop = false;
  std::vector<double> latencies;  // all, or a uniform sample of KD_SRV_LAT_CAP
  unsigned long long lat_seen = 0;
  uint64_t lat_rng = 0x6b64696765737400ull;
  void record_latency(double x) {
    if (latencies.size() < KD_SRV_LAT_CAP) {
      latencies.push_back(x);
    } else {
      const uint64_t j = srv_rand(lat_rng) % (lat_seen + 1);
      if (j < KD_SRV_LAT_CAP) latencies[(size_t)j] = x;
    }
    ++lat_seen;
  }
  size_t buffered_dev = 0;   // device footprint of submitted, not yet completed requests
  std::map<long long, size_t> win_dev;  // the same, per window
  unsigned long long next_seq = 0, admit_seq = 0;  // admission in submit order
  size_t dev_base = 0;       // session device memory when the server started
  size_t dev_measured = 0;   // session device memory + staging after the last window
  size_t dev_peak = 0;       // the largest dev_base + buffered_dev seen
  long long completed = 0, windows_done = 0;
  long long groups = 0, windows_grouped = 0;  // groups run; windows run in groups of two or more
  double max_group_s = 0.0;  // the longest group, from its take to its completion
  long long slow_groups = 0; // groups that took longer than 10 ms
  double stage_s = 0.0;      // host packing and copy set-up of groups (allocation included)
  double busy_s = 0.0;
  int fatal = 0;
  char fatal_msg[256] = {0};
  cudaStream_t copy_stream = nullptr;
  KdErrHost* d_qerr = nullptr;  // status word of the query kernels (empty digests read as NaN)
  Buf buf[2];
  std::thread worker;

  long long window_of(double ts) const { return (long long)std::floor(ts / window_s); }
  // Whether the window of the oldest pending request may be processed.
  bool front_closed() const {
    if (pending.empty()) return false;
    const long long w = pending.front()->window;
    return flushing || stop || newest_window > w || clock_ts >= (double)(w + 1) * window_s;
  }
};

namespace {

// Takes the closed windows, oldest first, up to KD_SRV_GROUP of them (caller
// holds the lock, at least one window is closed), for buffer set `bi`.
std::unique_ptr<Staged> take_group(kd_server* v, int bi) {
  auto sg = std::make_unique<Staged>();
  sg->buf = bi;
  while (sg->wins.size() < KD_SRV_GROUP && v->front_closed()) {
    long long ing = 0;  // the front window's ingest pairs
    for (const auto& r : v->pending) {
      if (r->window != v->pending.front()->window) break;
      if (r->kind == KD_REQ_INGEST) ing += (long long)r->vals.size();
    }
    if (!sg->wins.empty() && ing > KD_SRV_GROUP_BIG) break;  // a large window runs alone
    Win w;
    w.window = v->pending.front()->window;
    w.r0 = sg->reqs.size();
    w.oi = sg->n_ing;
    w.oq = sg->n_q;
    while (!v->pending.empty() && v->pending.front()->window == w.window) {
      auto r = v->pending.front();
      v->pending.pop_front();
      const long long n = (long long)r->vals.size();
      if (r->kind == KD_REQ_INGEST) {
        w.n_ing += n;
        w.ts = r->ts;
      } else if (r->kind == KD_REQ_QUANTILE) {
        w.n_qq += n;
      } else {
        w.n_qc += n;
      }
      sg->reqs.push_back(std::move(r));
    }
    w.r1 = sg->reqs.size();
    sg->n_ing += w.n_ing;
    sg->n_q += w.n_qq + w.n_qc;
    sg->wins.push_back(w);
    if (w.n_ing > KD_SRV_GROUP_BIG) break;  // and nothing joins it
  }
  return sg;
}

// Packs the group into its pinned buffers and starts the host->device copy.
int stage_copy(kd_server* v, Staged& sg) {
  Buf& b = v->buf[sg.buf];
  if (!grow_buf(b, (size_t)sg.n_ing, (size_t)sg.n_q)) return KD_ENOMEM;
  for (const Win& w : sg.wins) {
    long long oi = w.oi, oq = w.oq, oc = w.oq + w.n_qq;
    for (size_t j = w.r0; j < w.r1; ++j) {
      const Req& r = *sg.reqs[j];
      const size_t n = r.vals.size();
      if (r.kind == KD_REQ_INGEST) {
        memcpy(b.h_ik + oi, r.keys.data(), n * 4);
        memcpy(b.h_iv + oi, r.vals.data(), n * 8);
        oi += (long long)n;
      } else {
        long long& o = r.kind == KD_REQ_QUANTILE ? oq : oc;
        memcpy(b.h_qk + o, r.keys.data(), n * 4);
        memcpy(b.h_qv + o, r.vals.data(), n * 8);
        o += (long long)n;
      }
    }
  }
  cudaStream_t cs = v->copy_stream;
  if (sg.n_ing) {
    cudaMemcpyAsync(b.d_ik, b.h_ik, (size_t)sg.n_ing * 4, cudaMemcpyHostToDevice, cs);
    cudaMemcpyAsync(b.d_iv, b.h_iv, (size_t)sg.n_ing * 8, cudaMemcpyHostToDevice, cs);
  }
  if (sg.n_q) {
    cudaMemcpyAsync(b.d_qk, b.h_qk, (size_t)sg.n_q * 4, cudaMemcpyHostToDevice, cs);
    cudaMemcpyAsync(b.d_qv, b.h_qv, (size_t)sg.n_q * 8, cudaMemcpyHostToDevice, cs);
  }
  cudaEventRecord(b.copied, cs);
  return cudaGetLastError() == cudaSuccess ? KD_OK : KD_ECUDA;
}

struct HookCtx {
  kd_server* v;
  Staged* sg;
  Buf* b;
};

// Window i's queries and their read-back, on the ingest's main stream after
// the commit of window i - 1 and before that of window i.
void before_window(void* ctx, long long i, cudaStream_t str) {
  const HookCtx& h = *(const HookCtx*)ctx;
  const Win& w = h.sg->wins[(size_t)i];
  const long long nq = w.n_qq + w.n_qc;
  if (!nq) return;
  Buf& b = *h.b;
  const long long oc = w.oq + w.n_qq;
  kd_pipeline_query2_enqueue(h.v->s, h.v->st, b.d_qk + w.oq, b.d_qv + w.oq, w.n_qq, b.d_qo + w.oq,
                             b.d_qk + oc, b.d_qv + oc, w.n_qc, b.d_qo + oc, h.v->d_qerr, str);
  cudaMemcpyAsync(b.h_qo + w.oq, b.d_qo + w.oq, (size_t)nq * 8, cudaMemcpyDeviceToHost, str);
}

// Runs a staged group: every window's queries (against the state before the
// window's ingests) and ingest, through the pipelined multi-batch ingest.
void run_group(kd_server* v, Staged& sg, int stage_rc, std::unique_ptr<Staged>* next) {
  KdSession* s = v->s;
  Buf& b = v->buf[sg.buf];
  const double t0 = now_s();
  const long long nw = (long long)sg.wins.size();
  if (stage_rc == KD_OK) cudaStreamWaitEvent(s->stream, b.copied, 0);
  // The next group is packed now and its copy runs while this one computes.
  {
    std::unique_lock<std::mutex> lk(v->mu);
    if (!*next && v->front_closed()) {
      *next = take_group(v, sg.buf ^ 1);
      lk.unlock();
      const double ts0 = now_s();
      const int rc = stage_copy(v, **next);
      v->stage_s += now_s() - ts0;  // the worker thread alone writes it
      if (rc) (*next)->buf = -rc - 1;  // remember the failure for its turn
    }
  }
  int rc = stage_rc;
  long long done = 0;  // windows whose ingest committed
  if (stage_rc == KD_OK) {
    std::vector<const uint32_t*> dk((size_t)nw);
    std::vector<const double*> dv((size_t)nw);
    std::vector<long long> ns((size_t)nw);
    std::vector<double> ts((size_t)nw);
    for (long long i = 0; i < nw; ++i) {
      const Win& w = sg.wins[(size_t)i];
      dk[(size_t)i] = b.d_ik + w.oi;
      dv[(size_t)i] = b.d_iv + w.oi;
      ns[(size_t)i] = w.n_ing;
      ts[(size_t)i] = w.ts;
    }
    HookCtx hc{v, &sg, &b};
    if (nw == 1) {  // one window: its queries, then the one-call ingest
      before_window(&hc, 0, s->stream);
      if (ns[0]) rc = kd_pipeline_ingest(s, v->st, dk[0], dv[0], nullptr, ns[0], KD_MODE_TIME, ts[0],
                                         nullptr, nullptr, nullptr);
    } else {
      KdBatchHook hook;
      hook.ctx = &hc;
      hook.before = before_window;
      rc = kd_pipeline_ingest_many(s, v->st, nw, dk.data(), dv.data(), ns.data(), KD_MODE_TIME,
                                   ts.data(), &done, false, &hook);
    }
    if (cudaStreamSynchronize(s->stream) != cudaSuccess && rc == KD_OK) rc = KD_ECUDA;
    if (rc == KD_OK) done = nw;
  }
  const double t1 = now_s();
  // Outside the lock: each request's status and query results (written to the
  // caller's buffer before the status is published), and its consumed data
  // moved out, to be freed after the lock is released (freeing a large
  // request unmaps pages, which a submit waiting on the lock would wait for).
  std::vector<int> status(sg.reqs.size(), KD_OK);
  std::vector<std::vector<uint32_t>> dead_keys(sg.reqs.size());
  std::vector<std::vector<double>> dead_vals(sg.reqs.size());
  for (long long i = 0; i < nw; ++i) {
    const Win& w = sg.wins[(size_t)i];
    // A failed window fails its requests and every later window's (whose
    // queries would have seen a store without it).
    const int wrc = (rc != KD_OK && i >= done) ? rc : KD_OK;
    long long oq = w.oq, oc = w.oq + w.n_qq;
    for (size_t j = w.r0; j < w.r1; ++j) {
      Req& r = *sg.reqs[j];
      const size_t n = r.vals.size();
      int stt = wrc;
      if (r.kind != KD_REQ_INGEST) {
        long long& o = r.kind == KD_REQ_QUANTILE ? oq : oc;
        if (wrc == KD_OK) {
          for (size_t k = 0; k < n; ++k)
            if (std::isnan(b.h_qo[o + (long long)k])) stt = KD_EEMPTY;  // inputs were validated
          if (r.out) memcpy(r.out, b.h_qo + o, n * 8);
        }
        o += (long long)n;
      }
      status[j] = stt;
      dead_keys[j].swap(r.keys);
      dead_vals[j].swap(r.vals);
    }
  }
  {
    std::lock_guard<std::mutex> lk(v->mu);
    for (size_t j = 0; j < sg.reqs.size(); ++j) {
      Req& r = *sg.reqs[j];
      r.status = status[j];
      r.t_done = t1;
      v->record_latency(t1 - r.t_submit);
      v->buffered_dev -= std::min(v->buffered_dev, r.dev_bytes);
      auto wi = v->win_dev.find(r.window);
      if (wi != v->win_dev.end() && (wi->second -= std::min(wi->second, r.dev_bytes)) == 0)
        v->win_dev.erase(wi);
      ++v->completed;
    }
    v->dev_measured = v->s->mem_used + buf_dev_bytes(v->buf[0]) + buf_dev_bytes(v->buf[1]);
    v->windows_done += nw;
    ++v->groups;
    if (nw > 1) v->windows_grouped += nw;
    v->busy_s += t1 - t0;
    v->max_group_s = std::max(v->max_group_s, t1 - t0);
    if (t1 - t0 > 0.010) ++v->slow_groups;
    v->cv.notify_all();
  }
}

void worker_main(kd_server* v) {
  cudaSetDevice(v->s->device);
  std::unique_ptr<Staged> cur;
  int bi = 0;
  for (;;) {
    if (!cur) {
      std::unique_lock<std::mutex> lk(v->mu);
      v->cv.wait(lk, [&] { return v->front_closed() || (v->stop && v->pending.empty()); });
      if (v->pending.empty()) return;  // stopping
      cur = take_group(v, bi);
      lk.unlock();
      const double ts0 = now_s();
      const int rc = stage_copy(v, *cur);
      v->stage_s += now_s() - ts0;
      if (rc) cur->buf = -rc - 1;
    }
    int stage_rc = KD_OK;
    if (cur->buf < 0) {  // staging failed: report it on the group's requests
      stage_rc = -cur->buf - 1;
      cur->buf = bi;
    }
    std::unique_ptr<Staged> next;
    run_group(v, *cur, stage_rc, &next);
    bi = cur->buf ^ 1;
    cur = std::move(next);
  }
}

int srv_fail(char* dst, const char* msg, int code) {
  if (dst) snprintf(dst, 256, "%s", msg);
  return code;
}

}  // namespace

extern "C" {

KD_API int kd_server_create(kd_store* store, double window_s, size_t budget_bytes, kd_server** out) {
  if (!store || !out) return KD_EINVAL;
  *out = nullptr;
  KdSession* s = store->st.sess;
  if (!s) return KD_EINVAL;  // the store's session was destroyed
  if (!(window_s > 0.0) || !kd_isfinite(window_s)) return srv_fail(s->last_error, "window must be positive", KD_EINVAL);
  kd_server* v = new (std::nothrow) kd_server();
  if (!v) return KD_ENOMEM;
  v->st = &store->st;
  v->s = s;
  v->window_s = window_s;
  v->budget = budget_bytes ? budget_bytes : ((size_t)1 << 40);
  v->dev_base = v->dev_measured = s->mem_used;
  cudaSetDevice(s->device);
  int rc = kd_pipeline_prepare_device(s);
  // Samples a one-key store buffered on the single-sample path are merged
  // first (as any read does); the server's batches then go through the batch
  // path with the centroids as their priors.
  if (rc == KD_OK) rc = kd_spath_flush(s, &store->st);
  if (rc == KD_OK && cudaStreamCreateWithFlags(&v->copy_stream, cudaStreamNonBlocking) != cudaSuccess) rc = KD_ECUDA;
  if (rc == KD_OK && cudaMalloc(&v->d_qerr, sizeof(KdErrHost)) != cudaSuccess) rc = KD_ECUDA;
  // Staging for groups of up to 2^22 ingest and 2^20 query pairs, pinned now:
  // pinning or unpinning tens of megabytes while serving holds the process's
  // memory map and stalls every thread, clients included.  Larger groups
  // still grow the buffers (geometrically); a failure here only defers that.
  if (rc == KD_OK)
    for (Buf& b : v->buf) grow_buf(b, (size_t)1 << 22, (size_t)1 << 20);
  if (rc == KD_OK && cudaMemset(v->d_qerr, 0, sizeof(KdErrHost)) != cudaSuccess) rc = KD_ECUDA;
  if (rc) {
    cudaGetLastError();
    if (v->copy_stream) cudaStreamDestroy(v->copy_stream);
    if (v->d_qerr) cudaFree(v->d_qerr);
    delete v;
    return rc;
  }
  v->worker = std::thread(worker_main, v);
  s->servers.push_back(v);
  *out = v;
  return KD_OK;
}

KD_API int kd_server_submit(kd_server* v, int kind, double timestamp, const uint32_t* keys,
                            const double* vals, int64_t n, double* out, int64_t* ticket) {
  if (!v || !ticket) return KD_EINVAL;
  *ticket = 0;
  if (kind != KD_REQ_INGEST && kind != KD_REQ_QUANTILE && kind != KD_REQ_CDF) return KD_EINVAL;
  if (n < 0 || (n > 0 && !vals) || (kind != KD_REQ_INGEST && n > 0 && !out)) return KD_EINVAL;
  if (!kd_isfinite(timestamp)) return KD_EINVAL;
  const long long K = v->st->d.K;
  // validate before admission: a bad request never reaches a batch
  for (int64_t i = 0; i < n; ++i) {
    if (keys && (long long)keys[i] >= K) return KD_EINVAL;
    const double x = vals[i];
    if (!kd_isfinite(x)) return KD_EINVAL;
    if (kind == KD_REQ_QUANTILE && !(x >= 0.0 && x <= 1.0)) return KD_EINVAL;
  }
  auto r = std::make_shared<Req>();
  r->kind = kind;
  r->ts = timestamp;
  r->window = v->window_of(timestamp);
  r->keys.assign((size_t)n, 0u);
  if (keys && n) memcpy(r->keys.data(), keys, (size_t)n * 4);
  if (n) r->vals.assign(vals, vals + n);
  r->out = out;
  r->dev_bytes = req_dev_bytes(kind, n);
  std::unique_lock<std::mutex> lk(v->mu);
  if (v->stop) return KD_EINVAL;
  if (timestamp < v->last_ts) return KD_EINVAL;  // timestamps must not decrease
  if (r->window < v->newest_window || (double)(r->window + 1) * v->window_s <= v->clock_ts)
    return KD_EINVAL;  // its window is already closed
  // a request that could not fit even with nothing else buffered
  if (v->dev_base + r->dev_bytes > v->budget) return KD_ENOMEM;
  // The request takes its place in the stream now: its timestamp closes every
  // earlier window, so those drain while it waits for room.  Requests are
  // admitted in submit order.  Its own window closes only on a later request,
  // an advance or a flush, so if the earlier windows have all drained and its
  // window still leaves no room, waiting cannot help: KD_ENOMEM.
  r->t_submit = now_s();
  v->last_ts = timestamp;
  v->newest_window = std::max(v->newest_window, r->window);
  const unsigned long long seq = v->next_seq++;
  v->cv.notify_all();
  auto own = [&]() -> size_t {
    auto it = v->win_dev.find(r->window);
    return it == v->win_dev.end() ? 0 : it->second;
  };
  auto room = [&] { return v->dev_base + v->buffered_dev + r->dev_bytes <= v->budget; };
  v->cv.wait(lk, [&] {
    return v->stop || (v->admit_seq == seq && (room() || v->buffered_dev == own()));
  });
  if (v->stop) return KD_EINVAL;
  if (!room()) {  // only its own window holds the budget
    ++v->admit_seq;
    v->cv.notify_all();
    return KD_ENOMEM;
  }
  ++v->admit_seq;
  r->id = v->next_id++;
  v->buffered_dev += r->dev_bytes;
  v->win_dev[r->window] += r->dev_bytes;
  v->dev_peak = std::max(v->dev_peak, v->dev_base + v->buffered_dev);
  v->live[r->id] = r;
  v->pending.push_back(r);
  *ticket = r->id;
  v->cv.notify_all();
  return KD_OK;
}

KD_API int kd_server_advance(kd_server* v, double now_ts) {
  if (!v || !kd_isfinite(now_ts)) return KD_EINVAL;
  std::lock_guard<std::mutex> lk(v->mu);
  v->clock_ts = std::max(v->clock_ts, now_ts);
  v->cv.notify_all();
  return KD_OK;
}

KD_API int kd_server_wait(kd_server* v, int64_t ticket, double timeout_s, int* status) {
  if (!v || !status) return KD_EINVAL;
  std::unique_lock<std::mutex> lk(v->mu);
  auto it = v->live.find(ticket);
  if (it == v->live.end()) return KD_EINVAL;
  auto r = it->second;
  auto done = [&] { return r->status >= 0; };
  if (timeout_s < 0) {
    v->cv.wait(lk, done);
  } else if (!v->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
    return KD_ETIMEOUT;
  }
  *status = r->status;
  v->live.erase(ticket);
  return KD_OK;
}

KD_API int kd_server_latency(kd_server* v, int64_t ticket, double* seconds) {
  if (!v || !seconds) return KD_EINVAL;
  std::lock_guard<std::mutex> lk(v->mu);
  auto it = v->live.find(ticket);
  if (it == v->live.end()) return KD_EINVAL;
  *seconds = it->second->status >= 0 ? it->second->t_done - it->second->t_submit : -1.0;
  return KD_OK;
}

KD_API int kd_server_memory(kd_server* v, size_t* in_use, size_t* peak, size_t* budget,
                            size_t* measured) {
  if (!v) return KD_EINVAL;
  std::lock_guard<std::mutex> lk(v->mu);
  if (in_use) *in_use = v->dev_base + v->buffered_dev;
  if (measured) *measured = v->dev_measured;
  if (peak) *peak = v->dev_peak;
  if (budget) *budget = v->budget;
  return KD_OK;
}

KD_API int kd_server_flush(kd_server* v) {
  if (!v) return KD_EINVAL;
  std::unique_lock<std::mutex> lk(v->mu);
  v->flushing = true;
  v->cv.notify_all();
  v->cv.wait(lk, [&] { return v->pending.empty() && v->buffered_dev == 0; });
  v->flushing = false;
  // later requests open new windows after the flushed ones
  v->clock_ts = std::max(v->clock_ts, (double)(v->newest_window + 1) * v->window_s);
  return KD_OK;
}

KD_API int kd_server_stats(kd_server* v, double* lat3, int64_t* completed, int64_t* windows,
                           double* busy_s) {
  if (!v) return KD_EINVAL;
  std::vector<double> l;
  {
    std::lock_guard<std::mutex> lk(v->mu);
    if (lat3) l = v->latencies;
    if (completed) *completed = v->completed;
    if (windows) *windows = v->windows_done;
    if (busy_s) *busy_s = v->busy_s;
  }
  if (lat3) {  // sorted outside the lock: the worker publishes results meanwhile
    std::sort(l.begin(), l.end());
    const double ps[3] = {0.50, 0.99, 0.999};
    for (int i = 0; i < 3; ++i) {
      if (l.empty()) {
        lat3[i] = 0.0;
        continue;
      }
      size_t k = (size_t)std::ceil(ps[i] * (double)l.size());  // nearest rank
      lat3[i] = l[std::min(l.size() - 1, k == 0 ? 0 : k - 1)];
    }
  }
  return KD_OK;
}

KD_API int kd_server_groups(kd_server* v, int64_t* groups, int64_t* windows_grouped,
                            double* max_group_s, int64_t* slow_groups, double* stage_s) {
  if (!v) return KD_EINVAL;
  std::lock_guard<std::mutex> lk(v->mu);
  if (groups) *groups = v->groups;
  if (windows_grouped) *windows_grouped = v->windows_grouped;
  if (max_group_s) *max_group_s = v->max_group_s;
  if (slow_groups) *slow_groups = v->slow_groups;
  if (stage_s) *stage_s = v->stage_s;
  return KD_OK;
}

// Drains and stops the worker, then frees the device resources; the handle
// stays valid for waits and stats.
static void server_stop(kd_server* v) {
  {
    std::lock_guard<std::mutex> lk(v->mu);
    v->stop = true;  // remaining windows are processed before the worker exits
    v->cv.notify_all();
  }
  if (v->worker.joinable()) v->worker.join();
  if (!v->s) return;
  cudaSetDevice(v->s->device);
  cudaStreamSynchronize(v->s->stream);
  for (Buf& b : v->buf) free_buf(b);
  if (v->copy_stream) cudaStreamDestroy(v->copy_stream);
  v->copy_stream = nullptr;
  if (v->d_qerr) cudaFree(v->d_qerr);
  v->d_qerr = nullptr;
}

KD_API void kd_server_destroy(kd_server* v) {
  if (!v) return;
  if (v->s) {  // an orphan was already stopped by its session's destruction
    auto& list = v->s->servers;
    list.erase(std::remove(list.begin(), list.end(), v), list.end());
    server_stop(v);
  }
  delete v;
}

}  // extern "C"

void kd_server_orphan(kd_server* v) {
  server_stop(v);
  std::lock_guard<std::mutex> lk(v->mu);
  v->s = nullptr;
  v->st = nullptr;
}
