// kd_engine.h — host-side engine objects behind the C-ABI (sessions, resident
// stores, workspaces) and the pipeline entry points implemented in kd_pipeline.cu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

// Device view of a resident per-key digest store (the grouped layout).
// Every key owns two fixed slots of KD_TILE centroids (the P-path never emits
// more than one tile's worth), so an ingest writes the new centroids of a key
// into its back slot and a commit flips the key's `cur` bit only when the whole
// batch succeeded: a failed batch leaves every digest unchanged.
struct KdStoreDev {
  long long K;
  int scale;
  double compression;
  double lambda;        // decay rate; 0 = no decay
  double* slot_m;       // [2][K][1024] centroid means
  double* slot_w;       // [2][K][1024] centroid stored weights
  double* prefix;       // [K][1024] quantile-walk prefix of the live slot
  unsigned char* cur;   // [K] live slot
  int* count;           // [K]
  double* total;        // [K] stored total weight
  double* log_scale;    // [K]
  double* clock;        // [K]
  double* min_v;        // [K]
  double* max_v;        // [K]
  double* dfac;         // [K] e^{-log_scale} (singleton test of queries)
  // Single-sample path (TDigest.add / add_at): samples wait in a per-key buffer
  // of buf_cap entries until it fills and the sequential merge pass runs.
  // Null until a store first takes that path.
  int* bcount;          // [K] buffered samples
  double* buf_m;        // [K][buf_cap] their values
  double* buf_w;        // [K][buf_cap] their stored (decay-scaled) weights
  int buf_cap;          // 5 * int(compression), at least 1
};

struct KdErrHost {
  int code;
  int pad;
  long long index;
};

// Per-call inputs of an ingest, read by the kernels from device memory so that a
// captured ingest graph replays with new inputs: one copy (pinned host block ->
// device block) at the head of the step refreshes them together with the
// initial status word.
struct KdCallArgs {
  const uint32_t* keys;
  const double* vals;
  const double* wts;
  const double* merge_min;
  const double* merge_max;
  const double* merge_clock;
  double timestamp;
  // A batch of a one-key store whose digest came from the single-sample path:
  // the first `carry` inputs are its centroids and buffered samples (with their
  // stored weights in wts), the rest are the batch's unit-weight samples.
  long long carry;
  const unsigned long long* carry_mm;  // order keys of the batch's min and max
  KdErrHost err;  // the step's status word (device copy: KdWorkspace::err)
};

// Per-level plan of the P-path hierarchy.  Level 0 holds every touched key;
// level L >= 1 holds the keys whose input exceeded one tile at level L-1.  The
// input of a level is a dense array (means, weights): key a owns
// [base[a], base[a] + m[a]); its tiles are listed in `work` as (a, tile).
struct KdLevelDev {
  int* A;          // active keys (device scalar)
  int* j;          // touched ordinal of active key a
  int* src_base;   // first intermediate tile of the previous level holding its input
  int* src_tiles;  // number of those tiles
  int* mprev;      // input size at the previous level
  int* m;          // input size at this level
  int* base;       // offset of its input in the dense array
  int* inter_off;  // first intermediate output tile (when not final)
  int2* work_l;    // (a, tile) of tiles above KD_SERIAL_TILE_MAX elements (warp per tile)
  int2* work_s;    // (a, tile) of smaller tiles (lane per tile)
  int* Tl;         // large work tiles (device scalar)
  int* Ts;         // small work tiles (device scalar)
  int* I;          // intermediate tiles (device scalar)
  int* M;          // dense elements (device scalar)
};

#define KD_FIX_CAP 65536  // repair-list capacity of the packed sort (a full list re-sorts)

struct KdWorkspace {
  long long cap_n = 0;     // elements
  long long cap_keys = 0;  // touched-key capacity
  long long cap_inter = 0; // intermediate tiles per level
  // sort buffers
  uint64_t* k64[2] = {nullptr, nullptr};
  uint32_t* key[2] = {nullptr, nullptr};
  uint32_t* idx[2] = {nullptr, nullptr};
  unsigned* ghist = nullptr;             // digit counts of every radix pass
  unsigned long long* rs_state = nullptr; // look-back words, 256 per sort tile
  unsigned long long* rs_ticket = nullptr;
  long long cap_rs_tiles = 0;
  unsigned* rs_epoch_base = nullptr;        // device epoch base of the look-back words
  unsigned long long rs_epochs_used = 0;     // host bookkeeping of that base
  int4* partials = nullptr;
  long long cap_partials = 0;
  // touched keys
  uint32_t* tkey = nullptr;
  int* tstart = nullptr;
  int* tm = nullptr;
  int* tprior = nullptr;
  unsigned char* tbuf = nullptr;
  double* tsf = nullptr;
  double* tpscale = nullptr;
  uint32_t* tmap = nullptr;  // key -> touched ordinal (valid for touched keys only)
  long long cap_tmap = 0;
  // Key-level touched detection (cap_tmap entries each): the sort's unpack
  // stamps every key that starts a run with the step's epoch and records the
  // run's start; a scan over the keys then lists the touched ones.  Null in
  // workspaces without them (the element-level scan is used).
  int* kfirst = nullptr;
  unsigned long long* kstamp = nullptr;
  unsigned long long* kepoch = nullptr;  // advanced by every step's k_prep
  int* chain = nullptr;  // batch chain flag of a pipelined multi-batch ingest
  double* st_clock = nullptr;
  double* st_ls = nullptr;
  double* st_min = nullptr;
  double* st_max = nullptr;
  int* st_count = nullptr;
  // merge inputs (per touched key, optional)
  double* tm_min = nullptr;
  double* tm_max = nullptr;
  double* tm_clock = nullptr;
  // levels
  KdLevelDev lv[2];
  int* lv_storage = nullptr;
  long long cap_work = 0;      // work tiles per level
  long long cap_merged = 0;    // dense elements per level
  int2* work[4] = {nullptr, nullptr, nullptr, nullptr};  // (large, small) x 2 levels
  double* dx[2] = {nullptr, nullptr};  // dense level inputs (ping-pong)
  double* dw[2] = {nullptr, nullptr};
  // intermediate tile outputs (one set: a level's outputs are compacted into
  // the next dense input before the next level writes again)
  double* scr_m = nullptr;
  double* scr_w = nullptr;
  int* tcount = nullptr;
  int* doff = nullptr;
  int* needs = nullptr;  // device: required (work, merged, inter) capacities
  int* fix = nullptr;    // repair list of the packed sort: count, then positions
  long long cap_fix = 0;
  // scalars: U, T0, I0, A1 ... (int4 totals)
  int4* totals = nullptr;
  KdCallArgs* d_call = nullptr;  // device per-call block (err lives inside it)
  KdCallArgs* h_call = nullptr;  // pinned host mirror
  KdErrHost* err = nullptr;   // device: &d_call->err
  KdErrHost* h_err = nullptr; // pinned host: &h_call->err
  int* h_scalars = nullptr;   // pinned host scalars
  unsigned long long generation = 0;  // bumped whenever buffers move (graphs bake pointers)
  // host staging (pinned) for host-pointer inputs / outputs
  void* h_stage = nullptr;
  size_t h_stage_bytes = 0;
  void* d_in = nullptr;
  size_t d_in_bytes = 0;
};

// Per-stage device timing of ingests (CUDA events on the session stream).
#define KD_NSTAGES 6  // prep, sort, plan, level0, levels, commit
struct KdStageStats {
  int enabled = 0;
  cudaEvent_t ev[KD_NSTAGES + 1] = {};
  double ms[KD_NSTAGES] = {};
  long long launches = 0;  // kernels launched by the engine
  long long ingests = 0;
};

struct KdSession {
  int device = 0;
  cudaStream_t stream = nullptr;
  size_t mem_budget = 0;
  size_t mem_used = 0;
  long long ws_grows = 0;   // ingest workspace (re)allocations
  double ws_grow_s = 0.0;   // host seconds spent in them (frees synchronise the device)
  int num_sms = 0;
  int force_exact = 0;
  int max_levels = 32;
  int use_graphs = 1;  // capture repeated ingest steps as CUDA graphs
  // Launch tuning (results never depend on these): the largest partial tile
  // sent to the small-tile kernel, and resident blocks per SM of the two tile
  // kernels.  Defaults are the committed autotuner choice for GB300.
  int small_cap = 128;
  int large_bps = 6;
  // resident blocks per SM of the large-tile kernel, narrow and wide blocks
  // (0: not queried yet)
  int large_resident[2] = {0, 0};
  int small_bps = 8;
  // Run a level's two tile kernels on two streams (the second joins back
  // before anything reads their outputs).  Also a launch setting only.
  int concurrent_tiles = 1;
  // Tests only (KD_OPT_TEST_WAIT): when non-zero, one bounded device wait per
  // sort pass or key-map call waits on a word that nothing publishes, with
  // this many polls, so that the wait runs out and KD_ETIMEOUT comes back.
  int wait_test = 0;
  cudaStream_t side = nullptr;  // second stream for the small-tile kernel
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  char last_error[256] = {0};  // fixed buffer: reporting an error never allocates
  KdWorkspace ws;
  // Pipelined multi-batch ingest: two more workspaces, so that batches sort
  // (on `ahead`, up to two ahead) while an earlier one compresses (on
  // `stream`); events ordering the two; pinned host slots for every batch's
  // status.
#define KD_PIPE_WS 3
  KdWorkspace ws_more[KD_PIPE_WS - 1];
  cudaStream_t ahead = nullptr, ahead2 = nullptr;  // fronts alternate between the two
  int front_streams = 2;  // 1: every front on `ahead` (a launch setting only)
  // start; per workspace: front done, free, call block copied, inputs staged
  cudaEvent_t pipe_ev[1 + 4 * KD_PIPE_WS] = {};
  // Host inputs of a multi-batch ingest are copied by the copy engine (on
  // `copy`) into one device staging buffer per workspace, ahead of the front.
  cudaStream_t copy = nullptr;
  void* d_stage[KD_PIPE_WS] = {};
  size_t stage_bytes = 0;  // bytes of each staging buffer
  KdErrHost* h_many = nullptr;
  long long cap_many = 0;
  KdStageStats stats;
  struct KdStore* scratch_store = nullptr;  // 1-key store for stateless compress
  struct KdStore* scratch_many = nullptr;   // K-key store for the stateless grouped calls
  void* sl_buf = nullptr;                   // device working memory of the stateless calls
  size_t sl_bytes = 0;
  std::vector<struct KdStore*> stores;         // live stores of this session
  std::vector<struct kd_server*> servers;      // live serving loops over them
  std::vector<struct kd_keymap*> keymaps;      // live key dictionaries
};

// Stops a server whose session is being destroyed (drains it, joins its
// worker, frees its buffers); kd_server_destroy then only frees the handle.
void kd_server_orphan(struct kd_server* v);

// Frees the device tables of a key dictionary whose session is being
// destroyed; kd_keymap_destroy then only frees the handle.
void kd_keymap_orphan(struct kd_keymap* m);

// What a captured ingest step depends on besides the per-call block: launch
// shapes, kernel arguments that are baked in, and the buffers.
struct KdGraphKey {
  long long n = -1;
  int key_bits = 0, with_idx = 0, mode = 0, levels = 0, force_exact = 0, timing = 0;
  int scale = 0;
  int tuning = 0;
  double compression = 0.0;
  unsigned long long generation = 0;
  bool operator==(const KdGraphKey& o) const {
    return n == o.n && key_bits == o.key_bits && with_idx == o.with_idx && mode == o.mode &&
           levels == o.levels && force_exact == o.force_exact && timing == o.timing &&
           scale == o.scale && tuning == o.tuning && compression == o.compression &&
           generation == o.generation;
  }
};
struct KdGraphEntry {
  KdGraphKey key;
  cudaGraphExec_t exec = nullptr;
  // host view after the captured levels (for an eager continuation)
  const int* curA = nullptr;
  const int* Iprev = nullptr;
  long long launches = 0;
};
#define KD_GRAPH_CACHE 4

// Arguments of a batched quantile + cdf call; the same arguments twice in a row
// capture the call (one kernel and its status copies) as a CUDA graph.
struct KdQueryArgs {
  const void* p[6] = {};
  long long nq = -1, nc = -1;
  bool operator==(const KdQueryArgs& o) const {
    for (int i = 0; i < 6; ++i)
      if (p[i] != o.p[i]) return false;
    return nq == o.nq && nc == o.nc;
  }
};

struct KdStore {
  KdSession* sess = nullptr;
  KdStoreDev d{};
  size_t bytes = 0;
  int levels_hint = 3;  // hierarchy levels >= 1 the last ingest needed
  // Ingest steps captured as CUDA graphs: a step shape seen twice in a row is
  // captured, later steps of that shape replay it.
  KdGraphEntry graphs[KD_GRAPH_CACHE];
  int graph_next = 0;
  KdGraphKey last_eager;
  // The pipelined multi-batch ingest's graphs: per workspace, its front and
  // its back (with the chain flag the back's commit was captured with).
  KdGraphEntry pipe_graphs[KD_PIPE_WS][2];
  const int* pipe_chain[KD_PIPE_WS] = {};
  long long pipe_last_n = -1;  // size of the last batch of the last multi-batch call
  // Single-sample path state (one-key stores).  `pending`: samples wait in the
  // buffer.  `carry`: the next batch must carry the centroids and buffer in
  // its input (their order is the sequential pass's, not the batch path's).
  bool pending = false;
  bool carry = false;
  void* sp_scratch = nullptr;  // working memory of the pass when shared memory is too small
  size_t sp_scratch_bytes = 0;
  KdQueryArgs q_last, q_graph_args;
  cudaGraphExec_t q_graph = nullptr;
};

// The opaque handles of the C-ABI.
struct kd_session {
  KdSession s;
};
struct kd_store {
  KdStore st;
};

// Pipeline entry points (kd_pipeline.cu).  All work is enqueued on sess->stream.
// Return KD_* status; on error sess->last_error holds a message.
enum KdIngestMode { KD_MODE_COUNT = 0, KD_MODE_TIME = 1, KD_MODE_REPLACE = 2, KD_MODE_MERGE = 3 };

int kd_pipeline_ingest(KdSession* s, KdStore* st, const uint32_t* d_keys, const double* d_vals,
                       const double* d_wts, long long n, int mode, double timestamp,
                       const double* d_merge_min, const double* d_merge_max,
                       const double* d_merge_clock, long long carry = 0,
                       const unsigned long long* d_carry_mm = nullptr);
// Single-sample path (kd_spath.cu).  Merges the buffered samples of a one-key
// store (TDigest.merge, tdigest.mojo:391-439) when any wait; a no-op otherwise.
int kd_spath_flush(KdSession* s, KdStore* st);
// A batch into a one-key store with `carry` set: the centroids and buffer go
// into the batch's input ahead of its samples.
int kd_spath_carry_ingest(KdSession* s, KdStore* st, const double* d_vals, long long n, int mode,
                          double timestamp);
void kd_spath_free(KdSession* s, KdStore* st);
int kd_pipeline_quantile(KdSession* s, KdStore* st, const uint32_t* d_keys, const double* d_q,
                         long long nq, double* d_out, int is_cdf);
// Quantiles (qk/qs/qout, nq) and cdfs (ck/xs/cout, nc) of a store in one
// kernel launch, device pointers; captured as a graph when the same arguments
// recur.
int kd_pipeline_query2(KdSession* s, KdStore* st, const uint32_t* qk, const double* qs, long long nq,
                       double* qout, const uint32_t* ck, const double* xs, long long nc, double* cout);
// The same kernel enqueued on `str` with no synchronisation; failures (empty
// digests) go to the caller's device status word `err`.
int kd_pipeline_query2_enqueue(KdSession* s, KdStore* st, const uint32_t* qk, const double* qs,
                               long long nq, double* qout, const uint32_t* ck, const double* xs,
                               long long nc, double* cout, KdErrHost* err, cudaStream_t str);
// Session device memory with budget accounting (kd_capi.cu).
int kd_dalloc(KdSession* s, void** p, size_t bytes);
void kd_dfree(KdSession* s, void* p, size_t bytes);
int kd_pipeline_merge(KdSession* s, KdStore* dst, KdStore* src, const long long* h_group_off,
                      const uint32_t* h_parts, long long ngroups);
int kd_store_alloc(KdSession* s, KdStore* st);
void kd_store_free(KdStore* st);
// The batch capacity a workspace is sized for: its own when the batch fits,
// else at least twice it.  Callers derive every other capacity from it, so a
// run of ever larger batches reallocates once per doubling of the batch.
inline long long kd_ws_batch_cap(long long n, long long cap_n) {
  if (n <= cap_n) return cap_n;
  const long long twice = cap_n < (1LL << 30) ? 2 * cap_n : (1LL << 31) - 1;
  return n > twice ? n : twice;
}
int kd_ws_reserve(KdSession* s, long long n, long long keys, long long inter, long long work,
                  long long merged, long long tmap, KdWorkspace* wp = nullptr);
// Batches folded in order as if by one kd_pipeline_ingest each (unit weights),
// with the front of batch i + 1 (prep, sort) overlapping the back of batch i.
// On failure *done is the failing batch: batches before it are committed, it
// and every later one are not.
// With `host_inputs`, the key and value pointers are host memory (pinned or
// pageable): each batch is first copied into a device staging buffer.
// Work a caller interleaves with the batches of a multi-batch ingest: before(i)
// enqueues on `str` what must see the store after batch i - 1 and before batch
// i (the serving loop's queries of window i).  It is called for every batch,
// empty ones included, in batch order; after a retry of batch j the batches
// from j + 1 on are enqueued, and their before() called, once more.
struct KdBatchHook {
  void* ctx = nullptr;
  void (*before)(void* ctx, long long i, cudaStream_t str) = nullptr;
};
int kd_pipeline_ingest_many(KdSession* s, KdStore* st, long long nb, const uint32_t* const* d_keys,
                            const double* const* d_vals, const long long* ns, int mode,
                            const double* timestamps, long long* done, bool host_inputs = false,
                            const KdBatchHook* hook = nullptr);
void kd_ws_free(KdWorkspace& ws);
void kd_store_drop_graphs(KdStore* st);
int kd_cuda_fail(KdSession* s, cudaError_t e, const char* what);
void kd_set_msg(KdSession* s, const char* msg);
// One-time kernel attributes (shared-memory opt-ins); no allocation.
int kd_pipeline_prepare_device(KdSession* s);

// One ingest attempt on a caller-provided workspace (allocates nothing).
// Returns a KD_* status, or KD_ERANGE_SCRATCH_INTERNAL when a capacity of `w`
// was too small (w.h_scalars[0..2] then hold the needed work / dense /
// intermediate capacities).
#define KD_ERANGE_SCRATCH_INTERNAL 100
int kd_pipeline_attempt(KdSession* s, KdStore* st, KdWorkspace& w, const uint32_t* d_keys,
                        const double* d_vals, const double* d_wts, long long n, int mode,
                        double timestamp, const double* d_merge_min, const double* d_merge_max,
                        const double* d_merge_clock, long long carry = 0,
                        const unsigned long long* d_carry_mm = nullptr);
