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
};

struct KdErrHost {
  int code;
  int pad;
  long long index;
};

// Per-level plan of the P-path hierarchy (levels >= 1 hold only the keys whose
// input exceeded one tile at the previous level).
struct KdLevelDev {
  int* A;          // number of active keys (device scalar)
  int* j;          // touched ordinal
  int* src_base;   // first intermediate tile (previous level) holding the input
  int* src_tiles;  // number of those tiles
  int* mprev;      // input size at the previous level
  int* m;          // input size at this level
  int* tile_off;   // exclusive prefix of tiles over active keys
  int* inter_off;  // exclusive prefix of intermediate tiles
  int* T;          // total tiles (device scalar)
  int* I;          // total intermediate tiles (device scalar)
};

struct KdWorkspace {
  long long cap_n = 0;     // elements
  long long cap_keys = 0;  // touched-key capacity
  long long cap_inter = 0; // intermediate tiles per level
  // sort buffers
  uint64_t* k64[2] = {nullptr, nullptr};
  uint32_t* key[2] = {nullptr, nullptr};
  uint32_t* idx[2] = {nullptr, nullptr};
  int* hist = nullptr;
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
  int* ttiles = nullptr;
  int* ttile_off = nullptr;
  int* tinter_off = nullptr;
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
  // intermediate tiles (ping-pong)
  double* scr_m[2] = {nullptr, nullptr};
  double* scr_w[2] = {nullptr, nullptr};
  int* tcount[2] = {nullptr, nullptr};
  int* doff[2] = {nullptr, nullptr};
  // scalars: U, T0, I0, A1 ... (int4 totals)
  int4* totals = nullptr;
  KdErrHost* err = nullptr;   // device
  KdErrHost* h_err = nullptr; // pinned host mirror
  int* h_scalars = nullptr;   // pinned host scalars
  // host staging (pinned) for host-pointer inputs / outputs
  void* h_stage = nullptr;
  size_t h_stage_bytes = 0;
  void* d_in = nullptr;
  size_t d_in_bytes = 0;
};

struct KdSession {
  int device = 0;
  cudaStream_t stream = nullptr;
  size_t mem_budget = 0;
  size_t mem_used = 0;
  int num_sms = 0;
  int force_exact = 0;
  int max_levels = 8;
  std::string last_error;
  KdWorkspace ws;
  struct KdStore* scratch_store = nullptr;  // 1-key store for stateless compress
};

struct KdStore {
  KdSession* sess = nullptr;
  KdStoreDev d{};
  size_t bytes = 0;
};

// Pipeline entry points (kd_pipeline.cu).  All work is enqueued on sess->stream.
// Return KD_* status; on error sess->last_error holds a message.
enum KdIngestMode { KD_MODE_COUNT = 0, KD_MODE_TIME = 1, KD_MODE_REPLACE = 2, KD_MODE_MERGE = 3 };

int kd_pipeline_ingest(KdSession* s, KdStore* st, const uint32_t* d_keys, const double* d_vals,
                       const double* d_wts, long long n, int mode, double timestamp,
                       const double* d_merge_min, const double* d_merge_max,
                       const double* d_merge_clock);
int kd_pipeline_quantile(KdSession* s, KdStore* st, const uint32_t* d_keys, const double* d_q,
                         long long nq, double* d_out, int is_cdf);
int kd_pipeline_merge(KdSession* s, KdStore* dst, KdStore* src, const long long* h_group_off,
                      const uint32_t* h_parts, long long ngroups);
int kd_store_alloc(KdSession* s, KdStore* st);
void kd_store_free(KdStore* st);
int kd_ws_reserve(KdSession* s, long long n, long long keys, long long inter);
void kd_ws_free(KdWorkspace& ws);
int kd_cuda_fail(KdSession* s, cudaError_t e, const char* what);
