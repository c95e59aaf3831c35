/*
 * kdigest_gb300.h — C-ABI of the GB300 (sm_103a) t-digest engine.
 *
 * Plain pointers and sizes only.  Every entry point returns an int status
 * (KD_OK on success) and leaves a message readable through kd_last_error().
 * Digest state, centroid arithmetic, decay factors and scale evaluations are
 * FP64 throughout.
 *
 * Each declaration cites the reference interface it replaces (paths inside the
 * kdigest project, src/kdigest/...).  The reference's GPU backend is Mojo/MAX;
 * its host code would bind these symbols with external_call.
 */
#ifndef KDIGEST_GB300_H
#define KDIGEST_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define KD_API __attribute__((visibility("default")))
#else
#define KD_API
#endif

/* Status codes.  The reference raises Error(String); each raise site maps to one
 * code (tdigest.mojo:317-322, grouped.mojo:74-97, tdigest.mojo:492-498,545-546,
 * tdigest.mojo:661-662, gpu/primitives.mojo:260-268). */
#define KD_OK 0
#define KD_EINVAL 1     /* non-finite value, weight <= 0, key out of range, q outside [0,1] */
#define KD_EEMPTY 2     /* quantile / cdf of an empty digest */
#define KD_ERANGE 3     /* output capacity too small (needed size returned), truncated bytes */
#define KD_ECONVERGE 4  /* P-path pass could not shrink a key (the reference loops forever) */
#define KD_ENOMEM 5     /* over the session's device-memory budget / allocation failure */
#define KD_ECUDA 6      /* CUDA runtime error */
#define KD_ETIMEOUT 7   /* a bounded device wait gave up (sort look-back, key map, serving loop) */

/* Scale functions — src/kdigest/scale.mojo:78-200 (ScaleK0..ScaleK3). */
#define KD_K0 0
#define KD_K1 1
#define KD_K2 2
#define KD_K3 3

/* Clock modes of an ingest: count clock (add_batch, tdigest.mojo:177-296) or
 * time clock (add_at semantics with one timestamp per batch, :163-175). */
#define KD_CLOCK_COUNT 0
#define KD_CLOCK_TIME 1

/* Pointer flag: inputs/outputs of the call are device pointers (no H2D/D2H). */
#define KD_PTR_DEVICE 1

/* Session options (kd_session_set_option). */
#define KD_OPT_FORCE_EXACT_K 1 /* evaluate every bucket id in FP64 (no FP32 filter) */
#define KD_OPT_MAX_LEVELS 2    /* cap on tile-hierarchy levels per ingest (default 32) */
#define KD_OPT_STAGE_TIMING 3  /* record CUDA events between ingest stages */
#define KD_OPT_GRAPHS 4        /* capture repeated ingest steps as CUDA graphs (default on) */
/* Launch tuning; results never depend on it (kdigest_gb300/tuning/ holds the
 * autotuner's record for GB300, whose choice is the default). */
#define KD_OPT_SMALL_TILE_CAP 5       /* largest tile for the small-tile kernel, 1..128 */
#define KD_OPT_LARGE_BLOCKS_PER_SM 6  /* grid of the large-tile kernel, blocks per SM */
#define KD_OPT_SMALL_BLOCKS_PER_SM 7  /* grid of the small-tile kernel, blocks per SM */
#define KD_OPT_CONCURRENT_TILES 8     /* run the two tile kernels of a level on two streams */
#define KD_OPT_FRONT_STREAMS 9        /* multi-batch ingest: fronts (prep, sort) on 1 or 2 streams */
/* Tests only: with a value v > 0, every radix pass leaves its first tile's
 * look-back word unpublished, kd_keymap_map leaves the id of its first input
 * key unpublished when it inserts that key, and the waits on those words give
 * up after v polls: an ingest returns KD_ETIMEOUT and changes no digest; a map
 * call returns KD_ETIMEOUT when the key occurs again in the call, and the map
 * keeps the key without a published id (later lookups of it time out too).
 * 0 (default) is off. */
#define KD_OPT_TEST_WAIT 10

typedef struct kd_session kd_session;
typedef struct kd_store kd_store;

KD_API int kd_version(void);
KD_API const char* kd_status_string(int status);

/* GpuSession (gpu/session.mojo:19-27): device context + reusable workspaces.
 * mem_budget = 0 means no limit.  Not thread-safe (as the reference). */
KD_API int kd_session_create(int device, size_t mem_budget, kd_session** out);
KD_API void kd_session_destroy(kd_session* s);
KD_API const char* kd_last_error(kd_session* s);
KD_API int kd_session_sync(kd_session* s);
KD_API int kd_session_set_option(kd_session* s, int option, int value);
/* Ingest workspace (re)allocations of this session so far and the host seconds
 * they took (each frees the old buffers, which waits for the device).  Either
 * pointer may be NULL. */
KD_API int kd_session_alloc_stats(kd_session* s, int64_t* grows, double* seconds);
/* The CUDA stream (cudaStream_t) all work of this session is ordered on.  It
 * is created at the device's highest stream priority, so work a caller
 * enqueues on other streams yields SMs to it. */
KD_API void* kd_session_stream(kd_session* s);
/* Accumulated per-stage device milliseconds of ingests (prep, sort, plan, level0,
 * levels, commit; recorded when KD_OPT_STAGE_TIMING is on), kernels launched and
 * ingests run since the last reset.  Returns the number of stages.  No reference
 * counterpart (the reference times with perf_counter_ns, bench/bench_gpu.mojo:72). */
KD_API int kd_session_stats(kd_session* s, double* stage_ms, int cap, int64_t* launches,
                            int64_t* ingests);
KD_API void kd_session_reset_stats(kd_session* s);

/* gpu_compress_batch[S] (gpu/add_batch.mojo:629-663): P-path compress of an
 * arbitrary (mean, weight) set -> mean-sorted centroids.  out arrays hold cap
 * entries; KD_ERANGE with *out_n = needed when cap is too small. */
KD_API int kd_compress(kd_session* s, int scale, double compression, const double* means,
                       const double* weights, int64_t n, int flags, double* out_means,
                       double* out_weights, int64_t cap, int64_t* out_n);

/* Stateless entry points over caller-held digests: the reference's host state
 * keeps its digests on the host and passes their centroid arrays per call.
 * Digests and groups are CSR: digest d is entries [offsets[d], offsets[d+1]) of
 * the means / weights arrays (offsets[0] = 0, non-decreasing).
 *
 * gpu_grouped_compress_weighted (gpu/grouped.mojo:415-427, called from
 * grouped.mojo:144-157): for every key k < num_keys, the P-path compress of its
 * prior centroids (prior CSR, NULL prior_offsets: none) followed by its new
 * samples in batch order, each of weight new_weights[k] (NULL: 1).  A key with
 * neither gets no centroids.  The result is the output CSR over keys:
 * out_offsets (num_keys + 1, always filled), out_means / out_weights of cap
 * entries (KD_ERANGE with *out_n = the needed total when cap is too small).
 * out_min / out_max (num_keys, may be NULL): the range of each key's new
 * samples (0 without).  Everything is validated before any work (KD_EINVAL:
 * key out of range, non-finite value, weight <= 0).  Host pointers. */
KD_API int kd_grouped_compress(kd_session* s, int scale, double compression, int64_t num_keys,
                               const uint32_t* keys, const double* values, int64_t n,
                               const double* new_weights, const int64_t* prior_offsets,
                               const double* prior_means, const double* prior_weights,
                               int64_t* out_offsets, double* out_means, double* out_weights,
                               int64_t cap, int64_t* out_n, double* out_min, double* out_max);
/* gpu_quantile / gpu_cdf (gpu/query.mojo:320-342) for many digests at once:
 * query i reads digest ids[i] (ids NULL: digest 0) of the caller's CSR, with
 * that digest's min_v / max_v.  As the reference kernels: the walk's total is
 * the digest's weights summed in order (<= 0 -> 1), a tail centroid of raw
 * weight <= 1 + 1e-6 is a singleton, q <= 0 / q >= 1 give min / max (no range
 * error).  An empty digest gives KD_EEMPTY, one above 1024 centroids KD_ERANGE,
 * an id out of range KD_EINVAL (NaN for those queries; the first status is
 * returned).  Host pointers, or device pointers with KD_PTR_DEVICE. */
KD_API int kd_quantile(kd_session* s, const int64_t* offsets, int64_t ndigests, const double* means,
                       const double* weights, const double* min_v, const double* max_v,
                       const uint32_t* ids, const double* qs, int64_t nq, double* out, int flags);
KD_API int kd_cdf(kd_session* s, const int64_t* offsets, int64_t ndigests, const double* means,
                  const double* weights, const double* min_v, const double* max_v,
                  const uint32_t* ids, const double* xs, int64_t nx, double* out, int flags);
/* gpu_merge_digests (gpu/query.mojo:348-369), batched: group g is the P-path
 * compress of the centroids of parts part_ids[group_offsets[g] ..
 * group_offsets[g+1]) (part_ids NULL: parts group_offsets[g] .. in order),
 * concatenated in that order.  Parts are a CSR (part_offsets, nparts + 1).
 * Output CSR over groups as kd_grouped_compress.  Host pointers. */
KD_API int kd_merge(kd_session* s, int scale, double compression, const int64_t* part_offsets,
                    int64_t nparts, const double* means, const double* weights,
                    const int64_t* group_offsets, int64_t ngroups, const uint32_t* part_ids,
                    int64_t* out_offsets, double* out_means, double* out_weights, int64_t cap,
                    int64_t* out_n);

/* Self-test of the integer-pipe FP64 helpers the query kernels use (no
 * counterpart in the reference): element by element over device arrays,
 * op 0 writes kd_div(a, b), 1 the FP64 a / b, 2 kd_half(a), 3 the FP64
 * a * 0.5, 4 the order of the helpers' keys of a and b (1 less, 0.5 equal,
 * 0 greater), 5 the FP64 order of a and b.  Synchronous; b unused by 2 and 3. */
KD_API int kd_selftest_fp64(int op, const double* a, const double* b, int64_t n, double* out);

/* Resident per-key digests (GroupedTDigest, grouped.mojo:30-58; one key is a
 * TDigest, tdigest.mojo:135-151): num_keys dense ids, shared scale, compression
 * and decay rate (Decay.rate / half_life, decay.mojo:24-47; 0 = none). */
KD_API int kd_store_create(kd_session* s, int64_t num_keys, int scale, double compression,
                           double decay_lambda, kd_store** out);
KD_API void kd_store_destroy(kd_store* st);

/* GroupedTDigest.add_batch (grouped.mojo:60-162) / TDigest.add_batch on the GPU
 * route (tdigest.mojo:223-315): unit-weight samples; keys may be NULL (all key 0).
 * The whole batch is validated before any digest changes. */
KD_API int kd_store_ingest(kd_store* st, const uint32_t* keys, const double* values, int64_t n,
                           int clock_mode, double timestamp, int flags);
/* A sequence of GroupedTDigest.add_batch calls (grouped.mojo:60-162), batch i
 * being keys[i] / values[i] / n[i] (keys NULL, or keys[i] NULL: all key 0) at
 * timestamps[i] (KD_CLOCK_TIME only).  Results are those of one
 * kd_store_ingest per batch, in order; the sort of each batch overlaps the
 * compress of the one before.  Stops at the first failing batch: the batches
 * before it stay committed, it and every later one change nothing, and
 * *batches_done (may be NULL) receives its position (nbatch on success).
 * Device pointers (KD_PTR_DEVICE) are read in place; host memory (pinned or
 * pageable) is copied batch by batch into device staging buffers by the copy
 * engine while earlier batches compute.  Under a session memory budget with
 * no room for the two extra ingest workspaces the batches run one
 * kd_store_ingest each (same results); a budget with no room for the staging
 * buffers of host inputs returns KD_ENOMEM before any batch runs.  No
 * reference counterpart beyond the add_batch loop it replaces. */
KD_API int kd_store_ingest_many(kd_store* st, int64_t nbatch, const uint32_t* const* keys,
                                const double* const* values, const int64_t* n, int clock_mode,
                                const double* timestamps, int flags, int64_t* batches_done);

/* The single-sample path of a one-key store (TDigest.add / add_at,
 * tdigest.mojo:153-175, 324-458): the reference's add loop over n samples in
 * order, which is also what TDigest.add_batch runs below its GPU crossover
 * (tdigest.mojo:177-221).  Each sample advances the clock by one (timestamps =
 * NULL) or to its timestamp when later (add_at), is buffered with weight *
 * e^{log_scale} (weights = NULL: 1.0), and a full buffer (5 * int(compression)
 * samples) runs the sequential merge pass.  As in the loop, samples before the
 * first invalid one (non-finite value, weight <= 0 or non-finite) stay applied
 * and the call returns KD_EINVAL.  quantile, cdf, to_bytes and export merge the
 * buffer first (tdigest.mojo:493, 542, 639); kd_store_ingest folds it into its
 * batch (tdigest.mojo:262-268).  Pointers are host or device (flags). */
KD_API int kd_store_add(kd_store* st, const double* values, const double* weights,
                        const double* timestamps, int64_t n, int flags);
/* TDigest.merge (tdigest.mojo:391-439): merges the buffered samples, if any. */
KD_API int kd_store_flush(kd_store* st);
/* TDigest.merge_into (tdigest.mojo:589-623) of two one-key stores: src is
 * merged and (with decay) renormalised in place, then its centroids join dst's
 * merge pass. */
KD_API int kd_store_merge_into(kd_store* dst, kd_store* src);

/* TDigest.quantile / cdf per (key, q|x) (tdigest.mojo:485-587); keys may be
 * NULL (all key 0).  Errors fill NaN and return the first failing status. */
KD_API int kd_store_quantile(kd_store* st, const uint32_t* keys, const double* qs, int64_t nq,
                             double* out, int flags);
KD_API int kd_store_cdf(kd_store* st, const uint32_t* keys, const double* xs, int64_t nx,
                        double* out, int flags);
/* kd_store_quantile and kd_store_cdf of one call in one kernel launch: nq
 * (qkeys, qs) quantile queries into qout and nc (ckeys, xs) cdf queries into
 * cout (keys NULL: all key 0).  With device pointers, a call with the same
 * arguments as the call before it is captured as a CUDA graph and replayed
 * from then on.  Errors fill NaN and return the first failing status.  Same
 * arithmetic as the two calls (tdigest.mojo:485-587). */
KD_API int kd_store_query_batch(kd_store* st, const uint32_t* qkeys, const double* qs, int64_t nq,
                                double* qout, const uint32_t* ckeys, const double* xs, int64_t nc,
                                double* cout, int flags);

/* gpu_merge_digests (gpu/query.mojo:348-369) with merge_into's rebasing
 * (tdigest.mojo:589-623), batched: dst key g becomes the P-path compress of the
 * concatenated centroids of src keys parts[group_offsets[g] .. group_offsets[g+1])
 * in order.  Host pointers. */
KD_API int kd_store_merge(kd_store* dst, kd_store* src, const int64_t* group_offsets,
                          const uint32_t* parts, int64_t ngroups);

/* One key's state.  header8 = compression, decay lambda, log_scale, clock,
 * stored_total, min, max, count (the to_bytes header, tdigest.mojo:634-648). */
KD_API int kd_store_get_digest(kd_store* st, uint32_t key, double* header8, double* means,
                               double* weights, int64_t cap, int64_t* out_count);
KD_API int kd_store_set_digest(kd_store* st, uint32_t key, const double* header8,
                               const double* means, const double* weights, int64_t count);

/* to_bytes / from_bytes wire format (tdigest.mojo:627-698). */
KD_API int kd_store_to_bytes(kd_store* st, uint32_t key, uint8_t* buf, int64_t cap,
                             int64_t* out_len);
KD_API int kd_store_from_bytes(kd_store* st, uint32_t key, const uint8_t* buf, int64_t len);

KD_API int kd_store_stats(kd_store* st, int64_t* num_keys, int64_t* total_centroids,
                          size_t* device_bytes);
/* Centroid count of every key (num_keys int32), e.g. GroupedTDigest.centroid_count
 * for all keys at once (grouped.mojo:182-185). */
KD_API int kd_store_counts(kd_store* st, int32_t* out, int flags);

/* to_bytes for many keys at once (tdigest.mojo:627-648 per record): the records
 * of keys[0..nkeys) (keys NULL: keys 0..nkeys-1) concatenated in buf;
 * offsets[i] (host, nkeys + 1 entries) is where record i starts and
 * offsets[nkeys] the total.  buf NULL computes the offsets only.  The reference
 * serialises one digest per call; batching the records is a checkpoint of a
 * resident store. */
KD_API int kd_store_export(kd_store* st, const uint32_t* keys, int64_t nkeys, uint8_t* buf,
                           int64_t cap, int64_t* offsets, int flags);
/* from_bytes for many keys (tdigest.mojo:650-698 per record): record i,
 * buf[offsets[i] .. offsets[i+1]), is installed as key keys[i] (keys NULL: i).
 * Every record is validated before any key changes (KD_EINVAL: version or key,
 * KD_ERANGE: truncated).  The store keeps its own compression and decay rate. */
KD_API int kd_store_import(kd_store* st, const uint32_t* keys, int64_t nkeys, const uint8_t* buf,
                           const int64_t* offsets, int flags);

/* Serving loop over a resident store (no counterpart in the reference, which
 * has none).  Client threads submit ingest and query requests with
 * non-decreasing timestamps; a worker thread serves them by continuous
 * batching in windows of `window_s` of the timestamp axis.  A window's queries
 * see the store as it was before the window's ingests; the window's ingests are
 * applied as one grouped batch (samples concatenated in arrival order, clocks
 * moved to the window's last ingest timestamp).  Windows close when a later
 * window's request arrives, on kd_server_advance past their end, or on flush, so
 * every result depends only on the request stream.  Requests are validated at
 * submit (KD_EINVAL: key out of range, non-finite value, q outside [0,1],
 * decreasing timestamp or a closed window) and admitted against a device-memory
 * budget (budget_bytes, 0 = 1 TiB): the session's device memory when the server
 * started (its stores and workspaces) plus the device footprint of every
 * buffered or in-flight request (its staging, and about 100 bytes of ingest
 * workspace per ingest pair) must stay within it; submit blocks until there is
 * room, and returns KD_ENOMEM for a request that could not fit alone.  The
 * server also holds two staging buffer sets, pinned host and device memory for
 * groups of 2^22 ingest and 2^20 query pairs (about 68 MB each, allocated at
 * creation; grown for larger groups).  The store's session belongs to the
 * server until it is destroyed.  Query outputs are written to `out` (n doubles, kept valid until
 * the request is waited for); a query of an empty digest completes with
 * KD_EEMPTY and NaN. */
#define KD_REQ_INGEST 0
#define KD_REQ_QUANTILE 1
#define KD_REQ_CDF 2
typedef struct kd_server kd_server;
KD_API int kd_server_create(kd_store* st, double window_s, size_t budget_bytes, kd_server** out);
KD_API int kd_server_submit(kd_server* srv, int kind, double timestamp, const uint32_t* keys,
                            const double* vals, int64_t n, double* out, int64_t* ticket);
/* The client's clock reached now_ts: windows ending at or before it close. */
KD_API int kd_server_advance(kd_server* srv, double now_ts);
/* Waits for a request (timeout_s < 0: no limit; KD_ETIMEOUT when it runs out);
 * *status receives the request's own status. */
KD_API int kd_server_wait(kd_server* srv, int64_t ticket, double timeout_s, int* status);
/* Submit-to-completion latency of a completed request not yet waited for
 * (-1 while it is pending); KD_EINVAL for an unknown ticket. */
KD_API int kd_server_latency(kd_server* srv, int64_t ticket, double* seconds);
/* Device bytes counted against the budget now (the baseline plus buffered
 * requests), their peak so far, the budget, and the session's device memory
 * plus the server's staging buffers measured after the last window.  Any
 * pointer may be NULL. */
KD_API int kd_server_memory(kd_server* srv, size_t* in_use, size_t* peak, size_t* budget,
                            size_t* measured);
/* Closes every open window and waits until all submitted requests completed. */
KD_API int kd_server_flush(kd_server* srv);
/* Submit-to-completion latency percentiles in seconds (p50, p99, p999), requests
 * completed, windows served and seconds the worker spent serving windows.  The
 * percentiles are exact over the first 2^20 completed requests; after that they
 * are taken over a uniform sample of 2^20 of all completed requests (reservoir
 * sampling, seeded: the same completions give the same sample). */
KD_API int kd_server_stats(kd_server* srv, double* lat3, int64_t* completed, int64_t* windows,
                           double* busy_s);
/* Windows that were closed together when the worker took them run as one
 * group through the pipelined ingest: one window's prep and sort on the device
 * beside the previous window's queries, compress and commit.  Groups run so
 * far, the windows that ran in groups of two or more, the longest group in
 * seconds (queries, ingest and completion), the groups that took longer than
 * 10 ms, and the seconds the worker spent packing groups and starting their
 * copies (buffer growth included).  Any pointer may be NULL. */
KD_API int kd_server_groups(kd_server* srv, int64_t* groups, int64_t* windows_grouped,
                            double* max_group_s, int64_t* slow_groups, double* stage_s);
KD_API void kd_server_destroy(kd_server* srv);

/* Key dictionary.  No counterpart in the reference: GroupedTDigest.add_batch
 * takes dense ids in [0, num_keys) (grouped.mojo:60-63) and leaves the mapping
 * from application keys to them to the caller.  A kd_keymap maps arbitrary
 * 64-bit keys to dense ids on the device, ready to pass to kd_store_ingest with
 * KD_PTR_DEVICE.  Ids are handed out in first-seen order across calls; within
 * one call, the order among keys new to the map is unspecified.  Once given, an
 * id never changes.  The key value UINT64_MAX is reserved (KD_EINVAL).  A map of
 * `capacity` ids holds 12 bytes per slot, with at least 2 * capacity slots.
 * kd_keymap_map inserts unknown keys; past capacity it returns KD_ENOMEM, and
 * the keys that did get ids keep them.  kd_keymap_lookup inserts nothing and
 * writes UINT32_MAX for unknown keys.  keys and ids are device pointers with
 * KD_PTR_DEVICE in flags, else host pointers. */
typedef struct kd_keymap kd_keymap;
KD_API int kd_keymap_create(kd_session* s, int64_t capacity, kd_keymap** out);
KD_API int kd_keymap_map(kd_keymap* m, const uint64_t* keys, int64_t n, uint32_t* ids, int flags);
KD_API int kd_keymap_lookup(kd_keymap* m, const uint64_t* keys, int64_t n, uint32_t* ids,
                            int flags);
/* Number of ids handed out; -1 for a map whose session is gone. */
KD_API int64_t kd_keymap_size(kd_keymap* m);
KD_API void kd_keymap_destroy(kd_keymap* m);

/* No counterpart in the reference.  kd_compress for callers that cannot call
 * cudaMalloc: a host program whose own pool owns all device memory (memory taken
 * behind its back is unaccounted and may not exist), or a latency-critical loop
 * where cudaMalloc/cudaFree would synchronise the device.  Same arguments and
 * results as kd_compress, without a session: work runs on `stream` (a
 * cudaStream_t; NULL = the legacy default stream) of the current device, and
 * the call returns once that work is done.  It allocates nothing: its working
 * memory is one fixed device array of KD_NOALLOC_SCRATCH_BYTES in the library,
 * held on every GPU that loads the library until the process exits.
 * n > KD_NOALLOC_MAX_N returns KD_ERANGE with *out_n = 0.  KD_ENOMEM would
 * mean an input needed more working memory than the array's fixed layout; no
 * input of at most KD_NOALLOC_MAX_N centroids does (each level of the tile
 * hierarchy holds at most what the level before it held).  The first call on a
 * device resolves that array's address and sets kernel attributes.  No call
 * can be captured in a CUDA graph: each one synchronises its stream and reads
 * results back through host memory, so a call on a capturing stream returns
 * KD_EINVAL without touching the stream.  All calls on a device share the array
 * (it keeps the last call's contents; each call clears what must start at
 * zero), so calls whose GPU work overlaps race and give wrong results.  On
 * failure, msg (may be NULL) receives up to msg_cap bytes of text. */
#define KD_NOALLOC_MAX_N 16384
#define KD_NOALLOC_SCRATCH_BYTES (2 * 1024 * 1024)
KD_API int kd_compress_noalloc(int scale, double compression, const double* means,
                               const double* weights, int64_t n, int flags, double* out_means,
                               double* out_weights, int64_t cap, int64_t* out_n, void* stream,
                               char* msg, int msg_cap);

#ifdef __cplusplus
}
#endif

#endif /* KDIGEST_GB300_H */
