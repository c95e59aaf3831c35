/*
 * kd_oracle.h — CPU restatement of the reference kdigest algorithms (TEST
 * INFRASTRUCTURE ONLY).
 *
 * This library is the correctness oracle for the GB300 kernels and the timed
 * CPU baseline.  It is never linked into, loaded by, or called from the
 * product library: only the tests, the smoke check and the benchmark's CPU
 * baseline leg use it, and only as a checker or a timed reference.
 *
 * Semantics follow the reference source (paths inside the kdigest project):
 *   src/kdigest/scale.mojo, decay.mojo, centroid.mojo, tdigest.mojo,
 *   grouped.mojo, gpu/add_batch.mojo, gpu/grouped.mojo, gpu/query.mojo,
 *   gpu/sort.mojo, gpu/primitives.mojo
 * in FP64 (the reference's GPU path is FP32).  Sums keep the reference's own
 * association order: the Hillis-Steele scans of the P-path tile kernels and
 * the serial loops of the host code.
 */
#ifndef KD_ORACLE_H
#define KD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KDO_OK 0
#define KDO_EINVAL 1
#define KDO_EEMPTY 2
#define KDO_ERANGE 3
#define KDO_ECONVERGE 4

#define KDO_BLOCK_CAP 1024

/* Transcendentals of the scale functions: the FP64 functions shared with the
 * kernels (default), or the C library's log / asin. */
#define KDO_MATH_SHARED 0
#define KDO_MATH_LIBM 1
void kdo_set_math(int mode);
int kdo_get_math(void);

/* Association of the segment sums of w*x: the kernels' order (default) or
 * the reference's segmented Hillis-Steele tree.  Prefix sums, tile totals and
 * segment weights always take the reference's association. */
#define KDO_SUMS_BUILD 0
#define KDO_SUMS_REFERENCE 1
void kdo_set_sums(int mode);
int kdo_get_sums(void);

/* One P-path tile (gpu/add_batch.mojo:45-222) of n <= 1024 mean-sorted pairs.
 * Returns the number of centroids written; ids_out (optional, n entries)
 * receives each element's bucket id. */
int kdo_tile_compress(int scale, double compression, const double* x, const double* w,
                      int n, double* out_m, double* out_w, int32_t* ids_out);
/* The same tile through the reference kernel's 1024-lane loops run literally
 * (ten scan rounds per sum, segment flags, zero-padded lanes). */
int kdo_tile_compress_literal(int scale, double compression, const double* x, const double* w,
                              int n, double* out_m, double* out_w, int32_t* ids_out);

/* P-path compress of an arbitrary (mean, weight) set: stable sort by mean, then
 * the 1024-tile hierarchy.  out_* need capacity n.  perm_out (optional, n
 * entries) receives the stable sort permutation.  Returns the centroid count,
 * or -KDO_ECONVERGE when a pass stops shrinking the set. */
int64_t kdo_ppath_compress(int scale, double compression, const double* means,
                           const double* weights, int64_t n, double* out_m, double* out_w,
                           int64_t* perm_out);

typedef struct kdo_digest kdo_digest;

kdo_digest* kdo_digest_new(int scale, double compression, double decay_lambda);
kdo_digest* kdo_digest_clone(const kdo_digest* d);
void kdo_digest_free(kdo_digest* d);

/* S-path (sequential greedy sweep) API — tdigest.mojo:153-175, 391-458. */
int kdo_add(kdo_digest* d, double value, double weight);
int kdo_add_at(kdo_digest* d, double value, double timestamp, double weight);
int kdo_add_many(kdo_digest* d, const double* values, int64_t n);
void kdo_merge(kdo_digest* d);
int kdo_merge_into(kdo_digest* d, kdo_digest* other);

/* P-path batch ingest (the GPU route of add_batch) — tdigest.mojo:223-315.
 * kdo_add_batch_p advances the clock by n (count clock); kdo_add_batch_p_at
 * moves it to `timestamp` when later (time clock, add_at semantics). */
int kdo_add_batch_p(kdo_digest* d, const double* values, int64_t n);
int kdo_add_batch_p_at(kdo_digest* d, const double* values, int64_t n, double timestamp);

/* Queries — tdigest.mojo:485-587.  Return KDO_EINVAL / KDO_EEMPTY on error. */
int kdo_quantile(kdo_digest* d, double q, double* out);
int kdo_cdf(kdo_digest* d, double x, double* out);

/* Serialization — tdigest.mojo:627-698.  kdo_to_bytes returns the byte count
 * (writing only when cap suffices). */
int64_t kdo_to_bytes(kdo_digest* d, uint8_t* buf, int64_t cap);
kdo_digest* kdo_from_bytes(const uint8_t* buf, int64_t len, int scale, int* err);

/* Accessors.  state8 = compression, lambda, log_scale, clock, stored_total,
 * min, max, centroid count. */
int64_t kdo_len(const kdo_digest* d);
double kdo_total_weight(const kdo_digest* d);
void kdo_state(const kdo_digest* d, double* state8);
int64_t kdo_centroids(const kdo_digest* d, double* means, double* weights, int64_t cap);
int kdo_set_state(kdo_digest* d, const double* means, const double* weights, int64_t n,
                  double stored_total, double log_scale, double clock, double min_v,
                  double max_v);

/* Grouped ingest — grouped.mojo:60-162: validate everything first, then each
 * touched key takes the P-path batch of its own samples (batch order kept).
 * mode 0 = count clock, 1 = time clock at `timestamp`.  threads > 1 partitions
 * keys over that many threads. */
int kdo_grouped_add_batch(kdo_digest** digests, int64_t num_keys, const uint32_t* keys,
                          const double* values, int64_t n, int mode, double timestamp,
                          int threads);

/* gpu_merge_digests semantics (query.mojo:348-369) applied through merge_into's
 * rebasing: parts are renormalised, their centroids concatenated in part order
 * and compressed once with the P-path into `dst` (which is reset first). */
int kdo_merge_parts_p(kdo_digest* dst, kdo_digest** parts, int64_t nparts);

/* Batched queries: out[i] = quantile (is_cdf = 0) or cdf of digests[ids[i]] at
 * x[i] (tdigest.mojo:485-587), split over `threads` threads.  Every digest is
 * merged first, so the queries only read.  A failing query gives NaN; the
 * first failing status is returned. */
int kdo_query_batch(kdo_digest** digests, int64_t nd, const int32_t* ids, const double* x,
                    int64_t n, int is_cdf, double* out, int threads);

/* Exports of the shared FP64 scale arithmetic (kd_math.h), for accuracy tests. */
double kdo_log(double x);
double kdo_exp(double x);
double kdo_asin(double x);
double kdo_normalizer(int scale, double compression, double n);
double kdo_k(int scale, double q, double nrm);
int32_t kdo_bucket(int scale, double cum, double tot, double nrm);

#ifdef __cplusplus
}
#endif

#endif
