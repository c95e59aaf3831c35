/*
 * kd_oracle.c — CPU restatement of the reference kdigest algorithms.
 *
 * TEST INFRASTRUCTURE ONLY: the correctness oracle and the timed CPU baseline.
 * The product library never links, loads or calls this file.
 *
 * Build: cc -O2 -std=c11 -ffp-contract=off -fPIC -shared -pthread (see Makefile).
 * -ffp-contract=off is required: the bucket ids must be computed with exactly
 * the rounding the device kernels use (kd_math.h).
 */
#include "kd_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../kdigest_gb300/csrc/kd_math.h"

/* tdigest.mojo:39-61 */
#define BUFFER_FACTOR 5
#define RENORM_LOG_THRESHOLD 400.0
#define PRUNE_EPSILON 1e-6
#define SERDE_VERSION 1

static double canon(double v) { return v == 0.0 ? 0.0 : v; } /* -0.0 -> +0.0 */

/* ------------------------------------------------------------------------- */
/* Scale arithmetic.  Default: the FP64 functions of kd_math.h (the kernels   */
/* compute the same bits).  KDO_MATH_LIBM evaluates the same formulas         */
/* (scale.mojo:78-192) with the C library's log / asin instead, which is what */
/* the reference's std.math calls lower to on its CPU; tests use it to        */
/* measure how many bucket ids depend on the transcendental implementation.   */
/* ------------------------------------------------------------------------- */
static int g_math = KDO_MATH_SHARED;

void kdo_set_math(int mode) { g_math = mode == KDO_MATH_LIBM ? KDO_MATH_LIBM : KDO_MATH_SHARED; }
int kdo_get_math(void) { return g_math; }

static double libm_normalizer(int scale, double compression, double n) {
  switch (scale) {
    case KD_SCALE_K0: return compression / 2.0;
    case KD_SCALE_K1: return compression / (2.0 * 3.141592653589793);
    case KD_SCALE_K2: return compression / (4.0 * log(n / compression) + 24.0);
    default: return compression / (4.0 * log(n / compression) + 21.0);
  }
}
static double libm_k(int scale, double q, double nrm) {
  switch (scale) {
    case KD_SCALE_K0: return nrm * q;
    case KD_SCALE_K1: return nrm * asin(2.0 * q - 1.0);
    case KD_SCALE_K2: {
      double qc = kd_clamp_q(q);
      return nrm * log(qc / (1.0 - qc));
    }
    default: {
      double qc = kd_clamp_q(q);
      if (qc <= 0.5) return nrm * log(2.0 * qc);
      return -nrm * log(2.0 * (1.0 - qc));
    }
  }
}
static double o_normalizer(int scale, double compression, double n) {
  return g_math == KDO_MATH_LIBM ? libm_normalizer(scale, compression, n)
                                 : kd_normalizer(scale, compression, n);
}
static double o_k(int scale, double q, double nrm) {
  return g_math == KDO_MATH_LIBM ? libm_k(scale, q, nrm) : kd_k(scale, q, nrm);
}
static int32_t o_bucket(int scale, double cum, double tot, double nrm) {
  return kd_floor_i32(o_k(scale, cum / tot, nrm));
}

/* ------------------------------------------------------------------------- */
/* P-path tile compress.                                                      */
/*                                                                            */
/* _compress_block_kernel (gpu/add_batch.mojo:45-222) and the grouped kernel  */
/* (gpu/grouped.mojo:128-276) compress a sorted tile of n <= 1024 pairs on    */
/* BLOCK_CAP = 1024 lanes (weights and means of lanes >= n are 0):            */
/*   1. cum = Hillis-Steele inclusive scan of w (:79-95), offsets 1,2,..,512  */
/*      (cum[i] += cum[i - off] for i >= off);                                */
/*   2. total = cum[1023] (:97-100; <= 0 -> 1), id = floor(k(cum[i]/total))   */
/*      (:102-112);                                                           */
/*   3. heads where the id changes (:114-121);                               */
/*   4. segmented Hillis-Steele scans of w and w*x (:123-160);              */
/*   5. segment ends emit mean = sum(wx)/sum(w) (0 for zero weight) clamped  */
/*      to the segment's [first, last] value, and sum(w) (:162-218).         */
/* kdo_tile_compress_literal below runs exactly those lane loops.            */
/* kdo_tile_compress computes the same prefix, total, ids and weights with   */
/* less work:                                                                 */
/*   - cum[i] is the Hillis-Steele value itself (all offsets, in place in    */
/*     descending index order, which reads only values of the previous       */
/*     round); with integral weights every partial sum is exact and a plain  */
/*     running sum gives the same bits;                                       */
/*   - total is the scan's lane 1023: a balanced pairwise tree over lanes     */
/*     [0, 1024), i.e. over [0, 2^ceil(log2 n)) since adding a zero lane is   */
/*     exact;                                                                 */
/*   - a segment's scan value at its end element e (head h) is the sum of     */
/*     x[h..e] in the right-aligned pairwise tree: level-1 pairs (e, e-1),    */
/*     (e-2, e-3), ..., each level pairing the previous level's nodes from   */
/*     the e side, a node without partner carried up unchanged (the scan      */
/*     stops adding once its window reaches the head), plus the zero the     */
/*     scan adds in its later rounds.  That is the reference scan's value at */
/*     e with e - h additions instead of ~10 per lane.                        */
/* Segment sums of w*x come in two associations (kdo_set_sums):              */
/*   - KDO_SUMS_REFERENCE: the reference's tree above;                        */
/*   - KDO_SUMS_BUILD (default): the order the kernels use, which keeps their */
/*     FP64 pipe busy: tiles of at most KD_SERIAL_TILE_MAX elements sum each  */
/*     segment serially, left to right; larger tiles cut the tile into 128    */
/*     chunks of E = ceil(n/128) consecutive elements (one per thread of a    */
/*     4-warp block), sum each piece of a segment inside a chunk serially,    */
/*     carry the trailing pieces across the 32 chunks of each warp with a     */
/*     segmented Kogge-Stone scan, then across the 4 warps in order.          */
/* The two differ by rounding in the means only: no prefix, id or weight     */
/* depends on sum(w*x).  The tests check the reference form against the lane */
/* loops bit for bit and the build form against the reference form.          */
/* ------------------------------------------------------------------------- */
static int g_sums = KDO_SUMS_BUILD;

void kdo_set_sums(int mode) { g_sums = mode == KDO_SUMS_REFERENCE ? KDO_SUMS_REFERENCE : KDO_SUMS_BUILD; }
int kdo_get_sums(void) { return g_sums; }

static int small_int(double w) { /* an integral weight in [1, 2^42), as the kernels test it */
  if (!(w >= 1.0 && w < 4398046511104.0)) return 0;
  return floor(w) == w;
}

/* Sum of v[0..len) in the right-aligned pairwise tree, v[len-1] being the
 * segment's end element.  tmp holds at least (len + 1) / 2 entries. */
static double rapt_sum(const double* v, int len, double* tmp) {
  if (len == 1) return v[0];
  int m = 0;
  for (int u = 0; u < len; u += 2) { /* u: distance from the end */
    const double a = v[len - 1 - u];
    tmp[m++] = u + 1 < len ? a + v[len - 2 - u] : a;
  }
  while (m > 1) {
    int k = 0;
    for (int u = 0; u < m; u += 2) tmp[k++] = u + 1 < m ? tmp[u] + tmp[u + 1] : tmp[u];
    m = k;
  }
  return tmp[0];
}

/* Total of the tile: the balanced tree over lanes [0, 2^ceil(log2 n)). */
static double tree_total(const double* w, int n, double* tmp) {
  if (n == 1) return w[0];
  int m = 0;
  for (int i = 0; i < n; i += 2) tmp[m++] = i + 1 < n ? w[i] + w[i + 1] : w[i];
  while (m > 1) {
    int k = 0;
    for (int i = 0; i < m; i += 2) tmp[k++] = i + 1 < m ? tmp[i] + tmp[i + 1] : tmp[i];
    m = k;
  }
  return tmp[0];
}

static int emit_segment(const double* x, int h, int e, double sw, double swx, double* out_m,
                        double* out_w, int cnt) {
  double mean = sw > 0.0 ? swx / sw : 0.0;
  double lo_v = x[h], hi_v = x[e];
  mean = mean < lo_v ? lo_v : mean;
  mean = mean > hi_v ? hi_v : mean;
  out_m[cnt] = mean;
  out_w[cnt] = sw;
  return cnt + 1;
}

/* sum(w*x) of every segment in the kernels' order (KDO_SUMS_BUILD), written
 * at each segment end e into swx[e]. */
static void build_order_wx(const double* wx, const int32_t* id, int n, double* swx) {
  if (n <= KD_SERIAL_TILE_MAX) {
    double a = 0.0;
    for (int i = 0; i < n; ++i) {
      a = (i == 0 || id[i] != id[i - 1]) ? wx[i] : a + wx[i];
      if (i == n - 1 || id[i] != id[i + 1]) swx[i] = a;
    }
    return;
  }
  enum { C = 128, G = 32 }; /* chunks, chunks per group (a warp of the block) */
  const int E = (n + C - 1) / C;
  double V[C];
  int F[C];
  int pend[C];
  double pendv[C];
  for (int c = 0; c < C; ++c) {
    V[c] = 0.0;
    F[c] = 0;
    pend[c] = -1;
    int lo = c * E, hi = lo + E < n ? lo + E : n;
    if (lo >= n) continue;
    double a = 0.0;
    for (int i = lo; i < hi; ++i) {
      const int head = (i == 0) || id[i] != id[i - 1];
      a = (head || i == lo) ? wx[i] : a + wx[i];
      if (head) F[c] = 1;
      if (i == n - 1 || id[i] != id[i + 1]) {
        if (F[c]) swx[i] = a;
        else { pend[c] = i; pendv[c] = a; } /* segment started in an earlier chunk */
      }
    }
    V[c] = a;
  }
  /* segmented inclusive Kogge-Stone over the chunks of each group */
  for (int g = 0; g < C / G; ++g) {
    double* Vg = V + g * G;
    int* Fg = F + g * G;
    for (int o = 1; o < G; o <<= 1) {
      double tv[G];
      int tf[G];
      for (int c = 0; c < G; ++c) { tv[c] = Vg[c]; tf[c] = Fg[c]; }
      for (int c = o; c < G; ++c) {
        if (!tf[c]) Vg[c] = tv[c] + tv[c - o];
        Fg[c] = tf[c] | tf[c - o];
      }
    }
  }
  /* carried across the groups in order: a chunk with no head since its group
   * began adds the final value of the previous group's last chunk */
  for (int g = 1; g < C / G; ++g) {
    const double carry = V[g * G - 1];
    for (int c = g * G; c < (g + 1) * G; ++c)
      if (!F[c]) V[c] = V[c] + carry;
  }
  for (int c = 1; c < C; ++c)
    if (pend[c] >= 0) swx[pend[c]] = V[c - 1] + pendv[c];
}

int kdo_tile_compress(int scale, double compression, const double* x, const double* w,
                      int n, double* out_m, double* out_w, int32_t* ids_out) {
  if (n <= 0) return 0;
  if (n > KDO_BLOCK_CAP) return -1;
  double cum[KDO_BLOCK_CAP], wx[KDO_BLOCK_CAP], seg[KDO_BLOCK_CAP], tmp[KDO_BLOCK_CAP];
  double swxb[KDO_BLOCK_CAP];
  int32_t id[KDO_BLOCK_CAP];
  int integral = 1;
  for (int i = 0; i < n; ++i) integral &= small_int(w[i]);
  double tot;
  if (integral) { /* exact: any order gives these bits */
    double acc = w[0];
    cum[0] = acc;
    for (int i = 1; i < n; ++i) {
      acc = acc + w[i];
      cum[i] = acc;
    }
    tot = cum[n - 1];
  } else {
    for (int i = 0; i < n; ++i) cum[i] = w[i];
    for (int off = 1; off < n; off <<= 1)
      for (int i = n - 1; i >= off; --i) cum[i] = cum[i] + cum[i - off];
    tot = tree_total(w, n, tmp);
  }
  if (!(tot > 0.0)) tot = 1.0; /* add_batch.mojo:98-100 */
  double nrm = o_normalizer(scale, compression, tot);
  for (int i = 0; i < n; ++i) id[i] = o_bucket(scale, cum[i], tot, nrm);
  if (ids_out)
    for (int i = 0; i < n; ++i) ids_out[i] = id[i];
  for (int i = 0; i < n; ++i) wx[i] = w[i] * x[i];
  if (g_sums == KDO_SUMS_BUILD) build_order_wx(wx, id, n, swxb);
  int cnt = 0;
  for (int h = 0; h < n;) {
    int e = h;
    while (e + 1 < n && id[e + 1] == id[h]) ++e;
    const int len = e - h + 1;
    double sw;
    if (integral) {
      sw = w[h];
      for (int i = h + 1; i <= e; ++i) sw = sw + w[i];
    } else {
      for (int i = 0; i < len; ++i) seg[i] = w[h + i];
      sw = rapt_sum(seg, len, tmp);
    }
    const double swx = g_sums == KDO_SUMS_BUILD ? swxb[e] : rapt_sum(wx + h, len, tmp) + 0.0;
    cnt = emit_segment(x, h, e, sw, swx, out_m, out_w, cnt);
    h = e + 1;
  }
  return cnt;
}

/* The reference's lane loops, literally (FP64; test use only). */
int kdo_tile_compress_literal(int scale, double compression, const double* x, const double* w,
                              int n, double* out_m, double* out_w, int32_t* ids_out) {
  enum { B = KDO_BLOCK_CAP };
  if (n <= 0) return 0;
  if (n > B) return -1;
  static _Thread_local double lw[B], cum[B], tmp[B], sw[B], smw[B], nw[B], nmw[B], seg_lo[B];
  static _Thread_local int32_t cid[B], fl[B], nfl[B], is_end[B], pos[B], npos[B];
  for (int t = 0; t < B; ++t) lw[t] = t < n ? w[t] : 0.0;
  for (int t = 0; t < B; ++t) cum[t] = lw[t];
  for (int off = 1; off < B; off *= 2) {
    for (int t = 0; t < B; ++t) tmp[t] = t >= off ? cum[t] + cum[t - off] : cum[t];
    for (int t = 0; t < B; ++t) cum[t] = tmp[t];
  }
  double total = cum[B - 1];
  if (total <= 0.0) total = 1.0;
  const double nrm = o_normalizer(scale, compression, total);
  for (int t = 0; t < B; ++t)
    cid[t] = t < n ? kd_floor_i32(o_k(scale, cum[t] / total, nrm)) : 2147483647;
  if (ids_out)
    for (int t = 0; t < n; ++t) ids_out[t] = cid[t];
  for (int t = 0; t < B; ++t) fl[t] = t == 0 ? 1 : (cid[t] != cid[t - 1] ? 1 : 0);
  for (int t = 0; t < B; ++t) {
    sw[t] = lw[t];
    smw[t] = lw[t] * (t < n ? x[t] : 0.0);
  }
  for (int voff = 1; voff < B; voff *= 2) {
    for (int t = 0; t < B; ++t) {
      double add_w = 0.0, add_mw = 0.0;
      if (t >= voff && fl[t] == 0) {
        add_w = sw[t - voff];
        add_mw = smw[t - voff];
      }
      nfl[t] = t >= voff ? ((fl[t] != 0 || fl[t - voff] != 0) ? 1 : 0) : fl[t];
      nw[t] = sw[t] + add_w;
      nmw[t] = smw[t] + add_mw;
    }
    for (int t = 0; t < B; ++t) {
      sw[t] = nw[t];
      smw[t] = nmw[t];
      fl[t] = nfl[t];
    }
  }
  for (int t = 0; t < B; ++t) {
    is_end[t] = 0;
    if (t < n) is_end[t] = (t == n - 1 || cid[t] != cid[t + 1]) ? 1 : 0;
  }
  for (int t = 0; t < B; ++t) pos[t] = is_end[t];
  for (int poff = 1; poff < B; poff *= 2) {
    for (int t = 0; t < B; ++t) npos[t] = t >= poff ? pos[t] + pos[t - poff] : pos[t];
    for (int t = 0; t < B; ++t) pos[t] = npos[t];
  }
  for (int t = 0; t < n; ++t) {
    const int is_head = t == 0 || cid[t] != cid[t - 1];
    if (is_head) seg_lo[t == 0 ? 0 : pos[t - 1]] = x[t];
  }
  int cnt = 0;
  for (int t = 0; t < n; ++t) {
    if (!is_end[t]) continue;
    const int slot = pos[t] - 1;
    double mean = sw[t] > 0.0 ? smw[t] / sw[t] : 0.0;
    const double lo_v = seg_lo[slot], hi_v = x[t];
    mean = mean < lo_v ? lo_v : mean;
    mean = mean > hi_v ? hi_v : mean;
    out_m[slot] = mean;
    out_w[slot] = sw[t];
    ++cnt;
  }
  return cnt;
}

/* ------------------------------------------------------------------------- */
/* Stable sort by mean (ties keep input order) — the order of gpu/sort.mojo   */
/* (_before: key, then original index) and cpu_sort_pairs (primitives.mojo:   */
/* 421-498).  Bottom-up merge sort on an index permutation.                   */
/* ------------------------------------------------------------------------- */
static void stable_sort_perm(const double* key, int64_t n, int64_t* perm) {
  for (int64_t i = 0; i < n; ++i) perm[i] = i;
  if (n < 2) return;
  int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
  int64_t* src = perm;
  int64_t* dst = tmp;
  for (int64_t width = 1; width < n; width *= 2) {
    for (int64_t lo = 0; lo < n; lo += 2 * width) {
      int64_t mid = lo + width < n ? lo + width : n;
      int64_t hi = lo + 2 * width < n ? lo + 2 * width : n;
      int64_t a = lo, b = mid, o = lo;
      while (a < mid && b < hi) {
        if (key[src[a]] <= key[src[b]]) dst[o++] = src[a++];
        else dst[o++] = src[b++];
      }
      while (a < mid) dst[o++] = src[a++];
      while (b < hi) dst[o++] = src[b++];
    }
    int64_t* t = src;
    src = dst;
    dst = t;
  }
  if (src != perm) memcpy(perm, src, sizeof(int64_t) * (size_t)n);
  free(tmp);
}

/* ------------------------------------------------------------------------- */
/* P-path hierarchy — gpu_compress_batch_host_tiled (add_batch.mojo:308-347): */
/* sort, compress every 1024 tile, concatenate, repeat while the pass input   */
/* exceeded one tile.  The reference loops forever when a pass cannot shrink  */
/* the set; the restatement reports KDO_ECONVERGE instead.                    */
/* ------------------------------------------------------------------------- */
int64_t kdo_ppath_compress(int scale, double compression, const double* means,
                           const double* weights, int64_t n, double* out_m, double* out_w,
                           int64_t* perm_out) {
  if (n <= 0) return 0;
  double* cm = (double*)malloc(sizeof(double) * (size_t)n);
  double* cw = (double*)malloc(sizeof(double) * (size_t)n);
  double* key = (double*)malloc(sizeof(double) * (size_t)n);
  int64_t* perm = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
  for (int64_t i = 0; i < n; ++i) key[i] = canon(means[i]);
  stable_sort_perm(key, n, perm);
  if (perm_out) memcpy(perm_out, perm, sizeof(int64_t) * (size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    cm[i] = key[perm[i]];
    cw[i] = weights[perm[i]];
  }
  free(key);
  free(perm);
  int64_t m = n;
  double* nm = (double*)malloc(sizeof(double) * (size_t)n);
  double* nw = (double*)malloc(sizeof(double) * (size_t)n);
  for (;;) {
    /* The survivors of a pass are non-decreasing (each mean is clamped to its
     * segment), so the reference's re-sort between passes is the identity. */
    int64_t next = 0;
    for (int64_t p = 0; p < m; p += KDO_BLOCK_CAP) {
      int t = (int)(m - p < KDO_BLOCK_CAP ? m - p : KDO_BLOCK_CAP);
      next += kdo_tile_compress(scale, compression, cm + p, cw + p, t, nm + next, nw + next, NULL);
    }
    int done = m <= KDO_BLOCK_CAP;
    if (!done && next == m) {
      free(cm); free(cw); free(nm); free(nw);
      return -KDO_ECONVERGE;
    }
    double* t1 = cm; cm = nm; nm = t1;
    double* t2 = cw; cw = nw; nw = t2;
    m = next;
    if (done) break;
  }
  memcpy(out_m, cm, sizeof(double) * (size_t)m);
  memcpy(out_w, cw, sizeof(double) * (size_t)m);
  free(cm); free(cw); free(nm); free(nw);
  return m;
}

/* ------------------------------------------------------------------------- */
/* TDigest — tdigest.mojo:97-726.                                             */
/* ------------------------------------------------------------------------- */
struct kdo_digest {
  int scale;
  double compression;
  double lambda;
  double *cm, *cw;
  int64_t nc, capc;
  double *bm, *bw;
  int64_t nb, capb;
  int64_t buffer_limit;
  double stored_total, log_scale, clock, min_v, max_v;
};

static void reserve_c(kdo_digest* d, int64_t n) {
  if (n <= d->capc) return;
  int64_t cap = d->capc * 2 > n ? d->capc * 2 : n;
  d->cm = (double*)realloc(d->cm, sizeof(double) * (size_t)cap);
  d->cw = (double*)realloc(d->cw, sizeof(double) * (size_t)cap);
  d->capc = cap;
}
static void reserve_b(kdo_digest* d, int64_t n) {
  if (n <= d->capb) return;
  int64_t cap = d->capb * 2 > n ? d->capb * 2 : n;
  d->bm = (double*)realloc(d->bm, sizeof(double) * (size_t)cap);
  d->bw = (double*)realloc(d->bw, sizeof(double) * (size_t)cap);
  d->capb = cap;
}

kdo_digest* kdo_digest_new(int scale, double compression, double decay_lambda) {
  kdo_digest* d = (kdo_digest*)calloc(1, sizeof(kdo_digest));
  d->scale = scale;
  d->compression = compression;
  d->lambda = decay_lambda;
  d->buffer_limit = (int64_t)compression * BUFFER_FACTOR; /* tdigest.mojo:146 */
  return d;
}

kdo_digest* kdo_digest_clone(const kdo_digest* s) {
  kdo_digest* d = kdo_digest_new(s->scale, s->compression, s->lambda);
  reserve_c(d, s->nc > 0 ? s->nc : 1);
  reserve_b(d, s->nb > 0 ? s->nb : 1);
  memcpy(d->cm, s->cm, sizeof(double) * (size_t)s->nc);
  memcpy(d->cw, s->cw, sizeof(double) * (size_t)s->nc);
  memcpy(d->bm, s->bm, sizeof(double) * (size_t)s->nb);
  memcpy(d->bw, s->bw, sizeof(double) * (size_t)s->nb);
  d->nc = s->nc;
  d->nb = s->nb;
  d->buffer_limit = s->buffer_limit;
  d->stored_total = s->stored_total;
  d->log_scale = s->log_scale;
  d->clock = s->clock;
  d->min_v = s->min_v;
  d->max_v = s->max_v;
  return d;
}

void kdo_digest_free(kdo_digest* d) {
  if (!d) return;
  free(d->cm); free(d->cw); free(d->bm); free(d->bw);
  free(d);
}

static int decay_active(const kdo_digest* d) { return d->lambda > 0.0; } /* decay.mojo:49-51 */

static int validate(double value, double weight) { /* tdigest.mojo:317-322 */
  if (!kd_isfinite(value)) return KDO_EINVAL;
  if (!(weight > 0.0) || !kd_isfinite(weight)) return KDO_EINVAL;
  return KDO_OK;
}

static void renormalize(kdo_digest* d) { /* tdigest.mojo:359-371 */
  double factor = kd_exp(-d->log_scale);
  for (int64_t i = 0; i < d->nc; ++i) d->cw[i] *= factor;
  for (int64_t i = 0; i < d->nb; ++i) d->bw[i] *= factor;
  d->stored_total *= factor;
  d->log_scale = 0.0;
}

static void advance_clock(kdo_digest* d, double new_clock) { /* tdigest.mojo:324-332 */
  if (decay_active(d) && new_clock > d->clock) {
    d->log_scale += d->lambda * (new_clock - d->clock);
    if (d->log_scale > RENORM_LOG_THRESHOLD) renormalize(d);
  }
  d->clock = new_clock;
}

static double scale_factor(const kdo_digest* d) { /* tdigest.mojo:352-357 */
  return decay_active(d) ? kd_exp(d->log_scale) : 1.0;
}

static double effective_count(const kdo_digest* d) { /* tdigest.mojo:373-377 */
  return decay_active(d) ? d->stored_total * kd_exp(-d->log_scale) : d->stored_total;
}

static void prune(kdo_digest* d) { /* tdigest.mojo:441-458 */
  double floor_w = PRUNE_EPSILON * kd_exp(d->log_scale);
  int64_t k = 0;
  double removed = 0.0;
  for (int64_t i = 0; i < d->nc; ++i) {
    if (d->cw[i] >= floor_w) {
      d->cm[k] = d->cm[i];
      d->cw[k] = d->cw[i];
      ++k;
    } else {
      removed += d->cw[i];
    }
  }
  if (removed > 0.0) {
    d->stored_total -= removed;
    d->nc = k;
  }
}

/* S-path merge pass — tdigest.mojo:391-439 (insertion sort :64-77 is stable). */
void kdo_merge(kdo_digest* d) {
  if (d->nb == 0) return;
  int64_t n = d->nc + d->nb;
  double* m = (double*)malloc(sizeof(double) * (size_t)n);
  double* w = (double*)malloc(sizeof(double) * (size_t)n);
  memcpy(m, d->cm, sizeof(double) * (size_t)d->nc);
  memcpy(w, d->cw, sizeof(double) * (size_t)d->nc);
  memcpy(m + d->nc, d->bm, sizeof(double) * (size_t)d->nb);
  memcpy(w + d->nc, d->bw, sizeof(double) * (size_t)d->nb);
  d->nb = 0;
  for (int64_t i = 1; i < n; ++i) {
    double km = m[i], kw = w[i];
    int64_t j = i - 1;
    while (j >= 0 && m[j] > km) {
      m[j + 1] = m[j];
      w[j + 1] = w[j];
      --j;
    }
    m[j + 1] = km;
    w[j + 1] = kw;
  }
  double effective_n = effective_count(d);
  double stored_n = d->stored_total;
  double nrm = o_normalizer(d->scale, d->compression, effective_n);
  reserve_c(d, n);
  int64_t k = 0;
  double cur_m = m[0], cur_w = w[0];
  double wsf = 0.0;
  for (int64_t i = 1; i < n; ++i) {
    double q_left = wsf / stored_n;
    double q_right = (wsf + cur_w + w[i]) / stored_n;
    double k_span = o_k(d->scale, q_right, nrm) - o_k(d->scale, q_left, nrm);
    if (m[i] == cur_m || k_span <= 1.0) {
      /* Centroid.add_sample — centroid.mojo:279-290 */
      double new_w = cur_w + w[i];
      cur_m += (m[i] - cur_m) * (w[i] / new_w);
      cur_w = new_w;
    } else {
      d->cm[k] = cur_m;
      d->cw[k] = cur_w;
      ++k;
      wsf += cur_w;
      cur_m = m[i];
      cur_w = w[i];
    }
  }
  d->cm[k] = cur_m;
  d->cw[k] = cur_w;
  ++k;
  d->nc = k;
  free(m);
  free(w);
  if (decay_active(d)) prune(d);
}

static void insert(kdo_digest* d, double value, double weight) { /* tdigest.mojo:334-350 */
  if (d->stored_total == 0.0 && d->nb == 0) {
    d->min_v = value;
    d->max_v = value;
  } else {
    if (value < d->min_v) d->min_v = value;
    if (value > d->max_v) d->max_v = value;
  }
  double scaled = weight * scale_factor(d);
  reserve_b(d, d->nb + 1);
  d->bm[d->nb] = value;
  d->bw[d->nb] = scaled;
  d->nb++;
  d->stored_total += scaled;
  if (d->nb >= d->buffer_limit) kdo_merge(d);
}

int kdo_add(kdo_digest* d, double value, double weight) { /* tdigest.mojo:153-161 */
  int e = validate(value, weight);
  if (e) return e;
  advance_clock(d, d->clock + 1.0);
  insert(d, value, weight);
  return KDO_OK;
}

/* The reference's add loop over an array of unit-weight samples (what
 * TDigest.add_batch runs below its GPU crossover, tdigest.mojo:199-202). */
int kdo_add_many(kdo_digest* d, const double* values, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    int e = kdo_add(d, values[i], 1.0);
    if (e) return e;
  }
  return KDO_OK;
}

int kdo_add_at(kdo_digest* d, double value, double timestamp, double weight) {
  int e = validate(value, weight); /* tdigest.mojo:163-175 */
  if (e) return e;
  if (timestamp > d->clock) advance_clock(d, timestamp);
  insert(d, value, weight);
  return KDO_OK;
}

/* _gpu_batch_prepare + P-path compress + _gpu_batch_finish
 * (tdigest.mojo:236-315).  new_clock_mode 0: clock += n; 1: clock = t if later. */
static int add_batch_p(kdo_digest* d, const double* values, int64_t n, int time_mode,
                       double timestamp) {
  if (n == 0) return KDO_OK;
  for (int64_t i = 0; i < n; ++i)
    if (validate(values[i], 1.0)) return KDO_EINVAL;
  if (time_mode) {
    if (timestamp > d->clock) advance_clock(d, timestamp);
  } else {
    advance_clock(d, d->clock + (double)n);
  }
  double sf = scale_factor(d);
  int64_t total_in = d->nc + d->nb + n;
  double* m = (double*)malloc(sizeof(double) * (size_t)total_in);
  double* w = (double*)malloc(sizeof(double) * (size_t)total_in);
  int64_t k = 0;
  for (int64_t i = 0; i < d->nc; ++i, ++k) { m[k] = d->cm[i]; w[k] = d->cw[i]; }
  for (int64_t i = 0; i < d->nb; ++i, ++k) { m[k] = d->bm[i]; w[k] = d->bw[i]; }
  int had_centroids = d->nc > 0;
  d->nb = 0;
  double vmin = values[0], vmax = values[0];
  for (int64_t i = 0; i < n; ++i, ++k) {
    double v = values[i];
    m[k] = v;
    w[k] = sf;
    if (v < vmin) vmin = v;
    if (v > vmax) vmax = v;
  }
  d->stored_total += (double)n * sf;
  if (d->stored_total == (double)n * sf && !had_centroids) {
    d->min_v = vmin;
    d->max_v = vmax;
  } else {
    if (vmin < d->min_v) d->min_v = vmin;
    if (vmax > d->max_v) d->max_v = vmax;
  }
  double* om = (double*)malloc(sizeof(double) * (size_t)total_in);
  double* ow = (double*)malloc(sizeof(double) * (size_t)total_in);
  int64_t cnt = kdo_ppath_compress(d->scale, d->compression, m, w, total_in, om, ow, NULL);
  free(m);
  free(w);
  if (cnt < 0) {
    free(om);
    free(ow);
    return KDO_ECONVERGE;
  }
  reserve_c(d, cnt > 0 ? cnt : 1);
  double total = 0.0;
  for (int64_t i = 0; i < cnt; ++i) {
    d->cm[i] = om[i];
    d->cw[i] = ow[i];
    total += ow[i];
  }
  d->nc = cnt;
  d->stored_total = total;
  free(om);
  free(ow);
  if (decay_active(d)) prune(d);
  return KDO_OK;
}

int kdo_add_batch_p(kdo_digest* d, const double* values, int64_t n) {
  return add_batch_p(d, values, n, 0, 0.0);
}
int kdo_add_batch_p_at(kdo_digest* d, const double* values, int64_t n, double timestamp) {
  return add_batch_p(d, values, n, 1, timestamp);
}

static double effective_weight(const kdo_digest* d, double stored) { /* :475-479 */
  return decay_active(d) ? stored * kd_exp(-d->log_scale) : stored;
}
static int is_singleton(const kdo_digest* d, double stored) { /* :481-483 */
  return effective_weight(d, stored) <= 1.0 + 1e-9;
}

int kdo_quantile(kdo_digest* d, double q, double* out) { /* tdigest.mojo:485-538 */
  if (q < 0.0 || q > 1.0 || kd_isnan(q)) return KDO_EINVAL;
  kdo_merge(d);
  int64_t nc = d->nc;
  if (nc == 0) return KDO_EEMPTY;
  const double* cm = d->cm;
  const double* cw = d->cw;
  if (nc == 1) { *out = cm[0]; return KDO_OK; }
  double n = d->stored_total;
  if (q <= 0.0) { *out = d->min_v; return KDO_OK; }
  if (q >= 1.0) { *out = d->max_v; return KDO_OK; }
  double target = q * n;
  double first_half = cw[0] / 2.0;
  if (target < first_half) {
    if (is_singleton(d, cw[0])) *out = d->min_v;
    else *out = d->min_v + (cm[0] - d->min_v) * (target / first_half);
    return KDO_OK;
  }
  double last_m = cm[nc - 1], last_w = cw[nc - 1];
  double last_half = last_w / 2.0;
  if (target > n - last_half) {
    if (is_singleton(d, last_w)) { *out = d->max_v; return KDO_OK; }
    double frac = (target - (n - last_half)) / last_half;
    *out = last_m + (d->max_v - last_m) * frac;
    return KDO_OK;
  }
  double wsf = cw[0] / 2.0;
  for (int64_t i = 0; i < nc - 1; ++i) {
    double dw = (cw[i] + cw[i + 1]) / 2.0;
    if (target <= wsf + dw) {
      double frac = (target - wsf) / dw;
      *out = cm[i] + (cm[i + 1] - cm[i]) * frac;
      return KDO_OK;
    }
    wsf += dw;
  }
  *out = last_m;
  return KDO_OK;
}

int kdo_cdf(kdo_digest* d, double x, double* out) { /* tdigest.mojo:540-587 */
  kdo_merge(d);
  int64_t nc = d->nc;
  if (nc == 0) return KDO_EEMPTY;
  const double* cm = d->cm;
  const double* cw = d->cw;
  if (x < d->min_v) { *out = 0.0; return KDO_OK; }
  if (x > d->max_v) { *out = 1.0; return KDO_OK; }
  if (nc == 1) {
    *out = x < cm[0] ? 0.0 : (x > cm[0] ? 1.0 : 0.5);
    return KDO_OK;
  }
  double n = d->stored_total;
  if (x < cm[0]) {
    if (d->min_v == cm[0]) { *out = 0.0; return KDO_OK; }
    double frac = (x - d->min_v) / (cm[0] - d->min_v);
    *out = (cw[0] / 2.0) * frac / n;
    return KDO_OK;
  }
  double last_m = cm[nc - 1], last_w = cw[nc - 1];
  if (x > last_m) {
    if (d->max_v == last_m) { *out = 1.0; return KDO_OK; }
    double frac = (x - last_m) / (d->max_v - last_m);
    *out = (n - last_w / 2.0 + (last_w / 2.0) * frac) / n;
    return KDO_OK;
  }
  double wsf = cw[0] / 2.0;
  for (int64_t i = 0; i < nc - 1; ++i) {
    if (x <= cm[i + 1]) {
      double dw = (cw[i] + cw[i + 1]) / 2.0;
      if (cm[i + 1] == cm[i]) { *out = (wsf + dw / 2.0) / n; return KDO_OK; }
      double frac = (x - cm[i]) / (cm[i + 1] - cm[i]);
      *out = (wsf + dw * frac) / n;
      return KDO_OK;
    }
    wsf += (cw[i] + cw[i + 1]) / 2.0;
  }
  *out = 1.0;
  return KDO_OK;
}

int kdo_merge_into(kdo_digest* d, kdo_digest* o) { /* tdigest.mojo:589-623 */
  kdo_merge(o);
  if (effective_count(o) == 0.0) return KDO_OK;
  kdo_merge(d);
  if (decay_active(d)) renormalize(d);
  if (decay_active(o)) renormalize(o);
  int was_empty = d->stored_total == 0.0;
  reserve_b(d, d->nb + o->nc);
  for (int64_t i = 0; i < o->nc; ++i) {
    d->bm[d->nb] = o->cm[i];
    d->bw[d->nb] = o->cw[i];
    d->nb++;
  }
  d->stored_total += o->stored_total;
  if (was_empty) {
    d->min_v = o->min_v;
    d->max_v = o->max_v;
  } else {
    d->min_v = d->min_v < o->min_v ? d->min_v : o->min_v;
    d->max_v = d->max_v > o->max_v ? d->max_v : o->max_v;
  }
  d->clock = d->clock > o->clock ? d->clock : o->clock;
  kdo_merge(d);
  return KDO_OK;
}

/* Serialization — tdigest.mojo:627-698. */
static void put_f64(uint8_t* p, double v) {
  uint64_t b = kd_bits(v);
  for (int i = 0; i < 8; ++i) p[i] = (uint8_t)(b >> (8 * i));
}
static double get_f64(const uint8_t* p) {
  uint64_t b = 0;
  for (int i = 0; i < 8; ++i) b |= (uint64_t)p[i] << (8 * i);
  return kd_from_bits(b);
}

int64_t kdo_to_bytes(kdo_digest* d, uint8_t* buf, int64_t cap) {
  kdo_merge(d);
  int64_t need = 1 + 8 * 8 + 16 * d->nc;
  if (!buf || cap < need) return need;
  buf[0] = SERDE_VERSION;
  double hdr[8] = {d->compression, d->lambda, d->log_scale, d->clock,
                   d->stored_total, d->min_v, d->max_v, (double)d->nc};
  for (int i = 0; i < 8; ++i) put_f64(buf + 1 + 8 * i, hdr[i]);
  for (int64_t i = 0; i < d->nc; ++i) {
    put_f64(buf + 65 + 16 * i, d->cm[i]);
    put_f64(buf + 73 + 16 * i, d->cw[i]);
  }
  return need;
}

kdo_digest* kdo_from_bytes(const uint8_t* buf, int64_t len, int scale, int* err) {
  *err = KDO_OK;
  if (len <= 0 || buf[0] != SERDE_VERSION) { *err = KDO_EINVAL; return NULL; }
  if (len < 65) { *err = KDO_ERANGE; return NULL; }
  double h[8];
  for (int i = 0; i < 8; ++i) h[i] = get_f64(buf + 1 + 8 * i);
  int64_t count = (int64_t)h[7];
  if (count < 0 || 65 + 16 * count > len) { *err = KDO_ERANGE; return NULL; }
  kdo_digest* d = kdo_digest_new(scale, h[0], h[1]);
  reserve_c(d, count > 0 ? count : 1);
  for (int64_t i = 0; i < count; ++i) {
    d->cm[i] = get_f64(buf + 65 + 16 * i);
    d->cw[i] = get_f64(buf + 73 + 16 * i);
  }
  d->nc = count;
  d->log_scale = h[2];
  d->clock = h[3];
  d->stored_total = h[4];
  d->min_v = h[5];
  d->max_v = h[6];
  return d;
}

int64_t kdo_len(const kdo_digest* d) { return d->nc; }
double kdo_total_weight(const kdo_digest* d) { return effective_count(d); }
void kdo_state(const kdo_digest* d, double* s) {
  s[0] = d->compression; s[1] = d->lambda; s[2] = d->log_scale; s[3] = d->clock;
  s[4] = d->stored_total; s[5] = d->min_v; s[6] = d->max_v; s[7] = (double)d->nc;
}
int64_t kdo_centroids(const kdo_digest* d, double* m, double* w, int64_t cap) {
  int64_t k = d->nc < cap ? d->nc : cap;
  memcpy(m, d->cm, sizeof(double) * (size_t)k);
  memcpy(w, d->cw, sizeof(double) * (size_t)k);
  return d->nc;
}
int kdo_set_state(kdo_digest* d, const double* m, const double* w, int64_t n,
                  double stored_total, double log_scale, double clock, double min_v,
                  double max_v) {
  reserve_c(d, n > 0 ? n : 1);
  memcpy(d->cm, m, sizeof(double) * (size_t)n);
  memcpy(d->cw, w, sizeof(double) * (size_t)n);
  d->nc = n;
  d->nb = 0;
  d->stored_total = stored_total;
  d->log_scale = log_scale;
  d->clock = clock;
  d->min_v = min_v;
  d->max_v = max_v;
  return KDO_OK;
}

/* Grouped ingest — grouped.mojo:60-162. */
typedef struct {
  kdo_digest** digests;
  const int64_t* order;   /* sample indices grouped by key, batch order kept */
  const int64_t* offsets; /* per key start into order */
  int64_t k0, k1;
  const double* values;
  int mode;
  double timestamp;
  int err;
} grp_job;

static void* grp_worker(void* arg) {
  grp_job* j = (grp_job*)arg;
  double* buf = NULL;
  int64_t cap = 0;
  for (int64_t k = j->k0; k < j->k1; ++k) {
    int64_t s = j->offsets[k], e = j->offsets[k + 1];
    if (e == s) continue;
    if (e - s > cap) {
      cap = e - s;
      buf = (double*)realloc(buf, sizeof(double) * (size_t)cap);
    }
    for (int64_t i = s; i < e; ++i) buf[i - s] = j->values[j->order[i]];
    int r = add_batch_p(j->digests[k], buf, e - s, j->mode, j->timestamp);
    if (r) j->err = r;
  }
  free(buf);
  return NULL;
}

int kdo_grouped_add_batch(kdo_digest** digests, int64_t num_keys, const uint32_t* keys,
                          const double* values, int64_t n, int mode, double timestamp,
                          int threads) {
  if (n == 0) return KDO_OK;
  for (int64_t i = 0; i < n; ++i) { /* validate everything first (:91-97) */
    if ((int64_t)keys[i] >= num_keys) return KDO_EINVAL;
    if (validate(values[i], 1.0)) return KDO_EINVAL;
  }
  int64_t* offsets = (int64_t*)calloc((size_t)num_keys + 1, sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) offsets[keys[i] + 1]++;
  for (int64_t k = 0; k < num_keys; ++k) offsets[k + 1] += offsets[k];
  int64_t* cursor = (int64_t*)malloc(sizeof(int64_t) * (size_t)num_keys);
  memcpy(cursor, offsets, sizeof(int64_t) * (size_t)num_keys);
  int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
  for (int64_t i = 0; i < n; ++i) order[cursor[keys[i]]++] = i;
  free(cursor);
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  grp_job jobs[256];
  pthread_t tids[256];
  /* Balance threads by sample count, not key count (Zipf keys). */
  int64_t per = (n + threads - 1) / threads;
  int64_t k = 0;
  int used = 0;
  for (int t = 0; t < threads && k < num_keys; ++t) {
    int64_t k0 = k;
    int64_t target = offsets[k0] + per;
    while (k < num_keys && (offsets[k + 1] <= target || k == k0)) ++k;
    if (t == threads - 1) k = num_keys;
    jobs[t] = (grp_job){digests, order, offsets, k0, k, values, mode, timestamp, 0};
    ++used;
  }
  if (used == 1) {
    grp_worker(&jobs[0]);
  } else {
    for (int t = 0; t < used; ++t) pthread_create(&tids[t], NULL, grp_worker, &jobs[t]);
    for (int t = 0; t < used; ++t) pthread_join(tids[t], NULL);
  }
  int err = KDO_OK;
  for (int t = 0; t < used; ++t)
    if (jobs[t].err) err = jobs[t].err;
  free(order);
  free(offsets);
  return err;
}

int kdo_merge_parts_p(kdo_digest* dst, kdo_digest** parts, int64_t nparts) {
  int64_t total = 0;
  for (int64_t p = 0; p < nparts; ++p) {
    kdo_merge(parts[p]);
    total += parts[p]->nc;
  }
  double* m = (double*)malloc(sizeof(double) * (size_t)(total > 0 ? total : 1));
  double* w = (double*)malloc(sizeof(double) * (size_t)(total > 0 ? total : 1));
  int64_t k = 0;
  int seen = 0;
  double mn = 0.0, mx = 0.0, clock = 0.0;
  for (int64_t p = 0; p < nparts; ++p) {
    kdo_digest* o = parts[p];
    if (effective_count(o) == 0.0) continue; /* merge_into early return */
    if (decay_active(o)) renormalize(o);
    for (int64_t i = 0; i < o->nc; ++i, ++k) { m[k] = o->cm[i]; w[k] = o->cw[i]; }
    if (!seen) { mn = o->min_v; mx = o->max_v; seen = 1; }
    else { mn = mn < o->min_v ? mn : o->min_v; mx = mx > o->max_v ? mx : o->max_v; }
    clock = clock > o->clock ? clock : o->clock;
  }
  double* om = (double*)malloc(sizeof(double) * (size_t)(k > 0 ? k : 1));
  double* ow = (double*)malloc(sizeof(double) * (size_t)(k > 0 ? k : 1));
  int64_t cnt = kdo_ppath_compress(dst->scale, dst->compression, m, w, k, om, ow, NULL);
  free(m);
  free(w);
  if (cnt < 0) { free(om); free(ow); return KDO_ECONVERGE; }
  double total_w = 0.0;
  for (int64_t i = 0; i < cnt; ++i) total_w += ow[i];
  kdo_set_state(dst, om, ow, cnt, total_w, 0.0, clock, mn, mx);
  free(om);
  free(ow);
  return KDO_OK;
}

/* Thin exports of the shared FP64 scale arithmetic, for accuracy tests. */
double kdo_log(double x) { return kd_log(x); }
double kdo_exp(double x) { return kd_exp(x); }
double kdo_asin(double x) { return kd_asin(x); }
double kdo_normalizer(int scale, double compression, double n) {
  return kd_normalizer(scale, compression, n);
}
double kdo_k(int scale, double q, double nrm) { return kd_k(scale, q, nrm); }
int32_t kdo_bucket(int scale, double cum, double tot, double nrm) {
  return kd_bucket(scale, cum, tot, nrm);
}

typedef struct {
  kdo_digest** digests;
  int64_t nd;
  const int32_t* ids;
  const double* x;
  int64_t i0, i1;
  int is_cdf;
  double* out;
  int err;
} qry_job;

static void* qry_worker(void* p) {
  qry_job* j = (qry_job*)p;
  for (int64_t i = j->i0; i < j->i1; ++i) {
    const int32_t id = j->ids[i];
    int e = KDO_EINVAL;
    double v = kd_from_bits(0x7ff8000000000000ULL);
    if (id >= 0 && id < j->nd) {
      e = j->is_cdf ? kdo_cdf(j->digests[id], j->x[i], &v) : kdo_quantile(j->digests[id], j->x[i], &v);
      if (e) v = kd_from_bits(0x7ff8000000000000ULL);
    }
    j->out[i] = v;
    if (e && !j->err) j->err = e;
  }
  return NULL;
}

int kdo_query_batch(kdo_digest** digests, int64_t nd, const int32_t* ids, const double* x,
                    int64_t n, int is_cdf, double* out, int threads) {
  for (int64_t k = 0; k < nd; ++k) kdo_merge(digests[k]);
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  qry_job jobs[256];
  pthread_t tids[256];
  const int64_t per = (n + threads - 1) / threads;
  int used = 0;
  for (int t = 0; t < threads; ++t) {
    const int64_t i0 = (int64_t)t * per, i1 = i0 + per < n ? i0 + per : n;
    if (i0 >= i1) break;
    jobs[t] = (qry_job){digests, nd, ids, x, i0, i1, is_cdf, out, 0};
    ++used;
  }
  if (used == 1) {
    qry_worker(&jobs[0]);
  } else {
    for (int t = 0; t < used; ++t) pthread_create(&tids[t], NULL, qry_worker, &jobs[t]);
    for (int t = 0; t < used; ++t) pthread_join(tids[t], NULL);
  }
  int err = KDO_OK;
  for (int t = 0; t < used; ++t)
    if (jobs[t].err && !err) err = jobs[t].err;
  return err;
}
