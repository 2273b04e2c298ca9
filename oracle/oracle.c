/*
 * oracle.c -- CPU restatement of ManifoldANN's hot-path semantics.
 *
 * THIS IS TEST INFRASTRUCTURE (see oracle.h): the checker for the GPU
 * library and the timed CPU baseline, never part of the product path.
 *
 * Build: make -C oracle   (gcc, -ffp-contract=off so that every fused
 * multiply-add below is an explicit fmaf/fma call and nothing else is fused).
 *
 * Ordering rule used everywhere: Julia's partialsortperm over a Float vector
 * orders by (isless(value), index): NaN after every number, -0.0 before +0.0,
 * equal values by lower index (src/indices/bruteforce.jl:65,
 * src/indices/ivf_flat.jl:150, src/indices/multilevel/routing.jl:115).
 * fkey32/fkey64 map a float to an unsigned integer with exactly that order.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ keys */

static inline uint32_t fkey32(float f) {
  uint32_t b;
  memcpy(&b, &f, 4);
  if (isnan(f)) b = 0x7FC00000u;
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

static inline uint64_t fkey64(double f) {
  uint64_t b;
  memcpy(&b, &f, 8);
  if (isnan(f)) b = 0x7FF8000000000000ull;
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

/* (value, index) pair in the partialsortperm order */
typedef struct {
  uint64_t key;
  int64_t idx;
} kv_t;

static inline int kv_less(kv_t a, kv_t b) {
  return a.key < b.key || (a.key == b.key && a.idx < b.idx);
}

/* Keep the best `k` pairs in a sorted array (ascending).  `cnt` entries used. */
static inline void topk_push(kv_t* list, int32_t k, int32_t* cnt, kv_t c) {
  int32_t m = *cnt;
  if (m == k) {
    if (!kv_less(c, list[k - 1])) return;
    m = k - 1;
  }
  int32_t p = m;
  while (p > 0 && kv_less(c, list[p - 1])) {
    list[p] = list[p - 1];
    --p;
  }
  list[p] = c;
  if (*cnt < k) ++(*cnt);
}

/* ------------------------------------------------------------- distances */
/* Distances.jl 0.10.12 definitions (src/utils/distances.jl:15-18):
 *   SqEuclidean  sum((x_i - y_i)^2)
 *   Euclidean    sqrt(SqEuclidean)
 *   CosineDist   max(1 - x.y / (sqrt(x.x) * sqrt(y.y)), 0)   (NaN for a zero norm)
 * Summation: sequential over i = 0..d-1 with one fused multiply-add per term. */

float orc_dist_f32(const float* x, const float* y, int32_t d, int32_t metric) {
  if (metric == ORC_COSINE) {
    float ab = 0.0f, aa = 0.0f, bb = 0.0f;
    for (int32_t i = 0; i < d; ++i) {
      ab = fmaf(x[i], y[i], ab);
      aa = fmaf(x[i], x[i], aa);
      bb = fmaf(y[i], y[i], bb);
    }
    float den = sqrtf(aa) * sqrtf(bb);
    float r = 1.0f - ab / den;
    if (r < 0.0f) r = 0.0f; /* NaN stays NaN, as Julia's max(NaN, 0) */
    return r;
  }
  float s = 0.0f;
  for (int32_t i = 0; i < d; ++i) {
    float t = x[i] - y[i];
    s = fmaf(t, t, s);
  }
  return metric == ORC_EUCLIDEAN ? sqrtf(s) : s;
}

double orc_dist_f64(const float* x, const float* y, int32_t d, int32_t metric) {
  if (metric == ORC_COSINE) {
    double ab = 0.0, aa = 0.0, bb = 0.0;
    for (int32_t i = 0; i < d; ++i) {
      double xi = (double)x[i], yi = (double)y[i];
      ab = fma(xi, yi, ab);
      aa = fma(xi, xi, aa);
      bb = fma(yi, yi, bb);
    }
    double den = sqrt(aa) * sqrt(bb);
    double r = 1.0 - ab / den;
    if (r < 0.0) r = 0.0;
    return r;
  }
  double s = 0.0;
  for (int32_t i = 0; i < d; ++i) {
    double t = (double)x[i] - (double)y[i];
    s = fma(t, t, s);
  }
  return metric == ORC_EUCLIDEAN ? sqrt(s) : s;
}

int32_t orc_max_threads(void) {
#ifdef _OPENMP
  return (int32_t)omp_get_max_threads();
#else
  return 1;
#endif
}

static int resolve_threads(int32_t t) {
  int m = (int)orc_max_threads();
  if (t <= 0 || t > m) t = m;
  return t;
}

static inline float key_to_f32(uint64_t key) {
  uint32_t k = (uint32_t)key;
  uint32_t b = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
  float f;
  memcpy(&f, &b, 4);
  return f;
}

static inline double key_to_f64(uint64_t k) {
  uint64_t b = (k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  double f;
  memcpy(&f, &b, 8);
  return f;
}

/* ------------------------------------------------------------- exact kNN */

/* Four pairs at a time: the same sequential per-pair sums as orc_dist_f32 /
 * orc_dist_f64 (one fused multiply-add per dimension, in dimension order),
 * interleaved so four independent chains are in flight.  Results are those
 * of four separate orc_dist_* calls. */
static void dist4_f32(const float* b0, const float* b1, const float* b2, const float* b3,
                      const float* y, int32_t d, int32_t metric, float* out) {
  if (metric == ORC_COSINE) {
    float ab0 = 0.0f, ab1 = 0.0f, ab2 = 0.0f, ab3 = 0.0f;
    float aa0 = 0.0f, aa1 = 0.0f, aa2 = 0.0f, aa3 = 0.0f, bb = 0.0f;
    for (int32_t i = 0; i < d; ++i) {
      const float yi = y[i];
      ab0 = fmaf(b0[i], yi, ab0);
      ab1 = fmaf(b1[i], yi, ab1);
      ab2 = fmaf(b2[i], yi, ab2);
      ab3 = fmaf(b3[i], yi, ab3);
      aa0 = fmaf(b0[i], b0[i], aa0);
      aa1 = fmaf(b1[i], b1[i], aa1);
      aa2 = fmaf(b2[i], b2[i], aa2);
      aa3 = fmaf(b3[i], b3[i], aa3);
      bb = fmaf(yi, yi, bb);
    }
    const float ab[4] = {ab0, ab1, ab2, ab3}, aa[4] = {aa0, aa1, aa2, aa3};
    for (int j = 0; j < 4; ++j) {
      float r = 1.0f - ab[j] / (sqrtf(aa[j]) * sqrtf(bb));
      if (r < 0.0f) r = 0.0f;
      out[j] = r;
    }
    return;
  }
  float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
  for (int32_t i = 0; i < d; ++i) {
    const float yi = y[i];
    const float t0 = b0[i] - yi, t1 = b1[i] - yi, t2 = b2[i] - yi, t3 = b3[i] - yi;
    s0 = fmaf(t0, t0, s0);
    s1 = fmaf(t1, t1, s1);
    s2 = fmaf(t2, t2, s2);
    s3 = fmaf(t3, t3, s3);
  }
  out[0] = s0;
  out[1] = s1;
  out[2] = s2;
  out[3] = s3;
  if (metric == ORC_EUCLIDEAN)
    for (int j = 0; j < 4; ++j) out[j] = sqrtf(out[j]);
}

static void dist4_f64(const float* b0, const float* b1, const float* b2, const float* b3,
                      const float* y, int32_t d, int32_t metric, double* out) {
  if (metric == ORC_COSINE) {
    double ab0 = 0.0, ab1 = 0.0, ab2 = 0.0, ab3 = 0.0;
    double aa0 = 0.0, aa1 = 0.0, aa2 = 0.0, aa3 = 0.0, bb = 0.0;
    for (int32_t i = 0; i < d; ++i) {
      const double yi = (double)y[i];
      const double x0 = (double)b0[i], x1 = (double)b1[i], x2 = (double)b2[i], x3 = (double)b3[i];
      ab0 = fma(x0, yi, ab0);
      ab1 = fma(x1, yi, ab1);
      ab2 = fma(x2, yi, ab2);
      ab3 = fma(x3, yi, ab3);
      aa0 = fma(x0, x0, aa0);
      aa1 = fma(x1, x1, aa1);
      aa2 = fma(x2, x2, aa2);
      aa3 = fma(x3, x3, aa3);
      bb = fma(yi, yi, bb);
    }
    const double ab[4] = {ab0, ab1, ab2, ab3}, aa[4] = {aa0, aa1, aa2, aa3};
    for (int j = 0; j < 4; ++j) {
      double r = 1.0 - ab[j] / (sqrt(aa[j]) * sqrt(bb));
      if (r < 0.0) r = 0.0;
      out[j] = r;
    }
    return;
  }
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  for (int32_t i = 0; i < d; ++i) {
    const double yi = (double)y[i];
    const double t0 = (double)b0[i] - yi, t1 = (double)b1[i] - yi;
    const double t2 = (double)b2[i] - yi, t3 = (double)b3[i] - yi;
    s0 = fma(t0, t0, s0);
    s1 = fma(t1, t1, s1);
    s2 = fma(t2, t2, s2);
    s3 = fma(t3, t3, s3);
  }
  out[0] = s0;
  out[1] = s1;
  out[2] = s2;
  out[3] = s3;
  if (metric == ORC_EUCLIDEAN)
    for (int j = 0; j < 4; ++j) out[j] = sqrt(out[j]);
}

static void knn_row_f32(const float* base, int64_t n, const float* qv, int32_t d, int32_t k,
                        int32_t metric, int32_t* ids, float* dists, kv_t* scratch) {
  int32_t ke = (int32_t)(k < n ? k : n);
  int32_t cnt = 0;
  int64_t j = 0;
  for (; j + 4 <= n; j += 4) {
    float v[4];
    const float* b = base + j * (int64_t)d;
    dist4_f32(b, b + d, b + 2 * (int64_t)d, b + 3 * (int64_t)d, qv, d, metric, v);
    for (int u = 0; u < 4; ++u) {
      kv_t c = {fkey32(v[u]), j + u};
      topk_push(scratch, ke, &cnt, c);
    }
  }
  for (; j < n; ++j) {
    float v = orc_dist_f32(base + j * (int64_t)d, qv, d, metric);
    kv_t c = {fkey32(v), j};
    topk_push(scratch, ke, &cnt, c);
  }
  for (int32_t i = 0; i < k; ++i) {
    if (i < cnt) {
      ids[i] = (int32_t)scratch[i].idx;
      dists[i] = key_to_f32(scratch[i].key);
    } else {
      ids[i] = -1;
      dists[i] = INFINITY;
    }
  }
}

static void knn_row_f64(const float* base, int64_t n, const float* qv, int32_t d, int32_t k,
                        int32_t metric, int32_t* ids, double* dists, kv_t* scratch) {
  int32_t ke = (int32_t)(k < n ? k : n);
  int32_t cnt = 0;
  int64_t j = 0;
  for (; j + 4 <= n; j += 4) {
    double v[4];
    const float* b = base + j * (int64_t)d;
    dist4_f64(b, b + d, b + 2 * (int64_t)d, b + 3 * (int64_t)d, qv, d, metric, v);
    for (int u = 0; u < 4; ++u) {
      kv_t c = {fkey64(v[u]), j + u};
      topk_push(scratch, ke, &cnt, c);
    }
  }
  for (; j < n; ++j) {
    double v = orc_dist_f64(base + j * (int64_t)d, qv, d, metric);
    kv_t c = {fkey64(v), j};
    topk_push(scratch, ke, &cnt, c);
  }
  for (int32_t i = 0; i < k; ++i) {
    if (i < cnt) {
      ids[i] = (int32_t)scratch[i].idx;
      dists[i] = key_to_f64(scratch[i].key);
    } else {
      ids[i] = -1;
      dists[i] = INFINITY;
    }
  }
}

int orc_knn_f32(const float* base, int64_t n, const float* q, int64_t nq, int32_t d, int32_t k,
                int32_t metric, int32_t* ids, float* dists, int32_t nthreads) {
  if (d <= 0 || n <= 0) return 2;
  if (k <= 0 || nq <= 0) return 0;
  int nt = resolve_threads(nthreads);
#pragma omp parallel num_threads(nt)
  {
    kv_t* scratch = (kv_t*)malloc(sizeof(kv_t) * (size_t)k);
#pragma omp for schedule(dynamic, 4)
    for (int64_t i = 0; i < nq; ++i)
      knn_row_f32(base, n, q + i * (int64_t)d, d, k, metric, ids + i * (int64_t)k,
                  dists + i * (int64_t)k, scratch);
    free(scratch);
  }
  return 0;
}

int orc_knn_f64(const float* base, int64_t n, const float* q, int64_t nq, int32_t d, int32_t k,
                int32_t metric, int32_t* ids, double* dists, int32_t nthreads) {
  if (d <= 0 || n <= 0) return 2;
  if (k <= 0 || nq <= 0) return 0;
  int nt = resolve_threads(nthreads);
#pragma omp parallel num_threads(nt)
  {
    kv_t* scratch = (kv_t*)malloc(sizeof(kv_t) * (size_t)k);
#pragma omp for schedule(dynamic, 4)
    for (int64_t i = 0; i < nq; ++i)
      knn_row_f64(base, n, q + i * (int64_t)d, d, k, metric, ids + i * (int64_t)k,
                  dists + i * (int64_t)k, scratch);
    free(scratch);
  }
  return 0;
}

/* ------------------------------------------------------------- kNN graph */

/* _prepare_neighbors (src/graphs/knn_graph.jl:105-130): drop `self` wherever
 * it appears in the (k+1)-list and keep the first k others.  With
 * include_self the first k entries are kept as they are (_trim_or_fail). */
static void prepare_row_i(const int32_t* in_ids, int32_t in_k, int64_t self, int32_t k,
                          int32_t include_self, int32_t* out_ids, int32_t* pos_map) {
  int32_t m = 0;
  for (int32_t i = 0; i < in_k && m < k; ++i) {
    if (!include_self && in_ids[i] == self) continue;
    pos_map[m] = i;
    out_ids[m++] = in_ids[i];
  }
}

/* rows == NULL: every point, output row i = point i; otherwise output row i
 * = point rows[i] (nrows rows) */
#define GRAPH_BODY(TYPE, ROWFN)                                                              \
  if (d <= 0 || n <= 0) return 2;                                                            \
  int64_t maxk = n - (include_self ? 0 : 1);                                                 \
  if (!(k > 0 && k <= maxk)) return 2;                                                       \
  int32_t req = k + (include_self ? 0 : 1);                                                  \
  int nt = resolve_threads(nthreads);                                                        \
  const int64_t nout = rows ? nrows : n;                                                     \
  for (int64_t i = 0; rows && i < nrows; ++i)                                                \
    if (rows[i] < 0 || rows[i] >= n) return 2;                                               \
  _Pragma("omp parallel num_threads(nt)") {                                                  \
    kv_t* scratch = (kv_t*)malloc(sizeof(kv_t) * (size_t)req);                               \
    int32_t* tid = (int32_t*)malloc(sizeof(int32_t) * (size_t)req);                          \
    TYPE* td = (TYPE*)malloc(sizeof(TYPE) * (size_t)req);                                    \
    int32_t* pos = (int32_t*)malloc(sizeof(int32_t) * (size_t)req);                          \
    _Pragma("omp for schedule(dynamic, 1)") for (int64_t i = 0; i < nout; ++i) {             \
      const int64_t r = rows ? (int64_t)rows[i] : i;                                         \
      ROWFN(data, n, data + r * (int64_t)d, d, req, metric, tid, td, scratch);               \
      prepare_row_i(tid, req, r, k, include_self, ids + i * (int64_t)k, pos);                \
      for (int32_t j = 0; j < k; ++j) dists[i * (int64_t)k + j] = td[pos[j]];                \
    }                                                                                        \
    free(scratch);                                                                           \
    free(tid);                                                                               \
    free(td);                                                                                \
    free(pos);                                                                               \
  }                                                                                          \
  return 0;

int orc_knn_graph_f32(const float* data, int64_t n, int32_t d, int32_t k, int32_t include_self,
                      int32_t metric, int32_t* ids, float* dists, int32_t nthreads) {
  const int32_t* rows = NULL;
  const int64_t nrows = 0;
  GRAPH_BODY(float, knn_row_f32)
}

int orc_knn_graph_f64(const float* data, int64_t n, int32_t d, int32_t k, int32_t include_self,
                      int32_t metric, int32_t* ids, double* dists, int32_t nthreads) {
  const int32_t* rows = NULL;
  const int64_t nrows = 0;
  GRAPH_BODY(double, knn_row_f64)
}

int orc_knn_graph_rows_f32(const float* data, int64_t n, int32_t d, int32_t k,
                           int32_t include_self, int32_t metric, const int32_t* rows,
                           int64_t nrows, int32_t* ids, float* dists, int32_t nthreads) {
  if (!rows) return 2;
  GRAPH_BODY(float, knn_row_f32)
}

int orc_knn_graph_rows_f64(const float* data, int64_t n, int32_t d, int32_t k,
                           int32_t include_self, int32_t metric, const int32_t* rows,
                           int64_t nrows, int32_t* ids, double* dists, int32_t nthreads) {
  if (!rows) return 2;
  GRAPH_BODY(double, knn_row_f64)
}

/* --------------------------------------------------------- KMeans assign */

int orc_kmeans_assign_gemm_f32(const float* X, int64_t n, const float* C, int32_t nlist, int32_t d,
                               int32_t metric, int32_t* assign, float* out_dist,
                               int32_t nthreads) {
  if (d <= 0 || n <= 0 || nlist <= 0) return 2;
  float* cn = (float*)malloc(sizeof(float) * (size_t)nlist);
  for (int32_t c = 0; c < nlist; ++c) {
    float s = 0.0f;
    for (int32_t i = 0; i < d; ++i) s = fmaf(C[c * (int64_t)d + i], C[c * (int64_t)d + i], s);
    cn[c] = s;
  }
  int nt = resolve_threads(nthreads);
#pragma omp parallel for num_threads(nt) schedule(static)
  for (int64_t j = 0; j < n; ++j) {
    const float* x = X + j * (int64_t)d;
    float xn = 0.0f;
    for (int32_t i = 0; i < d; ++i) xn = fmaf(x[i], x[i], xn);
    float best = 0.0f;
    int32_t bi = 0;
    for (int32_t c = 0; c < nlist; ++c) {
      const float* cc = C + c * (int64_t)d;
      float dot = 0.0f;
      for (int32_t i = 0; i < d; ++i) dot = fmaf(cc[i], x[i], dot);
      float sq = (cn[c] + xn) - 2.0f * dot;
      if (!(sq > 0.0f)) sq = (sq != sq) ? sq : 0.0f;
      float v = metric == ORC_EUCLIDEAN ? sqrtf(sq) : sq;
      /* strict < : lowest centroid id wins ties (distance.jl:299) */
      if (c == 0 || v < best) {
        best = v;
        bi = c;
      }
    }
    assign[j] = bi;
    if (out_dist) out_dist[j] = best;
  }
  free(cn);
  return 0;
}

int orc_kmeans_assign_f64(const float* X, int64_t n, const float* C, int32_t nlist, int32_t d,
                          int32_t metric, int32_t* assign, double* out_dist, int32_t nthreads) {
  if (d <= 0 || n <= 0 || nlist <= 0) return 2;
  int nt = resolve_threads(nthreads);
#pragma omp parallel for num_threads(nt) schedule(static)
  for (int64_t j = 0; j < n; ++j) {
    const float* x = X + j * (int64_t)d;
    double best = 0.0;
    int32_t bi = 0;
    for (int32_t c = 0; c < nlist; ++c) {
      double v = orc_dist_f64(C + c * (int64_t)d, x, d,
                              metric == ORC_EUCLIDEAN ? ORC_SQEUCLIDEAN : metric);
      if (c == 0 || v < best) {
        best = v;
        bi = c;
      }
    }
    assign[j] = bi;
    if (out_dist) out_dist[j] = metric == ORC_EUCLIDEAN ? sqrt(best) : best;
  }
  return 0;
}

/* ------------------------------------------------------------ k-means++ */

#define ORC_SCAN_BLOCK 1024

int orc_kmeanspp(const float* X, int64_t n, int32_t d, int32_t k, int64_t first, const double* u,
                 int64_t* out_idx) {
  if (n <= 0 || d <= 0 || k <= 0 || k > n) return 2;
  float* mind = (float*)malloc(sizeof(float) * (size_t)n);
  int64_t nb = (n + ORC_SCAN_BLOCK - 1) / ORC_SCAN_BLOCK;
  double* bsum = (double*)malloc(sizeof(double) * (size_t)nb);
  for (int64_t j = 0; j < n; ++j) mind[j] = INFINITY;
  out_idx[0] = first;
  for (int32_t i = 1; i < k; ++i) {
    const float* c = X + out_idx[i - 1] * (int64_t)d;
    for (int64_t j = 0; j < n; ++j) {
      float v = orc_dist_f32(X + j * (int64_t)d, c, d, ORC_SQEUCLIDEAN);
      if (v < mind[j]) mind[j] = v;
    }
    for (int64_t b = 0; b < nb; ++b) {
      double s = 0.0;
      int64_t e = (b + 1) * ORC_SCAN_BLOCK < n ? (b + 1) * ORC_SCAN_BLOCK : n;
      for (int64_t j = b * ORC_SCAN_BLOCK; j < e; ++j) s += (double)mind[j];
      bsum[b] = s;
    }
    double total = 0.0;
    for (int64_t b = 0; b < nb; ++b) total += bsum[b];
    const double thr = u[i] * total;
    double acc = 0.0;
    int64_t pick = n - 1;
    for (int64_t b = 0; b < nb; ++b) {
      if (acc + bsum[b] >= thr) {
        int64_t e = (b + 1) * ORC_SCAN_BLOCK < n ? (b + 1) * ORC_SCAN_BLOCK : n;
        double a2 = acc;
        for (int64_t j = b * ORC_SCAN_BLOCK; j < e; ++j) {
          a2 += (double)mind[j];
          if (a2 >= thr) {
            pick = j;
            break;
          }
        }
        break;
      }
      acc += bsum[b];
    }
    out_idx[i] = pick;
  }
  free(mind);
  free(bsum);
  return 0;
}

/* ------------------------------------------------------------------ Lloyd */

int orc_kmeans_lloyd(const float* X, int64_t n, int32_t d, int32_t k, float* C, int32_t max_iters,
                     double tol, int32_t metric, int32_t* assign, int32_t* iters, int32_t nthreads) {
  if (n <= 0 || d <= 0 || k <= 0) return 2;
  double* dist = (double*)malloc(sizeof(double) * (size_t)n);
  float* nc = (float*)malloc(sizeof(float) * (size_t)k * d);
  int64_t* cnt = (int64_t*)malloc(sizeof(int64_t) * (size_t)k);
  const int32_t am = metric == ORC_EUCLIDEAN ? ORC_EUCLIDEAN : ORC_SQEUCLIDEAN;
  int32_t it = 0;
  for (int32_t step = 1; step <= max_iters; ++step) {
    it = step;
    orc_kmeans_assign_f64(X, n, C, k, d, am, assign, dist, nthreads);
    memset(nc, 0, sizeof(float) * (size_t)k * d);
    memset(cnt, 0, sizeof(int64_t) * (size_t)k);
    for (int64_t j = 0; j < n; ++j) {
      float* dst = nc + (int64_t)assign[j] * d;
      const float* x = X + j * (int64_t)d;
      for (int32_t r = 0; r < d; ++r) dst[r] += x[r];
      cnt[assign[j]] += 1;
    }
    for (int32_t c = 0; c < k; ++c) {
      float* dst = nc + (int64_t)c * d;
      if (cnt[c] == 0) {
        double best = -INFINITY;
        int64_t far = 0;
        for (int64_t j = 0; j < n; ++j)
          if (dist[j] > best) {
            best = dist[j];
            far = j;
          }
        memcpy(dst, X + far * (int64_t)d, sizeof(float) * (size_t)d);
        cnt[c] = 1;
        dist[far] = -INFINITY;
      } else {
        const float cf = (float)cnt[c];
        for (int32_t r = 0; r < d; ++r) dst[r] = dst[r] / cf;
      }
    }
    double move = 0.0;
    for (int32_t c = 0; c < k; ++c) {
      double m = (double)orc_dist_f32(C + (int64_t)c * d, nc + (int64_t)c * d, d, am);
      if (m > move) move = m;
    }
    memcpy(C, nc, sizeof(float) * (size_t)k * d);
    if (move < tol) break;
  }
  orc_kmeans_assign_f64(X, n, C, k, d, am, assign, dist, nthreads);
  *iters = it;
  free(dist);
  free(nc);
  free(cnt);
  return 0;
}

/* ------------------------------------------------------------- routing */

int32_t orc_topk_route(const float* dists, int32_t n_dist, int32_t n_children, int32_t k,
                       int32_t* out) {
  if (n_children <= 0) return 0;
  int32_t avail = n_dist < n_children ? n_dist : n_children;
  if (avail <= 0) return -2;
  int32_t kk = k < avail ? k : avail;
  if (kk <= 0) return 0;
  kv_t* list = (kv_t*)malloc(sizeof(kv_t) * (size_t)kk);
  int32_t cnt = 0;
  for (int32_t i = 0; i < avail; ++i) {
    kv_t c = {fkey32(dists[i]), i};
    topk_push(list, kk, &cnt, c);
  }
  for (int32_t i = 0; i < cnt; ++i) out[i] = (int32_t)list[i].idx;
  free(list);
  return cnt;
}

/* ------------------------------------------------------------------ IVF */

/* BoundedMaxHeap (src/utils/neighbor_heaps.jl:58-190): binary max-heap on
 * dist only, strict < admission when full, sift comparisons with strict >. */
typedef struct {
  float dist;
  int64_t id;
} nb_t;

static void heap_sift_up(nb_t* h, int32_t i) { /* 1-based i */
  while (i > 1) {
    int32_t p = i >> 1;
    if (h[i - 1].dist > h[p - 1].dist) {
      nb_t t = h[i - 1];
      h[i - 1] = h[p - 1];
      h[p - 1] = t;
      i = p;
    } else {
      break;
    }
  }
}

static void heap_sift_down(nb_t* h, int32_t len, int32_t i) {
  for (;;) {
    int32_t l = i << 1, r = l + 1, g = i;
    if (l <= len && h[l - 1].dist > h[g - 1].dist) g = l;
    if (r <= len && h[r - 1].dist > h[g - 1].dist) g = r;
    if (g == i) break;
    nb_t t = h[i - 1];
    h[i - 1] = h[g - 1];
    h[g - 1] = t;
    i = g;
  }
}

static int nb_cmp(const void* a, const void* b) {
  const nb_t* x = (const nb_t*)a;
  const nb_t* y = (const nb_t*)b;
  uint32_t kx = fkey32(x->dist), ky = fkey32(y->dist);
  if (kx != ky) return kx < ky ? -1 : 1;
  return (x->id > y->id) - (x->id < y->id);
}

/* _centroid_distances (src/indices/ivf_flat.jl:103-131), GEMV form:
 * ||c||^2 + ||q||^2 - 2 c.q with the caller's centroid norms, clamped at 0,
 * sqrt for Euclidean; other metrics per pair. */
static void centroid_dists_gemv(const float* qv, int32_t d, const float* centroids,
                                const float* centroid_norms, int32_t nlist, int32_t centroid_metric,
                                float* cd) {
  float xn = 0.0f;
  for (int32_t i = 0; i < d; ++i) xn = fmaf(qv[i], qv[i], xn);
  for (int32_t c = 0; c < nlist; ++c) {
    const float* cc = centroids + c * (int64_t)d;
    if (centroid_metric == ORC_COSINE) {
      cd[c] = orc_dist_f32(cc, qv, d, ORC_COSINE);
      continue;
    }
    float dot = 0.0f;
    for (int32_t i = 0; i < d; ++i) dot = fmaf(cc[i], qv[i], dot);
    float sq = (centroid_norms[c] + xn) - 2.0f * dot;
    if (!(sq > 0.0f)) sq = (sq != sq) ? sq : 0.0f;
    cd[c] = centroid_metric == ORC_EUCLIDEAN ? sqrtf(sq) : sq;
  }
}

int orc_ivf_route_gemv_f32(const float* centroids, const float* centroid_norms, int32_t nlist,
                           int32_t d, const float* q, int64_t nq, int32_t nprobe,
                           int32_t centroid_metric, int32_t* probes, int32_t nthreads) {
  if (d <= 0 || nlist <= 0) return 2;
  if (nq <= 0) return 0;
  int32_t np = nprobe < 1 ? 1 : (nprobe > nlist ? nlist : nprobe);
  int nt = resolve_threads(nthreads);
#pragma omp parallel num_threads(nt)
  {
    float* cd = (float*)malloc(sizeof(float) * (size_t)nlist);
#pragma omp for schedule(dynamic, 16)
    for (int64_t qi = 0; qi < nq; ++qi) {
      centroid_dists_gemv(q + qi * (int64_t)d, d, centroids, centroid_norms, nlist, centroid_metric, cd);
      orc_topk_route(cd, nlist, nlist, np, probes + qi * (int64_t)np);
    }
    free(cd);
  }
  return 0;
}

int orc_ivf_query_f32(const float* data, int32_t d, const float* centroids,
                      const float* centroid_norms, int32_t nlist, const int64_t* list_offsets,
                      const int32_t* list_ids, const float* q, int64_t nq, int32_t k,
                      int32_t nprobe, int32_t metric, int32_t centroid_metric, int32_t* ids,
                      float* dists, int32_t nthreads) {
  if (d <= 0 || nlist <= 0) return 2;
  if (k <= 0 || nq <= 0) return 0;
  int32_t np = nprobe < 1 ? 1 : (nprobe > nlist ? nlist : nprobe);
  int nt = resolve_threads(nthreads);
#pragma omp parallel num_threads(nt)
  {
    float* cd = (float*)malloc(sizeof(float) * (size_t)nlist);
    int32_t* probe = (int32_t*)malloc(sizeof(int32_t) * (size_t)np);
    nb_t* heap = (nb_t*)malloc(sizeof(nb_t) * (size_t)k);
#pragma omp for schedule(dynamic, 4)
    for (int64_t qi = 0; qi < nq; ++qi) {
      const float* qv = q + qi * (int64_t)d;
      centroid_dists_gemv(qv, d, centroids, centroid_norms, nlist, centroid_metric, cd);
      int32_t got = orc_topk_route(cd, nlist, nlist, np, probe);
      int64_t avail = 0;
      for (int32_t p = 0; p < got; ++p)
        avail += list_offsets[probe[p] + 1] - list_offsets[probe[p]];
      int32_t ke = (int32_t)(k < avail ? k : avail);
      int32_t len = 0;
      for (int32_t p = 0; p < got && ke > 0; ++p) {
        int32_t c = probe[p];
        for (int64_t t = list_offsets[c]; t < list_offsets[c + 1]; ++t) {
          int32_t id = list_ids[t];
          float v = orc_dist_f32(data + (int64_t)id * d, qv, d, metric);
          if (len < ke) {
            heap[len].dist = v;
            heap[len].id = id;
            ++len;
            heap_sift_up(heap, len);
          } else if (v < heap[0].dist) {
            heap[0].dist = v;
            heap[0].id = id;
            heap_sift_down(heap, len, 1);
          }
        }
      }
      qsort(heap, (size_t)len, sizeof(nb_t), nb_cmp);
      for (int32_t i = 0; i < k; ++i) {
        ids[qi * (int64_t)k + i] = i < len ? (int32_t)heap[i].id : -1;
        dists[qi * (int64_t)k + i] = i < len ? heap[i].dist : INFINITY;
      }
    }
    free(cd);
    free(probe);
    free(heap);
  }
  return 0;
}

int orc_ivf_scan_f32(const float* data, int32_t d, const int64_t* list_offsets,
                     const int32_t* list_ids, const float* q, int64_t nq, const int32_t* probes,
                     int32_t nprobe, int32_t k, int32_t metric, int32_t* ids, float* dists,
                     int32_t nthreads) {
  if (d <= 0) return 2;
  if (k <= 0 || nq <= 0) return 0;
  int nt = resolve_threads(nthreads);
#pragma omp parallel num_threads(nt)
  {
    nb_t* heap = (nb_t*)malloc(sizeof(nb_t) * (size_t)k);
#pragma omp for schedule(dynamic, 4)
    for (int64_t qi = 0; qi < nq; ++qi) {
      const float* qv = q + qi * (int64_t)d;
      const int32_t* pr = probes + qi * (int64_t)nprobe;
      int64_t avail = 0;
      for (int32_t p = 0; p < nprobe; ++p)
        if (pr[p] >= 0) avail += list_offsets[pr[p] + 1] - list_offsets[pr[p]];
      int32_t ke = (int32_t)(k < avail ? k : avail);
      int32_t len = 0;
      for (int32_t p = 0; p < nprobe && ke > 0; ++p) {
        const int32_t c = pr[p];
        if (c < 0) continue;
        for (int64_t t = list_offsets[c]; t < list_offsets[c + 1]; ++t) {
          int32_t id = list_ids[t];
          float v = orc_dist_f32(data + (int64_t)id * d, qv, d, metric);
          if (len < ke) {
            heap[len].dist = v;
            heap[len].id = id;
            ++len;
            heap_sift_up(heap, len);
          } else if (v < heap[0].dist) {
            heap[0].dist = v;
            heap[0].id = id;
            heap_sift_down(heap, len, 1);
          }
        }
      }
      qsort(heap, (size_t)len, sizeof(nb_t), nb_cmp);
      for (int32_t i = 0; i < k; ++i) {
        ids[qi * (int64_t)k + i] = i < len ? (int32_t)heap[i].id : -1;
        dists[qi * (int64_t)k + i] = i < len ? heap[i].dist : INFINITY;
      }
    }
    free(heap);
  }
  return 0;
}

/* ------------------------------------------------------ CPU baseline */

static inline float dist_simd16(const float* x, const float* y, int32_t d, int32_t metric) {
  if (metric == ORC_COSINE) {
    float ab[16] = {0}, aa[16] = {0}, bb[16] = {0};
    int32_t i = 0;
    for (; i + 16 <= d; i += 16)
      for (int l = 0; l < 16; ++l) {
        ab[l] += x[i + l] * y[i + l];
        aa[l] += x[i + l] * x[i + l];
        bb[l] += y[i + l] * y[i + l];
      }
    float sab = 0, saa = 0, sbb = 0;
    for (int l = 0; l < 16; ++l) {
      sab += ab[l];
      saa += aa[l];
      sbb += bb[l];
    }
    for (; i < d; ++i) {
      sab += x[i] * y[i];
      saa += x[i] * x[i];
      sbb += y[i] * y[i];
    }
    float r = 1.0f - sab / (sqrtf(saa) * sqrtf(sbb));
    return r < 0.0f ? 0.0f : r;
  }
  float acc[16] = {0};
  int32_t i = 0;
  for (; i + 16 <= d; i += 16)
    for (int l = 0; l < 16; ++l) {
      float t = x[i + l] - y[i + l];
      acc[l] += t * t;
    }
  float s = 0.0f;
  for (int l = 0; l < 16; ++l) s += acc[l];
  for (; i < d; ++i) {
    float t = x[i] - y[i];
    s += t * t;
  }
  return metric == ORC_EUCLIDEAN ? sqrtf(s) : s;
}

static void select_row(const float* dv, int64_t n, int32_t k, int32_t* ids, float* dists,
                       kv_t* scratch) {
  int32_t ke = (int32_t)(k < n ? k : n);
  int32_t cnt = 0;
  for (int64_t j = 0; j < n; ++j) {
    kv_t c = {fkey32(dv[j]), j};
    if (cnt == ke && !kv_less(c, scratch[ke - 1])) continue;
    topk_push(scratch, ke, &cnt, c);
  }
  for (int32_t i = 0; i < k; ++i) {
    ids[i] = i < cnt ? (int32_t)scratch[i].idx : -1;
    dists[i] = i < cnt ? key_to_f32(scratch[i].key) : INFINITY;
  }
}

int cpu_bruteforce_batch(const float* base, int64_t n, const float* q, int64_t nq, int32_t d,
                         int32_t k, int32_t metric, int32_t* ids, float* dists,
                         int32_t nthreads) {
  if (d <= 0 || n <= 0) return 2;
  if (k <= 0 || nq <= 0) return 0;
  int nt = resolve_threads(nthreads);
  if (nq >= 64 && nt > 1) {
#pragma omp parallel num_threads(nt)
    {
      float* dv = (float*)malloc(sizeof(float) * (size_t)n);
      kv_t* scratch = (kv_t*)malloc(sizeof(kv_t) * (size_t)k);
#pragma omp for schedule(dynamic, 1)
      for (int64_t i = 0; i < nq; ++i) {
        const float* qv = q + i * (int64_t)d;
        for (int64_t j = 0; j < n; ++j) dv[j] = dist_simd16(base + j * (int64_t)d, qv, d, metric);
        select_row(dv, n, k, ids + i * (int64_t)k, dists + i * (int64_t)k, scratch);
      }
      free(dv);
      free(scratch);
    }
  } else {
    float* dv = (float*)malloc(sizeof(float) * (size_t)n);
    kv_t* scratch = (kv_t*)malloc(sizeof(kv_t) * (size_t)k);
    for (int64_t i = 0; i < nq; ++i) {
      const float* qv = q + i * (int64_t)d;
#pragma omp parallel for num_threads(nt) schedule(static)
      for (int64_t j = 0; j < n; ++j) dv[j] = dist_simd16(base + j * (int64_t)d, qv, d, metric);
      select_row(dv, n, k, ids + i * (int64_t)k, dists + i * (int64_t)k, scratch);
    }
    free(dv);
    free(scratch);
  }
  return 0;
}
