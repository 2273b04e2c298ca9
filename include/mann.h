/*
 * mann.h -- C ABI of libmanngpu.so, the GB300 (sm_103a) implementation of
 * ManifoldANN's exact-kNN / kNN-graph / KMeans-assignment hot path.
 *
 * Layout: a Julia Matrix{Float32} of size d x n (column-major, one point per
 * column) is, byte for byte, a row-major [n][d] array; pass pointer(data).
 * Ids are 0-based int32 (a Julia shim adds 1).  Outputs are caller-allocated
 * [q][k] arrays.  Every entry point returns a mann_status; MANN_OK is 0 and
 * mann_last_error() gives the calling thread's last message.
 *
 * Entry points with host pointers copy inputs to the GPU and results back on
 * every call (the reference passes `data` on every query,
 * src/ann_index.jl:1-10).  The *_device variants take device pointers on the
 * current device and a cudaStream_t (NULL = the legacy default stream); they
 * return once the work is enqueued, results are valid after the stream
 * synchronises.
 *
 * All entry points are thread-safe; calls on one device are serialised
 * internally (the reference's re-entrancy contract, src/ann_index.jl:60-66).
 */
#ifndef MANN_H
#define MANN_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t mann_status;
#define MANN_OK 0
#define MANN_EINVAL_DIM 1 /* Julia: DimensionMismatch (src/utils/validation.jl:8-12) */
#define MANN_EINVAL_ARG 2 /* Julia: ArgumentError (validation.jl:13-17, knn_graph.jl:55-59) */
#define MANN_ENOMEM 3
#define MANN_ECUDA 4
#define MANN_ETIMEOUT 5 /* a bounded device-side wait ran out; the context stays usable */
#define MANN_ENODEV 6

/* Distances.jl metrics aliased in src/utils/distances.jl:15-18 */
#define MANN_METRIC_EUCLIDEAN 0   /* Euclidean()   sqrt(sum((x-y)^2)) -- the reference default */
#define MANN_METRIC_SQEUCLIDEAN 1 /* SqEuclidean() sum((x-y)^2) */
#define MANN_METRIC_COSINE 2      /* CosineDist()  max(1 - x.y/(|x||y|), 0) */

/* Arithmetic forms of the exact search */
#define MANN_PREC_FP32 0 /* FP32 difference-form tiles + fused top-k (reference semantics) */
#define MANN_PREC_BF16 1 /* BF16 tcgen05 tiles, certified top-(k+m), exact FP32 rerank */
#define MANN_PREC_FP8 2  /* FP8-e4m3 tcgen05 tiles with per-row power-of-two scales, certified
                            top-(k+m), exact FP32 rerank (never chosen by AUTO: its certified
                            window is far wider than BF16's on the measured sets) */
#define MANN_PREC_AUTO 3 /* library picks: the tensor-core form when k <= 24, d >= 128 and n >= 4096
                            (FP16 rows when BF16 cannot hold the centred, scaled data exactly, BF16
                            rows otherwise), else the FP32 form */
#define MANN_PREC_FP16 4 /* FP16 tcgen05 tiles: rows centred and scaled by a power of two into
                            FP16's range (operand rounding 2^-11, one product per term at the
                            16-bit tensor rate, where data that BF16 cannot hold exactly needs
                            the three-product BF16 split), the norm fold as one BF16 step,
                            certified top-(k+m), exact FP32 rerank */

/* Flags */
#define MANN_FLAG_FP64_TIES 1u   /* order near-ties at the k-th boundary by FP64 distances */
#define MANN_FLAG_TIME_KERNEL 2u /* time the call's dominant kernel into report->kernel_ms
                                    (synchronises the stream before returning) */
#define MANN_FLAG_FP64_ERR 4u    /* report->max_abs_err_fp64 = max over the returned neighbours of
                                    |returned distance - FP64 distance| (synchronises the stream) */

typedef struct {
  int32_t metric;    /* MANN_METRIC_* */
  int32_t k;         /* neighbours per query; k <= 0 writes nothing (bruteforce.jl:55-56) */
  int32_t precision; /* MANN_PREC_* */
  int32_t margin;    /* extra candidates kept by reduced-precision forms; 0 = autotuned */
  uint32_t flags;    /* MANN_FLAG_* */
  int32_t reserved[3];
} mann_knn_params;

/* Optional per-call report (pass NULL to skip). */
typedef struct {
  int64_t rows;              /* query rows processed */
  int64_t rows_fallback;     /* rows whose reduced-precision candidate set could not be
                                certified and that were re-run by the exact FP32 scan */
  int64_t rows_fp64_ties;    /* rows where an FP64 recompute ordered a near-tie */
  int64_t candidates;        /* candidates reranked in exact FP32 */
  double max_abs_err_fp64;   /* with MANN_FLAG_FP64_ERR: max |returned - FP64| distance; else -1 */
  int32_t precision_used;    /* MANN_PREC_* actually run */
  int32_t margin_used;       /* candidates kept beyond k by the reduced-precision form */
  double kernel_ms;          /* dominant kernel's CUDA-event time (MANN_FLAG_TIME_KERNEL), else -1 */
  int64_t launches;          /* kernels this call launched */
  int64_t rows_ties_widened; /* MANN_FLAG_FP64_TIES: rows whose tie at the k-th distance reached
                                past the candidate list and were re-ordered from their exact
                                FP32 top-64 (top-256 when longer) */
  int64_t rows_unresolved;   /* MANN_FLAG_FP64_TIES: rows whose tie cluster is longer than that
                                (they keep the FP32 (distance, id) order); 0 in every test */
} mann_knn_report;

const char* mann_version(void);
/* Message for the calling thread's last non-OK status ("" if none). */
const char* mann_last_error(void);
mann_status mann_device_count(int32_t* out_count);

/* Page-lock (pin) a caller buffer so host<->device copies run at full speed
 * (Julia: call once on a long-lived Matrix). */
mann_status mann_host_register(void* ptr, int64_t bytes);
mann_status mann_host_unregister(void* ptr);

/* Exact kNN of q queries against n points (d dims each).
 * Replaces query(::BruteForceIndex, data, Q::AbstractMatrix, k)
 * (src/ann_index.jl:71-101 looping src/indices/bruteforce.jl:46-71).
 * out_ids/out_dists: [q][k]; columns >= min(k, n) are written as -1 / +inf.
 * Order: ascending (distance, id) -- partialsortperm, bruteforce.jl:65. */
mann_status mann_knn(const mann_knn_params* p, const float* base, int64_t n,
                     const float* queries, int64_t q, int32_t d, int32_t* out_ids,
                     float* out_dists, mann_knn_report* report);
mann_status mann_knn_device(const mann_knn_params* p, const float* base, int64_t n,
                            const float* queries, int64_t q, int32_t d, int32_t* out_ids,
                            float* out_dists, mann_knn_report* report, void* stream);

/* kNN graph of n points against themselves.
 * Replaces the column loop of build_knn_graph (src/graphs/knn_graph.jl:42-81):
 * each point queries k+1 neighbours (k when include_self), the point itself is
 * dropped wherever it appears and the first k others are kept
 * (_prepare_neighbors, knn_graph.jl:105-130).  MANN_EINVAL_ARG unless
 * 0 < k <= n - (include_self ? 0 : 1).  out: [n][k]. */
mann_status mann_knn_graph(const mann_knn_params* p, const float* data, int64_t n, int32_t d,
                           int32_t include_self, int32_t* out_ids, float* out_dists,
                           mann_knn_report* report);
mann_status mann_knn_graph_device(const mann_knn_params* p, const float* data, int64_t n,
                                  int32_t d, int32_t include_self, int32_t* out_ids,
                                  float* out_dists, mann_knn_report* report, void* stream);

/* Device-resident point set.  The reference keeps the data matrix with the
 * caller and passes it to every query (src/ann_index.jl:1-10); a dataset
 * handle is the explicit device copy of such a matrix, so repeated searches
 * over the same points copy only their queries.  The copy goes stale when the
 * caller changes the points: re-upload after insert!
 * (src/indices/bruteforce.jl:82-95).  A handle belongs to the device that
 * was current at create; calls from another device fail with MANN_EINVAL_ARG.
 * Searches may share a handle across threads; an upload or destroy must not
 * overlap a search on the same handle (the handle has no lock).  The first
 * BF16 / FP16 / AUTO search of an upload also keeps the points' prepared
 * tensor-core operand on the device (about 2 bytes per value, three times
 * that for data the BF16 form splits), which later searches of the same
 * upload, metric and form reuse; the next upload retires it (its memory is
 * reused) and mann_dataset_destroy frees it. */
typedef struct mann_dataset mann_dataset;
/* data: host [n][d] FP32; copied to the device before the call returns. */
mann_status mann_dataset_create(const float* data, int64_t n, int32_t d, mann_dataset** out);
/* Replace the contents with n new rows of the same width (n may grow). */
mann_status mann_dataset_upload(mann_dataset* ds, const float* data, int64_t n);
mann_status mann_dataset_destroy(mann_dataset* ds);
/* mann_knn / mann_knn_graph over a dataset's points: host queries and
 * outputs, the points already on the device. */
mann_status mann_knn_dataset(const mann_knn_params* p, const mann_dataset* ds, const float* queries,
                             int64_t q, int32_t* out_ids, float* out_dists, mann_knn_report* report);
mann_status mann_knn_graph_dataset(const mann_knn_params* p, const mann_dataset* ds, int32_t include_self,
                                   int32_t* out_ids, float* out_dists, mann_knn_report* report);

/* kNN graphs of nsets independent point sets stored back to back: set c is
 * rows [set_offsets[c], set_offsets[c+1]) of data (set_offsets[0] = 0, host
 * array of nsets+1).  Replaces a loop of build_knn_graph calls, one per set
 * (src/graphs/knn_graph.jl:42-81), with one launch over all sets (FP32 form,
 * Euclidean / SqEuclidean, k + (include_self ? 0 : 1) <= 32); row r of out
 * holds the graph row of point r with ids local to its set.  The launches of
 * a (buffers, sizes) signature are captured into a CUDA graph on first use
 * and replayed; the tile height and split count come from a measuring
 * autotuner (first call of a signature runs each candidate once). */
mann_status mann_knn_graph_batched(const mann_knn_params* p, const float* data, const int64_t* set_offsets,
                                   int32_t nsets, int32_t d, int32_t include_self, int32_t* out_ids,
                                   float* out_dists, mann_knn_report* report);
/* Same with device data and outputs (set_offsets stays a host array). */
mann_status mann_knn_graph_batched_device(const mann_knn_params* p, const float* data, const int64_t* set_offsets,
                                          int32_t nsets, int32_t d, int32_t include_self, int32_t* out_ids,
                                          float* out_dists, mann_knn_report* report, void* stream);

/* Undirected kNN graph: _symmetrize_adjacency (src/graphs/knn_graph.jl:196-210)
 * as CSR.  ids[n][k] 0-based (-1 = none); row i of the result is
 * out(i) ∪ in(i), ascending, without repeats.  out_row_offsets[n+1];
 * out_cols needs room for 2 n k entries; *out_nnz = entries written.
 * MANN_EINVAL_ARG if a vertex has more than 16384 distinct neighbours. */
mann_status mann_knn_graph_symmetrize(const int32_t* ids, int64_t n, int32_t k, int64_t* out_row_offsets,
                                      int32_t* out_cols, int64_t* out_nnz);
/* Same on device buffers (ids, out_row_offsets, out_cols); *out_nnz is a host
 * pointer, written once the stream has finished. */
mann_status mann_knn_graph_symmetrize_device(const int32_t* ids, int64_t n, int32_t k,
                                             int64_t* out_row_offsets, int32_t* out_cols, int64_t* out_nnz,
                                             void* stream);

/* ------------------------------------------------------------ KMeans (KMeansTransform) */

typedef struct {
  int32_t k;          /* clusters */
  int32_t metric;     /* MANN_METRIC_EUCLIDEAN or MANN_METRIC_SQEUCLIDEAN */
  int32_t init;       /* 0 random points, 1 k-means++ */
  int32_t max_iters;  /* Lloyd iterations (> 0) */
  double tol;         /* stop when the largest centroid movement is below tol */
  int64_t subsample;  /* > 0 and < n: Lloyd on that many random points, then a full assignment */
  uint64_t seed;      /* seed of the library's own generator (Julia's streams are not reproduced) */
} mann_kmeans_params;

/* D[n][k] = dist(X[i], C[j]) -- pairwise_distances! (src/transforms/kmeans/distance.jl:28-165).
 * Julia's k x n matrix D has the same bytes as this [n][k] array. */
mann_status mann_pairwise_distances(const float* X, int64_t n, const float* C, int32_t k, int32_t d,
                                    int32_t metric, float* D);

/* Nearest centroid of every point -- assign_clusters! on pairwise distances
 * (distance.jl:287-310): the exact arg-min (near-ties ordered in FP64, lowest
 * centroid id on exact ties), 0-based; out_dist (nullable) = its distance. */
mann_status mann_kmeans_assign(const float* X, int64_t n, const float* C, int32_t k, int32_t d,
                               int32_t metric, int32_t* out_assign, float* out_dist);

/* k-means++ seeding with the caller's randomness -- init_kmeans_plus_plus
 * (src/transforms/kmeans/init.jl:56-102): first = first point, u[i] in [0,1)
 * the i-th draw (u[0] unused).  out_idx[k] = chosen point indices. */
mann_status mann_kmeanspp(const float* X, int64_t n, int32_t d, int32_t k, int64_t first,
                          const double* u, int64_t* out_idx);

/* lloyd! (src/transforms/kmeans/lloyd.jl:36-134) from the given centroids
 * [k][d] (updated in place); out_assign[n] 0-based; *out_iters = iterations. */
mann_status mann_kmeans_lloyd(const float* X, int64_t n, int32_t d, int32_t k, float* centroids,
                              int32_t max_iters, double tol, int32_t metric, int32_t* out_assign,
                              int32_t* out_iters);

/* fit! of KMeansTransform (src/transforms/KMeansTransform.jl:106-161). */
mann_status mann_kmeans_fit(const mann_kmeans_params* p, const float* X, int64_t n, int32_t d,
                            float* out_centroids, int32_t* out_assign, int32_t* out_iters);

/* ---------------------------------------------------------------- IVF-Flat
 * build_index(IVFFlatIndex, ...) and query (src/indices/ivf_flat.jl:30-93,
 * :135-168).  Lists are CSR: list c holds list_ids[list_offsets[c] ..
 * list_offsets[c+1]) (0-based point ids, ascending within a list, as the
 * reference's counting pass leaves them); points stay the caller's [n][d]. */
typedef struct {
  int32_t nlist;
  int32_t centroid_metric;   /* MANN_METRIC_EUCLIDEAN (default) or _SQEUCLIDEAN */
  int32_t kmeans_max_iters;  /* <= 0: 25 */
  int32_t reserved;
  double kmeans_tol;         /* <= 0: 1e-4 */
  int64_t kmeans_subsample;  /* Lloyd sample; the reference's default is max(256 nlist, 32768) */
  uint64_t seed;
} mann_ivf_build_params;

/* KMeans (k-means++, Lloyd on the subsample, full assignment) + inverted lists.
 * out_centroids[nlist][d], out_offsets[nlist+1], out_ids[n]. */
mann_status mann_ivf_build(const mann_ivf_build_params* p, const float* data, int64_t n, int32_t d,
                           float* out_centroids, int64_t* out_offsets, int32_t* out_ids,
                           int32_t* out_iters);

/* query of IVFFlatIndex for q queries: route each query to its nprobe
 * (clamped to nlist) nearest centroids by exact centroid_metric distance,
 * scan those lists with p->metric (Euclidean / SqEuclidean, FP32 form), keep
 * the top p->k (1..64) by (distance, id).  Rows with fewer candidates than k
 * are padded with -1 / +inf (the reference returns the shorter list). */
mann_status mann_ivf_search(const mann_knn_params* p, int32_t nprobe, int32_t centroid_metric,
                            const float* data, int64_t n, int32_t d, const float* centroids,
                            int32_t nlist, const int64_t* list_offsets, const int32_t* list_ids,
                            const float* queries, int64_t q, int32_t* out_ids, float* out_dists);
/* Same with device pointers, ordered on `stream`. */
mann_status mann_ivf_search_device(const mann_knn_params* p, int32_t nprobe, int32_t centroid_metric,
                                   const float* data, int64_t n, int32_t d, const float* centroids,
                                   int32_t nlist, const int64_t* list_offsets,
                                   const int32_t* list_ids, const float* queries, int64_t q,
                                   int32_t* out_ids, float* out_dists, void* stream);
/* The list scan alone for a routing chosen by the caller (select_indices of
 * any routing policy, src/indices/multilevel/routing.jl): probes[q][nprobe]
 * (device) holds distinct list ids per query, -1 = unused slot. */
mann_status mann_ivf_scan_device(const mann_knn_params* p, const int32_t* probes, int32_t nprobe,
                                 const float* data, int64_t n, int32_t d, int32_t nlist,
                                 const int64_t* list_offsets, const int32_t* list_ids,
                                 const float* queries, int64_t q, int32_t* out_ids,
                                 float* out_dists, void* stream);

/* ----------------------------------------------------- learned coarse probe
 * No counterpart in the reference: a routing strategy beside TopKRouting
 * (select_indices, src/indices/multilevel/routing.jl:91-118) that ranks the
 * IVF lists of a query with a BF16 MLP din -> hidden1 -> hidden2 -> nout
 * (GELU after both hidden layers), trained on the GPU with softmax
 * cross-entropy against the lists holding the query's exact neighbours.
 * With use_prior the score of list c is MLP(q)_c - beta ||q - c||^2, beta =
 * exp(theta) learned with the rest.
 * Flat FP32 parameters (mann_probe_param_count floats): W1[hidden1][din],
 * b1[hidden1], W2[hidden2][hidden1], b2[hidden2], W3[nout][hidden2], b3[nout],
 * theta. */
typedef struct {
  int32_t din, hidden1, hidden2, nout;
  int32_t batch;      /* training rows per step (<= 0: 1024) */
  int32_t use_prior;  /* 1: add the distance prior (needs the centroids) */
  float lr, beta1, beta2, eps, weight_decay; /* AdamW (<= 0: 1e-3, 0.9, 0.999, 1e-8; decay as given) */
  float beta_init;    /* initial beta of the prior (<= 0: 1) */
  uint64_t seed;      /* initialisation and shuffling */
} mann_probe_params;

typedef struct mann_probe mann_probe; /* device-resident model */

int64_t mann_probe_param_count(const mann_probe_params* p);
/* Seeded initialisation (uniform +-1/sqrt(fan_in); with the prior the output
 * layer starts 20x smaller and its bias at zero). */
mann_status mann_probe_init(const mann_probe_params* p, float* params);
/* Model on the current device from flat params; centroids [nout][din] for the prior. */
mann_status mann_probe_create(const mann_probe_params* p, const float* params, const float* centroids,
                              mann_probe** out);
mann_status mann_probe_destroy(mann_probe* m);
mann_status mann_probe_get_params(mann_probe* m, float* params);
/* AdamW training on host queries [nq][din], labels [nq][nlabel] (list ids,
 * -1 = none); out_loss[epochs] = mean loss of each epoch (nullable). */
mann_status mann_probe_train(mann_probe* m, const float* queries, int64_t nq, const int32_t* labels,
                             int32_t nlabel, int32_t epochs, float* out_loss);
/* Loss and gradient of one batch (nq <= 65536) without an update. */
mann_status mann_probe_grad(mann_probe* m, const float* queries, int64_t nq, const int32_t* labels,
                            int32_t nlabel, float* out_grad, float* out_loss);
/* Scores [nq][nout] of host queries. */
mann_status mann_probe_scores(mann_probe* m, const float* queries, int64_t nq, float* out_scores);
/* Device queries [q][din] -> probes [q][nprobe] (best list first; ties to the
 * lower id) and the softmax mass of the chosen lists (nullable). */
mann_status mann_probe_route_device(mann_probe* m, const float* queries, int64_t q, int32_t nprobe,
                                    int32_t* out_probes, float* out_coverage, void* stream);
/* IVF search routed by the model (device pointers): mann_ivf_search_device
 * with the probes chosen by the scores instead of the centroid distances. */
mann_status mann_ivf_search_learned_device(mann_probe* m, const mann_knn_params* p, int32_t nprobe,
                                           const float* data, int64_t n, int32_t d, int32_t nlist,
                                           const int64_t* list_offsets, const int32_t* list_ids,
                                           const float* queries, int64_t q, int32_t* out_ids,
                                           float* out_dists, void* stream);
/* Same with host buffers. */
mann_status mann_ivf_search_learned(mann_probe* m, const mann_knn_params* p, int32_t nprobe, const float* data,
                                    int64_t n, int32_t d, int32_t nlist, const int64_t* list_offsets,
                                    const int32_t* list_ids, const float* queries, int64_t q,
                                    int32_t* out_ids, float* out_dists);

/* ------------------------------------------------------ local PCA (batched)
 * fit_geometry(::PCAMethod, data, center, neighbor_indices)
 * (src/geometry/pca.jl:101-241) for m centres at once -- the per-node fits of
 * LocalGeometryEstimator in build_weighted_graph
 * (src/graphs/weighted_knn_graph.jl:247-264).  Centre i is data row
 * centres[i], or query_points[i] (row-major [m][d]) when centres is NULL;
 * neighbors[m][k] (k <= 32) are data row ids, -1 = none.  Outputs:
 * out_dim[m], out_eigvals[m][maxd] (descending; zero past the dimension),
 * out_basis[m][maxd][d] (principal directions as rows, i.e. the bytes of
 * Julia's d x dim basis).  FP32, one-sided Jacobi; the eigenvalues are the
 * squared singular values of the centred neighbours, as the reference's. */
typedef struct {
  int32_t intrinsic_dim;      /* > 0: fixed dimension; 0: by variance ratio */
  int32_t reserved;
  double min_variance_ratio;  /* (0, 1], default 0.95 */
} mann_pca_params;

mann_status mann_local_pca(const mann_pca_params* p, const float* data, int64_t n, int32_t d,
                           const int32_t* centres, const float* query_points, int64_t m,
                           const int32_t* neighbors, int32_t k, int32_t maxd, int32_t* out_dim,
                           float* out_eigvals, float* out_basis);
mann_status mann_local_pca_device(const mann_pca_params* p, const float* data, int64_t n, int32_t d,
                                  const int32_t* centres, const float* query_points, int64_t m,
                                  const int32_t* neighbors, int32_t k, int32_t maxd, int32_t* out_dim,
                                  float* out_eigvals, float* out_basis, void* stream);

/* ---------------------------------------------------------- edge weights
 * compute_edge_weight for every edge of a kNN graph
 * (src/graphs/edge_weight.jl:163-262, src/graphs/weighted_knn_graph.jl:194-236):
 * nbrs[n][k] (0-based, -1 = none -> NaN weight), per-vertex tangent estimates
 * as written by mann_local_pca (dims[n], basis[n][maxd][d]); out_weights[n][k];
 * *out_negative = edges where the curvature-free estimator fell back to the
 * Euclidean chord (EstimatorDiagnostics.n_negative_fallbacks). */
#define MANN_EDGE_EUCLIDEAN_CHORD 0  /* ||x_j - x_i|| */
#define MANN_EDGE_TANGENT_SOURCE 1   /* d_T^(i) */
#define MANN_EDGE_TANGENT_MEAN 2     /* (d_T^(i) + d_T^(j)) / 2 */
#define MANN_EDGE_TANGENT_MAX 3      /* max(d_T^(i), d_T^(j)) */
#define MANN_EDGE_CURVATURE_FREE 4   /* (8 d_E - d_T^(i) - d_T^(j)) / 6, d_E when negative */

mann_status mann_edge_weights(int32_t rule, const float* data, int64_t n, int32_t d, const int32_t* nbrs,
                              int32_t k, const int32_t* dims, const float* basis, int32_t maxd,
                              float* out_weights, int64_t* out_negative);
mann_status mann_edge_weights_device(int32_t rule, const float* data, int64_t n, int32_t d,
                                     const int32_t* nbrs, int32_t k, const int32_t* dims,
                                     const float* basis, int32_t maxd, float* out_weights,
                                     int64_t* out_negative, void* stream);

/* Measured FP32 fused multiply-add rate of the current device (TFLOP/s,
 * 2 flops per FMA): independent fma.rn.f32x2 / fmaf chains on every lane,
 * timed with CUDA events, the faster form reported.  The denominator of the
 * FP32 kernels' rooflines.  No reference counterpart (device
 * characterisation).  out_ms (nullable): the timed launch. */
mann_status mann_measure_fp32_peak(double* out_tflops, double* out_ms);

/* Host-side fault injection for tests (no reference counterpart; the
 * reference reports failures as Julia exceptions, src/utils/validation.jl).
 * MANN_INJECT_ALLOC: the next `count` requests for the library's device
 * scratch fail as an out-of-memory cudaMalloc would (the call returns
 * MANN_ENOMEM; buffers already held stay valid).
 * MANN_INJECT_LAUNCH: the next `count` checked kernel launches report a CUDA
 * error (the call returns MANN_ECUDA; the work already enqueued completes).
 * MANN_INJECT_QUEUE: the next `count` batched-graph calls skip publishing
 * their device work queue (a producer that never delivers); the persistent
 * kernel's consumers give up after a short bounded wait and the call returns
 * MANN_ETIMEOUT with the context still usable.
 * count = 0 clears the kind.  Arming touches no GPU. */
#define MANN_INJECT_ALLOC 1
#define MANN_INJECT_LAUNCH 2
#define MANN_INJECT_QUEUE 3
mann_status mann_debug_inject(int32_t kind, int32_t count);

/* Exact kNN in the FP32 form for callers that cannot allocate device memory.
 * No counterpart in the reference: it is an addition of this library for
 * hosts that own all device memory through their own pool (a Julia or Python
 * runtime that reserved the GPU's memory), code that must not stall the
 * device with cudaMalloc/cudaFree (both synchronise it), and callers that
 * must not run out of memory mid-job.  Arguments as mann_knn_device (device
 * pointers; precision FP32 or AUTO, no MANN_FLAG_FP64_TIES).  It allocates
 * nothing: its scratch is one 16 MiB array the library holds on every device
 * it is loaded on until exit; a search that needs more is rejected with
 * MANN_EINVAL_ARG (pass fewer queries per call).  The first call on a device
 * looks up that array's address and should come before any stream capture.
 * All calls on a device share the array, so calls that overlap on the GPU
 * race: serialise them.  The array's address is looked up once per device
 * and kept for the life of the process: after a cudaDeviceReset the process
 * must be restarted before this entry point is called again. */
mann_status mann_knn_device_noalloc(const mann_knn_params* p, const float* base, int64_t n,
                                    const float* queries, int64_t q, int32_t d, int32_t* out_ids,
                                    float* out_dists, void* stream);

#ifdef __cplusplus
}
#endif
#endif
