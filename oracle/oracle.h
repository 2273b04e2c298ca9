/*
 * oracle.h -- CPU restatement of ManifoldANN's exact-kNN / kNN-graph /
 * KMeans-assignment / IVF semantics.
 *
 * THIS IS TEST INFRASTRUCTURE.  Only the test-suite, the smoke check and the
 * CPU-baseline leg of bench.py load it, and only as the checker or as the
 * timed CPU baseline.  The GPU library never links, loads or calls it.
 *
 * Parity pins: the known answers of the reference's own tests
 *   test/unit/indices/bruteforce_tests.jl:22-27   ([0 1 2;0 0 0], q=[.25,0], k=2 -> [1,2])
 *   test/unit/graphs/graph_tests.jl:4-48           (collinear equal-gap points, ties -> lower id)
 *   test/unit/indices/multilevel/routing_tests.jl:8-56 ([5,4,3], [4,3,2,1])
 *   test/unit/transforms/test_kmeans_optimizations.jl:107-122 (clamp >= 0)
 * are checked against this file by tests/test_oracle.py.  The Float32
 * summation order of Distances.jl 0.10.12 (an un-vendored Julia package) is
 * not pinned by any reference test; this restatement fixes it to a
 * sequential fused multiply-add over dimensions 0..d-1, which the GPU FP32
 * kernels reproduce bit for bit.
 */
#ifndef MANN_ORACLE_H
#define MANN_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* metric codes (same values as include/mann.h) */
#define ORC_EUCLIDEAN 0
#define ORC_SQEUCLIDEAN 1
#define ORC_COSINE 2

/* Per-pair distances, FP32 and FP64 (src/utils/distances.jl:15-18). */
float orc_dist_f32(const float* x, const float* y, int32_t d, int32_t metric);
double orc_dist_f64(const float* x, const float* y, int32_t d, int32_t metric);

/* Exact kNN of every query (src/indices/bruteforce.jl:46-71 per query,
 * src/ann_index.jl:71-101 over the batch).  Points and queries are row-major
 * [n][d] (= Julia column-major d x n).  Output [nq][k]; columns at or beyond
 * min(k, n) get id -1 and +inf.  Ids are 0-based. */
int orc_knn_f32(const float* base, int64_t n, const float* q, int64_t nq, int32_t d,
                int32_t k, int32_t metric, int32_t* ids, float* dists, int32_t nthreads);
int orc_knn_f64(const float* base, int64_t n, const float* q, int64_t nq, int32_t d,
                int32_t k, int32_t metric, int32_t* ids, double* dists, int32_t nthreads);

/* build_knn_graph (src/graphs/knn_graph.jl:42-81, _prepare_neighbors :105-130):
 * query k+1 (k when include_self), drop the point itself wherever it sits,
 * keep the first k.  Returns 0, or 2 (ArgumentError) when k is out of range. */
int orc_knn_graph_f32(const float* data, int64_t n, int32_t d, int32_t k, int32_t include_self,
                      int32_t metric, int32_t* ids, float* dists, int32_t nthreads);
int orc_knn_graph_f64(const float* data, int64_t n, int32_t d, int32_t k, int32_t include_self,
                      int32_t metric, int32_t* ids, double* dists, int32_t nthreads);
/* The same rows of the graph for the points rows[0..nrows) only (output row
 * i = point rows[i]): sampled rows of a graph too large for the full oracle. */
int orc_knn_graph_rows_f32(const float* data, int64_t n, int32_t d, int32_t k,
                           int32_t include_self, int32_t metric, const int32_t* rows,
                           int64_t nrows, int32_t* ids, float* dists, int32_t nthreads);
int orc_knn_graph_rows_f64(const float* data, int64_t n, int32_t d, int32_t k,
                           int32_t include_self, int32_t metric, const int32_t* rows,
                           int64_t nrows, int32_t* ids, double* dists, int32_t nthreads);

/* KMeans assignment.
 * _gemm_f32: the reference's GEMM-form distances (src/transforms/kmeans/distance.jl:68-143:
 *   ||c||^2 + ||x||^2 - 2 c.x, clamped at 0, sqrt for Euclidean) followed by the
 *   strict-< arg-min of assign_clusters! (:287-310).  Sums are sequential.
 * _f64: the exact answer: FP64 difference-form distances, strict-< arg-min
 *   (lowest centroid id wins ties).  out_dist holds the winning distance. */
int orc_kmeans_assign_gemm_f32(const float* X, int64_t n, const float* C, int32_t nlist, int32_t d,
                               int32_t metric, int32_t* assign, float* out_dist, int32_t nthreads);
int orc_kmeans_assign_f64(const float* X, int64_t n, const float* C, int32_t nlist, int32_t d,
                          int32_t metric, int32_t* assign, double* out_dist, int32_t nthreads);

/* k-means++ seeding (src/transforms/kmeans/init.jl:56-102) with the
 * randomness supplied: first = index of the first centroid, u[i] uniform in
 * [0,1) for the i-th draw (i = 1..k-1).  D^2 is the FP32 difference form; the
 * running sums are FP64 over blocks of 1024 points (block sums sequential,
 * then a sequential prefix over blocks) -- the same order as the GPU.  The
 * next centroid is the first point whose cumulative D^2 reaches u*total
 * (searchsortedfirst).  out_idx[0..k-1] = chosen point indices. */
int orc_kmeanspp(const float* X, int64_t n, int32_t d, int32_t k, int64_t first, const double* u,
                 int64_t* out_idx);

/* Lloyd iterations (src/transforms/kmeans/lloyd.jl:36-134) from the given
 * centroids C [k][d] (updated in place): exact assignment (FP64 difference
 * form, strict <), per-cluster FP32 sums in point order, division by the
 * count, empty clusters refilled with the point farthest from its assigned
 * centroid (first maximum; a chosen point is marked -inf), stop when the
 * largest centroid movement (metric) is below tol; final assignment.
 * Returns the iterations run in *iters. */
int orc_kmeans_lloyd(const float* X, int64_t n, int32_t d, int32_t k, float* C, int32_t max_iters,
                     double tol, int32_t metric, int32_t* assign, int32_t* iters, int32_t nthreads);

/* select_indices(::TopKRouting, ::KMeansAssignment, domain)
 * (src/indices/multilevel/routing.jl:94-118).  Writes up to k 0-based
 * positions; returns the count, or -2 for the ArgumentError case (no
 * distances while children exist). */
int32_t orc_topk_route(const float* dists, int32_t n_dist, int32_t n_children, int32_t k,
                       int32_t* out);

/* The routing step of that query alone: the nprobe lists of every query by
 * the GEMV-form centroid distances (ivf_flat.jl:103-131) and partialsortperm
 * (:150).  probes: [nq][min(nprobe, nlist)]. */
int orc_ivf_route_gemv_f32(const float* centroids, const float* centroid_norms, int32_t nlist,
                           int32_t d, const float* q, int64_t nq, int32_t nprobe,
                           int32_t centroid_metric, int32_t* probes, int32_t nthreads);

/* IVF-Flat query (src/indices/ivf_flat.jl:103-168): SqEuclidean / Euclidean
 * centroid distances in GEMV form, partialsortperm(nprobe), scan of the probed
 * lists into a bounded max-heap (strict < admission) and a final sort by
 * (dist, id).  lists are CSR: list_offsets[nlist+1], list_ids[n] (0-based).
 * Output [nq][k]; short rows padded with -1/+inf. */
int orc_ivf_query_f32(const float* data, int32_t d, const float* centroids,
                      const float* centroid_norms, int32_t nlist, const int64_t* list_offsets,
                      const int32_t* list_ids, const float* q, int64_t nq, int32_t k,
                      int32_t nprobe, int32_t metric, int32_t centroid_metric, int32_t* ids,
                      float* dists, int32_t nthreads);

/* The list scan of the IVF-Flat query (src/indices/ivf_flat.jl:153-167) for
 * given probes [nq][nprobe] (0-based list ids, -1 = none): k_eff =
 * min(k, points in the probed lists), BoundedMaxHeap admission, final (dist,
 * id) sort.  Output [nq][k] padded with -1 / +inf. */
int orc_ivf_scan_f32(const float* data, int32_t d, const int64_t* list_offsets,
                     const int32_t* list_ids, const float* q, int64_t nq, const int32_t* probes,
                     int32_t nprobe, int32_t k, int32_t metric, int32_t* ids, float* dists,
                     int32_t nthreads);

/* Reference-algorithm CPU baseline (timed, not a parity oracle): per query all
 * n distances into a vector, then a (dist, index) selection; threads over the
 * queries when there are at least 64 of them, else over the points
 * (src/ann_index.jl:91-98, src/indices/bruteforce.jl:59-65).  The per-pair
 * reduction uses 16 independent partial sums, as a vectorised @simd loop does. */
int cpu_bruteforce_batch(const float* base, int64_t n, const float* q, int64_t nq, int32_t d,
                         int32_t k, int32_t metric, int32_t* ids, float* dists, int32_t nthreads);

int32_t orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
