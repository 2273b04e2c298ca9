// kernels.cuh -- internal launchers shared by the entry points.
#pragma once
#include "context.cuh"

namespace mann {

// Squared norms of n rows of d floats (sequential fused multiply-add over the
// dimensions, the same order as every FP32 distance in this library).
mann_status launch_row_sqnorm(const float* x, int64_t n, int d, float* out, cudaStream_t s);

// Exact FP32 top-kk of every query (difference-form distances, fused top-k).
// Result: sorted (distance, id) keys [nq][kk] in `out_keys` (device scratch
// owned by the context, valid until the next call).  `rows` optionally maps
// result row i to query row rows[i] (nq entries); NULL = identity.  Cosine
// needs the squared row norms of the points (bn) and of the query matrix (qn,
// indexed by query row).
mann_status knn_fp32_keys(Context* ctx, cudaStream_t s, const float* base, int64_t n,
                          const float* qs, int64_t nq, int d, int metric, int kk,
                          const int32_t* rows, const float* qn, const float* bn,
                          uint64_t** out_keys, int slot_partial, int slot_keys);

// Keys [nq][kk] -> ids/dists [*][kout].  Key row i goes to output row
// rows[i] (identity when rows is NULL).  With graph_self >= 0 the query of
// output row r is point (graph_self + r) and is dropped wherever it appears
// (_prepare_neighbors, src/graphs/knn_graph.jl:105-130); entries without a key
// become id -1 / +inf.
mann_status launch_finish(const uint64_t* keys, int64_t nq, int kk, int kout, int64_t graph_self,
                          const int32_t* rows, int32_t* ids, float* dists, cudaStream_t s);

// Operand forms of the tensor-core search: BF16 rows (the three-product split
// when BF16 cannot hold the data), E4M3 rows with per-row power-of-two scales
// (kind::f8f6f4), FP16 rows scaled by one power of two into FP16's range.
// FORM_AUTO16: FP16 rows when BF16 cannot hold the data exactly (one
// product per term instead of the split's three), BF16 rows otherwise.
enum : int { FORM_BF16 = 0, FORM_FP8 = 1, FORM_FP16 = 2, FORM_AUTO16 = 3 };

// Tensor-core form (SqEuclidean / Euclidean / cosine): certified candidates,
// exact FP32 rerank, optional FP64 near-tie order.  Result: keys [nq][kreq].
mann_status knn_bf16_keys(Context* ctx, cudaStream_t s, const float* base, int64_t n,
                          const float* qs, int64_t nq, int d, int metric, int kreq, int margin,
                          bool fp64, uint64_t** out_keys, mann_knn_report* rep, int form = FORM_BF16);

// Self-kNN keys [N][kreq] (global ids, the row itself included) of many point
// sets stored back to back (set c = rows [offs[c], offs[c+1])), each against
// its own points, in the BF16 form (offs on the host and on the device).
mann_status knn_bf16_batched_keys(Context* ctx, cudaStream_t s, const float* data, const int64_t* offs_host,
                                  const int64_t* offs_dev, int nsets, int d, int metric, int kreq, int margin,
                                  uint64_t** out_keys, mann_knn_report* rep, int form = FORM_BF16);

// Orders near-ties of sorted FP32 candidate lists as the FP64 oracle does
// (when fp64) and truncates them to kreq keys.  counters[0] += rows with a
// tie, counters[1] += rows whose boundary tie could not be settled (their
// query rows appended to unres_rows when it is not NULL), counters[2] is
// scratch of the call (Euclidean / SqEuclidean: += rows that needed FP64
// sequential sums; cosine: the FP64 task cursor, reset by the call).
// Candidate row i belongs to query / output row rows[i] (identity when rows
// is NULL).
mann_status launch_resolve(Context* ctx, const float* base, const float* qs, int d, int metric, int64_t nq, int L,
                           int kreq, int fp64, const uint64_t* cand, const int* cand_count,
                           const float* floor_val, uint64_t* keys_out, unsigned long long* counters,
                           cudaStream_t s, const int32_t* rows = nullptr, int32_t* unres_rows = nullptr);

// Exact FP32 top-kk lists -> FP64-ordered near-ties, truncated to kreq; rows
// whose boundary tie reaches past kk are widened to the top-KMAX_FUSED.
// Cosine needs the squared row norms (qn, bn) for that widening.
mann_status fp32_then_resolve(Context* ctx, cudaStream_t s, const float* base, const float* qs,
                              int64_t n, int64_t nq, int d, int metric, int kk, int kreq,
                              const uint64_t* fkeys, const float* qn, const float* bn,
                              uint64_t** out_keys, mann_knn_report* rep);

// Rows listed in unres_rows (h_unres, device) re-resolved from their exact
// FP32 top-min(n, KMAX_FUSED); the rows still unsettled are counted.
mann_status widen_unresolved(Context* ctx, cudaStream_t s, const float* base, const float* qs,
                             int64_t n, int d, int metric, int kreq, const float* qn,
                             const float* bn, const int32_t* unres_rows, int64_t h_unres,
                             uint64_t* keys_out, int64_t* still_unresolved);

// Plan and scratch-free variant of knn_fp32_keys (caller supplies `words`
// uint64 of device scratch).
void knn_fp32_plan(int num_sms, int64_t n, int64_t nq, int kk, int* nsplit_out, size_t* words_out);
mann_status knn_fp32_keys_on(int num_sms, cudaStream_t s, const float* base, int64_t n,
                             const float* qs, int64_t nq, int d, int metric, int kk,
                             const float* qn, const float* bn, uint64_t* scratch, size_t words,
                             uint64_t** out_keys);

// The exact search of mann_knn_device / mann_knn_graph_device on device
// buffers, inside a caller's CallScope (ids/dists [nq][kout]).
mann_status exact_search_device(Context* ctx, cudaStream_t s, const mann_knn_params* p,
                                const float* base, int64_t n, const float* qs, int64_t nq, int d,
                                int64_t graph_self, int kreq, int kout, int32_t* ids, float* dists,
                                mann_knn_report* rep);

// Merge nsplit sorted key lists of k per query (nsplit <= 128) into one.
// Work item of the segmented FP32 tile kernel (batched point sets).
struct SegItem {
  int64_t q0, qend, nb0, nb1;
  int32_t split, pad;
};
// Device work queue of the persistent segmented kernel: `count` items, taken
// in order through the atomic `head`; `epoch` publishes the queue of one call
// (consumers wait, bounded, for it); `status` receives MANN_ETIMEOUT when
// that wait runs out.
struct SegQueue {
  unsigned long long head;
  int count;
  unsigned epoch;
  int status;
  int pad[3];
};
// Persistent segmented kernel: resident CTAs consume the items of `q` (k <= 64).
// `qrows` (optional) maps an item's query index i to the query row qrows[i]
// (the lists still go to slot i).
mann_status launch_k1_persistent(int num_sms, const float* data, const SegItem* items, SegQueue* q, unsigned epoch,
                                 long long wait_cycles, int d, int metric, int bq, int k, int nsplit,
                                 uint64_t* partial, cudaStream_t s, const int32_t* qrows = nullptr);
// Publishes a work queue of `count` items (head 0, status 0, then the epoch).
// count_dev (optional) supplies the count from device memory instead.
mann_status launch_publish_queue(SegQueue* q, int count, const int* count_dev, unsigned epoch, cudaStream_t s);
mann_status knn_graph_batched_device(Context* ctx, cudaStream_t s, const mann_knn_params* p, const float* data,
                                     const int64_t* offs, int nsets, int d, int include_self, int32_t* ids,
                                     float* dists, mann_knn_report* rep);
mann_status fp64_max_error(Context* ctx, cudaStream_t s, const float* base, const float* qs, int d, int metric,
                           int64_t nq, int kout, const int32_t* ids, const float* dists, double* out);
mann_status launch_merge_lists(const uint64_t* partial, int64_t nq, int nsplit, int k, uint64_t* out,
                               cudaStream_t s);

// KMeans pieces (kmeans.cu) used by the IVF index.
mann_status kmeans_fit_device(Context* ctx, cudaStream_t s, const float* X, int64_t n, int d, int k,
                              int metric, int init, int max_iters, double tol, int64_t subsample,
                              uint64_t seed, float* C, int32_t* assign, int* iters_out);
mann_status group_by_cluster_device(Context* ctx, cudaStream_t s, const int32_t* assign, int64_t n,
                                    int k, int64_t* start, int64_t* count, int64_t* members);

// Largest k handled by the fused top-k kernels.
constexpr int KMAX_FUSED = 256;

}  // namespace mann
