// context.cuh -- per-device state of libmanngpu: stream, grow-only scratch
// buffers, device properties and the autotune cache.
#pragma once
#include <mutex>
#include <unordered_map>
#include <vector>

#include "common.cuh"

namespace mann {

// Named scratch slots.  Each slot is one grow-only device allocation that is
// reused by every call on the device; calls are serialised by Context::mu and
// ordered on the GPU through Context::last_use.
enum ScratchSlot : int {
  SLOT_BASE = 0,      // host-pointer calls: device copy of the points
  SLOT_QUERIES,       // host-pointer calls: device copy of the queries
  SLOT_OUT_IDS,       // host-pointer calls: device ids
  SLOT_OUT_DISTS,     // host-pointer calls: device distances
  SLOT_PARTIAL,       // per-split top-k lists (uint64 keys)
  SLOT_KEYS,          // merged top-k lists (uint64 keys)
  SLOT_NORMS_Q,       // per-row squared norms of the queries
  SLOT_NORMS_B,       // per-row squared norms of the points
  SLOT_BF16_Q,        // BF16 copy of the (centred) queries
  SLOT_BF16_B,        // BF16 copy of the (centred) points
  SLOT_ROWINFO_Q,     // per-row bound terms of the queries
  SLOT_ROWINFO_B,     // per-row bound terms of the points
  SLOT_CENTRE,        // per-dimension centre (float) + reduction partials
  SLOT_CAND,          // candidate lists of the reduced-precision forms
  SLOT_FALLBACK,      // rows that need the exact FP32 scan
  SLOT_FALLBACK_KEYS, // their FP32 top-k lists
  SLOT_COUNTERS,      // small counters (report, status words)
  SLOT_MISC0,
  SLOT_MISC1,
  SLOT_MISC2,
  SLOT_MISC3,
  SLOT_OUT_KEYS_BF16, // final sorted keys of the BF16 form
  SLOT_SEED_PARTIAL,  // seed pass: per-CTA lists
  SLOT_SEED_LISTS,    // seed pass: merged lists
  SLOT_SEED,          // per-query admission seeds
  SLOT_KM_A,          // KMeans work buffers (k-means++ / Lloyd)
  SLOT_KM_B,
  SLOT_KM_C,
  SLOT_KM_D,
  SLOT_KM_E,
  SLOT_KM_F,
  SLOT_KM_G,
  SLOT_KM_H,
  SLOT_KM_I,
  SLOT_KM_J,
  SLOT_KM_DIST,       // assignment distances
  SLOT_KM_X,          // host-pointer KMeans calls: points
  SLOT_KM_CENT,       // centroids
  SLOT_KM_ASSIGN,     // assignments
  SLOT_IVF_CNT,       // IVF search: per-list query counts and cursors
  SLOT_IVF_OFF,       // IVF search: per-list query and chunk offsets
  SLOT_IVF_PAIRS,     // IVF search: (query, probe rank) pairs grouped by list
  SLOT_IVF_PARTIAL,   // IVF search: per-probe top-k lists
  SLOT_IVF_KEYS,      // IVF search: merged top-k lists
  SLOT_IVF_PROBES,    // IVF search: routed lists
  SLOT_IVF_ROUTE_D,   // IVF search: routing distances
  SLOT_IVF_ASSIGN,    // IVF build: cluster of every point
  SLOT_IVF_START,     // IVF build: list starts and sizes
  SLOT_IVF_MEMBERS,   // IVF build: members grouped by list
  SLOT_IVF_LOFF,      // host-pointer IVF calls: list offsets
  SLOT_IVF_LIDS,      // host-pointer IVF calls: list ids
  SLOT_PROBE_X,       // learned probe: BF16 queries
  SLOT_PROBE_H1,      // learned probe: first hidden layer
  SLOT_PROBE_H2,      // learned probe: second hidden layer
  SLOT_PROBE_LOGITS,  // learned probe: output scores
  SLOT_PROBE_D,       // learned probe: squared distances to the centroids
  SLOT_BATCH_ITEMS,   // batched graphs: work items
  SLOT_BATCH_OFFS,    // batched graphs: set offsets
  SLOT_BATCH_QUEUE,   // batched graphs: work-queue header
  SLOT_SEG_ITEMS,     // batched BF16 graphs: (set, block, tile) items
  SLOT_SEG_RUNS,      // batched BF16 graphs: the items of each block
  SLOT_SEG_ROWRUN,    // batched BF16 graphs: each row's block
  SLOT_SEG_QUEUE,     // batched BF16 graphs: fallback work-queue header
  SLOT_SEG_SITEMS,    // batched BF16 graphs: seed-pass items
  SLOT_SEG_SRUNS,     // batched BF16 graphs: seed-pass items of each block
  SLOT_SEG_SROWRUN,   // batched BF16 graphs: seed pass, each row's block
  SLOT_FP8_SCALE_B,   // FP8 form: per-point 1/f
  SLOT_FP8_SCALE_Q,   // FP8 form: per-query 1/f
  SLOT_COS_B,         // BF16 cosine: unit-normalised points
  SLOT_COS_Q,         // BF16 cosine: unit-normalised queries
  SLOT_COS_NB,        // BF16 cosine: squared norms of the points
  SLOT_COS_NQ,        // BF16 cosine: squared norms of the queries
  SLOT_PCA_IDX,       // host-pointer local PCA: neighbour and centre ids, dimensions
  SLOT_PCA_BASIS,     // host-pointer local PCA: bases
  SLOT_EDGE_COUNT,    // edge weights: negative-fallback counter
  SLOT_CSR_COUNTS,    // union graph: degrees, cursors, long rows
  SLOT_CSR_OFFS,      // union graph: row capacities
  SLOT_CSR_BUF,       // union graph: unsorted rows
  SLOT_CSR_COLS,      // host-pointer union graph: columns
  SLOT_CSR_ROWS,      // host-pointer union graph: row offsets
  SLOT_FP64_ERR,      // maximum FP64 error of the returned distances
  SLOT_TIES_ROWS,     // FP64 ties: rows whose boundary tie reached past the candidates
  SLOT_TIES_ROWS2,    // FP64 ties: rows still unsettled after the top-64 widening
  SLOT_TIES_ROWS3,    // FP64 ties: rows still unsettled after the top-256 widening
  SLOT_TIES_PARTIAL,  // FP64 ties: their wider FP32 lists (per split)
  SLOT_TIES_KEYS,     // FP64 ties: their wider FP32 lists (merged)
  SLOT_TIES_CNT,      // FP64 ties: candidate counts of the wider lists
  SLOT_TIES_FLOOR,    // FP64 ties: floors of the wider lists
  SLOT_TIES_COUNTERS, // FP64 ties: counters of the second resolve
  SLOT_TIES_TASKS,    // FP64 ties: (row, position, point) tasks
  SLOT_TIES_VALS,     // FP64 ties: FP64 distances by (row, position)
  SLOT_TIES_STATE,    // FP64 ties: rows to reorder
  SLOT_COUNT
};

// Prepared tensor-core operand of a dataset handle's points, kept between
// calls on the handle: the converted rows with their bound terms and norms
// (`rows`), and the centre, scales, bounds and cosine row norms (`misc`).
// `key` names the upload generation, metric and form it was prepared for
// (0: empty); knn_bf16.cu fills and reads it, the handle's destruction frees it.
struct PointsOperand {
  uint64_t key = 0;
  int64_t n = 0;
  int d = 0;
  void* rows = nullptr;
  size_t rows_bytes = 0;
  float* misc = nullptr;
  size_t misc_bytes = 0;
  int split = 0, f16 = 0, dp = 0, dpe = 0, width = 0, mainw = 0, augx = 0;
};

struct Context {
  int device = 0;
  int num_sms = 0;
  int cc_major = 0, cc_minor = 0;
  size_t smem_optin = 0;
  std::mutex mu;
  cudaStream_t stream = nullptr;   // used by the host-pointer entry points
  cudaEvent_t last_use = nullptr;  // recorded after every call that used scratch
  void* slot_ptr[SLOT_COUNT] = {};
  size_t slot_bytes[SLOT_COUNT] = {};
  // optional timing of the call's dominant kernel (MANN_FLAG_TIME_KERNEL)
  cudaEvent_t time_a = nullptr, time_b = nullptr;
  bool timing = false;  // requested for the current call
  bool timed = false;   // the dominant kernel has been bracketed
  void time_begin(cudaStream_t s);
  void time_end(cudaStream_t s);
  // autotune cache: shape class -> chosen configuration word
  std::unordered_map<uint64_t, uint64_t> tune;
  // prepared points of dataset handles (by handle), and the handle, its
  // points and upload generation during a call on a handle (owner NULL: none)
  std::unordered_map<const void*, PointsOperand> points_cache;
  const void* points_owner = nullptr;
  const float* points_base = nullptr;
  uint64_t points_generation = 0;  // the handle's serial and upload generation
  // frees a handle's prepared points (the handle is going away)
  void release_points(const void* owner);

  // Device buffer of at least `bytes` for `slot`.  Grows by reallocation
  // (cudaFree synchronises the device, so no kernel still uses the old one).
  mann_status scratch(int slot, size_t bytes, void** out);
  template <typename T>
  mann_status scratch_t(int slot, size_t count, T** out) {
    void* p = nullptr;
    mann_status s = scratch(slot, count * sizeof(T), &p);
    *out = static_cast<T*>(p);
    return s;
  }
};

// The context of the current device (created on first use).
mann_status get_context(Context** out);

// Scope guard for one entry-point call: locks the context, orders the call's
// stream after the previous call's use of scratch, and records the new use.
class CallScope {
 public:
  CallScope(Context* ctx, cudaStream_t s);
  ~CallScope();
  cudaStream_t stream() const { return s_; }

 private:
  Context* ctx_;
  cudaStream_t s_;
  std::unique_lock<std::mutex> lock_;
};

}  // namespace mann
