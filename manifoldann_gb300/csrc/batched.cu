// batched.cu -- kNN graphs of many independent point sets of uneven size in
// one persistent launch replayed from a captured CUDA graph, with the tile
// height and split count picked by a measuring autotuner.
//
// Replaces a caller's loop of build_knn_graph(BruteForceIndex, cloud; k)
// (src/graphs/knn_graph.jl:42-81), one call per cloud: every set's graph has
// the reference's semantics (k+1 neighbours per point, the point itself
// dropped wherever it appears, (distance, id) order; ids local to the set).
//
// Work items are (set, block of BQ query rows, split of the set's points),
// largest first, in a device work queue.  A call runs: [memset of the split
// lists] -> publish (writes the queue header: item count, head 0, the call's
// epoch) -> k1_persistent (resident CTAs take items through an atomic head
// until the queue is empty; each waits, bounded, for the header of its epoch)
// -> [merge of splits] -> finish (drops the point itself) -> local ids.  The
// launches of one (buffers, sizes, plan) signature are captured once into a
// CUDA graph and replayed by later calls; the queue's status word is read
// after every call (MANN_ETIMEOUT when the consumers' wait ran out).
#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.cuh"

namespace mann {
namespace {

__global__ void localize_ids_kernel(int32_t* __restrict__ ids, int64_t nrows, int k,
                                    const int64_t* __restrict__ offs, int nsets) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  int lo = 0, hi = nsets - 1;
  while (lo < hi) {  // last set whose offset <= r
    const int mid = (lo + hi + 1) >> 1;
    if (offs[mid] <= r) lo = mid;
    else hi = mid - 1;
  }
  const int32_t base = (int32_t)offs[lo];
  int32_t* row = ids + r * k;
  for (int j = 0; j < k; ++j)
    if (row[j] >= 0) row[j] -= base;
}

__global__ void publish_queue_kernel(SegQueue* q, int count, const int* count_dev, unsigned epoch) {
  q->head = 0;
  q->count = count_dev ? *count_dev : count;
  q->status = 0;
  __threadfence();
  q->epoch = epoch;
}

struct Plan {
  int bq = 128, S = 1;
  std::vector<SegItem> items;
  uint64_t hash = 0;
};

// the consumers' wait for a published queue: about a second at 2 GHz
constexpr long long QUEUE_WAIT_CYCLES = 1ll << 31;
// with an injected dropped publish: about 50 us
constexpr long long QUEUE_WAIT_CYCLES_SHORT = 100000;

constexpr int64_t MIN_SPLIT_POINTS = 8192;

void make_plan(const int64_t* offs, int nsets, int bq, int S, Plan* p) {
  p->bq = bq;
  p->S = S;
  p->items.clear();
  for (int c = 0; c < nsets; ++c) {
    const int64_t o = offs[c], n = offs[c + 1] - offs[c];
    if (n <= 0) continue;
    const int sc = (int)std::max<int64_t>(1, std::min<int64_t>(S, n / MIN_SPLIT_POINTS));
    const int64_t len = (n + sc - 1) / sc;
    for (int64_t q = 0; q < n; q += bq)
      for (int sp = 0; sp < sc; ++sp) {
        SegItem it{};
        it.q0 = o + q;
        it.qend = o + n;
        it.nb0 = o + sp * len;
        it.nb1 = std::min(o + n, it.nb0 + len);
        it.split = sp;
        if (it.nb0 < it.nb1) p->items.push_back(it);
      }
  }
  std::stable_sort(p->items.begin(), p->items.end(), [](const SegItem& a, const SegItem& b) {
    return (a.nb1 - a.nb0) > (b.nb1 - b.nb0);
  });
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) {
    h ^= v;
    h *= 1099511628211ull;
  };
  mix((uint64_t)bq);
  mix((uint64_t)S);
  for (int c = 0; c <= nsets; ++c) mix((uint64_t)offs[c]);
  p->hash = h;
}

struct Bufs {
  SegItem* items = nullptr;
  int64_t* offs = nullptr;
  uint64_t* partial = nullptr;
  uint64_t* keys = nullptr;
  SegQueue* queue = nullptr;
};

struct Shape {
  const float* data;
  int64_t N;
  int nsets, d, metric, k, kk, include_self;
  int32_t* ids;
  float* dists;
};

// The launches of one call (no allocation, no synchronisation: capturable).
// `publish` = false leaves the queue unpublished (injected dropped publish);
// the consumers then give up after `wait_cycles`.
mann_status issue(int num_sms, const Shape& sh, const Plan& pl, const Bufs& b, unsigned epoch, bool publish,
                  long long wait_cycles, cudaStream_t s) {
  const int nitems = (int)pl.items.size();
  if (pl.S > 1) MANN_CUDA_TRY(cudaMemsetAsync(b.partial, 0xFF, sizeof(uint64_t) * sh.N * pl.S * sh.kk, s));
  if (publish) MANN_TRY(launch_publish_queue(b.queue, nitems, nullptr, epoch, s));
  MANN_TRY(launch_k1_persistent(num_sms, sh.data, b.items, b.queue, epoch, wait_cycles, sh.d, sh.metric, pl.bq,
                                sh.kk, pl.S, pl.S > 1 ? b.partial : b.keys, s));
  if (pl.S > 1) MANN_TRY(launch_merge_lists(b.partial, sh.N, pl.S, sh.kk, b.keys, s));
  MANN_TRY(launch_finish(b.keys, sh.N, sh.kk, sh.k, sh.include_self ? -1 : 0, nullptr, sh.ids, sh.dists, s));
  localize_ids_kernel<<<(unsigned)ceil_div(sh.N, 256), 256, 0, s>>>(sh.ids, sh.N, sh.k, b.offs, sh.nsets);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

struct GraphEntry {
  cudaGraphExec_t exec = nullptr;
  uint64_t last_use = 0;
  unsigned epoch = 0;
};

struct BatchState {
  std::mutex mu;
  std::map<std::string, GraphEntry> graphs;
  std::map<std::string, std::pair<int, int>> tuned;  // signature -> (bq, S)
  uint64_t clock = 0;
  cudaStream_t cap = nullptr;
  const void* uploaded_items = nullptr;  // device buffer holding the plan with hash uploaded_hash
  uint64_t uploaded_hash = 0;
  unsigned epoch = 0;  // last epoch handed to a queue
};

BatchState& state_of(Context* ctx) {
  static std::mutex mu;
  static std::map<Context*, BatchState*> all;
  std::lock_guard<std::mutex> lk(mu);
  BatchState*& st = all[ctx];
  if (!st) st = new BatchState();
  return *st;
}

constexpr size_t MAX_GRAPHS = 16;

mann_status prepare(Context* ctx, cudaStream_t s, const Shape& sh, const int64_t* offs_host, const Plan& pl,
                    Bufs* b, BatchState& st) {
  MANN_TRY(ctx->scratch_t(SLOT_BATCH_ITEMS, std::max<size_t>(pl.items.size(), 1), &b->items));
  MANN_TRY(ctx->scratch_t(SLOT_BATCH_OFFS, (size_t)sh.nsets + 1, &b->offs));
  MANN_TRY(ctx->scratch_t(SLOT_KEYS, (size_t)sh.N * sh.kk, &b->keys));
  MANN_TRY(ctx->scratch_t(SLOT_BATCH_QUEUE, 1, &b->queue));
  if (pl.S > 1) MANN_TRY(ctx->scratch_t(SLOT_PARTIAL, (size_t)sh.N * pl.S * sh.kk, &b->partial));
  if (st.uploaded_items != b->items || st.uploaded_hash != pl.hash) {
    MANN_CUDA_TRY(cudaMemcpyAsync(b->items, pl.items.data(), sizeof(SegItem) * pl.items.size(),
                                  cudaMemcpyHostToDevice, s));
    MANN_CUDA_TRY(cudaMemcpyAsync(b->offs, offs_host, sizeof(int64_t) * (sh.nsets + 1), cudaMemcpyHostToDevice, s));
    // the copies read pageable host memory: finish them before the plan can change
    MANN_CUDA_TRY(cudaStreamSynchronize(s));
    st.uploaded_items = b->items;
    st.uploaded_hash = pl.hash;
  }
  return MANN_OK;
}

std::string graph_key(const Shape& sh, const Plan& pl, const Bufs& b) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%p|%lld|%d|%d|%d|%d|%d|%p|%p|%p|%p|%p|%p|%p|%d|%d|%llu|%zu", (const void*)sh.data,
           (long long)sh.N, sh.nsets, sh.d, sh.metric, sh.k, sh.include_self, (void*)sh.ids, (void*)sh.dists,
           (void*)b.items, (void*)b.offs, (void*)b.partial, (void*)b.keys, (void*)b.queue, pl.bq, pl.S,
           (unsigned long long)pl.hash, pl.items.size());
  return buf;
}

mann_status run_graph(Context* ctx, cudaStream_t s, const Shape& sh, const Plan& pl, const Bufs& b,
                      BatchState& st) {
  const std::string key = graph_key(sh, pl, b);
  auto it = st.graphs.find(key);
  if (it == st.graphs.end()) {
    // captured on the library's own stream (the caller's may be the legacy
    // default stream, which cannot be captured); replayed on the caller's.
    // The graph's publish and consumers share its own epoch.
    if (!st.cap) MANN_CUDA_TRY(cudaStreamCreateWithFlags(&st.cap, cudaStreamNonBlocking));
    const unsigned epoch = ++st.epoch;
    cudaGraph_t g = nullptr;
    MANN_CUDA_TRY(cudaStreamBeginCapture(st.cap, cudaStreamCaptureModeThreadLocal));
    const mann_status rc = issue(ctx->num_sms, sh, pl, b, epoch, true, QUEUE_WAIT_CYCLES, st.cap);
    const cudaError_t ce = cudaStreamEndCapture(st.cap, &g);
    if (rc != MANN_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    MANN_CUDA_TRY(ce);
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    MANN_CUDA_TRY(ie);
    if (st.graphs.size() >= MAX_GRAPHS) {
      auto victim = st.graphs.begin();
      for (auto j = st.graphs.begin(); j != st.graphs.end(); ++j)
        if (j->second.last_use < victim->second.last_use) victim = j;
      cudaGraphExecDestroy(victim->second.exec);
      st.graphs.erase(victim);
    }
    it = st.graphs.emplace(key, GraphEntry{exec, 0, epoch}).first;
  }
  it->second.last_use = ++st.clock;
  MANN_CUDA_TRY(cudaGraphLaunch(it->second.exec, s));
  for (int i = 0; i < (pl.S > 1 ? 5 : 4); ++i) note_launch();  // kernels in the graph
  return MANN_OK;
}

// The queue's status word after the call's kernels: MANN_ETIMEOUT when the
// consumers' wait for a published queue ran out.
mann_status check_queue(const Bufs& b, cudaStream_t s) {
  int h = 0;
  MANN_CUDA_TRY(cudaMemcpyAsync(&h, &b.queue->status, sizeof(int), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  if (h != 0)
    return fail(MANN_ETIMEOUT, "batched graphs: the work queue was not published before the consumers' "
                               "bounded wait ran out");
  return MANN_OK;
}

}  // namespace

mann_status launch_publish_queue(SegQueue* q, int count, const int* count_dev, unsigned epoch, cudaStream_t s) {
  publish_queue_kernel<<<1, 1, 0, s>>>(q, count, count_dev, epoch);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

mann_status knn_graph_batched_device(Context* ctx, cudaStream_t s, const mann_knn_params* p, const float* data,
                                     const int64_t* offs, int nsets, int d, int include_self, int32_t* ids,
                                     float* dists, mann_knn_report* rep) {
  if (p->metric != MANN_METRIC_EUCLIDEAN && p->metric != MANN_METRIC_SQEUCLIDEAN)
    return fail(MANN_EINVAL_ARG, "batched graphs: Euclidean or SqEuclidean");
  const int k = p->k;
  Shape sh{data, offs[nsets], nsets, d, p->metric, k, include_self ? k : k + 1, include_self ? 1 : 0, ids, dists};
  if (p->precision == MANN_PREC_BF16 || p->precision == MANN_PREC_FP16) {
    // the tensor-core form: one segmented pass over every set's (block, tile) items
    int64_t* offs_dev = nullptr;
    MANN_TRY(ctx->scratch_t(SLOT_BATCH_OFFS, (size_t)nsets + 1, &offs_dev));
    MANN_CUDA_TRY(cudaMemcpyAsync(offs_dev, offs, sizeof(int64_t) * (nsets + 1), cudaMemcpyHostToDevice, s));
    uint64_t* keys = nullptr;
    ctx->time_begin(s);
    MANN_TRY(knn_bf16_batched_keys(ctx, s, data, offs, offs_dev, nsets, d, p->metric, sh.kk, p->margin, &keys, rep,
                                   p->precision == MANN_PREC_FP16 ? FORM_FP16 : FORM_BF16));
    ctx->time_end(s);
    MANN_TRY(launch_finish(keys, sh.N, sh.kk, k, include_self ? -1 : 0, nullptr, ids, dists, s));
    localize_ids_kernel<<<(unsigned)ceil_div(sh.N, 256), 256, 0, s>>>(ids, sh.N, k, offs_dev, nsets);
    MANN_CHECK_LAUNCH();
    BatchState& st = state_of(ctx);
    std::lock_guard<std::mutex> lk(st.mu);
    st.uploaded_items = nullptr;  // the offsets buffer was rewritten: the FP32 plan re-uploads
    return MANN_OK;
  }
  if (sh.kk > 64) return fail(MANN_EINVAL_ARG, "batched graphs support k <= 63 (64 with include_self)");
  BatchState& st = state_of(ctx);
  std::lock_guard<std::mutex> lk(st.mu);
  char sig[128];
  snprintf(sig, sizeof(sig), "%lld|%d|%d|%d|%d", (long long)sh.N, nsets, d, sh.kk, p->metric);
  auto tuned = st.tuned.find(sig);
  Plan pl;
  Bufs b;
  if (tuned == st.tuned.end()) {
    // measure every candidate once on this call's data (each run writes the
    // full result): tile heights (64-row tiles for k+1 > 32) x point splits
    static const int cand32[][2] = {{128, 1}, {64, 1}, {128, 2}, {64, 2}, {128, 4}};
    static const int cand64[][2] = {{64, 1}, {32, 1}, {64, 2}, {64, 4}};
    const int ncand = sh.kk > 32 ? 4 : 5;
    float best = 1e30f;
    std::pair<int, int> pick{sh.kk > 32 ? 64 : 128, 1};
    cudaEvent_t e0, e1;
    MANN_CUDA_TRY(cudaEventCreate(&e0));
    MANN_CUDA_TRY(cudaEventCreate(&e1));
    for (int ci = 0; ci < ncand; ++ci) {
      const int* c = sh.kk > 32 ? cand64[ci] : cand32[ci];
      make_plan(offs, nsets, c[0], c[1], &pl);
      MANN_TRY(prepare(ctx, s, sh, offs, pl, &b, st));
      cudaEventRecord(e0, s);
      MANN_TRY(issue(ctx->num_sms, sh, pl, b, ++st.epoch, true, QUEUE_WAIT_CYCLES, s));
      cudaEventRecord(e1, s);
      MANN_CUDA_TRY(cudaEventSynchronize(e1));
      MANN_TRY(check_queue(b, s));
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) {
        best = ms;
        pick = {c[0], c[1]};
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tuned = st.tuned.emplace(sig, pick).first;
  }
  make_plan(offs, nsets, tuned->second.first, tuned->second.second, &pl);
  MANN_TRY(prepare(ctx, s, sh, offs, pl, &b, st));
  if (rep) rep->margin_used = pl.bq * 100 + pl.S;  // chosen configuration: tile height * 100 + splits
  if (injected_dropped_publish()) {
    // the queue's producer "fails": the consumers find no published queue and
    // return MANN_ETIMEOUT after a short bounded wait (no kernel is left waiting)
    MANN_TRY(issue(ctx->num_sms, sh, pl, b, ++st.epoch, false, QUEUE_WAIT_CYCLES_SHORT, s));
    return check_queue(b, s);
  }
  ctx->time_begin(s);
  MANN_TRY(run_graph(ctx, s, sh, pl, b, st));
  ctx->time_end(s);
  return check_queue(b, s);
}

}  // namespace mann

using namespace mann;

extern "C" {

static mann_status batched_check(const mann_knn_params* p, const float* data, const int64_t* offs, int32_t nsets,
                                 int32_t d, int32_t include_self, const int32_t* ids, const float* dists) {
  if (!p) return fail(MANN_EINVAL_ARG, "params must not be NULL");
  if (d <= 0) return fail(MANN_EINVAL_ARG, "Dataset must have at least one dimension");
  if (nsets <= 0 || !offs) return fail(MANN_EINVAL_ARG, "at least one point set is needed");
  if (offs[0] != 0) return fail(MANN_EINVAL_ARG, "set offsets must start at 0");
  for (int c = 0; c < nsets; ++c) {
    const int64_t n = offs[c + 1] - offs[c];
    if (n <= 0) return fail(MANN_EINVAL_ARG, "Dataset must contain at least one point");
    const int64_t max_neighbors = n - (include_self ? 0 : 1);
    if (!(0 < p->k && p->k <= max_neighbors))
      return fail(MANN_EINVAL_ARG, "k must satisfy 0 < k <= " + std::to_string(max_neighbors) +
                                       " for dataset with " + std::to_string(n) + " points");
  }
  if (offs[nsets] > INT32_MAX) return fail(MANN_EINVAL_ARG, "at most 2^31-1 points in a batch");
  if (!data || !ids || !dists) return fail(MANN_EINVAL_ARG, "NULL buffer");
  return MANN_OK;
}

mann_status mann_knn_graph_batched_device(const mann_knn_params* p, const float* data, const int64_t* set_offsets,
                                          int32_t nsets, int32_t d, int32_t include_self, int32_t* out_ids,
                                          float* out_dists, mann_knn_report* report, void* stream) {
  clear_error();
  MANN_TRY(batched_check(p, data, set_offsets, nsets, d, include_self, out_ids, out_dists));
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CallScope scope(ctx, s);
  const int64_t l0 = launch_count();
  ctx->timing = report && (p->flags & MANN_FLAG_TIME_KERNEL);
  ctx->timed = false;
  MANN_TRY(knn_graph_batched_device(ctx, s, p, data, set_offsets, nsets, d, include_self, out_ids, out_dists,
                                    report));
  if (report) {
    report->rows = set_offsets[nsets];
    report->precision_used =
        (p->precision == MANN_PREC_BF16 || p->precision == MANN_PREC_FP16) ? p->precision : MANN_PREC_FP32;
    report->launches = launch_count() - l0;
    report->kernel_ms = -1;
    if (ctx->timing && ctx->timed) {
      MANN_CUDA_TRY(cudaEventSynchronize(ctx->time_b));
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, ctx->time_a, ctx->time_b);
      report->kernel_ms = ms;
    }
  }
  ctx->timing = false;
  return MANN_OK;
}

mann_status mann_knn_graph_batched(const mann_knn_params* p, const float* data, const int64_t* set_offsets,
                                   int32_t nsets, int32_t d, int32_t include_self, int32_t* out_ids,
                                   float* out_dists, mann_knn_report* report) {
  clear_error();
  MANN_TRY(batched_check(p, data, set_offsets, nsets, d, include_self, out_ids, out_dists));
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  const int64_t N = set_offsets[nsets];
  float *dx = nullptr, *dd = nullptr;
  int32_t* di = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_BASE, (size_t)N * d, &dx));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_IDS, (size_t)N * p->k, &di));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_DISTS, (size_t)N * p->k, &dd));
  MANN_CUDA_TRY(cudaMemcpyAsync(dx, data, sizeof(float) * N * d, cudaMemcpyHostToDevice, s));
  const int64_t l0 = launch_count();
  MANN_TRY(knn_graph_batched_device(ctx, s, p, dx, set_offsets, nsets, d, include_self, di, dd, report));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_ids, di, sizeof(int32_t) * N * p->k, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_dists, dd, sizeof(float) * N * p->k, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  if (report) {
    report->rows = N;
    report->precision_used =
        (p->precision == MANN_PREC_BF16 || p->precision == MANN_PREC_FP16) ? p->precision : MANN_PREC_FP32;
    report->launches = launch_count() - l0;
    report->kernel_ms = -1;
  }
  return MANN_OK;
}

}  // extern "C"
