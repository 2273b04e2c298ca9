// api.cu -- extern "C" entry points of libmanngpu (declared in include/mann.h).
#include <atomic>
#include <new>
#include <string>

#include "kernels.cuh"

namespace mann {
const char* last_error_cstr();

namespace {

bool valid_metric(int m) {
  return m == MANN_METRIC_EUCLIDEAN || m == MANN_METRIC_SQEUCLIDEAN || m == MANN_METRIC_COSINE;
}

mann_status check_common(const mann_knn_params* p, int64_t n, int32_t d) {
  if (!p) return fail(MANN_EINVAL_ARG, "params must not be NULL");
  if (d <= 0) return fail(MANN_EINVAL_ARG, "Dataset must have at least one dimension");
  if (n <= 0) return fail(MANN_EINVAL_ARG, "Dataset must contain at least one point");
  if (n > 0x7FFFFFFFll) return fail(MANN_EINVAL_ARG, "at most 2^31-1 points (int32 ids)");
  if (!valid_metric(p->metric)) return fail(MANN_EINVAL_ARG, "unknown metric code");
  if (p->precision != MANN_PREC_FP32 && p->precision != MANN_PREC_BF16 && p->precision != MANN_PREC_FP8 &&
      p->precision != MANN_PREC_AUTO && p->precision != MANN_PREC_FP16)
    return fail(MANN_EINVAL_ARG, "unknown precision code");
  return MANN_OK;
}

mann_status search_device_body(Context* ctx, cudaStream_t s, const mann_knn_params* p,
                               const float* base, int64_t n, const float* qs, int64_t nq, int d,
                               int64_t graph_self, int kreq, int kout, int32_t* ids, float* dists,
                               mann_knn_report* rep);

// One exact search on device buffers.  graph_self >= 0: the queries are the
// points themselves (row r is point r) and `kreq` = k+1 lists drop the self id.
mann_status search_device(Context* ctx, cudaStream_t s, const mann_knn_params* p,
                          const float* base, int64_t n, const float* qs, int64_t nq, int d,
                          int64_t graph_self, int kreq, int kout, int32_t* ids, float* dists,
                          mann_knn_report* rep) {
  const int64_t launches0 = launch_count();
  ctx->timing = (p->flags & MANN_FLAG_TIME_KERNEL) != 0;
  ctx->timed = false;
  mann_status st = search_device_body(ctx, s, p, base, n, qs, nq, d, graph_self, kreq, kout, ids,
                                      dists, rep);
  if (rep) {
    rep->launches = launch_count() - launches0;
    rep->kernel_ms = -1.0;
    if (st == MANN_OK && ctx->timing && ctx->timed) {
      float ms = 0.0f;
      MANN_CUDA_TRY(cudaEventSynchronize(ctx->time_b));
      MANN_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->time_a, ctx->time_b));
      rep->kernel_ms = ms;
    }
  }
  ctx->timing = false;
  return st;
}

mann_status search_device_body(Context* ctx, cudaStream_t s, const mann_knn_params* p,
                               const float* base, int64_t n, const float* qs, int64_t nq, int d,
                               int64_t graph_self, int kreq, int kout, int32_t* ids, float* dists,
                               mann_knn_report* rep) {
  if (rep) {
    *rep = mann_knn_report{};
    rep->rows = nq;
    rep->max_abs_err_fp64 = -1.0;
    rep->precision_used = MANN_PREC_FP32;
  }
  if (nq <= 0 || kout <= 0) return MANN_OK;
  if (kreq > KMAX_FUSED)
    return fail(MANN_EINVAL_ARG, "k = " + std::to_string(kreq) + " exceeds the fused top-k limit " +
                                     std::to_string(KMAX_FUSED));
  bool use_bf16 = false;
  const int form = p->precision == MANN_PREC_FP8 ? FORM_FP8 : (p->precision == MANN_PREC_FP16 ? FORM_FP16 : FORM_BF16);
  if (p->precision == MANN_PREC_BF16 || form != FORM_BF16) {
    if (kreq > 24)
      return fail(MANN_EINVAL_ARG, "the BF16, FP16 and FP8 forms support k <= 24 (k+1 for graphs)");
    use_bf16 = true;
  } else if (p->precision == MANN_PREC_AUTO) {
    use_bf16 = kreq <= 24 && d >= 128 && n >= 4096;
  }
  const int form_used = p->precision == MANN_PREC_AUTO ? FORM_AUTO16 : form;
  const float* qn = nullptr;
  const float* bn = nullptr;
  if (p->metric == MANN_METRIC_COSINE && !use_bf16) {
    float *db = nullptr, *dq = nullptr;
    MANN_TRY(ctx->scratch_t(SLOT_NORMS_B, (size_t)n, &db));
    MANN_TRY(launch_row_sqnorm(base, n, d, db, s));
    bn = db;
    if (qs == base) {
      qn = db;
    } else {
      MANN_TRY(ctx->scratch_t(SLOT_NORMS_Q, (size_t)nq, &dq));
      MANN_TRY(launch_row_sqnorm(qs, nq, d, dq, s));
      qn = dq;
    }
  }
  uint64_t* keys = nullptr;
  if (use_bf16) {
    MANN_TRY(knn_bf16_keys(ctx, s, base, n, qs, nq, d, p->metric, kreq, p->margin,
                           (p->flags & MANN_FLAG_FP64_TIES) != 0, &keys, rep, form_used));
    if (rep) rep->rows = nq;
  } else if (p->flags & MANN_FLAG_FP64_TIES) {
    // FP32 scan with a few extra entries, then FP64 order for near-ties
    const int kk = (int)std::min<int64_t>(std::min<int64_t>(n, KMAX_FUSED), (int64_t)kreq + 32);
    uint64_t* fkeys = nullptr;
    MANN_TRY(knn_fp32_keys(ctx, s, base, n, qs, nq, d, p->metric, kk, nullptr, qn, bn, &fkeys,
                           SLOT_PARTIAL, SLOT_KEYS));
    MANN_TRY(fp32_then_resolve(ctx, s, base, qs, n, nq, d, p->metric, kk, kreq, fkeys, qn, bn, &keys, rep));
  } else {
    MANN_TRY(knn_fp32_keys(ctx, s, base, n, qs, nq, d, p->metric, kreq, nullptr, qn, bn, &keys,
                           SLOT_PARTIAL, SLOT_KEYS));
  }
  MANN_TRY(launch_finish(keys, nq, kreq, kout, graph_self, nullptr, ids, dists, s));
  if (rep && (p->flags & MANN_FLAG_FP64_ERR))
    MANN_TRY(fp64_max_error(ctx, s, base, qs, d, p->metric, nq, kout, ids, dists, &rep->max_abs_err_fp64));
  return MANN_OK;
}

mann_status knn_impl(const mann_knn_params* p, const float* base, int64_t n, const float* qs,
                     int64_t q, int32_t d, int32_t* ids, float* dists, mann_knn_report* rep,
                     bool host, cudaStream_t user_stream) {
  clear_error();
  MANN_TRY(check_common(p, n, d));
  if (q < 0) return fail(MANN_EINVAL_ARG, "negative query count");
  if (rep) *rep = mann_knn_report{};
  if (p->k <= 0 || q == 0) return MANN_OK;
  if (!base || !qs || !ids || !dists) return fail(MANN_EINVAL_ARG, "NULL buffer");
  const int kout = p->k;
  const int kreq = (int)std::min<int64_t>(p->k, n);
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = host ? ctx->stream : user_stream;
  CallScope scope(ctx, s);
  if (!host) return search_device(ctx, s, p, base, n, qs, q, d, -1, kreq, kout, ids, dists, rep);

  float *db = nullptr, *dq = nullptr, *dd = nullptr;
  int32_t* di = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_BASE, (size_t)n * d, &db));
  MANN_TRY(ctx->scratch_t(SLOT_QUERIES, (size_t)q * d, &dq));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_IDS, (size_t)q * kout, &di));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_DISTS, (size_t)q * kout, &dd));
  MANN_CUDA_TRY(cudaMemcpyAsync(db, base, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dq, qs, sizeof(float) * q * d, cudaMemcpyHostToDevice, s));
  MANN_TRY(search_device(ctx, s, p, db, n, dq, q, d, -1, kreq, kout, di, dd, rep));
  MANN_CUDA_TRY(cudaMemcpyAsync(ids, di, sizeof(int32_t) * q * kout, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dists, dd, sizeof(float) * q * kout, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  return MANN_OK;
}

mann_status graph_impl(const mann_knn_params* p, const float* data, int64_t n, int32_t d,
                       int32_t include_self, int32_t* ids, float* dists, mann_knn_report* rep,
                       bool host, cudaStream_t user_stream) {
  clear_error();
  MANN_TRY(check_common(p, n, d));
  if (rep) *rep = mann_knn_report{};
  const int64_t max_neighbors = n - (include_self ? 0 : 1);
  if (!(p->k > 0 && p->k <= max_neighbors))
    return fail(MANN_EINVAL_ARG, "k must satisfy 0 < k <= " + std::to_string(max_neighbors) +
                                     " for dataset with " + std::to_string(n) + " points");
  if (!data || !ids || !dists) return fail(MANN_EINVAL_ARG, "NULL buffer");
  const int kout = p->k;
  const int kreq = p->k + (include_self ? 0 : 1);
  const int64_t self = include_self ? -1 : 0;
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = host ? ctx->stream : user_stream;
  CallScope scope(ctx, s);
  if (!host) return search_device(ctx, s, p, data, n, data, n, d, self, kreq, kout, ids, dists, rep);

  float *db = nullptr, *dd = nullptr;
  int32_t* di = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_BASE, (size_t)n * d, &db));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_IDS, (size_t)n * kout, &di));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_DISTS, (size_t)n * kout, &dd));
  MANN_CUDA_TRY(cudaMemcpyAsync(db, data, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  MANN_TRY(search_device(ctx, s, p, db, n, db, n, d, self, kreq, kout, di, dd, rep));
  MANN_CUDA_TRY(cudaMemcpyAsync(ids, di, sizeof(int32_t) * n * kout, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dists, dd, sizeof(float) * n * kout, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  return MANN_OK;
}

// Names the dataset handle of the current call to the tensor-core forms
// (which keep the handle's prepared points between calls) while it lives.
struct PointsOwnerScope {
  Context* ctx;
  PointsOwnerScope(Context* c, const void* owner, const float* base, uint64_t generation) : ctx(c) {
    ctx->points_owner = owner;
    ctx->points_base = base;
    ctx->points_generation = generation;
  }
  ~PointsOwnerScope() {
    ctx->points_owner = nullptr;
    ctx->points_base = nullptr;
  }
};

// the points of a dataset handle are device memory; queries and outputs are host
mann_status knn_dataset_impl(const mann_knn_params* p, const void* owner, uint64_t generation, const float* dbase,
                             int64_t n, const float* qs, int64_t q, int32_t d, int64_t graph_self, int kreq,
                             int32_t* ids, float* dists, mann_knn_report* rep) {
  const int kout = p->k;
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  PointsOwnerScope owner_scope(ctx, owner, dbase, generation);
  const int64_t rows = qs ? q : n;
  float *dq = nullptr, *dd = nullptr;
  int32_t* di = nullptr;
  if (qs) {
    MANN_TRY(ctx->scratch_t(SLOT_QUERIES, (size_t)q * d, &dq));
    MANN_CUDA_TRY(cudaMemcpyAsync(dq, qs, sizeof(float) * q * d, cudaMemcpyHostToDevice, s));
  }
  MANN_TRY(ctx->scratch_t(SLOT_OUT_IDS, (size_t)rows * kout, &di));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_DISTS, (size_t)rows * kout, &dd));
  MANN_TRY(search_device(ctx, s, p, dbase, n, qs ? dq : dbase, rows, d, graph_self, kreq, kout, di, dd, rep));
  MANN_CUDA_TRY(cudaMemcpyAsync(ids, di, sizeof(int32_t) * rows * kout, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dists, dd, sizeof(float) * rows * kout, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  return MANN_OK;
}

}  // namespace

mann_status exact_search_device(Context* ctx, cudaStream_t s, const mann_knn_params* p,
                                const float* base, int64_t n, const float* qs, int64_t nq, int d,
                                int64_t graph_self, int kreq, int kout, int32_t* ids, float* dists,
                                mann_knn_report* rep) {
  return search_device(ctx, s, p, base, n, qs, nq, d, graph_self, kreq, kout, ids, dists, rep);
}

}  // namespace mann

using namespace mann;

extern "C" {

const char* mann_version(void) { return "manifoldann-gb300 0.1.0 (sm_103a)"; }

const char* mann_last_error(void) { return last_error_cstr(); }

mann_status mann_device_count(int32_t* out_count) {
  clear_error();
  if (!out_count) return fail(MANN_EINVAL_ARG, "out_count must not be NULL");
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    *out_count = 0;
    return MANN_OK;
  }
  *out_count = c;
  return MANN_OK;
}

mann_status mann_host_register(void* ptr, int64_t bytes) {
  clear_error();
  if (!ptr || bytes <= 0) return fail(MANN_EINVAL_ARG, "bad buffer");
  MANN_CUDA_TRY(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault));
  return MANN_OK;
}

mann_status mann_host_unregister(void* ptr) {
  clear_error();
  if (!ptr) return fail(MANN_EINVAL_ARG, "bad buffer");
  MANN_CUDA_TRY(cudaHostUnregister(ptr));
  return MANN_OK;
}

}  // extern "C"

struct mann_dataset {
  float* dev = nullptr;
  int64_t n = 0, cap = 0;
  int32_t d = 0;
  int device = -1;
  uint64_t serial = 0;      // never reused, unlike the handle's address
  uint64_t generation = 0;  // bumped by every upload: prepared points of an older one are stale
};

namespace {
std::atomic<uint64_t> g_dataset_serial{0};
// the name of a handle's current upload in the prepared-points cache
uint64_t upload_name(const mann_dataset* ds) { return (ds->serial << 24) ^ ds->generation; }
}  // namespace

namespace {

mann_status dataset_device_check(const mann_dataset* ds) {
  int dev = -1;
  MANN_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != ds->device) return fail(MANN_EINVAL_ARG, "dataset belongs to another device");
  return MANN_OK;
}

mann_status dataset_copy_in(mann_dataset* ds, const float* data, int64_t n) {
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  if (n > ds->cap) {
    if (ds->dev) MANN_CUDA_TRY(cudaFree(ds->dev));
    ds->dev = nullptr;
    ds->cap = 0;
    if (cudaMalloc(&ds->dev, sizeof(float) * (size_t)n * ds->d) != cudaSuccess) {
      (void)cudaGetLastError();
      ds->dev = nullptr;
      return fail(MANN_ENOMEM, "dataset: device allocation failed");
    }
    ds->cap = n;
  }
  CallScope scope(ctx, ctx->stream);
  MANN_CUDA_TRY(cudaMemcpyAsync(ds->dev, data, sizeof(float) * (size_t)n * ds->d, cudaMemcpyHostToDevice,
                                ctx->stream));
  MANN_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  ds->n = n;
  ++ds->generation;
  return MANN_OK;
}

}  // namespace

extern "C" {

mann_status mann_dataset_create(const float* data, int64_t n, int32_t d, mann_dataset** out) {
  clear_error();
  if (!out) return fail(MANN_EINVAL_ARG, "out must not be NULL");
  *out = nullptr;
  if (n <= 0 || d <= 0) return fail(MANN_EINVAL_ARG, "a dataset needs n > 0 points of d > 0 values");
  if (!data) return fail(MANN_EINVAL_ARG, "NULL buffer");
  auto* ds = new (std::nothrow) mann_dataset();
  if (!ds) return fail(MANN_ENOMEM, "dataset: host allocation failed");
  ds->d = d;
  ds->serial = ++g_dataset_serial;
  if (cudaGetDevice(&ds->device) != cudaSuccess) {
    (void)cudaGetLastError();
    delete ds;
    return fail(MANN_ECUDA, "no CUDA device");
  }
  const mann_status st = dataset_copy_in(ds, data, n);
  if (st != MANN_OK) {
    if (ds->dev) (void)cudaFree(ds->dev);
    delete ds;
    return st;
  }
  *out = ds;
  return MANN_OK;
}

mann_status mann_dataset_upload(mann_dataset* ds, const float* data, int64_t n) {
  clear_error();
  if (!ds || !data) return fail(MANN_EINVAL_ARG, "NULL argument");
  if (n <= 0) return fail(MANN_EINVAL_ARG, "a dataset needs n > 0 points");
  MANN_TRY(dataset_device_check(ds));
  return dataset_copy_in(ds, data, n);
}

mann_status mann_dataset_destroy(mann_dataset* ds) {
  clear_error();
  if (!ds) return MANN_OK;
  if (ds->dev) {
    int prev = -1;
    (void)cudaGetDevice(&prev);
    if (prev != ds->device) (void)cudaSetDevice(ds->device);
    Context* ctx = nullptr;
    if (get_context(&ctx) == MANN_OK) {
      CallScope scope(ctx, ctx->stream);
      ctx->release_points(ds);  // the handle's prepared tensor-core operand
    } else {
      clear_error();
    }
    (void)cudaFree(ds->dev);
    if (prev >= 0 && prev != ds->device) (void)cudaSetDevice(prev);
  }
  delete ds;
  return MANN_OK;
}

mann_status mann_knn_dataset(const mann_knn_params* p, const mann_dataset* ds, const float* queries,
                             int64_t q, int32_t* out_ids, float* out_dists, mann_knn_report* report) {
  clear_error();
  if (!ds) return fail(MANN_EINVAL_ARG, "NULL dataset");
  MANN_TRY(check_common(p, ds->n, ds->d));
  if (q < 0) return fail(MANN_EINVAL_ARG, "negative query count");
  if (report) *report = mann_knn_report{};
  if (p->k <= 0 || q == 0) return MANN_OK;
  if (!queries || !out_ids || !out_dists) return fail(MANN_EINVAL_ARG, "NULL buffer");
  MANN_TRY(dataset_device_check(ds));
  const int kreq = (int)std::min<int64_t>(p->k, ds->n);
  return knn_dataset_impl(p, ds, upload_name(ds), ds->dev, ds->n, queries, q, ds->d, -1, kreq, out_ids, out_dists,
                          report);
}

mann_status mann_knn_graph_dataset(const mann_knn_params* p, const mann_dataset* ds, int32_t include_self,
                                   int32_t* out_ids, float* out_dists, mann_knn_report* report) {
  clear_error();
  if (!ds) return fail(MANN_EINVAL_ARG, "NULL dataset");
  MANN_TRY(check_common(p, ds->n, ds->d));
  if (report) *report = mann_knn_report{};
  const int64_t n = ds->n;
  const int64_t max_neighbors = n - (include_self ? 0 : 1);
  if (!(p->k > 0 && p->k <= max_neighbors))
    return fail(MANN_EINVAL_ARG, "k must satisfy 0 < k <= " + std::to_string(max_neighbors) +
                                     " for dataset with " + std::to_string(n) + " points");
  if (!out_ids || !out_dists) return fail(MANN_EINVAL_ARG, "NULL buffer");
  MANN_TRY(dataset_device_check(ds));
  const int kreq = p->k + (include_self ? 0 : 1);
  return knn_dataset_impl(p, ds, upload_name(ds), ds->dev, n, nullptr, n, ds->d, include_self ? -1 : 0, kreq,
                          out_ids, out_dists, report);
}

mann_status mann_knn(const mann_knn_params* p, const float* base, int64_t n, const float* queries,
                     int64_t q, int32_t d, int32_t* out_ids, float* out_dists,
                     mann_knn_report* report) {
  return knn_impl(p, base, n, queries, q, d, out_ids, out_dists, report, true, nullptr);
}

mann_status mann_knn_device(const mann_knn_params* p, const float* base, int64_t n,
                            const float* queries, int64_t q, int32_t d, int32_t* out_ids,
                            float* out_dists, mann_knn_report* report, void* stream) {
  return knn_impl(p, base, n, queries, q, d, out_ids, out_dists, report, false,
                  static_cast<cudaStream_t>(stream));
}

mann_status mann_knn_graph(const mann_knn_params* p, const float* data, int64_t n, int32_t d,
                           int32_t include_self, int32_t* out_ids, float* out_dists,
                           mann_knn_report* report) {
  return graph_impl(p, data, n, d, include_self, out_ids, out_dists, report, true, nullptr);
}

mann_status mann_knn_graph_device(const mann_knn_params* p, const float* data, int64_t n,
                                  int32_t d, int32_t include_self, int32_t* out_ids,
                                  float* out_dists, mann_knn_report* report, void* stream) {
  return graph_impl(p, data, n, d, include_self, out_ids, out_dists, report, false,
                    static_cast<cudaStream_t>(stream));
}

}  // extern "C"
