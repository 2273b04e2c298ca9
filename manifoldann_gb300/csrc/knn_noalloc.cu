// knn_noalloc.cu -- the exact FP32 kNN (the same kernels as mann_knn_device
// with MANN_PREC_FP32) for callers that cannot allocate device memory.
//
// Who needs it: a host that owns all device memory through its own pool and
// forbids other allocators (e.g. a Julia or Python runtime that reserved the
// GPU's memory for its arrays), code that runs where allocating would stall
// other work (cudaMalloc/cudaFree synchronise the whole device), and callers
// that must not fail with out-of-memory once started.  Such callers pass
// their inputs and outputs in device memory they already own; the scratch
// the search needs comes from one array of NOALLOC_WORDS uint64 words
// (16 MiB) that the library holds on every device it is loaded on until the
// process exits.
//
// Rules of use:
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture.  The address is kept for the life of the
//     process, so a cudaDeviceReset (which drops the device's module and
//     its arrays) needs a process restart before the next call;
//   * every call on a device shares the one array: calls whose work overlaps
//     on the GPU (different streams, or threads racing on one stream) corrupt
//     each other's results -- serialise them;
//   * a search whose scratch does not fit is rejected with MANN_EINVAL_ARG
//     (split the queries into smaller batches).  Nothing in the array has to
//     start at zero: every word a call reads was written earlier by the same
//     call.
#include <mutex>

#include "kernels.cuh"

namespace mann {
namespace {

constexpr size_t NOALLOC_WORDS = size_t(1) << 21;  // 2 Mi uint64 = 16 MiB

static __device__ __align__(256) uint64_t g_noalloc_scratch[NOALLOC_WORDS];

struct NoallocDevice {
  bool ready = false;
  uint64_t* scratch = nullptr;  // device address of g_noalloc_scratch on this device
  int num_sms = 0;
};

std::mutex g_noalloc_mu;
NoallocDevice g_noalloc_dev[64];

// Set-up of the current device, once: the array's device address and the SM count.
mann_status noalloc_device(NoallocDevice** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return fail(MANN_ENODEV, std::string("no CUDA device: ") + cudaGetErrorString(e));
  }
  if (dev < 0 || dev >= 64) return fail(MANN_ENODEV, "device ordinal out of range");
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  NoallocDevice& nd = g_noalloc_dev[dev];
  if (!nd.ready) {
    int major = 0;
    MANN_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    if (major != 10) return fail(MANN_ENODEV, "libmanngpu is built for sm_103a (GB300)");
    MANN_CUDA_TRY(cudaDeviceGetAttribute(&nd.num_sms, cudaDevAttrMultiProcessorCount, dev));
    void* p = nullptr;
    MANN_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    nd.scratch = static_cast<uint64_t*>(p);
    nd.ready = true;
  }
  *out = &nd;
  return MANN_OK;
}

}  // namespace
}  // namespace mann

using namespace mann;

extern "C" mann_status mann_knn_device_noalloc(const mann_knn_params* p, const float* base,
                                               int64_t n, const float* queries, int64_t q,
                                               int32_t d, int32_t* out_ids, float* out_dists,
                                               void* stream) {
  clear_error();
  if (!p) return fail(MANN_EINVAL_ARG, "params must not be NULL");
  if (d <= 0) return fail(MANN_EINVAL_ARG, "Dataset must have at least one dimension");
  if (n <= 0) return fail(MANN_EINVAL_ARG, "Dataset must contain at least one point");
  if (n > 0x7FFFFFFFll) return fail(MANN_EINVAL_ARG, "at most 2^31-1 points (int32 ids)");
  if (q < 0) return fail(MANN_EINVAL_ARG, "negative query count");
  if (p->metric != MANN_METRIC_EUCLIDEAN && p->metric != MANN_METRIC_SQEUCLIDEAN &&
      p->metric != MANN_METRIC_COSINE)
    return fail(MANN_EINVAL_ARG, "unknown metric code");
  if (p->precision != MANN_PREC_FP32 && p->precision != MANN_PREC_AUTO)
    return fail(MANN_EINVAL_ARG, "the allocation-free entry point runs the FP32 form only");
  if (p->flags & MANN_FLAG_FP64_TIES)
    return fail(MANN_EINVAL_ARG, "the allocation-free entry point does not order ties in FP64");
  if (p->k <= 0 || q == 0) return MANN_OK;
  if (!base || !queries || !out_ids || !out_dists) return fail(MANN_EINVAL_ARG, "NULL buffer");
  const int kout = p->k;
  const int kreq = (int)std::min<int64_t>(p->k, n);
  if (kreq > KMAX_FUSED)
    return fail(MANN_EINVAL_ARG, "k = " + std::to_string(kreq) + " exceeds the fused top-k limit " +
                                     std::to_string(KMAX_FUSED));
  NoallocDevice* nd = nullptr;
  MANN_TRY(noalloc_device(&nd));
  // scratch: [row norms (cosine only)] [per-split lists] [merged lists]
  const bool cosine = p->metric == MANN_METRIC_COSINE;
  const size_t norm_words = cosine ? (size_t)(n + q + 1) / 2 + 1 : 0;
  int nsplit = 1;
  size_t list_words = 0;
  knn_fp32_plan(nd->num_sms, n, q, kreq, &nsplit, &list_words);
  if (norm_words + list_words > NOALLOC_WORDS)
    return fail(MANN_EINVAL_ARG, "this search needs " + std::to_string(norm_words + list_words) +
                                     " words of scratch; the allocation-free entry point has " +
                                     std::to_string(NOALLOC_WORDS) +
                                     ": pass fewer queries per call");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const float* qn = nullptr;
  const float* bn = nullptr;
  if (cosine) {
    float* norms = reinterpret_cast<float*>(nd->scratch);
    MANN_TRY(launch_row_sqnorm(base, n, d, norms, s));
    MANN_TRY(launch_row_sqnorm(queries, q, d, norms + n, s));
    bn = norms;
    qn = norms + n;
  }
  uint64_t* keys = nullptr;
  MANN_TRY(knn_fp32_keys_on(nd->num_sms, s, base, n, queries, q, d, p->metric, kreq, qn, bn,
                            nd->scratch + norm_words, NOALLOC_WORDS - norm_words, &keys));
  MANN_TRY(launch_finish(keys, q, kreq, kout, -1, nullptr, out_ids, out_dists, s));
  return MANN_OK;
}
