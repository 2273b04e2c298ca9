// peaks.cu -- measured FP32 fused multiply-add rate of the current GPU, the
// denominator of the FP32-form rooflines (the plain tiled kernel, the
// batched segmented kernel, the IVF list scan's arithmetic).  No counterpart
// in the reference: it characterises the device the kernels run on.
//
// Every thread runs 16 independent FMA chains (eight fma.rn.f32x2 pairs, the
// instruction the FP32 kernels of this library use, or sixteen scalar
// fmaf) for `iters` steps; a grid of 8 blocks of 256 threads per SM keeps
// every FP32 lane busy.  Two flops per FMA.  The host times one launch of
// each form with CUDA events after a warm-up launch and reports the faster.
#include "f32x2.cuh"
#include "kernels.cuh"

namespace mann {
namespace {

constexpr int PEAK_THREADS = 256;
constexpr int PEAK_BLOCKS_PER_SM = 8;
constexpr int PEAK_CHAINS = 16;

__global__ void __launch_bounds__(PEAK_THREADS) fma_rate_pairs(float* out, int iters, float a, float b) {
  uint64_t x[PEAK_CHAINS / 2];
  const float t = (float)threadIdx.x * 1e-7f;
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS / 2; ++c) x[c] = f2::pack(t + (float)c, t - (float)c);
  const uint64_t av = f2::pack(a, a), bv = f2::pack(b, b);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS / 2; ++c) x[c] = f2::fma(x[c], av, bv);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS / 2; ++c) {
    float lo, hi;
    f2::unpack(x[c], lo, hi);
    s += lo + hi;
  }
  if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

__global__ void __launch_bounds__(PEAK_THREADS) fma_rate_scalar(float* out, int iters, float a, float b) {
  float x[PEAK_CHAINS];
  const float t = (float)threadIdx.x * 1e-7f;
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS; ++c) x[c] = t + (float)c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; ++c) x[c] = __fmaf_rn(x[c], a, b);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS; ++c) s += x[c];
  if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace mann

using namespace mann;

extern "C" mann_status mann_measure_fp32_peak(double* out_tflops, double* out_ms) {
  clear_error();
  if (!out_tflops) return fail(MANN_EINVAL_ARG, "out_tflops must not be NULL");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  CallScope scope(ctx, ctx->stream);
  cudaStream_t s = ctx->stream;
  float* sink = nullptr;
  const int grid = ctx->num_sms * PEAK_BLOCKS_PER_SM;
  MANN_TRY(ctx->scratch_t(SLOT_MISC2, (size_t)grid * PEAK_THREADS, &sink));
  const int iters = 1 << 14;
  const double flops = 2.0 * PEAK_CHAINS * (double)iters * (double)grid * PEAK_THREADS;
  cudaEvent_t e0, e1;
  MANN_CUDA_TRY(cudaEventCreate(&e0));
  MANN_CUDA_TRY(cudaEventCreate(&e1));
  double best_ms = 1e30;
  for (int form = 0; form < 2; ++form) {
    for (int rep = 0; rep < 3; ++rep) {  // rep 0 is the warm-up
      cudaEventRecord(e0, s);
      if (form == 0)
        fma_rate_pairs<<<grid, PEAK_THREADS, 0, s>>>(sink, iters, 0.9999999f, 1e-7f);
      else
        fma_rate_scalar<<<grid, PEAK_THREADS, 0, s>>>(sink, iters, 0.9999999f, 1e-7f);
      cudaEventRecord(e1, s);
      cudaError_t le = cudaGetLastError();
      if (le != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return fail(MANN_ECUDA, std::string("fma rate kernel: ") + cudaGetErrorString(le));
      }
      note_launch();
      float ms = 0.0f;
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && ms > 0.0f) best_ms = std::min(best_ms, (double)ms);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *out_tflops = flops / (best_ms * 1e-3) / 1e12;
  if (out_ms) *out_ms = best_ms;
  return MANN_OK;
}
