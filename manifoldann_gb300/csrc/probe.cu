// probe.cu -- the learned coarse probe: a BF16 MLP din -> h1 -> h2 -> nlist
// (GELU after both hidden layers) that scores the inverted lists of an
// IVF-Flat index for a query, trained on the GPU by the kernels below.
//
// No counterpart in the reference: it is a new routing strategy beside
// TopKRouting (select_indices, src/indices/multilevel/routing.jl:91-118).
//
// score_c(q) = MLP(q)_c - beta * ||q - c||^2     (prior on; beta = exp(theta) learned)
// score_c(q) = MLP(q)_c                            (prior off)
// Training: softmax cross-entropy of the scores against the distribution of
// the lists that hold the query's exact nearest neighbours; AdamW.
//
// Kernels:
//  * probe_gemm<EPI>  C[M][N] = A[M][K] B[N][K]^T on tcgen05 (BF16 operands by
//    TMA with 128-byte swizzle, FP32 accumulators in TMEM), one 128 x 128
//    tile per CTA, with fused epilogues (bias + GELU writing the activation in
//    both layouts, logits, GELU-derivative product, plain FP32 gradients);
//  * softmax statistics / gradient (deterministic, no float atomics);
//  * bias gradients as fixed-order row sums; AdamW over the flat parameters;
//    BF16 weight copies in both layouts;
//  * top-nprobe selection of lists per query (radix select, ties -> lower id).
//
// Every wait on an mbarrier is bounded; a timeout sets the model's error word
// and the host reports MANN_ETIMEOUT after the call.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "ptx.cuh"

namespace mann {

mann_status pairwise_device(Context* ctx, cudaStream_t s, const float* X, int64_t n, const float* C,
                            int k, int d, int metric, float* D);
mann_status ivf_scan_device(Context* ctx, cudaStream_t s, const float* data, int64_t n, int d,
                            int metric, const int64_t* loff, const int32_t* lids, int nlist,
                            const float* qs, int64_t nq, const int32_t* probes, int nprobe, int k,
                            int32_t* out_ids, float* out_dists);

namespace {

typedef __nv_bfloat16 bf16;

constexpr int GM = 128, GN = 128, GK = 64;
constexpr int GSTAGES = 4;
constexpr int G_A_BYTES = GM * GK * 2;
constexpr int G_STAGE = G_A_BYTES + GN * GK * 2;
constexpr int G_THREADS = 192;
constexpr size_t G_SMEM = 1024 + (size_t)GSTAGES * G_STAGE + (2 * GSTAGES + 2) * 8 + 16;

enum { EPI_F32 = 0, EPI_BIAS_GELU = 1, EPI_LOGITS = 2, EPI_DGELU = 3 };
enum { PERR_TIMEOUT = 1 };

struct GemmArgs {
  int M, N, K;
  const float* bias;  // [N]
  float* outf;        // [M][N]: gradient / logits / pre-activation (nullable for GELU)
  bf16* outh;         // [M][N]
  bf16* outt;         // [N][M] (nullable)
  const float* zin;   // [M][N] pre-activation (DGELU)
  int* err;
};

__device__ __forceinline__ float gelu_f(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

template <int EPI>
__global__ void __launch_bounds__(G_THREADS, 1)
    probe_gemm(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
               GemmArgs g) {
  extern __shared__ __align__(1024) uint8_t g_smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(g_smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + GSTAGES * G_STAGE);
  uint64_t* full_bar = bars;
  uint64_t* empty_bar = bars + GSTAGES;
  uint64_t* done_bar = bars + 2 * GSTAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * GSTAGES + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * GM, n0 = blockIdx.x * GN;
  const int nkb = g.K / GK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < GSTAGES; ++s) {
      ptx::mbar_init(&full_bar[s], 1);
      ptx::mbar_init(&empty_bar[s], 1);
    }
    ptx::mbar_init(done_bar, 1);
    ptx::fence_mbar_init();
    ptx::prefetch_tensormap(&mapA);
    ptx::prefetch_tensormap(&mapB);
  }
  if (warp == 1) {
    ptx::tmem_alloc(tmem_slot, GN);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % GSTAGES;
        const uint32_t ph = (kb / GSTAGES) & 1;
        if (!ptx::mbar_wait(&empty_bar[s], ph ^ 1, g.err, PERR_TIMEOUT)) break;
        uint8_t* sa = smem + s * G_STAGE;
        ptx::mbar_arrive_expect_tx(&full_bar[s], G_STAGE);
        ptx::tma_load_2d(sa, &mapA, &full_bar[s], kb * GK, m0);
        ptx::tma_load_2d(sa + G_A_BYTES, &mapB, &full_bar[s], kb * GK, n0);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = ptx::idesc_bf16_f32(GM, GN);
      bool ok = true;
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % GSTAGES;
        const uint32_t ph = (kb / GSTAGES) & 1;
        if (!ptx::mbar_wait(&full_bar[s], ph, g.err, PERR_TIMEOUT)) {
          ok = false;
          break;
        }
        ptx::tc_fence_after();
        const uint32_t sa = ptx::smem_u32(smem + s * G_STAGE);
        const uint32_t sb = sa + G_A_BYTES;
#pragma unroll
        for (int kk = 0; kk < GK / 16; ++kk)
          ptx::mma_f16(tmem_base, ptx::sw128_desc(sa + kk * 32), ptx::sw128_desc(sb + kk * 32), idesc,
                       (kb > 0 || kk > 0) ? 1u : 0u);
        ptx::mma_commit(&empty_bar[s]);
      }
      if (ok) ptx::mma_commit(done_bar);
    }
  } else {
    const int quad = warp & 3;
    const int row = quad * 32 + lane;
    const int gm = m0 + row;
    if (ptx::mbar_wait(done_bar, 0, g.err, PERR_TIMEOUT)) {
      ptx::tc_fence_after();
      const uint32_t taddr = tmem_base + ((uint32_t)(quad * 32) << 16);
#pragma unroll 1
      for (int ch = 0; ch < GN / 16; ++ch) {
        uint32_t r[16];
        ptx::tmem_ld16(taddr + ch * 16, r);
        ptx::tmem_ld_wait();
        const int gc = n0 + ch * 16;
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
        const size_t o = (size_t)gm * g.N + gc;
        if (EPI == EPI_F32 || EPI == EPI_LOGITS) {
          if (EPI == EPI_LOGITS)
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] += __ldg(&g.bias[gc + j]);
          float4* dst = reinterpret_cast<float4*>(g.outf + o);
#pragma unroll
          for (int j = 0; j < 4; ++j) dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        } else {
          if (EPI == EPI_BIAS_GELU) {
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] += __ldg(&g.bias[gc + j]);
            if (g.outf) {
              float4* dst = reinterpret_cast<float4*>(g.outf + o);
#pragma unroll
              for (int j = 0; j < 4; ++j)
                dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = gelu_f(v[j]);
          } else {  // EPI_DGELU
            const float4* zp = reinterpret_cast<const float4*>(g.zin + o);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const float4 z = __ldg(&zp[j]);
              v[4 * j] *= gelu_grad(z.x);
              v[4 * j + 1] *= gelu_grad(z.y);
              v[4 * j + 2] *= gelu_grad(z.z);
              v[4 * j + 3] *= gelu_grad(z.w);
            }
          }
          __align__(16) bf16 h[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) h[j] = __float2bfloat16_rn(v[j]);
          uint4* dst = reinterpret_cast<uint4*>(g.outh + o);
          dst[0] = reinterpret_cast<const uint4*>(h)[0];
          dst[1] = reinterpret_cast<const uint4*>(h)[1];
          if (g.outt)
#pragma unroll
            for (int j = 0; j < 16; ++j) g.outt[(size_t)(gc + j) * g.M + gm] = h[j];
        }
      }
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem_base, GN);
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult qr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &qr) ==
            cudaSuccess &&
        qr == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// K-major BF16 matrix [rows][cols], boxes of 64 columns x 128 rows
mann_status map_kmajor(CUtensorMap* m, const bf16* ptr, int64_t rows, int64_t cols) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return fail(MANN_ECUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {(cuuint32_t)GK, 128u};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(ptr), dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(MANN_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return MANN_OK;
}

template <int EPI>
mann_status launch_gemm_t(cudaStream_t s, const bf16* A, const bf16* B, const GemmArgs& g) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(probe_gemm<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G_SMEM);
  });
  MANN_CUDA_TRY(attr);
  CUtensorMap ma, mb;
  MANN_TRY(map_kmajor(&ma, A, g.M, g.K));
  MANN_TRY(map_kmajor(&mb, B, g.N, g.K));
  dim3 grid((unsigned)(g.N / GN), (unsigned)(g.M / GM));
  probe_gemm<EPI><<<grid, G_THREADS, G_SMEM, s>>>(ma, mb, g);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

// C[M][N] = A[M][K] B[N][K]^T with the given epilogue; M, N multiples of 128, K of 64.
mann_status gemm(cudaStream_t s, int epi, const bf16* A, const bf16* B, int M, int N, int K,
                 const float* bias, float* outf, bf16* outh, bf16* outt, const float* zin, int* err) {
  if (M % GM || N % GN || K % GK || K <= 0)
    return fail(MANN_EINVAL_ARG, "probe GEMM shape must be multiples of 128 x 128 x 64");
  GemmArgs g{M, N, K, bias, outf, outh, outt, zin, err};
  switch (epi) {
    case EPI_F32: return launch_gemm_t<EPI_F32>(s, A, B, g);
    case EPI_BIAS_GELU: return launch_gemm_t<EPI_BIAS_GELU>(s, A, B, g);
    case EPI_LOGITS: return launch_gemm_t<EPI_LOGITS>(s, A, B, g);
    default: return launch_gemm_t<EPI_DGELU>(s, A, B, g);
  }
}

// ------------------------------------------------------------ batch staging
// X bf16 [Bp][dinp] and X^T [dinp][Bp]; Xf f32 [Bp][din]; labels [Bp][L].
// Rows past nb (and columns past din) are zero; their labels are -1.
__global__ void stage_batch_kernel(const float* __restrict__ q, int din, const int32_t* __restrict__ idx,
                                   int nb, int Bp, int dinp, const int32_t* __restrict__ labels, int L,
                                   bf16* __restrict__ X, bf16* __restrict__ Xt, float* __restrict__ Xf,
                                   int32_t* __restrict__ lb) {
  __shared__ float tile[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int i = ty; i < 32; i += 8) {
    const int r = r0 + i, c = c0 + tx;
    float v = 0.0f;
    if (r < nb && c < din) {
      const int64_t src = idx ? (int64_t)idx[r] : (int64_t)r;
      v = q[src * din + c];
    }
    tile[i][tx] = v;
    X[(size_t)r * dinp + c] = __float2bfloat16_rn(v);
    if (Xf && c < din) Xf[(size_t)r * din + c] = v;
  }
  __syncthreads();
  if (Xt)
    for (int i = ty; i < 32; i += 8) Xt[(size_t)(c0 + i) * Bp + r0 + tx] = __float2bfloat16_rn(tile[tx][i]);
  if (lb && blockIdx.x == 0)
    for (int i = ty; i < 32; i += 8) {
      const int r = r0 + i;
      for (int l = tx; l < L; l += 32) {
        int32_t v = -1;
        if (r < nb) v = labels[(idx ? (int64_t)idx[r] : (int64_t)r) * L + l];
        lb[(size_t)r * L + l] = v;
      }
    }
}

// ------------------------------------------------------------ softmax loss
struct SoftmaxArgs {
  const float* logits;  // [Bp][noutp]
  const float* D;       // [Bp][nout] squared distances to the centroids (prior) or null
  const float* theta;   // log beta (device scalar)
  const int32_t* lb;    // [Bp][L]
  int L, nb, nout, noutp, Bp;
  float* lse;           // [Bp]
  float* loss_row;      // [Bp]
  bf16* dL;             // [Bp][noutp]
  bf16* dLt;            // [noutp][Bp]
  float* theta_part;    // [gridDim] partial d loss / d theta
};

__device__ __forceinline__ float score_at(const SoftmaxArgs& a, int r, int c, float beta) {
  float v = a.logits[(size_t)r * a.noutp + c];
  if (a.D) v -= beta * a.D[(size_t)r * a.nout + c];
  return v;
}

// one warp per row: log-sum-exp of the scores and the row's loss
__global__ void softmax_stats_kernel(SoftmaxArgs a) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= a.Bp) return;
  const float beta = a.D ? expf(*a.theta) : 0.0f;
  float mx = -INFINITY;
  for (int c = lane; c < a.nout; c += 32) mx = fmaxf(mx, score_at(a, r, c, beta));
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  float sm = 0.0f;
  for (int c = lane; c < a.nout; c += 32) sm += expf(score_at(a, r, c, beta) - mx);
  for (int o = 16; o; o >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, o);
  const float lse = mx + logf(sm);
  if (lane == 0) {
    a.lse[r] = lse;
    float loss = 0.0f;
    if (r < a.nb) {
      int nv = 0;
      float acc = 0.0f;
      for (int l = 0; l < a.L; ++l) {
        const int c = a.lb[(size_t)r * a.L + l];
        if (c >= 0 && c < a.nout) {
          acc += score_at(a, r, c, beta);
          ++nv;
        }
      }
      loss = nv ? lse - acc / nv : 0.0f;
    }
    a.loss_row[r] = loss;
  }
}

// 32 x 32 tiles: dL = (softmax - y) / nb in both layouts, and the tile's
// share of d loss / d theta (theta = log beta).
__global__ void softmax_grad_kernel(SoftmaxArgs a) {
  __shared__ bf16 tile[32][34];
  __shared__ float red[8];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const float beta = a.D ? expf(*a.theta) : 0.0f;
  const float inv_nb = 1.0f / (float)max(a.nb, 1);
  float th = 0.0f;
  for (int i = ty; i < 32; i += 8) {
    const int r = r0 + i, c = c0 + tx;
    float gv = 0.0f;
    if (r < a.nb && c < a.nout) {
      int nv = 0, hit = 0;
      for (int l = 0; l < a.L; ++l) {
        const int lc = a.lb[(size_t)r * a.L + l];
        if (lc >= 0 && lc < a.nout) {
          ++nv;
          hit += lc == c;
        }
      }
      const float sc = score_at(a, r, c, beta);
      const float p = expf(sc - a.lse[r]);
      const float y = nv ? (float)hit / nv : 0.0f;
      gv = nv ? (p - y) * inv_nb : 0.0f;
      if (a.D) th += gv * (-beta * a.D[(size_t)r * a.nout + c]);
    }
    const bf16 h = __float2bfloat16_rn(gv);
    a.dL[(size_t)r * a.noutp + c] = h;
    tile[i][tx] = h;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) a.dLt[(size_t)(c0 + i) * a.Bp + r0 + tx] = tile[tx][i];
  if (a.theta_part) {
    for (int o = 16; o; o >>= 1) th += __shfl_xor_sync(0xffffffffu, th, o);
    if (tx == 0) red[ty] = th;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.0f;
      for (int i = 0; i < 8; ++i) t += red[i];
      a.theta_part[blockIdx.y * gridDim.x + blockIdx.x] = t;
    }
  }
}

// Row sums (fixed order) of up to three transposed BF16 matrices into the
// bias gradients; the block past them reduces theta's partials and the loss.
struct BiasGradArgs {
  const bf16* src[3];
  float* dst[3];
  int rows[3];
  int Bp;
  const float* theta_part;
  int ntheta;
  float* dtheta;
  const float* loss_row;
  int nb;
  float* loss_acc;  // += mean loss of the batch (nullable)
};

__global__ void bias_grad_kernel(BiasGradArgs a) {
  const int lane = threadIdx.x & 31;
  int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int total = a.rows[0] + a.rows[1] + a.rows[2];
  if (r < total) {
    int m = 0;
    while (r >= a.rows[m]) r -= a.rows[m++];
    const bf16* p = a.src[m] + (size_t)r * a.Bp;
    float s = 0.0f;
    for (int i = lane; i < a.Bp; i += 32) s += __bfloat162float(p[i]);
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) a.dst[m][r] = s;
  } else if (r == total && lane == 0) {
    if (a.dtheta) {
      float t = 0.0f;
      for (int i = 0; i < a.ntheta; ++i) t += a.theta_part[i];
      *a.dtheta = t;
    }
    if (a.loss_acc) {
      float l = 0.0f;
      for (int i = 0; i < a.nb; ++i) l += a.loss_row[i];
      *a.loss_acc += l / (float)max(a.nb, 1);
    }
  }
}

// ------------------------------------------------------------ AdamW
struct AdamArgs {
  float* w;
  const float* g;
  float* m;
  float* v;
  int64_t n;
  float lr, b1, b2, eps, wd, bc1, bc2;
  int64_t decay_end[3];    // [decay_begin[i], decay_end[i]) take weight decay
  int64_t decay_begin[3];
};

__global__ void adamw_kernel(AdamArgs a) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
    const float g = a.g[i];
    const float m = a.b1 * a.m[i] + (1.0f - a.b1) * g;
    const float v = a.b2 * a.v[i] + (1.0f - a.b2) * g * g;
    a.m[i] = m;
    a.v[i] = v;
    float w = a.w[i];
    bool dec = false;
#pragma unroll
    for (int j = 0; j < 3; ++j) dec |= (i >= a.decay_begin[j] && i < a.decay_end[j]);
    if (dec) w -= a.lr * a.wd * w;
    w -= a.lr * (m / a.bc1) / (sqrtf(v / a.bc2) + a.eps);
    a.w[i] = w;
  }
}

// BF16 copies W [rows][cols] and W^T [cols][rows] of an FP32 matrix
__global__ void weights_bf16_kernel(const float* __restrict__ w, int rows, int cols, bf16* __restrict__ wb,
                                    bf16* __restrict__ wt) {
  __shared__ bf16 tile[32][34];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int i = ty; i < 32; i += 8) {
    const bf16 h = __float2bfloat16_rn(w[(size_t)(r0 + i) * cols + c0 + tx]);
    wb[(size_t)(r0 + i) * cols + c0 + tx] = h;
    tile[i][tx] = h;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) wt[(size_t)(c0 + i) * rows + r0 + tx] = tile[tx][i];
}

// ------------------------------------------------------------ top-nprobe
// Order key of a score: ascending key = descending score (NaN last).
__device__ __forceinline__ uint32_t score_key(float s) {
  const uint32_t b = __float_as_uint(-s);
  if ((b & 0x7F800000u) == 0x7F800000u && (b & 0x7FFFFFu)) return 0xFFFFFFFFu;
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

constexpr int ROUTE_THREADS = 256;
constexpr int ROUTE_MAXCOLS = 16384;

// Block per query: the nprobe best lists by (score desc, id asc), and the
// softmax mass they hold (coverage).
__global__ void __launch_bounds__(ROUTE_THREADS)
    route_topk_kernel(const float* __restrict__ logits, int noutp, const float* __restrict__ D,
                      const float* __restrict__ theta, int nout, int64_t nq, int nprobe,
                      int32_t* __restrict__ probes, float* __restrict__ coverage) {
  extern __shared__ uint32_t rk[];  // [nout] keys
  __shared__ uint32_t hist[256];
  __shared__ uint32_t sel_key[128];
  __shared__ int32_t sel_id[128];
  __shared__ uint32_t s_prefix, s_need;
  __shared__ float red[ROUTE_THREADS / 32];
  __shared__ int cnt_lt[ROUTE_THREADS], cnt_eq[ROUTE_THREADS];
  const int64_t q = blockIdx.x;
  if (q >= nq) return;
  const int t = threadIdx.x;
  const float beta = D ? expf(*theta) : 0.0f;
  float mx = -INFINITY;
  for (int c = t; c < nout; c += ROUTE_THREADS) {
    float sc = logits[q * noutp + c];
    if (D) sc -= beta * D[q * nout + c];
    rk[c] = score_key(sc);
    mx = fmaxf(mx, sc);
  }
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((t & 31) == 0) red[t >> 5] = mx;
  __syncthreads();
  mx = red[0];
  for (int i = 1; i < ROUTE_THREADS / 32; ++i) mx = fmaxf(mx, red[i]);
  __syncthreads();
  float sm = 0.0f;
  for (int c = t; c < nout; c += ROUTE_THREADS) {
    float sc = logits[q * noutp + c];
    if (D) sc -= beta * D[q * nout + c];
    sm += expf(sc - mx);
  }
  for (int o = 16; o; o >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, o);
  if ((t & 31) == 0) red[t >> 5] = sm;
  // radix select of the nprobe-th smallest key
  if (t == 0) {
    s_prefix = 0;
    s_need = (uint32_t)nprobe;
  }
  __syncthreads();
  float total = 0.0f;
  for (int i = 0; i < ROUTE_THREADS / 32; ++i) total += red[i];
  uint32_t mask = 0;
  for (int shift = 24; shift >= 0; shift -= 8) {
    hist[t] = 0;
    __syncthreads();
    const uint32_t prefix = s_prefix;
    for (int c = t; c < nout; c += ROUTE_THREADS) {
      const uint32_t k = rk[c];
      if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 255u], 1u);
    }
    __syncthreads();
    if (t == 0) {
      uint32_t need = s_need, cum = 0;
      int b = 0;
      for (; b < 255; ++b) {
        if (cum + hist[b] >= need) break;
        cum += hist[b];
      }
      s_need = need - cum;
      s_prefix = prefix | ((uint32_t)b << shift);
    }
    mask |= 255u << shift;
    __syncthreads();
  }
  const uint32_t kth = s_prefix;
  const uint32_t need_eq = s_need;             // how many keys equal to kth are taken
  const int per = (nout + ROUTE_THREADS - 1) / ROUTE_THREADS;
  const int cb = min(nout, t * per), ce = min(nout, cb + per);
  int lt = 0, eq = 0;
  for (int c = cb; c < ce; ++c) {
    lt += rk[c] < kth;
    eq += rk[c] == kth;
  }
  cnt_lt[t] = lt;
  cnt_eq[t] = eq;
  __syncthreads();
  if (t == 0) {  // exclusive scans in index order
    int a = 0, b = 0;
    for (int i = 0; i < ROUTE_THREADS; ++i) {
      const int x = cnt_lt[i], y = cnt_eq[i];
      cnt_lt[i] = a;
      cnt_eq[i] = b;
      a += x;
      b += y;
    }
  }
  __syncthreads();
  const int n_lt = nprobe - (int)need_eq;
  int pl = cnt_lt[t], pe = cnt_eq[t];
  for (int c = cb; c < ce; ++c) {
    const uint32_t k = rk[c];
    if (k < kth) {
      sel_key[pl] = k;
      sel_id[pl] = c;
      ++pl;
    } else if (k == kth) {
      if (pe < (int)need_eq) {
        sel_key[n_lt + pe] = k;
        sel_id[n_lt + pe] = c;
      }
      ++pe;
    }
  }
  __syncthreads();
  // rank the selected entries by (key, id)
  float covp = 0.0f;
  if (t < nprobe) {
    const uint32_t k = sel_key[t];
    const int id = sel_id[t];
    int rank = 0;
    for (int j = 0; j < nprobe; ++j) {
      const uint32_t kj = sel_key[j];
      rank += (kj < k) || (kj == k && sel_id[j] < id);
    }
    probes[q * nprobe + rank] = id;
    float sc = logits[q * noutp + id];
    if (D) sc -= beta * D[q * nout + id];
    covp = expf(sc - mx) / total;
  }
  if (coverage) {
    __syncthreads();
    for (int o = 16; o; o >>= 1) covp += __shfl_xor_sync(0xffffffffu, covp, o);
    if ((t & 31) == 0) red[t >> 5] = covp;
    __syncthreads();
    if (t == 0) {
      float c = 0.0f;
      for (int i = 0; i < ROUTE_THREADS / 32; ++i) c += red[i];
      coverage[q] = c;
    }
  }
}

// Warp per query for small nprobe: every lane keeps the NP best keys of its
// columns (key = score order << 32 | list id) and, when coverage is asked for
// (COV), an online softmax sum; the warp then pops the nprobe smallest heads.
// Without the distance prior the logits are read as float4, four per lane in
// flight (a lane's columns are 4g .. 4g+3 for its groups g).
template <int NP, bool COV>
__global__ void route_topk_warp_kernel(const float* __restrict__ logits, int noutp, const float* __restrict__ D,
                                       const float* __restrict__ theta, int nout, int64_t nq, int nprobe,
                                       int32_t* __restrict__ probes, float* __restrict__ coverage) {
  const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= nq) return;
  const float beta = D ? expf(*theta) : 0.0f;
  uint64_t lst[NP];
#pragma unroll
  for (int i = 0; i < NP; ++i) lst[i] = KEY_NONE;
  float mx = -INFINITY, sm = 0.0f;
  const float* lrow = logits + q * noutp;
  const float* drow = D ? D + q * nout : nullptr;
  // wthr: the NP-th smallest of the lanes' best keys -- NP distinct columns
  // are at or below it, so no larger key can be among the warp's NP best
  uint64_t wthr = KEY_NONE;
  auto consider = [&](float sc, int c) {
    if (COV) {
      if (sc > mx) {
        sm = (mx == -INFINITY ? 0.0f : sm * expf(mx - sc)) + 1.0f;
        mx = sc;
      } else if (sc > -INFINITY) {
        sm += expf(sc - mx);
      }
    }
    const uint64_t key = ((uint64_t)score_key(sc) << 32) | (uint32_t)c;
    if (key < lst[NP - 1] && key < wthr) {
      lst[NP - 1] = key;
#pragma unroll
      for (int i = NP - 1; i > 0; --i)
        if (lst[i] < lst[i - 1]) {
          const uint64_t x = lst[i];
          lst[i] = lst[i - 1];
          lst[i - 1] = x;
        }
    }
  };
  if (!D) {
    const float4* l4 = reinterpret_cast<const float4*>(lrow);  // noutp % 4 == 0, rows 16-byte aligned
    const int n4 = (nout + 3) >> 2;
    constexpr int U = 4;
    // every lane runs the same number of passes (the bitonic exchange below
    // uses full-mask shuffles); lanes past the end only skip their loads
    for (int b = 0; b < n4; b += 32 * U) {
      const int g0 = b + lane;
      float4 v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int g = g0 + 32 * u;
        v[u] = g < n4 ? __ldg(l4 + g) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int g = g0 + 32 * u;
        if (g < n4) {
          const int c = 4 * g;
          consider(v[u].x, c);
          if (c + 1 < nout) consider(v[u].y, c + 1);
          if (c + 2 < nout) consider(v[u].z, c + 2);
          if (c + 3 < nout) consider(v[u].w, c + 3);
        }
      }
      // tighten the warp bound: sort the lanes' best keys across the warp
      uint64_t h = lst[0];
#pragma unroll
      for (int kk = 2; kk <= 32; kk <<= 1) {
#pragma unroll
        for (int j = kk >> 1; j > 0; j >>= 1) {
          const uint64_t o = __shfl_xor_sync(0xffffffffu, (unsigned long long)h, j);
          const bool keep_min = ((lane & j) == 0) == ((lane & kk) == 0);
          h = keep_min ? (o < h ? o : h) : (o > h ? o : h);
        }
      }
      wthr = __shfl_sync(0xffffffffu, (unsigned long long)h, NP - 1);
    }
  } else {
    for (int c = lane; c < nout; c += 32) consider(lrow[c] - beta * drow[c], c);
  }
  float gmx = 0.0f, gs = 1.0f;
  if (COV) {
    gmx = mx;
    for (int o = 16; o; o >>= 1) gmx = fmaxf(gmx, __shfl_xor_sync(0xffffffffu, gmx, o));
    gs = (mx == -INFINITY) ? 0.0f : sm * expf(mx - gmx);
    for (int o = 16; o; o >>= 1) gs += __shfl_xor_sync(0xffffffffu, gs, o);
  }
  float cov = 0.0f;
  for (int r = 0; r < nprobe; ++r) {
    uint64_t m = lst[0];
    for (int o = 16; o; o >>= 1) {
      const uint64_t x = __shfl_xor_sync(0xffffffffu, m, o);
      m = x < m ? x : m;
    }
    if (lst[0] == m) {  // keys are unique: exactly one lane pops
#pragma unroll
      for (int i = 0; i < NP - 1; ++i) lst[i] = lst[i + 1];
      lst[NP - 1] = KEY_NONE;
    }
    if (lane == 0) {
      const int id = (int)(uint32_t)(m & 0xFFFFFFFFu);
      probes[q * nprobe + r] = id;
      if (COV) {
        float sc = lrow[id];
        if (D) sc -= beta * drow[id];
        cov += expf(sc - gmx);
      }
    }
  }
  if (COV && lane == 0) coverage[q] = cov / gs;
}

// ------------------------------------------------------------ host model
struct Splitmix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

struct Layout {  // flat FP32 parameter vector, padded dimensions
  int din, h1, h2, nout;
  int dinp, h1p, h2p, noutp;
  int64_t w1, b1, w2, b2, w3, b3, theta, total;
  void set(int din_, int h1_, int h2_, int nout_, bool padded) {
    din = din_;
    h1 = h1_;
    h2 = h2_;
    nout = nout_;
    dinp = padded ? round_up(din, 128) : din;
    h1p = padded ? round_up(h1, 128) : h1;
    h2p = padded ? round_up(h2, 128) : h2;
    noutp = padded ? round_up(nout, 128) : nout;
    w1 = 0;
    b1 = w1 + (int64_t)h1p * dinp;
    w2 = b1 + h1p;
    b2 = w2 + (int64_t)h2p * h1p;
    w3 = b2 + h2p;
    b3 = w3 + (int64_t)noutp * h2p;
    theta = b3 + noutp;
    total = theta + (padded ? 4 : 1);
  }
};

}  // namespace

struct ProbeModel {
  mann_probe_params p{};
  Layout user{}, pad{};
  int device = 0;
  float* master = nullptr;  // padded flat parameters (device)
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  float* grad = nullptr;
  bf16 *w1 = nullptr, *w1t = nullptr, *w2 = nullptr, *w2t = nullptr, *w3 = nullptr, *w3t = nullptr;
  float* cent = nullptr;  // [nout][din] centroids (prior)
  int* err = nullptr;
  int64_t step = 0;
  std::mutex mu;
};

namespace {

// user layout <-> padded device layout
void pad_params(const Layout& u, const Layout& p, const float* src, std::vector<float>& dst) {
  dst.assign((size_t)p.total, 0.0f);
  for (int o = 0; o < u.h1; ++o)
    std::memcpy(&dst[p.w1 + (int64_t)o * p.dinp], src + u.w1 + (int64_t)o * u.din, sizeof(float) * u.din);
  std::memcpy(&dst[p.b1], src + u.b1, sizeof(float) * u.h1);
  for (int o = 0; o < u.h2; ++o)
    std::memcpy(&dst[p.w2 + (int64_t)o * p.h1p], src + u.w2 + (int64_t)o * u.h1, sizeof(float) * u.h1);
  std::memcpy(&dst[p.b2], src + u.b2, sizeof(float) * u.h2);
  for (int o = 0; o < u.nout; ++o)
    std::memcpy(&dst[p.w3 + (int64_t)o * p.h2p], src + u.w3 + (int64_t)o * u.h2, sizeof(float) * u.h2);
  std::memcpy(&dst[p.b3], src + u.b3, sizeof(float) * u.nout);
  dst[p.theta] = src[u.theta];
}

void unpad_params(const Layout& u, const Layout& p, const float* src, float* dst) {
  for (int o = 0; o < u.h1; ++o)
    std::memcpy(dst + u.w1 + (int64_t)o * u.din, src + p.w1 + (int64_t)o * p.dinp, sizeof(float) * u.din);
  std::memcpy(dst + u.b1, src + p.b1, sizeof(float) * u.h1);
  for (int o = 0; o < u.h2; ++o)
    std::memcpy(dst + u.w2 + (int64_t)o * u.h1, src + p.w2 + (int64_t)o * p.h1p, sizeof(float) * u.h1);
  std::memcpy(dst + u.b2, src + p.b2, sizeof(float) * u.h2);
  for (int o = 0; o < u.nout; ++o)
    std::memcpy(dst + u.w3 + (int64_t)o * u.h2, src + p.w3 + (int64_t)o * p.h2p, sizeof(float) * u.h2);
  std::memcpy(dst + u.b3, src + p.b3, sizeof(float) * u.nout);
  dst[u.theta] = src[p.theta];
}

mann_status check_params(const mann_probe_params* p) {
  if (!p) return fail(MANN_EINVAL_ARG, "params must not be NULL");
  if (p->din <= 0 || p->hidden1 <= 0 || p->hidden2 <= 0 || p->nout <= 0)
    return fail(MANN_EINVAL_ARG, "probe layer widths must be positive");
  if (p->nout > ROUTE_MAXCOLS) return fail(MANN_EINVAL_ARG, "probe supports at most 16384 lists");
  if (p->din > 4096 || p->hidden1 > 8192 || p->hidden2 > 8192)
    return fail(MANN_EINVAL_ARG, "probe layer widths too large");
  return MANN_OK;
}

mann_status refresh_bf16(ProbeModel* m, cudaStream_t s) {
  const Layout& L = m->pad;
  const float* w = m->master;
  weights_bf16_kernel<<<dim3(L.dinp / 32, L.h1p / 32), 256, 0, s>>>(w + L.w1, L.h1p, L.dinp, m->w1, m->w1t);
  MANN_CHECK_LAUNCH();
  weights_bf16_kernel<<<dim3(L.h1p / 32, L.h2p / 32), 256, 0, s>>>(w + L.w2, L.h2p, L.h1p, m->w2, m->w2t);
  MANN_CHECK_LAUNCH();
  weights_bf16_kernel<<<dim3(L.h2p / 32, L.noutp / 32), 256, 0, s>>>(w + L.w3, L.noutp, L.h2p, m->w3, m->w3t);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

mann_status read_err(ProbeModel* m, cudaStream_t s) {
  int e = 0;
  MANN_CUDA_TRY(cudaMemcpyAsync(&e, m->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  if (e != 0) {
    cudaMemsetAsync(m->err, 0, sizeof(int), s);
    return fail(MANN_ETIMEOUT, "probe GEMM: a pipeline wait timed out");
  }
  return MANN_OK;
}

// Device buffers of one forward/backward over Bp rows.
struct Batch {
  int Bp = 0, L = 0;
  bf16 *X = nullptr, *Xt = nullptr, *H1 = nullptr, *H1t = nullptr, *H2 = nullptr, *H2t = nullptr;
  bf16 *dL = nullptr, *dLt = nullptr, *dZ2 = nullptr, *dZ2t = nullptr, *dZ1 = nullptr, *dZ1t = nullptr;
  float *Xf = nullptr, *D = nullptr, *Z1 = nullptr, *Z2 = nullptr, *logits = nullptr, *lse = nullptr,
        *loss_row = nullptr, *theta_part = nullptr, *loss_acc = nullptr;
  int32_t *lb = nullptr, *idx = nullptr;
  void* arena = nullptr;

  mann_status alloc(const Layout& P, int Bp_, int L_, int64_t nidx, bool prior) {
    Bp = Bp_;
    L = L_;
    size_t off = 0;
    std::vector<std::pair<void**, size_t>> want;
    auto add = [&](void** ptr, size_t bytes) { want.push_back({ptr, (bytes + 255) / 256 * 256}); };
    add((void**)&X, (size_t)Bp * P.dinp * 2);
    add((void**)&Xt, (size_t)Bp * P.dinp * 2);
    add((void**)&H1, (size_t)Bp * P.h1p * 2);
    add((void**)&H1t, (size_t)Bp * P.h1p * 2);
    add((void**)&H2, (size_t)Bp * P.h2p * 2);
    add((void**)&H2t, (size_t)Bp * P.h2p * 2);
    add((void**)&dL, (size_t)Bp * P.noutp * 2);
    add((void**)&dLt, (size_t)Bp * P.noutp * 2);
    add((void**)&dZ2, (size_t)Bp * P.h2p * 2);
    add((void**)&dZ2t, (size_t)Bp * P.h2p * 2);
    add((void**)&dZ1, (size_t)Bp * P.h1p * 2);
    add((void**)&dZ1t, (size_t)Bp * P.h1p * 2);
    add((void**)&Xf, (size_t)Bp * P.din * 4);
    if (prior) add((void**)&D, (size_t)Bp * P.nout * 4);
    add((void**)&Z1, (size_t)Bp * P.h1p * 4);
    add((void**)&Z2, (size_t)Bp * P.h2p * 4);
    add((void**)&logits, (size_t)Bp * P.noutp * 4);
    add((void**)&lse, (size_t)Bp * 4);
    add((void**)&loss_row, (size_t)Bp * 4);
    add((void**)&theta_part, (size_t)(Bp / 32) * (P.noutp / 32) * 4);
    add((void**)&loss_acc, 64 * 4);
    add((void**)&lb, (size_t)Bp * std::max(L, 1) * 4);
    add((void**)&idx, (size_t)std::max<int64_t>(nidx, 1) * 4);
    for (auto& w : want) off += w.second;
    MANN_CUDA_TRY(cudaMalloc(&arena, off));
    off = 0;
    for (auto& w : want) {
      *w.first = static_cast<uint8_t*>(arena) + off;
      off += w.second;
    }
    return MANN_OK;
  }
  ~Batch() {
    if (arena) cudaFree(arena);
  }
};

// Forward (and with `grad`, backward into m->grad) of the rows staged in b.
// The loss of the batch is added to *loss_slot when given.
mann_status fwd_bwd(ProbeModel* m, cudaStream_t s, Batch& b, int nb, bool grad, float* loss_slot) {
  const Layout& P = m->pad;
  const bool prior = m->p.use_prior != 0;
  const int Bp = b.Bp;
  const float* w = m->master;
  MANN_TRY(gemm(s, EPI_BIAS_GELU, b.X, m->w1, Bp, P.h1p, P.dinp, w + P.b1, grad ? b.Z1 : nullptr, b.H1,
                grad ? b.H1t : nullptr, nullptr, m->err));
  MANN_TRY(gemm(s, EPI_BIAS_GELU, b.H1, m->w2, Bp, P.h2p, P.h1p, w + P.b2, grad ? b.Z2 : nullptr, b.H2,
                grad ? b.H2t : nullptr, nullptr, m->err));
  MANN_TRY(gemm(s, EPI_LOGITS, b.H2, m->w3, Bp, P.noutp, P.h2p, w + P.b3, b.logits, nullptr, nullptr,
                nullptr, m->err));
  if (!grad) return MANN_OK;
  SoftmaxArgs sa{b.logits, prior ? b.D : nullptr, w + P.theta, b.lb, b.L, nb, P.nout, P.noutp, Bp,
                 b.lse, b.loss_row, b.dL, b.dLt, prior ? b.theta_part : nullptr};
  softmax_stats_kernel<<<(unsigned)ceil_div(Bp, 8), 256, 0, s>>>(sa);
  MANN_CHECK_LAUNCH();
  softmax_grad_kernel<<<dim3(P.noutp / 32, Bp / 32), 256, 0, s>>>(sa);
  MANN_CHECK_LAUNCH();
  float* g = m->grad;
  // dW3 = dL^T H2 ; dZ2 = (dL W3) * gelu'(Z2) ; dW2 = dZ2^T H1 ; dZ1 = (dZ2 W2) * gelu'(Z1) ; dW1 = dZ1^T X
  MANN_TRY(gemm(s, EPI_F32, b.dLt, b.H2t, P.noutp, P.h2p, Bp, nullptr, g + P.w3, nullptr, nullptr, nullptr, m->err));
  MANN_TRY(gemm(s, EPI_DGELU, b.dL, m->w3t, Bp, P.h2p, P.noutp, nullptr, nullptr, b.dZ2, b.dZ2t, b.Z2, m->err));
  MANN_TRY(gemm(s, EPI_F32, b.dZ2t, b.H1t, P.h2p, P.h1p, Bp, nullptr, g + P.w2, nullptr, nullptr, nullptr, m->err));
  MANN_TRY(gemm(s, EPI_DGELU, b.dZ2, m->w2t, Bp, P.h1p, P.h2p, nullptr, nullptr, b.dZ1, b.dZ1t, b.Z1, m->err));
  MANN_TRY(gemm(s, EPI_F32, b.dZ1t, b.Xt, P.h1p, P.dinp, Bp, nullptr, g + P.w1, nullptr, nullptr, nullptr, m->err));
  BiasGradArgs ba{};
  ba.src[0] = b.dLt;
  ba.dst[0] = g + P.b3;
  ba.rows[0] = P.noutp;
  ba.src[1] = b.dZ2t;
  ba.dst[1] = g + P.b2;
  ba.rows[1] = P.h2p;
  ba.src[2] = b.dZ1t;
  ba.dst[2] = g + P.b1;
  ba.rows[2] = P.h1p;
  ba.Bp = Bp;
  ba.theta_part = b.theta_part;
  ba.ntheta = (Bp / 32) * (P.noutp / 32);
  ba.dtheta = prior ? g + P.theta : nullptr;
  ba.loss_row = b.loss_row;
  ba.nb = nb;
  ba.loss_acc = loss_slot;
  const int rows = P.noutp + P.h2p + P.h1p + 1;
  bias_grad_kernel<<<(unsigned)ceil_div(rows, 8), 256, 0, s>>>(ba);
  MANN_CHECK_LAUNCH();
  if (!prior) MANN_CUDA_TRY(cudaMemsetAsync(g + P.theta, 0, sizeof(float), s));
  return MANN_OK;
}

mann_status stage(ProbeModel* m, cudaStream_t s, Batch& b, const float* q, const int32_t* idx, int nb,
                  const int32_t* labels) {
  const Layout& P = m->pad;
  stage_batch_kernel<<<dim3(P.dinp / 32, b.Bp / 32), 256, 0, s>>>(q, P.din, idx, nb, b.Bp, P.dinp, labels,
                                                                   b.L, b.X, b.Xt, b.Xf, labels ? b.lb : nullptr);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

mann_status prior_dist(Context* ctx, ProbeModel* m, cudaStream_t s, const float* Xf, int64_t rows, float* D) {
  return pairwise_device(ctx, s, Xf, rows, m->cent, m->pad.nout, m->pad.din, MANN_METRIC_SQEUCLIDEAN, D);
}

mann_status adam_step(ProbeModel* m, cudaStream_t s) {
  const Layout& P = m->pad;
  m->step += 1;
  AdamArgs a{};
  a.w = m->master;
  a.g = m->grad;
  a.m = m->adam_m;
  a.v = m->adam_v;
  a.n = P.total;
  a.lr = m->p.lr;
  a.b1 = m->p.beta1;
  a.b2 = m->p.beta2;
  a.eps = m->p.eps;
  a.wd = m->p.weight_decay;
  a.bc1 = (float)(1.0 - std::pow((double)a.b1, (double)m->step));
  a.bc2 = (float)(1.0 - std::pow((double)a.b2, (double)m->step));
  a.decay_begin[0] = P.w1;
  a.decay_end[0] = P.b1;
  a.decay_begin[1] = P.w2;
  a.decay_end[1] = P.b2;
  a.decay_begin[2] = P.w3;
  a.decay_end[2] = P.b3;
  adamw_kernel<<<(unsigned)std::min<int64_t>(ceil_div(P.total, 256), 4096), 256, 0, s>>>(a);
  MANN_CHECK_LAUNCH();
  return refresh_bf16(m, s);
}

}  // namespace

// Top-nprobe lists of device queries [nq][din] with the model (probes [nq][nprobe]).
mann_status probe_route_device(Context* ctx, ProbeModel* m, cudaStream_t s, const float* qs, int64_t nq,
                               int nprobe, int32_t* probes, float* coverage) {
  const Layout& P = m->pad;
  if (nprobe < 1 || nprobe > 128 || nprobe > P.nout)
    return fail(MANN_EINVAL_ARG, "learned routing supports 1 <= nprobe <= min(128, nlist)");
  const bool prior = m->p.use_prior != 0;
  constexpr int64_t CH = 16384;  // rows per pass
  for (int64_t r0 = 0; r0 < nq; r0 += CH) {
    const int nb = (int)std::min<int64_t>(CH, nq - r0);
    const int Bp = round_up(nb, 128);
    bf16 *X = nullptr, *H1 = nullptr, *H2 = nullptr;
    float *logits = nullptr, *D = nullptr;
    MANN_TRY(ctx->scratch_t(SLOT_PROBE_X, (size_t)Bp * P.dinp, &X));
    MANN_TRY(ctx->scratch_t(SLOT_PROBE_H1, (size_t)Bp * P.h1p, &H1));
    MANN_TRY(ctx->scratch_t(SLOT_PROBE_H2, (size_t)Bp * P.h2p, &H2));
    MANN_TRY(ctx->scratch_t(SLOT_PROBE_LOGITS, (size_t)Bp * P.noutp, &logits));
    stage_batch_kernel<<<dim3(P.dinp / 32, Bp / 32), 256, 0, s>>>(qs + r0 * P.din, P.din, nullptr, nb, Bp,
                                                                   P.dinp, nullptr, 0, X, nullptr, nullptr,
                                                                   nullptr);
    MANN_CHECK_LAUNCH();
    const float* w = m->master;
    MANN_TRY(gemm(s, EPI_BIAS_GELU, X, m->w1, Bp, P.h1p, P.dinp, w + P.b1, nullptr, H1, nullptr, nullptr, m->err));
    MANN_TRY(gemm(s, EPI_BIAS_GELU, H1, m->w2, Bp, P.h2p, P.h1p, w + P.b2, nullptr, H2, nullptr, nullptr, m->err));
    MANN_TRY(gemm(s, EPI_LOGITS, H2, m->w3, Bp, P.noutp, P.h2p, w + P.b3, logits, nullptr, nullptr, nullptr, m->err));
    if (prior) {
      MANN_TRY(ctx->scratch_t(SLOT_PROBE_D, (size_t)nb * P.nout, &D));
      MANN_TRY(prior_dist(ctx, m, s, qs + r0 * P.din, nb, D));
    }
    int32_t* pr = probes + r0 * nprobe;
    float* cv = coverage ? coverage + r0 : nullptr;
    const unsigned wgrid = (unsigned)ceil_div(nb, 8);
    if (nprobe <= 8) {
      if (cv)
        route_topk_warp_kernel<8, true><<<wgrid, 256, 0, s>>>(logits, P.noutp, D, w + P.theta, P.nout, nb, nprobe,
                                                              pr, cv);
      else
        route_topk_warp_kernel<8, false><<<wgrid, 256, 0, s>>>(logits, P.noutp, D, w + P.theta, P.nout, nb, nprobe,
                                                               pr, cv);
    } else if (nprobe <= 16) {
      if (cv)
        route_topk_warp_kernel<16, true><<<wgrid, 256, 0, s>>>(logits, P.noutp, D, w + P.theta, P.nout, nb, nprobe,
                                                               pr, cv);
      else
        route_topk_warp_kernel<16, false><<<wgrid, 256, 0, s>>>(logits, P.noutp, D, w + P.theta, P.nout, nb,
                                                                nprobe, pr, cv);
    } else {
      const size_t smem = sizeof(uint32_t) * P.nout;
      if (smem > 48 * 1024)
        MANN_CUDA_TRY(cudaFuncSetAttribute(route_topk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      route_topk_kernel<<<(unsigned)nb, ROUTE_THREADS, smem, s>>>(logits, P.noutp, D, w + P.theta, P.nout, nb,
                                                                  nprobe, pr, cv);
    }
    MANN_CHECK_LAUNCH();
  }
  return MANN_OK;
}

}  // namespace mann

using namespace mann;

struct mann_probe : ProbeModel {};

extern "C" {

int64_t mann_probe_param_count(const mann_probe_params* p) {
  if (!p || p->din <= 0 || p->hidden1 <= 0 || p->hidden2 <= 0 || p->nout <= 0) return -1;
  Layout L;
  L.set(p->din, p->hidden1, p->hidden2, p->nout, false);
  return L.total;
}

mann_status mann_probe_init(const mann_probe_params* p, float* params) {
  clear_error();
  MANN_TRY(check_params(p));
  if (!params) return fail(MANN_EINVAL_ARG, "NULL buffer");
  Layout L;
  L.set(p->din, p->hidden1, p->hidden2, p->nout, false);
  Splitmix r{p->seed ^ 0x5EEDC0DEull};
  auto fill = [&](int64_t off, int64_t n, double bound) {
    for (int64_t i = 0; i < n; ++i) params[off + i] = (float)((2.0 * r.uniform() - 1.0) * bound);
  };
  fill(L.w1, (int64_t)L.h1 * L.din, 1.0 / std::sqrt((double)L.din));
  fill(L.b1, L.h1, 1.0 / std::sqrt((double)L.din));
  fill(L.w2, (int64_t)L.h2 * L.h1, 1.0 / std::sqrt((double)L.h1));
  fill(L.b2, L.h2, 1.0 / std::sqrt((double)L.h1));
  if (p->use_prior) {  // start near the prior alone: small output layer, zero output bias
    fill(L.w3, (int64_t)L.nout * L.h2, 0.05 / std::sqrt((double)L.h2));
    std::fill(params + L.b3, params + L.b3 + L.nout, 0.0f);
  } else {
    fill(L.w3, (int64_t)L.nout * L.h2, 1.0 / std::sqrt((double)L.h2));
    fill(L.b3, L.nout, 1.0 / std::sqrt((double)L.h2));
  }
  params[L.theta] = (float)std::log(p->beta_init > 0 ? (double)p->beta_init : 1.0);
  return MANN_OK;
}

mann_status mann_probe_create(const mann_probe_params* p, const float* params, const float* centroids,
                              mann_probe** out) {
  clear_error();
  MANN_TRY(check_params(p));
  if (!params || !out) return fail(MANN_EINVAL_ARG, "NULL buffer");
  if (p->use_prior && !centroids) return fail(MANN_EINVAL_ARG, "the distance prior needs the centroids");
  *out = nullptr;
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  mann_probe* m = new mann_probe();
  m->p = *p;
  if (m->p.batch <= 0) m->p.batch = 1024;
  if (m->p.lr <= 0) m->p.lr = 1e-3f;
  if (m->p.beta1 <= 0) m->p.beta1 = 0.9f;
  if (m->p.beta2 <= 0) m->p.beta2 = 0.999f;
  if (m->p.eps <= 0) m->p.eps = 1e-8f;
  m->user.set(p->din, p->hidden1, p->hidden2, p->nout, false);
  m->pad.set(p->din, p->hidden1, p->hidden2, p->nout, true);
  cudaGetDevice(&m->device);
  const Layout& P = m->pad;
  auto bad = [&](cudaError_t e) {
    if (e == cudaSuccess) return false;
    mann_probe_destroy(m);
    set_error(std::string("probe allocation: ") + cudaGetErrorString(e));
    return true;
  };
  if (bad(cudaMalloc(&m->master, sizeof(float) * P.total)) || bad(cudaMalloc(&m->adam_m, sizeof(float) * P.total)) ||
      bad(cudaMalloc(&m->adam_v, sizeof(float) * P.total)) || bad(cudaMalloc(&m->grad, sizeof(float) * P.total)) ||
      bad(cudaMalloc(&m->w1, 2ull * P.h1p * P.dinp)) || bad(cudaMalloc(&m->w1t, 2ull * P.h1p * P.dinp)) ||
      bad(cudaMalloc(&m->w2, 2ull * P.h2p * P.h1p)) || bad(cudaMalloc(&m->w2t, 2ull * P.h2p * P.h1p)) ||
      bad(cudaMalloc(&m->w3, 2ull * P.noutp * P.h2p)) || bad(cudaMalloc(&m->w3t, 2ull * P.noutp * P.h2p)) ||
      bad(cudaMalloc(&m->err, sizeof(int))) ||
      (p->use_prior && bad(cudaMalloc(&m->cent, sizeof(float) * (size_t)P.nout * P.din))))
    return MANN_ECUDA;
  std::vector<float> hp;
  pad_params(m->user, P, params, hp);
  cudaStream_t s = ctx->stream;
  mann_status st = MANN_OK;
  {
    CallScope scope(ctx, s);
    if (cudaMemcpyAsync(m->master, hp.data(), sizeof(float) * P.total, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(m->adam_m, 0, sizeof(float) * P.total, s) != cudaSuccess ||
        cudaMemsetAsync(m->adam_v, 0, sizeof(float) * P.total, s) != cudaSuccess ||
        cudaMemsetAsync(m->grad, 0, sizeof(float) * P.total, s) != cudaSuccess ||
        cudaMemsetAsync(m->err, 0, sizeof(int), s) != cudaSuccess ||
        (m->cent && cudaMemcpyAsync(m->cent, centroids, sizeof(float) * (size_t)P.nout * P.din,
                                    cudaMemcpyHostToDevice, s) != cudaSuccess))
      st = fail(MANN_ECUDA, "probe upload failed");
    if (st == MANN_OK) st = refresh_bf16(m, s);
    if (st == MANN_OK && cudaStreamSynchronize(s) != cudaSuccess) st = fail(MANN_ECUDA, "probe upload failed");
  }
  if (st != MANN_OK) {
    mann_probe_destroy(m);
    return st;
  }
  *out = m;
  return MANN_OK;
}

mann_status mann_probe_destroy(mann_probe* m) {
  if (!m) return MANN_OK;
  cudaDeviceSynchronize();
  for (void* p : {(void*)m->master, (void*)m->adam_m, (void*)m->adam_v, (void*)m->grad, (void*)m->w1,
                  (void*)m->w1t, (void*)m->w2, (void*)m->w2t, (void*)m->w3, (void*)m->w3t, (void*)m->cent,
                  (void*)m->err})
    if (p) cudaFree(p);
  delete m;
  return MANN_OK;
}

mann_status mann_probe_get_params(mann_probe* m, float* params) {
  clear_error();
  if (!m || !params) return fail(MANN_EINVAL_ARG, "NULL argument");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(m->mu);
  std::vector<float> hp((size_t)m->pad.total);
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  MANN_CUDA_TRY(cudaMemcpyAsync(hp.data(), m->master, sizeof(float) * m->pad.total, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  unpad_params(m->user, m->pad, hp.data(), params);
  return MANN_OK;
}

// Train on host queries [nq][din] with labels [nq][nlabel] (list ids, -1 =
// none): `epochs` passes in a seeded shuffled order, batches of p.batch.
mann_status mann_probe_train(mann_probe* m, const float* queries, int64_t nq, const int32_t* labels,
                             int32_t nlabel, int32_t epochs, float* out_loss) {
  clear_error();
  if (!m || !queries || !labels) return fail(MANN_EINVAL_ARG, "NULL argument");
  if (nq <= 0 || nlabel <= 0 || epochs <= 0) return fail(MANN_EINVAL_ARG, "empty training set");
  if (nq > INT32_MAX) return fail(MANN_EINVAL_ARG, "too many training queries");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(m->mu);
  const Layout& P = m->pad;
  const int B = (int)std::min<int64_t>(m->p.batch, nq);
  const int Bp = round_up(B, 128);
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  Batch b;
  MANN_TRY(b.alloc(P, Bp, nlabel, nq, m->p.use_prior != 0));
  float *dq = nullptr;
  int32_t* dl = nullptr;
  MANN_CUDA_TRY(cudaMalloc(&dq, sizeof(float) * nq * P.din));
  struct Free {
    void* p;
    ~Free() {
      if (p) cudaFree(p);
    }
  } f1{dq};
  MANN_CUDA_TRY(cudaMalloc(&dl, sizeof(int32_t) * nq * nlabel));
  Free f2{dl};
  MANN_CUDA_TRY(cudaMemcpyAsync(dq, queries, sizeof(float) * nq * P.din, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dl, labels, sizeof(int32_t) * nq * nlabel, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemsetAsync(b.loss_acc, 0, sizeof(float) * 64, s));
  std::vector<int32_t> perm((size_t)nq);
  Splitmix r{m->p.seed ^ 0xC0FFEEull ^ (uint64_t)m->step};
  std::vector<float> losses((size_t)epochs, 0.0f);
  const int64_t steps_per_epoch = ceil_div(nq, B);
  for (int e = 0; e < epochs; ++e) {
    for (int64_t i = 0; i < nq; ++i) perm[i] = (int32_t)i;
    for (int64_t i = nq - 1; i > 0; --i) std::swap(perm[i], perm[r.next() % (uint64_t)(i + 1)]);
    MANN_CUDA_TRY(cudaMemcpyAsync(b.idx, perm.data(), sizeof(int32_t) * nq, cudaMemcpyHostToDevice, s));
    float* slot = b.loss_acc + (e % 64);
    MANN_CUDA_TRY(cudaMemsetAsync(slot, 0, sizeof(float), s));
    for (int64_t st = 0; st < steps_per_epoch; ++st) {
      const int nb = (int)std::min<int64_t>(B, nq - st * B);
      MANN_TRY(stage(m, s, b, dq, b.idx + st * B, nb, dl));
      if (m->p.use_prior) MANN_TRY(prior_dist(ctx, m, s, b.Xf, Bp, b.D));
      MANN_TRY(fwd_bwd(m, s, b, nb, true, slot));
      MANN_TRY(adam_step(m, s));
    }
    float l = 0.0f;
    MANN_CUDA_TRY(cudaMemcpyAsync(&l, slot, sizeof(float), cudaMemcpyDeviceToHost, s));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));
    losses[e] = l / (float)steps_per_epoch;
  }
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  MANN_TRY(read_err(m, s));
  if (out_loss) std::memcpy(out_loss, losses.data(), sizeof(float) * epochs);
  return MANN_OK;
}

// Loss and gradient (flat, user layout) of one batch, no update.
mann_status mann_probe_grad(mann_probe* m, const float* queries, int64_t nq, const int32_t* labels,
                            int32_t nlabel, float* out_grad, float* out_loss) {
  clear_error();
  if (!m || !queries || !labels || !out_grad) return fail(MANN_EINVAL_ARG, "NULL argument");
  if (nq <= 0 || nq > 65536 || nlabel <= 0) return fail(MANN_EINVAL_ARG, "batch must hold 1..65536 queries");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(m->mu);
  const Layout& P = m->pad;
  const int Bp = round_up((int)nq, 128);
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  Batch b;
  MANN_TRY(b.alloc(P, Bp, nlabel, 1, m->p.use_prior != 0));
  float* dq = nullptr;
  int32_t* dl = nullptr;
  MANN_CUDA_TRY(cudaMalloc(&dq, sizeof(float) * nq * P.din + sizeof(int32_t) * nq * nlabel));
  dl = reinterpret_cast<int32_t*>(dq + nq * P.din);
  MANN_CUDA_TRY(cudaMemcpyAsync(dq, queries, sizeof(float) * nq * P.din, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dl, labels, sizeof(int32_t) * nq * nlabel, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemsetAsync(b.loss_acc, 0, sizeof(float), s));
  mann_status st = stage(m, s, b, dq, nullptr, (int)nq, dl);
  if (st == MANN_OK && m->p.use_prior) st = prior_dist(ctx, m, s, b.Xf, Bp, b.D);
  if (st == MANN_OK) st = fwd_bwd(m, s, b, (int)nq, true, b.loss_acc);
  std::vector<float> hg((size_t)P.total);
  float loss = 0.0f;
  if (st == MANN_OK &&
      (cudaMemcpyAsync(hg.data(), m->grad, sizeof(float) * P.total, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
       cudaMemcpyAsync(&loss, b.loss_acc, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
       cudaStreamSynchronize(s) != cudaSuccess))
    st = fail(MANN_ECUDA, "probe gradient readback failed");
  cudaFree(dq);
  MANN_TRY(st);
  MANN_TRY(read_err(m, s));
  unpad_params(m->user, P, hg.data(), out_grad);
  if (out_loss) *out_loss = loss;
  return MANN_OK;
}

// Scores [nq][nout] of host queries (MLP output minus the prior term).
mann_status mann_probe_scores(mann_probe* m, const float* queries, int64_t nq, float* out_scores) {
  clear_error();
  if (!m || !queries || !out_scores) return fail(MANN_EINVAL_ARG, "NULL argument");
  if (nq <= 0) return MANN_OK;
  if (nq > 65536) return fail(MANN_EINVAL_ARG, "at most 65536 queries per call");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(m->mu);
  const Layout& P = m->pad;
  const int Bp = round_up((int)nq, 128);
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  Batch b;
  MANN_TRY(b.alloc(P, Bp, 1, 1, m->p.use_prior != 0));
  float* dq = nullptr;
  MANN_CUDA_TRY(cudaMalloc(&dq, sizeof(float) * nq * P.din));
  mann_status st = MANN_OK;
  if (cudaMemcpyAsync(dq, queries, sizeof(float) * nq * P.din, cudaMemcpyHostToDevice, s) != cudaSuccess)
    st = fail(MANN_ECUDA, "upload failed");
  if (st == MANN_OK) st = stage(m, s, b, dq, nullptr, (int)nq, nullptr);
  if (st == MANN_OK) st = fwd_bwd(m, s, b, (int)nq, false, nullptr);
  if (st == MANN_OK && m->p.use_prior) st = prior_dist(ctx, m, s, b.Xf, nq, b.D);
  std::vector<float> lg((size_t)nq * P.noutp), dd;
  float theta = 0.0f;
  if (m->p.use_prior) dd.resize((size_t)nq * P.nout);
  if (st == MANN_OK &&
      (cudaMemcpyAsync(lg.data(), b.logits, sizeof(float) * nq * P.noutp, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
       (m->p.use_prior &&
        cudaMemcpyAsync(dd.data(), b.D, sizeof(float) * nq * P.nout, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
       cudaMemcpyAsync(&theta, m->master + P.theta, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
       cudaStreamSynchronize(s) != cudaSuccess))
    st = fail(MANN_ECUDA, "readback failed");
  cudaFree(dq);
  MANN_TRY(st);
  MANN_TRY(read_err(m, s));
  const float beta = std::exp(theta);
  for (int64_t r = 0; r < nq; ++r)
    for (int c = 0; c < P.nout; ++c) {
      float v = lg[(size_t)r * P.noutp + c];
      if (m->p.use_prior) v -= beta * dd[(size_t)r * P.nout + c];
      out_scores[r * P.nout + c] = v;
    }
  return MANN_OK;
}

mann_status mann_probe_route_device(mann_probe* m, const float* queries, int64_t q, int32_t nprobe,
                                    int32_t* out_probes, float* out_coverage, void* stream) {
  clear_error();
  if (!m || (q > 0 && (!queries || !out_probes))) return fail(MANN_EINVAL_ARG, "NULL argument");
  if (q <= 0) return MANN_OK;
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(m->mu);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CallScope scope(ctx, s);
  return probe_route_device(ctx, m, s, queries, q, nprobe, out_probes, out_coverage);
}

// IVF search routed by the model: probes from the scores, then the list scan.
mann_status mann_ivf_search_learned_device(mann_probe* m, const mann_knn_params* p, int32_t nprobe,
                                           const float* data, int64_t n, int32_t d, int32_t nlist,
                                           const int64_t* list_offsets, const int32_t* list_ids,
                                           const float* queries, int64_t q, int32_t* out_ids,
                                           float* out_dists, void* stream) {
  clear_error();
  if (!m || !p) return fail(MANN_EINVAL_ARG, "NULL argument");
  if (d != m->p.din || nlist != m->p.nout) return fail(MANN_EINVAL_DIM, "probe model does not match the index");
  if (!data || !list_offsets || !list_ids || (q > 0 && (!queries || !out_ids || !out_dists)))
    return fail(MANN_EINVAL_ARG, "NULL buffer");
  if (p->k <= 0 || q <= 0) return MANN_OK;
  nprobe = std::min(nprobe, nlist);
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(m->mu);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CallScope scope(ctx, s);
  int32_t* probes = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_IVF_PROBES, (size_t)q * nprobe, &probes));
  MANN_TRY(probe_route_device(ctx, m, s, queries, q, nprobe, probes, nullptr));
  return ivf_scan_device(ctx, s, data, n, d, p->metric, list_offsets, list_ids, nlist, queries, q, probes,
                         nprobe, p->k, out_ids, out_dists);
}

// Host-pointer form of mann_ivf_search_learned_device.
mann_status mann_ivf_search_learned(mann_probe* m, const mann_knn_params* p, int32_t nprobe, const float* data,
                                    int64_t n, int32_t d, int32_t nlist, const int64_t* list_offsets,
                                    const int32_t* list_ids, const float* queries, int64_t q,
                                    int32_t* out_ids, float* out_dists) {
  clear_error();
  if (!m || !p) return fail(MANN_EINVAL_ARG, "NULL argument");
  if (d != m->p.din || nlist != m->p.nout) return fail(MANN_EINVAL_DIM, "probe model does not match the index");
  if (!data || !list_offsets || !list_ids || (q > 0 && (!queries || !out_ids || !out_dists)))
    return fail(MANN_EINVAL_ARG, "NULL buffer");
  if (p->k <= 0 || q <= 0) return MANN_OK;
  nprobe = std::min(nprobe, nlist);
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  std::lock_guard<std::mutex> lk(m->mu);
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  float *dx = nullptr, *dq = nullptr, *dd = nullptr;
  int64_t* doff = nullptr;
  int32_t *dids = nullptr, *dout = nullptr, *probes = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_BASE, (size_t)n * d, &dx));
  MANN_TRY(ctx->scratch_t(SLOT_QUERIES, (size_t)q * d, &dq));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_LOFF, (size_t)nlist + 1, &doff));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_LIDS, (size_t)n, &dids));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_IDS, (size_t)q * p->k, &dout));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_DISTS, (size_t)q * p->k, &dd));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_PROBES, (size_t)q * nprobe, &probes));
  MANN_CUDA_TRY(cudaMemcpyAsync(dx, data, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dq, queries, sizeof(float) * q * d, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(doff, list_offsets, sizeof(int64_t) * (nlist + 1), cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dids, list_ids, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
  MANN_TRY(probe_route_device(ctx, m, s, dq, q, nprobe, probes, nullptr));
  MANN_TRY(ivf_scan_device(ctx, s, dx, n, d, p->metric, doff, dids, nlist, dq, q, probes, nprobe, p->k, dout, dd));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_ids, dout, sizeof(int32_t) * q * p->k, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_dists, dd, sizeof(float) * q * p->k, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  return read_err(m, s);
}

}  // extern "C"
