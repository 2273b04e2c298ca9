// knn_bf16.cu -- exact kNN through BF16 tensor-core tiles (tcgen05 / TMEM),
// a certified top-(k+m) candidate set, exact FP32 rerank and FP64 near-tie
// resolution.  Metrics: SqEuclidean, Euclidean, and CosineDist (the passes run
// on unit-normalised rows; the rerank uses the FP32 form's cosine).
//
// Replaces the same reference sites as the FP32 form
// (src/indices/bruteforce.jl:59-65, src/ann_index.jl:91-98,
// src/graphs/knn_graph.jl:63-67) and returns the same answer:
//
//   1. prep      centre the points (x - mu, mu = mean of the points; distances
//                are unchanged), round to BF16, and record per row
//                ||x~||^2, ||x~|| and a bound R on ||(x - mu) - x~||.
//   2. main      est(q, p) = ||q~||^2 + ||p~||^2 - 2 q~.p~ with q~.p~ from
//                tcgen05.mma (BF16 x BF16 -> FP32 in TMEM); the epilogue
//                warps keep each query's L smallest est (L = k + margin).
//   3. merge     per query, the L smallest est over all CTAs.
//   4. rerank    threshold T(q) such that every point that can be in the
//                exact top-k (in FP32 or FP64) has est <= T (bound below);
//                the list is certified when its L-th est exceeds T.  Every
//                candidate with est <= T gets its exact FP32 difference-form
//                distance (the sequential sum of the FP32 form), and the
//                candidates are sorted by (distance, id).  Uncertified rows
//                are re-run by the exact FP32 scan.
//   5. resolve   (MANN_FLAG_FP64_TIES) adjacent candidates whose FP32
//                distances are within the FP32 rounding bound are re-ordered
//                by FP64 distances.
//
// Error bound used by the certificate (all in the centred, rounded space):
//   E = ||x~ - y~||, D = ||x - y||^2 exact.  |sqrt(D) - E| <= Rx + Ry.
//   |est - E^2| <= c1 * (||x~|| + ||y~||)^2,  c1 = 4u + 2*gamma_d,
//   u = 2^-24, gamma_d = (d + 32) * 2^-22 (FP32 tensor accumulation,
//   conservatively truncating).  With e_k the k-th smallest est of the row:
//   D_(k) <= U = (sqrt(e_k + c1 A) + Rs)^2 and any j in the exact top-k has
//   est_j <= (sqrt(U) + Rs)^2 + c1 A;  A = (||q~|| + max||p~||)^2,
//   Rs = R_q + max R_p.  A slack of 3 (d+2) u U keeps every point that could
//   enter the FP32 top-k or tie with its k-th FP32 distance.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "kernels.cuh"
#include "ptx.cuh"

namespace mann {

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr int BM = 128;          // queries per CTA tile (TMEM lanes)
constexpr int BN = 256;          // points per tile (TMEM columns per accumulator)
constexpr int BK = 64;           // BF16 elements per stage row (128 bytes, one swizzle span)
constexpr int A_STAGE_BYTES = BM * BK * 2;  // 16 KB
// One CTA: A 128 x 64 + B 256 x 64 per stage (48 KB), 4 stages.  A CTA pair
// (cta_group::2, M = 256): each CTA stages its own 128 query rows and half of
// the tile's 256 point rows (32 KB per stage), 6 stages.
template <bool PAIR>
struct Stg {
  static constexpr int B_ROWS = PAIR ? BN / 2 : BN;
  static constexpr int B_BYTES = B_ROWS * BK * 2;
  static constexpr int BYTES = A_STAGE_BYTES + B_BYTES;
  static constexpr int N = PAIR ? 6 : 4;
};

constexpr int AUG = 24;                              // norm-fold columns read after a BF16 row's main part
constexpr int LIST = 32;                             // candidates kept per query row
constexpr int SEED_SAMPLE = 2048;                    // points sampled by the seed pass
constexpr int SEED_DEPTH = 5;                        // the seed is the 5th smallest (chunk minimum)
constexpr int KREQ_MAX_BF16 = 24;                    // largest k (k+1 for graphs) of this form
constexpr int SEG_SEED_STRIDE = 32;                  // many point sets: the seed pass samples every 32nd point
constexpr uint32_t TMEM_COLS = 2 * BN;               // double-buffered accumulator
// Bands and CTA pairs are built but not selected: on one GB300 the
// phase-aligned single-band walk beat 48 MB bands (1M x 128: 8.2 vs 11.8 ms;
// 290k x 256 cosine: 5.5 vs 6.1 ms) and single CTAs beat cta_group::2 pairs
// (60k x 784 self graph: 4.50 vs 4.75 ms per main pass), CUDA events.
constexpr double BAND_MIN_BYTES = 1e30;          // point operands above this are walked in bands
constexpr double BAND_BYTES = 48.0 * (1 << 20);  // point-operand bytes per band
constexpr bool K2_USE_PAIRS = false;

enum : int { ERR_TIMEOUT_PRODUCER = 1, ERR_TIMEOUT_MMA = 2, ERR_TIMEOUT_EPI = 3 };

struct RowInfo {
  float nrm;    // ||x~||^2 (FP64 sum rounded to nearest)
  float xn_up;  // ||x~|| rounded up
  float r_up;   // bound on ||(x - mu) - x~|| (includes the FP32 rounding of x - mu)
  float lo_up;  // split form: ||x_lo|| rounded up (0 otherwise)
};

struct BaseMax {
  unsigned xn_bits;  // max over points of xn_up (positive float bits, integer max)
  unsigned r_bits;   // max over points of r_up
  unsigned lo_bits;  // max over points of lo_up
  unsigned pad;
};

// ---------------------------------------------------------------- prep kernels

// Unit-normalised copy of every row (cosine, FP8 form): x^ = x / sqrt(|x|^2)
// with |x|^2 the FP32 form's sequential sum (row_sqnorm_kernel, kept for the
// rerank); a zero row stays zero.  One warp per row, coalesced.
__global__ void scale_rows_kernel(const float* __restrict__ x, int64_t n, int d, const float* __restrict__ sqn,
                                  float* __restrict__ xh) {
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= n) return;
  const float nr = __fsqrt_rn(sqn[row]);
  const float* r = x + row * (int64_t)d;
  float* o = xh + row * (int64_t)d;
  for (int c = threadIdx.x & 31; c < d; c += 32) o[c] = nr > 0.0f ? __fdiv_rn(__ldg(r + c), nr) : 0.0f;
}

// Column means over an evenly spaced sample of rows (rows <= CENTRE_ROWS).
// Any centre keeps the distances unchanged; a good one shrinks the BF16
// values and their rounding.  Block (32 columns x 32 row groups): FP32
// partial sums per thread, FP64 across groups.  With row norms (cosine) each
// sampled row is scaled by one reciprocal, computed once per block: the
// centre only needs to be near the unit rows' mean, not their exact bits.
constexpr int CENTRE_ROWS = 4096;
__global__ void centre_sample_kernel(const float* __restrict__ x, int64_t n, int d, int64_t stride,
                                     int64_t rows, float* __restrict__ mu, const float* __restrict__ rnorm) {
  __shared__ double part[32][33];
  __shared__ float inv[CENTRE_ROWS];
  const int cl = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + cl;
  if (rnorm) {
    for (int64_t i = threadIdx.x; i < rows; i += blockDim.x) {
      const float nr = __fsqrt_rn(rnorm[i * stride]);
      inv[i] = nr > 0.0f ? 1.0f / nr : 0.0f;
    }
    __syncthreads();
  }
  float s = 0.0f;
  if (c < d)
    for (int64_t i = g; i < rows; i += 32) {
      const float xv = x[(i * stride) * d + c];
      s += rnorm ? xv * inv[i] : xv;
    }
  part[g][cl] = (double)s;
  __syncthreads();
  if (g == 0 && c < d) {
    double t = 0.0;
    for (int i = 0; i < 32; ++i) t += part[i][cl];
    mu[c] = (float)(t / (double)rows);
  }
}


// scale / centre candidates tried on a sample of rows: the one whose BF16
// rounding residual is smallest wins.  (1, mean) suits general data;
// (255, mean on the 1/255 grid) and (1, integer mean) make 8-bit-quantised
// data exactly representable, so its certificate is nearly exact.
constexpr int NUM_SCALES = 3;
__device__ __forceinline__ void scale_candidate(int i, float m, float* sc, float* mc) {
  if (i == 0) { *sc = 1.0f; *mc = m; }
  else if (i == 1) { *sc = 255.0f; *mc = rintf(m * 255.0f) / 255.0f; }
  else { *sc = 1.0f; *mc = rintf(m); }
}

// per candidate: sum over sampled rows of ||cv - bf16(cv)||^2 / ||cv||^2; the
// first candidate also records the sampled max |x - mu| (float bits, integer
// max) in score[NUM_SCALES] for the FP16 form's scale
__global__ void scale_probe_kernel(const float* __restrict__ x, int64_t n, int d,
                                   const float* __restrict__ mu, int64_t stride,
                                   double* __restrict__ score, const float* __restrict__ rnorm) {
  const int lane = threadIdx.x & 31;
  const int64_t row = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * stride;
  const int cand = blockIdx.y;
  if (row >= n) return;
  float rr = 0.0f, cc = 0.0f, mx = 0.0f;  // a heuristic score: FP32 is plenty
  float inv = 1.0f;  // unit rows: one reciprocal of the row's norm (a heuristic needs no exact division)
  if (rnorm) {
    const float nr = __fsqrt_rn(rnorm[row]);
    inv = nr > 0.0f ? 1.0f / nr : 0.0f;
  }
  for (int c = lane; c < d; c += 32) {
    float sc, mc;
    scale_candidate(cand, mu[c], &sc, &mc);
    const float cv = __fmul_rn(sc, __fsub_rn(x[row * d + c] * inv, mc));
    const float bv = __bfloat162float(__float2bfloat16_rn(cv));
    rr = __fmaf_rn(cv - bv, cv - bv, rr);
    cc = __fmaf_rn(cv, cv, cc);
    mx = fmaxf(mx, fabsf(cv));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    rr += __shfl_xor_sync(FULL, rr, o);
    cc += __shfl_xor_sync(FULL, cc, o);
    mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, o));
  }
  if (lane == 0) {
    atomicAdd(&score[cand], cc > 0.0f ? (double)rr / (double)cc : 0.0);
    if (cand == 0 && mx < 3.0e38f) atomicMax(reinterpret_cast<unsigned*>(&score[NUM_SCALES]), __float_as_uint(mx));
  }
}

// pick the candidate with the smallest residual (moving off the plain mean
// only for a clear win), replace mu by its centre and publish its scale
__global__ void choose_scale_kernel(const double* __restrict__ score, float* __restrict__ mu, int d,
                                    float* __restrict__ scale_out, int* __restrict__ inexact, int64_t nrows,
                                    float* __restrict__ f16_scale_out) {
  __shared__ int best;
  if (threadIdx.x == 0) {
    // FP16 form: the power of two that takes the sampled max |x - mu| into
    // [2^11, 2^12) -- 16x below FP16's largest value for rows off the sample
    // (a value that still overflows saturates, and its row's bound says so)
    const float smax = __uint_as_float(*reinterpret_cast<const unsigned*>(&score[NUM_SCALES]));
    int e = 0;
    if (smax > 0.0f) frexpf(smax, &e);  // smax in [2^(e-1), 2^e)
    *f16_scale_out = ldexpf(1.0f, max(-120, min(120, 12 - e)));
    int b = 0;
    for (int i = 1; i < NUM_SCALES; ++i)
      if (score[i] < 0.25 * score[b]) b = i;
    best = b;
    // the mean squared relative residual of the sampled rows: ~2^-18 for data
    // off any grid, ~1e-14 for grid data that FP32 centring merely blurs
    *inexact = score[b] > 1e-10 * (double)(nrows > 0 ? nrows : 1) ? 1 : 0;
    float sc, mc;
    scale_candidate(b, 0.0f, &sc, &mc);
    *scale_out = sc;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < d; c += blockDim.x) {
    float sc, mc;
    scale_candidate(best, mu[c], &sc, &mc);
    mu[c] = mc;
  }
}

// One warp per row: BF16 copy of scale*(x - mu) padded to dp, and the row's bound terms.
// FP16 form (f16 = 1): the main columns are FP16 instead (values beyond FP16's
// largest finite value saturate, and the row's residual bound becomes +inf,
// so its certificate fails and the exact scan answers it); the fold block
// stays BF16 (its K-step is a BF16 MMA of its own).
// Split form (split = 1): x~ = hi + lo with hi = bf16(cv), lo = bf16(cv - hi),
// written as three dp-wide segments -- [hi | hi | lo] for query rows (role 0),
// [hi | lo | hi] for point rows (role 1) -- so one MMA over 3dp columns gives
// hi.hi + hi.lo + lo.hi = q~.p~ - lo_q.lo_p.  The row (width = augx + 16
// columns) then holds zeros up to augx and the first 16 columns of the
// norm-fold block, [P0 P1 P2 1 1 1 0 0 | 1 1 1 P0 P1 P2 0 0], with P0 + P1 +
// P2 = -||x~||^2 / 2 exactly; its last 8 columns are zeros past the row.
__global__ void convert_rows_kernel(const float* __restrict__ x, int64_t n, int d, int dp, int augx, int width,
                                    const float* __restrict__ mu, const float* __restrict__ scale_ptr,
                                    __nv_bfloat16* __restrict__ xb, RowInfo* __restrict__ info,
                                    float* __restrict__ norms, BaseMax* __restrict__ bmax, int split,
                                    int role, int f16, const float* __restrict__ rnorm) {
  const int lane = threadIdx.x & 31;
  const float scale = *scale_ptr;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  __shared__ unsigned blk_max[3];
  if (threadIdx.x < 3) blk_max[threadIdx.x] = 0u;
  __syncthreads();
  const bool valid = row < n;
  const float* xr = x + (valid ? row : 0) * d;
  __nv_bfloat16* br = xb + (valid ? row : 0) * (int64_t)width;
  // cosine: the unit row x / sqrt(|x|^2), divided exactly as scale_rows_kernel
  // writes it (a zero or non-finite row gives 0)
  const float unr = (rnorm && valid) ? __fsqrt_rn(rnorm[row]) : 1.0f;
  // per-lane FP32 sums (ceil(dp/32) terms each), cross-lane sum in FP64: every
  // sum carries a relative error below (ceil(dp/32) + 2) u, which the
  // certificate adds to its bound (norm_rel_err)
  float f_b = 0.0f, f_r = 0.0f, f_c = 0.0f, f_l = 0.0f;
  bool sat = false;  // FP16 form: a value saturated (or was not a number)
  constexpr int PF = 8;  // loads in flight per lane (the kernel is latency-bound otherwise)
  for (int c0 = lane; valid && c0 < dp; c0 += 32 * PF) {
    float xv[PF], mv[PF];
#pragma unroll
    for (int u = 0; u < PF; ++u) {
      const int c = c0 + 32 * u;
      xv[u] = c < d ? __ldg(xr + c) : 0.0f;
      mv[u] = c < d ? __ldg(mu + c) : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < PF; ++u) {
    const int c = c0 + 32 * u;
    if (c >= dp) break;
    float cv = 0.0f;
    if (c < d) {
      const float uv = rnorm ? (unr > 0.0f ? __fdiv_rn(xv[u], unr) : 0.0f) : xv[u];
      cv = __fmul_rn(scale, __fsub_rn(uv, mv[u]));
    }
    float bv;
    if (f16) {
      const float cl = fminf(fmaxf(cv, -65504.0f), 65504.0f);
      const __half h = __float2half_rn(cl);
      bv = __half2float(h);
      sat |= !(cl == cv);
      reinterpret_cast<__half*>(br)[c] = h;
    } else {
    const __nv_bfloat16 b = __float2bfloat16_rn(cv);
    bv = __bfloat162float(b);
    if (split) {
      // cv - hi is exact in FP32; hi + lo spans at most 17 bits, also exact
      const __nv_bfloat16 lb = __float2bfloat16_rn(cv - bv);
      const float lv = __bfloat162float(lb);
      br[c] = b;
      br[dp + c] = role ? lb : b;
      br[2 * dp + c] = role ? b : lb;
      bv = bv + lv;
      f_l = __fmaf_rn(lv, lv, f_l);
    } else {
      br[c] = b;
    }
    }
    const float rv = cv - bv;  // exact: the rounding residual of a float fits in a float
    f_b = __fmaf_rn(bv, bv, f_b);
    f_r = __fmaf_rn(rv, rv, f_r);
    f_c = __fmaf_rn(cv, cv, f_c);
    }
  }
  const bool any_sat = __any_sync(FULL, sat);
  // cross-lane sums in FP32 (a 5-level tree of nonnegative terms adds at most
  // 5u of relative error; FP64 arithmetic is slow on this part)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    f_b += __shfl_xor_sync(FULL, f_b, o);
    f_r += __shfl_xor_sync(FULL, f_r, o);
    f_c += __shfl_xor_sync(FULL, f_c, o);
    f_l += __shfl_xor_sync(FULL, f_l, o);
  }
  if (valid) {
    // the butterfly leaves the same f_b in every lane (x + y == y + x); split
    // -f_b / 2 into three BF16 pieces: each remainder is exact (Sterbenz) and
    // the third holds at most 8 significant bits
    const float hn = -0.5f * f_b;
    const __nv_bfloat16 p0 = __float2bfloat16_rn(hn);
    const float r1 = __fsub_rn(hn, __bfloat162float(p0));
    const __nv_bfloat16 p1 = __float2bfloat16_rn(r1);
    const __nv_bfloat16 p2 = __float2bfloat16_rn(__fsub_rn(r1, __bfloat162float(p1)));
    const __nv_bfloat16 one = __float2bfloat16_rn(1.0f), zero = __float2bfloat16_rn(0.0f);
    for (int c = (split ? 3 * dp : dp) + lane; c < width; c += 32) {
      const int a = c - augx;  // < 0: zero padding of the main columns
      const int k = a < 8 ? a : a - 11;  // piece index in the first / second group
      __nv_bfloat16 val = zero;
      if ((a >= 0 && a < 3) || (a >= 11 && a < 14)) val = k == 0 ? p0 : (k == 1 ? p1 : p2);
      else if ((a >= 3 && a < 6) || (a >= 8 && a < 11)) val = one;
      br[c] = val;
    }
  }
  if (lane == 0 && valid) {
    // FP32 with directed rounding (FP64 is slow on this part): each bound is
    // rounded up at every step, so it stays an upper bound of the FP64 value
    const float rel = (float)((dp + 31) / 32 + 2 + 5) * 5.9604644775390625e-08f;  // exact
    const float onep = __fadd_ru(1.0f, rel);
    RowInfo ri;
    ri.nrm = f_b;
    ri.xn_up = __fsqrt_ru(__fmul_ru(f_b, onep));
    // ||s(x-mu)_exact - x~|| <= ||cv - x~|| + 2u ||cv|| (1+u), cv = fl(s fl(x-mu))
    ri.r_up = __fadd_ru(__fsqrt_ru(__fmul_ru(f_r, onep)),
                        __fmul_ru(__fmul_ru(1.1920928955078125e-07f, 1.0000002f), __fsqrt_ru(__fmul_ru(f_c, onep))));
    ri.lo_up = split ? __fsqrt_ru(__fmul_ru(f_l, onep)) : 0.0f;
    if (any_sat) ri.r_up = __int_as_float(0x7F800000);
    info[row] = ri;
    if (norms) norms[row] = ri.nrm;
    if (bmax) {  // one global atomic per block and field, not per row
      atomicMax(&blk_max[0], __float_as_uint(ri.xn_up));
      atomicMax(&blk_max[1], __float_as_uint(ri.r_up));
      atomicMax(&blk_max[2], __float_as_uint(ri.lo_up));
    }
  }
  if (bmax) {
    __syncthreads();
    if (threadIdx.x == 0) {
      atomicMax(&bmax->xn_bits, blk_max[0]);
      atomicMax(&bmax->r_bits, blk_max[1]);
      atomicMax(&bmax->lo_bits, blk_max[2]);
    }
  }
}

// One warp per row: the FP8 (e4m3) form of scale*(x - mu).  The row gets
// its own power-of-two factor f = 2^e with max|cv| f <= 448 (e4m3's largest
// finite value), x8 = e4m3(cv f) (round to nearest, finite), and x~ = x8 / f
// exactly; `rscale` receives 1/f, the factor that turns the tensor core's
// sum of x8 products back into x~ units.  Bound terms as convert_rows_kernel.
__global__ void convert_rows_fp8_kernel(const float* __restrict__ x, int64_t n, int d, int dp,
                                        const float* __restrict__ mu, const float* __restrict__ scale_ptr,
                                        uint8_t* __restrict__ x8, float* __restrict__ rscale,
                                        RowInfo* __restrict__ info, float* __restrict__ norms,
                                        BaseMax* __restrict__ bmax) {
  const int lane = threadIdx.x & 31;
  const float scale = *scale_ptr;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  __shared__ unsigned blk_max[2];
  if (threadIdx.x < 2) blk_max[threadIdx.x] = 0u;
  __syncthreads();
  const bool valid = row < n;
  const float* xr = x + (valid ? row : 0) * d;
  uint8_t* br = x8 + (valid ? row : 0) * (int64_t)dp;
  // the row's largest magnitude
  float amax = 0.0f;
  for (int c = lane; valid && c < d; c += 32)
    amax = fmaxf(amax, fabsf(__fmul_rn(scale, __fsub_rn(__ldg(xr + c), __ldg(mu + c)))));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(FULL, amax, o));
  float f = 1.0f;
  if (amax > 0.0f && amax < 3.0e38f) {
    f = exp2f(floorf(log2f(448.0f / amax)));
    while (amax * f > 448.0f) f *= 0.5f;
    while (amax * (2.0f * f) <= 448.0f) f *= 2.0f;
  }
  // keep the product of two rows' 1/f factors (and -2) a normal FP32 number
  f = fminf(fmaxf(f, 0x1p-40f), 0x1p40f);
  const float inv = 1.0f / f;  // a power of two: exact
  float f_b = 0.0f, f_r = 0.0f, f_c = 0.0f;
  for (int c = lane; valid && c < dp; c += 32) {
    float cv = 0.0f;
    if (c < d) cv = __fmul_rn(scale, __fsub_rn(__ldg(xr + c), __ldg(mu + c)));
    const __nv_fp8_storage_t q8 = __nv_cvt_float_to_fp8(cv * f, __NV_SATFINITE, __NV_E4M3);
    const float bv = __half2float(__half(__nv_cvt_fp8_to_halfraw(q8, __NV_E4M3))) * inv;
    br[c] = (uint8_t)q8;
    const float rv = cv - bv;  // exact: bv is cv rounded to fewer bits
    f_b = __fmaf_rn(bv, bv, f_b);
    f_r = __fmaf_rn(rv, rv, f_r);
    f_c = __fmaf_rn(cv, cv, f_c);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    f_b += __shfl_xor_sync(FULL, f_b, o);
    f_r += __shfl_xor_sync(FULL, f_r, o);
    f_c += __shfl_xor_sync(FULL, f_c, o);
  }
  if (lane == 0 && valid) {
    const float rel = (float)((dp + 31) / 32 + 2 + 5) * 5.9604644775390625e-08f;  // exact
    const float onep = __fadd_ru(1.0f, rel);
    RowInfo ri;
    ri.nrm = f_b;
    ri.xn_up = __fsqrt_ru(__fmul_ru(f_b, onep));
    ri.r_up = __fadd_ru(__fsqrt_ru(__fmul_ru(f_r, onep)),
                        __fmul_ru(__fmul_ru(1.1920928955078125e-07f, 1.0000002f), __fsqrt_ru(__fmul_ru(f_c, onep))));
    ri.lo_up = 0.0f;
    info[row] = ri;
    rscale[row] = inv;
    if (norms) norms[row] = ri.nrm;
    if (bmax) {
      atomicMax(&blk_max[0], __float_as_uint(ri.xn_up));
      atomicMax(&blk_max[1], __float_as_uint(ri.r_up));
    }
  }
  if (bmax) {
    __syncthreads();
    if (threadIdx.x == 0) {
      atomicMax(&bmax->xn_bits, blk_max[0]);
      atomicMax(&bmax->r_bits, blk_max[1]);
    }
  }
}

// ---------------------------------------------------------------- main kernel

// Order of the (query block, point tile) items.  With one band the items
// are query-block-major (item = qb * tiles + t).  With several bands the point
// tiles are cut into bands of band_tiles tiles (the last one shorter) and the
// items of band b -- every query block against the band's tiles, query-block
// major inside the band -- come before those of band b + 1, so all CTAs work
// inside one band at a time and a point operand larger than L2 is read from
// DRAM about once per launch instead of once per query block.  A segment is
// the run of one (band, query block) inside one CTA's range; each segment
// writes one partial list per epilogue set, at slot
// (band * span + (cta - first CTA of the (band, query block) run)) * nsets + set.
struct Walk {
  int64_t work;   // qblocks * tiles
  int grid;       // CTAs
  int tiles;      // point tiles of BN
  int qblocks;    // query blocks of BM
  int band_tiles; // tiles per band (== tiles: one band)
  int nbands;
  int span;       // most CTAs any (band, query block) run touches
  int qrows;      // query rows per query block (BM, or 2 BM for CTA pairs)
};

__host__ __device__ __forceinline__ int band_len(const Walk& w, int b) {
  return b == w.nbands - 1 ? w.tiles - b * w.band_tiles : w.band_tiles;
}
// first item of the (band b, query block qb) run
__host__ __device__ __forceinline__ int64_t run_begin(const Walk& w, int b, int qb) {
  return (int64_t)b * w.qblocks * w.band_tiles + (int64_t)qb * band_len(w, b);
}
// (query block, tile, band) of item i
__host__ __device__ __forceinline__ void item_pos(const Walk& w, int64_t i, int& qb, int& t, int& b) {
  if (w.nbands == 1) {
    qb = (int)(i / w.tiles);
    t = (int)(i % w.tiles);
    b = 0;
    return;
  }
  const int64_t per = (int64_t)w.qblocks * w.band_tiles;
  b = (int)(i / per);
  if (b > w.nbands - 1) b = w.nbands - 1;
  const int64_t r = i - (int64_t)b * per;
  const int tb = band_len(w, b);
  qb = (int)(r / tb);
  t = b * w.band_tiles + (int)(r % tb);
}

// Work item of a segmented pass (many independent point sets stored back to
// back, each searched against itself): a 128-row block of one set's rows
// against a 256-point tile of the same set's points.  Columns at or past
// `tend` and rows at or past `qend` belong to other sets and are masked.
// The items of one block are contiguous; `run_first` is the first of them.
struct TileItem {
  int64_t q0, qend;   // first row of the block; end of its set's rows
  int64_t t0, tend;   // first point of the tile; end of its set's points
  int64_t run_first;  // first item of this block's run
};

// a block's run of items: first item and count (segmented merge)
struct RunInfo {
  int64_t first, len;
};

struct MainArgs {
  int64_t nq, n;
  int d, dp, nkb;     // dp: main operand columns (zero-padded); nkb: K-stages per tile
  int augx;           // norm-folded form: first fold column (within the last stage); 0 = none
  Walk w;
  const TileItem* titems;  // segmented pass (NULL: the banded walk of `w`)
  const float* qscale;     // FP8 form: per query row, 1/f of its e4m3 scaling (NULL otherwise)
  const float* bscale;     // FP8 form: per point, 1/f (row p * bstride)
  int smax;           // partial-list slots per query
  int L;              // list capacity (32)
  int depth;          // admission depth = k + margin (<= L)
  const RowInfo* qinfo;
  const RowInfo* binfo;
  const float* bnorm; // ||p~||^2 of the points, contiguous
  int64_t bstride;    // point p of this launch is row p * bstride of binfo / bnorm (sampled passes)
  const float* seed;  // per query: admit only est' below this (NULL = no seed)
  uint64_t* partial;  // [nq][smax][L]
  int* err;
  int seedmode;       // keep the SEED_DEPTH smallest 32-column chunk minima instead of points
  int f16;            // FP16 main columns: their MMAs read FP16 (the fold step stays BF16)
};

// What one item means for the kernel's roles: rows [q0, qend), points
// [c0, cend), and where its block's run starts (segment identity and slot).
struct ItemView {
  int64_t q0, qend, c0, cend, run_first;
  int slot_base;  // band * span (banded walk), 0 (segmented)
};

__device__ __forceinline__ ItemView view_item(const MainArgs& a, int64_t item, int qrows) {
  ItemView v;
  if (a.titems) {
    const TileItem ti = a.titems[item];
    v.q0 = ti.q0;
    v.qend = ti.qend;
    v.c0 = ti.t0;
    v.cend = ti.tend;
    v.run_first = ti.run_first;
    v.slot_base = 0;
  } else {
    int qb, t, band;
    item_pos(a.w, item, qb, t, band);
    v.q0 = (int64_t)qb * qrows;
    v.qend = a.nq;
    v.c0 = (int64_t)t * BN;
    v.cend = a.n;
    v.run_first = run_begin(a.w, band, qb);
    v.slot_base = band * a.w.span;
  }
  return v;
}

// a * b / c for non-negative operands, without 128-bit division (a software
// routine of hundreds of instructions) unless the product needs 64 bits
__device__ __forceinline__ int64_t muldiv_nn(int64_t a, int64_t b, int64_t c) {
  const uint64_t ua = (uint64_t)a, ub = (uint64_t)b, uc = (uint64_t)c;
  if (__umul64hi(ua, ub) != 0) return (int64_t)((__int128)a * b / c);
  const uint64_t p = ua * ub;
  if (((p | uc) >> 32) == 0) return (int64_t)((uint32_t)p / (uint32_t)uc);
  return (int64_t)(p / uc);
}

__device__ __forceinline__ int64_t chunk_begin(int c, int64_t work, int grid) {
  return muldiv_nn(c, work, grid);
}

// Step s of CTA c's walk over its range [b0, b1) of items.  With one band
// the walk starts at the range's first item of tile 0 and wraps, so all CTAs
// stream the same point tiles at the same time (L2 reuse); each query block's
// items stay contiguous in the walk.  With several bands the walk is the
// range in order (a band fits in L2).
__device__ __forceinline__ int64_t walk_item(int64_t b0, int64_t b1, const Walk& w, int64_t s) {
  if (w.nbands > 1) return b0 + s;
  const int tiles = w.tiles;
  const int64_t f = ((b0 + tiles - 1) / tiles) * tiles;
  if (f >= b1 || f == b0) return b0 + s;
  const int64_t head = b1 - f;
  return s < head ? f + s : b0 + (s - head);
}

// the CTA whose work range contains item i
__device__ __forceinline__ int cta_of(int64_t i, int64_t work, int grid) {
  int c = (int)muldiv_nn(i, grid, work);
  while (c + 1 < grid && chunk_begin(c + 1, work, grid) <= i) ++c;
  while (c > 0 && chunk_begin(c, work, grid) > i) --c;
  return c;
}

template <int KW>
__device__ __forceinline__ void wl_insert(uint64_t (&Lr)[KW], uint64_t c, int lane) {
  int pos = 0;
#pragma unroll
  for (int s = 0; s < KW; ++s) pos += __popc(__ballot_sync(FULL, Lr[s] < c));
  uint64_t up[KW], last[KW];
#pragma unroll
  for (int s = 0; s < KW; ++s) {
    up[s] = __shfl_up_sync(FULL, Lr[s], 1);
    last[s] = __shfl_sync(FULL, Lr[s], 31);
  }
#pragma unroll
  for (int s = 0; s < KW; ++s) {
    const int e = s * 32 + lane;
    uint64_t shifted = up[s];
    if (lane == 0) shifted = (s == 0) ? KEY_NONE : last[s > 0 ? s - 1 : 0];
    if (e > pos) Lr[s] = shifted;
    else if (e == pos) Lr[s] = c;
  }
}

// a[i] for a run-time i without local memory
template <int N>
__device__ __forceinline__ float pick(const float (&a)[N], int i) {
  float r = a[0];
#pragma unroll
  for (int u = 1; u < N; ++u) r = i == u ? a[u] : r;
  return r;
}

// ascending bitonic sort of one key per lane across the warp
__device__ __forceinline__ uint64_t warp_sort32(uint64_t v, int lane) {
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const uint64_t o = __shfl_xor_sync(FULL, (unsigned long long)v, j);
      const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
      v = keep_min ? (o < v ? o : v) : (o > v ? o : v);
    }
  }
  return v;
}

// A row's list: the `depth` smallest keys seen, unsorted in shared memory
// (entry e at list[e * BM]).  While it fills (nfill < depth) a key takes the
// next slot and the threshold stays the row's seed key.  Once full, the
// threshold is the largest entry (slot lslot); the entries form LGROUPS
// groups of 8 whose maxima (and slots) stay in registers, so a new key that
// replaces the largest entry costs a rescan of its group (8 independent
// loads) and a 4-way compare instead of a rescan of all `depth` entries
// (GROUPED: the many-set pass, where rows admit many candidates; measured
// slower on the seeded single-set passes, so those keep the plain rescan).
constexpr int LGROUPS = 4;             // LIST / 8
constexpr int GROUPED_MIN_DEPTH = 24;  // single-set passes use the groups from this list depth

// List rescans compare the keys' distance words only (the high 32 bits, one
// 32-bit load and compare per entry): among entries of equal distance the
// first slot is taken as the largest.  The list then holds `depth` keys of
// the smallest distances with ties broken by slot instead of id, which keeps
// the certificate's premise (every point left out has a distance >= the
// depth-th entry's), so the candidate sets and answers are the same.
constexpr bool LIST_HI_SCAN = true;

__device__ __forceinline__ uint32_t key_hi(const uint64_t* __restrict__ list, int e) {
  return reinterpret_cast<const uint32_t*>(list)[2 * e * BM + 1];  // little-endian: the high word
}

__device__ __forceinline__ void list_group_max(const uint64_t* __restrict__ list, int g, int depth, uint64_t& m,
                                               int& ms) {
  ms = 8 * g;
  if constexpr (LIST_HI_SCAN) {
    uint32_t mh = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = 8 * g + i;
      const uint32_t h = e < depth ? key_hi(list, e) : 0u;
      if (h > mh) {
        mh = h;
        ms = e;
      }
    }
    m = ms < depth ? list[ms * BM] : 0ull;
    return;
  }
  m = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int e = 8 * g + i;
    const uint64_t v = e < depth ? list[e * BM] : 0ull;
    if (v > m) {
      m = v;
      ms = e;
    }
  }
}

template <bool GROUPED>
__device__ __forceinline__ void list_admit(uint64_t* __restrict__ list, uint64_t c, uint64_t& thr_key,
                                           float& thr_est, int& lslot, int& nfill, int depth,
                                           uint64_t (&gmax)[LGROUPS], int (&gidx)[LGROUPS]) {
  if (!(c < thr_key)) return;
  if (!GROUPED) {
    // plain form: the new key replaces the largest entry and all `depth`
    // entries are rescanned (independent loads; cheapest where admissions are
    // rare, e.g. rows with an admission seed)
    if (nfill < depth) {
      list[nfill * BM] = c;  // an empty slot: the threshold stays the seed until the list is full
      if (++nfill < depth) return;
    } else {
      list[lslot * BM] = c;  // the largest entry drops out
    }
    int ms = 0;
    uint64_t m = 0;
    if constexpr (LIST_HI_SCAN) {
      uint32_t mh = 0;
#pragma unroll 8
      for (int e2 = 0; e2 < depth; ++e2) {
        const uint32_t h = key_hi(list, e2);
        if (h > mh) {
          mh = h;
          ms = e2;
        }
      }
      m = list[ms * BM];
    } else {
#pragma unroll 8
      for (int e2 = 0; e2 < depth; ++e2) {
        const uint64_t v2 = list[e2 * BM];
        if (v2 > m) {
          m = v2;
          ms = e2;
        }
      }
    }
    lslot = ms;
    thr_key = m;
    thr_est = key_dist(thr_key);
    return;
  }
  if (nfill < depth) {
    list[nfill * BM] = c;  // an empty slot: the threshold stays the seed until the list is full
    if (++nfill < depth) return;
#pragma unroll
    for (int g = 0; g < LGROUPS; ++g) list_group_max(list, g, depth, gmax[g], gidx[g]);
  } else {
    list[lslot * BM] = c;  // the largest entry drops out
    const int g = lslot >> 3;
    uint64_t m;
    int ms;
    list_group_max(list, g, depth, m, ms);
#pragma unroll
    for (int gg = 0; gg < LGROUPS; ++gg)
      if (gg == g) {
        gmax[gg] = m;
        gidx[gg] = ms;
      }
  }
  uint64_t m = gmax[0];
  int ms = gidx[0];
#pragma unroll
  for (int g = 1; g < LGROUPS; ++g)
    if (gmax[g] > m) {
      m = gmax[g];
      ms = gidx[g];
    }
  lslot = ms;
  thr_key = m;
  thr_est = key_dist(thr_key);
}

// One 32-column chunk of the epilogue.  Lane r owns row r of the warp's 32
// rows: v holds the row's 32 accumulators of the chunk; lane j's nbv is the
// norm of the chunk's point j (read by shuffle).  The row's list lives in
// shared memory, entry e at mylist[e * BM], unsorted, filled in slot order
// (nfill slots in use); lslot is the slot of its largest entry and thr_key
// that entry, or the row's seed key (seed est', id 0) while the list has an
// empty slot, and thr_est that key's est'.  The common
// case -- no column of any row below its threshold -- costs a shuffle, an FMA
// and a min per value and one vote; a lane with candidates admits them one by
// one: the new key replaces the largest entry and the `depth` entries are
// rescanned for the new largest (independent loads, conflict-free while the
// lanes run in step; a sorted insert would be a chain of dependent
// shared-memory loads).
template <bool FP8, bool GROUPED>
__device__ __forceinline__ void epi_chunk(const uint32_t (&v)[32], float nbv, float csv, float rs,
                                          uint64_t* __restrict__ mylist,
                                          uint64_t& thr_key, float& thr_est, int& lslot, int& nfill,
                                          uint32_t col0, int depth, uint64_t (&gmax)[LGROUPS],
                                          int (&gidx)[LGROUPS]) {
  // est' = ||p~||^2 - 2 q~.p~; in the FP8 form the accumulator holds the sum of
  // e4m3 products and -2 (1/f_q) (1/f_p) = rs * csv (a power of two) rescales it
  float e[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    const float coef = FP8 ? rs * __shfl_sync(FULL, csv, j) : -2.0f;
    e[j] = __fmaf_rn(coef, __uint_as_float(v[j]), __shfl_sync(FULL, nbv, j));
  }
  float m4[8];
#pragma unroll
  for (int j4 = 0; j4 < 8; ++j4)
    m4[j4] = fminf(fminf(e[4 * j4 + 0], e[4 * j4 + 1]), fminf(e[4 * j4 + 2], e[4 * j4 + 3]));
  const float mn = fminf(fminf(fminf(m4[0], m4[1]), fminf(m4[2], m4[3])),
                         fminf(fminf(m4[4], m4[5]), fminf(m4[6], m4[7])));
  if (!__any_sync(FULL, mn < thr_est)) return;
  if (mn < thr_est) {
    unsigned mask = 0;
#pragma unroll
    for (int j = 0; j < 32; ++j) mask |= (e[j] < thr_est ? 1u : 0u) << j;
    while (mask) {
      const int j = __ffs(mask) - 1;
      mask &= mask - 1;
      float val = e[0];
#pragma unroll
      for (int u = 1; u < 32; ++u) val = j == u ? e[u] : val;
      const uint64_t c = make_key(val, col0 + (uint32_t)j);
      list_admit<GROUPED>(mylist, c, thr_key, thr_est, lslot, nfill, depth, gmax, gidx);
    }
  }
}

// Seed-pass form of epi_chunk: the row keeps, in registers and sorted, the
// SEED_DEPTH smallest minima of its 32-column chunks (keyed by the chunk's
// first column, so each comes from a distinct point).  SEED_DEPTH distinct
// points lie at or below the SEED_DEPTH-th of them, so it bounds the row's
// SEED_DEPTH-th smallest est' over the sample from above -- all a seed needs.
template <bool FP8>
__device__ __forceinline__ void seed_chunk(const uint32_t (&v)[32], float nbv, float csv, float rs,
                                           uint64_t (&top)[SEED_DEPTH], uint32_t col0) {
  float m4[8];
#pragma unroll
  for (int j4 = 0; j4 < 8; ++j4) {
    float e4[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = 4 * j4 + u;
      const float coef = FP8 ? rs * __shfl_sync(FULL, csv, j) : -2.0f;
      e4[u] = __fmaf_rn(coef, __uint_as_float(v[j]), __shfl_sync(FULL, nbv, j));
    }
    m4[j4] = fminf(fminf(e4[0], e4[1]), fminf(e4[2], e4[3]));
  }
  const float mn = fminf(fminf(fminf(m4[0], m4[1]), fminf(m4[2], m4[3])),
                         fminf(fminf(m4[4], m4[5]), fminf(m4[6], m4[7])));
  uint64_t c = make_key(mn, col0);
  if (c < top[SEED_DEPTH - 1]) {
    top[SEED_DEPTH - 1] = c;
#pragma unroll
    for (int i = SEED_DEPTH - 1; i > 0; --i) {
      const uint64_t lo = top[i - 1], hi = top[i];
      if (hi < lo) {
        top[i - 1] = hi;
        top[i] = lo;
      }
    }
  }
}

// In the plain-rescan instances, candidates of the norm-folded epilogue wait
// in a per-lane register stack of ADMIT_Q keys and are admitted after the
// tile's last chunk, when the lanes of a warp drain their stacks together
// (admissions in step, instead of one lane at a time per chunk); a full stack
// drains at once.  The list ends with the same keys: list_admit re-tests each
// key against the row's current threshold, and a top-`depth` set does not
// depend on the order.  Measured: the 60k x 784 self graph's main pass 4.40 ->
// 4.27 ms with a stack of 2 (4 or 8: slower).  The grouped-maxima instances
// serve the many-set segmented pass, whose rows admit many candidates per
// tile against a threshold that a stack leaves stale until the tile ends
// (42.8 -> 54.7 ms), and admit at once.
constexpr int ADMIT_Q = 2;
// the epilogue takes each 16-column half-chunk's largest accumulator from the
// max-reduction form of the TMEM load
constexpr bool LD_RED = true;
// single-matrix passes of at most this many K-stages per tile run the
// three-stage, two-set instance (their MMA per tile is short against the
// epilogue's work)
constexpr int SHORT_K_STAGES = 3;
// points per work item of the batched form's exact fallback scan
constexpr int64_t FB_CHUNK = 4096;

// v[j] for a lane-varying j in [0, 32): a five-level select tree on the bits of j
__device__ __forceinline__ uint32_t select32(const uint32_t (&v)[32], int j) {
  uint32_t t16[16], t8[8], t4[4];
#pragma unroll
  for (int i = 0; i < 16; ++i) t16[i] = (j & 1) ? v[2 * i + 1] : v[2 * i];
#pragma unroll
  for (int i = 0; i < 8; ++i) t8[i] = (j & 2) ? t16[2 * i + 1] : t16[2 * i];
#pragma unroll
  for (int i = 0; i < 4; ++i) t4[i] = (j & 4) ? t8[2 * i + 1] : t8[2 * i];
  const uint32_t a = (j & 8) ? t4[1] : t4[0], b = (j & 8) ? t4[3] : t4[2];
  return (j & 16) ? b : a;
}

template <bool GROUPED>
__device__ __forceinline__ void admit_drain(uint64_t (&dq)[ADMIT_Q], int& dn, uint64_t* __restrict__ mylist,
                                            uint64_t& thr_key, float& thr_est, int& lslot, int& nfill, int depth,
                                            uint64_t (&gmax)[LGROUPS], int (&gidx)[LGROUPS]) {
  while (dn > 0) {
    const uint64_t c = dq[0];
#pragma unroll
    for (int i = 0; i + 1 < ADMIT_Q; ++i) dq[i] = dq[i + 1];
    --dn;
    list_admit<GROUPED>(mylist, c, thr_key, thr_est, lslot, nfill, depth, gmax, gidx);
  }
}

// Norm-folded epilogue (BF16 form).  Every operand row carries, after its
// main columns, a 24-column block [P0 P1 P2 1 1 1 0 0 | 1 1 1 P0 P1 P2 0 0 |
// 0 ...] with P0 + P1 + P2 = -||x~||^2 / 2 exactly (three BF16 pieces of an
// FP32 value); one extra K-step reads the query block at its first column and
// the point block eight columns later, so it adds -(||q~||^2 + ||p~||^2) / 2 and the accumulator
// holds acc = q~.p~ - (||q~||^2 + ||p~||^2) / 2.  The estimate is then
// est = -2 acc = ||q~ - p~||^2 (an exact scaling): the chunk's smallest est is
// -2 max(acc), with no per-column norm.  With LD_RED the TMEM load returns
// that max (tcgen05.ld.red); a chunk with columns j >= nvalid (past the
// tile's last point, or in another point set) masks them and takes the max
// by a tree of FMNMX.
__device__ __forceinline__ float chunk_max(uint32_t (&v)[32], int nvalid, float rmax) {
  if (LD_RED && nvalid == 32) return rmax;
  if (nvalid < 32) {
#pragma unroll
    for (int j = 0; j < 32; ++j)
      if (j >= nvalid) v[j] = 0xFF800000u;  // -inf: est = +inf
  }
  float m4[8];
#pragma unroll
  for (int j4 = 0; j4 < 8; ++j4)
    m4[j4] = fmaxf(fmaxf(__uint_as_float(v[4 * j4 + 0]), __uint_as_float(v[4 * j4 + 1])),
                   fmaxf(__uint_as_float(v[4 * j4 + 2]), __uint_as_float(v[4 * j4 + 3])));
  return fmaxf(fmaxf(fmaxf(m4[0], m4[1]), fmaxf(m4[2], m4[3])), fmaxf(fmaxf(m4[4], m4[5]), fmaxf(m4[6], m4[7])));
}

template <bool GROUPED>
__device__ __forceinline__ void epi_chunk_fold(uint32_t (&v)[32], int nvalid, float rmax,
                                               uint64_t* __restrict__ mylist, uint64_t& thr_key, float& thr_est,
                                               int& lslot, int& nfill, uint32_t col0, int depth,
                                               uint64_t (&gmax)[LGROUPS], int (&gidx)[LGROUPS],
                                               uint64_t (&dq)[ADMIT_Q], int& dn) {
  const float mn = -2.0f * chunk_max(v, nvalid, rmax);
  if (!__any_sync(FULL, mn < thr_est)) return;
  if (mn < thr_est) {
    unsigned mask = 0;
#pragma unroll
    for (int j = 0; j < 32; ++j) mask |= (-2.0f * __uint_as_float(v[j]) < thr_est ? 1u : 0u) << j;
    while (mask) {
      const int j = __ffs(mask) - 1;
      mask &= mask - 1;
      const uint64_t c = make_key(-2.0f * __uint_as_float(select32(v, j)), col0 + (uint32_t)j);
      if constexpr (!GROUPED) {
        if (!(c < thr_key)) continue;
        if (dn == ADMIT_Q) admit_drain<GROUPED>(dq, dn, mylist, thr_key, thr_est, lslot, nfill, depth, gmax, gidx);
#pragma unroll
        for (int i = ADMIT_Q - 1; i > 0; --i) dq[i] = dq[i - 1];
        dq[0] = c;
        ++dn;
      } else {
        list_admit<GROUPED>(mylist, c, thr_key, thr_est, lslot, nfill, depth, gmax, gidx);
      }
    }
  }
}

// Seed-pass form of epi_chunk_fold (the chunk minimum of est = -2 max(acc)).
__device__ __forceinline__ void seed_chunk_fold(uint32_t (&v)[32], int nvalid, float rmax,
                                                uint64_t (&top)[SEED_DEPTH], uint32_t col0) {
  uint64_t c = make_key(-2.0f * chunk_max(v, nvalid, rmax), col0);
  if (c < top[SEED_DEPTH - 1]) {
    top[SEED_DEPTH - 1] = c;
#pragma unroll
    for (int i = SEED_DEPTH - 1; i > 0; --i) {
      const uint64_t lo = top[i - 1], hi = top[i];
      if (hi < lo) {
        top[i - 1] = hi;
        top[i] = lo;
      }
    }
  }
}

// Shared-memory footprint of k2_main<CAP, NSETS>.
template <bool PAIR>
__host__ __device__ constexpr size_t k2_smem_bytes(int cap, int nsets, int stages = Stg<PAIR>::N) {
  return 1024 /* alignment */ + (size_t)stages * Stg<PAIR>::BYTES +
         (size_t)nsets * BM * cap * 8 /* lists */ + (2 * stages + 4) * 8 + 16;
}
static_assert(k2_smem_bytes<false>(32, 1) <= 232448 && k2_smem_bytes<false>(16, 2) <= 232448, "k2_main shared memory");
static_assert(k2_smem_bytes<true>(32, 1) <= 232448 && k2_smem_bytes<true>(16, 2) <= 232448, "k2_main shared memory");
static_assert(k2_smem_bytes<false>(24, 2, 3) <= 232448 && k2_smem_bytes<false>(32, 2, 3) <= 232448,
              "k2_main shared memory");

// The list keys are (est', id) with est' = ||p~||^2 - 2 q~.p~ (the row's own
// ||q~||^2 is left out: it does not change the row's order).  A point is
// admitted when its key is below the row's `depth`-th entry, so the first
// `depth` entries of a list are exactly the segment's `depth` smallest keys and
// every point left out has est' >= the depth-th entry (the certificate's
// premise); entries past `depth` are admitted points kept while space lasts.
//
// Warps: 0 = TMA producer, 1 = MMA issuer (and TMEM owner), then NSETS sets
// of 4 epilogue warps.  With two sets, set h drains columns [128h, 128h + 128)
// of every tile, so a TMEM buffer is free again after half a tile of epilogue
// work (the MMA of the tile after next reuses it one tile-time later); each
// set keeps its own lists and writes them to its own partial slot.  A list is
// sorted when it is written out.
//
// PAIR: the kernel runs as clusters of two CTAs on two SMs that compute one
// 256-query x 256-point tile with tcgen05.mma.cta_group::2 (M = 256): CTA
// rank r stages query rows [128r, 128r + 128) of the pair's block and point
// rows [128r, 128r + 128) of the tile, so each SM writes and feeds the tensor
// core 32 KB per K-stage instead of 48 KB; the even CTA's thread issues the
// MMAs, both CTAs' TMA loads complete on the even CTA's full barrier, its
// commits arrive on the stage and accumulator barriers of both CTAs, and both
// CTAs' epilogue warps release an accumulator on the even CTA's barrier.  The
// work unit (a walk item) is then one pair tile and `a.w.grid` counts pairs.
template <int CAP, int NSETS, bool PAIR, bool FP8, bool GROUPED = false, int NST = 0>
__global__ void __launch_bounds__(64 + 128 * NSETS, 1)
    k2_main(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
            MainArgs a) {
  constexpr int NEPI = 4 * NSETS;
  constexpr int EPS = FP8 ? 128 : BK;  // operand elements per 128-byte stage row
  constexpr int EPK = EPS / 4;         // elements per MMA (K): 16 BF16 or 32 E4M3
  constexpr int STAGES = NST > 0 ? NST : Stg<PAIR>::N;
  constexpr int STAGE_BYTES = Stg<PAIR>::BYTES;
  constexpr int QROWS = PAIR ? 2 * BM : BM;  // query rows of one work unit
  extern __shared__ __align__(1024) uint8_t k2_smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(k2_smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* stage_base = smem;                                                   // STAGES * STAGE_BYTES
  uint64_t* lists = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);  // [NSETS][CAP][BM]
  uint64_t* bars = lists + NSETS * BM * CAP;
  uint64_t* full_bar = bars;
  uint64_t* empty_bar = bars + STAGES;
  uint64_t* tfull_bar = bars + 2 * STAGES;
  uint64_t* tempty_bar = bars + 2 * STAGES + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 4);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = PAIR ? ptx::cluster_ctarank() : 0u;
  const int cta = PAIR ? (int)ptx::cluster_id_x() : (int)blockIdx.x;  // work unit: pair or CTA
  const int64_t it0 = chunk_begin(cta, a.w.work, a.w.grid);
  const int64_t it1 = chunk_begin(cta + 1, a.w.work, a.w.grid);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full_bar[s], 1);
      ptx::mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(&tfull_bar[b], 1);
      // one arrival per epilogue warp of both CTAs (PAIR) or per epilogue thread
      ptx::mbar_init(&tempty_bar[b], PAIR ? 2 * NEPI : NEPI * 32);
    }
    ptx::fence_mbar_init();
    ptx::prefetch_tensormap(&mapA);
    ptx::prefetch_tensormap(&mapB);
  }
  if (warp == 1) {
    if (PAIR) {
      ptx::tmem_alloc_pair(tmem_slot, TMEM_COLS);
      ptx::tmem_relinquish_pair();
    } else {
      ptx::tmem_alloc(tmem_slot, TMEM_COLS);
      ptx::tmem_relinquish();
    }
  }
  ptx::tc_fence_before();
  if (PAIR)
    ptx::cluster_sync();  // both CTAs' barriers initialised before any cross-CTA arrival
  else
    __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      const uint32_t full0 = PAIR ? ptx::mapa(ptx::smem_u32(&full_bar[0]), 0) : 0u;  // even CTA's full_bar[0]
      for (int64_t st = 0; st < it1 - it0 && ok; ++st) {
        const ItemView v = view_item(a, walk_item(it0, it1, a.w, st), QROWS);
        for (int kb = 0; kb < a.nkb; ++kb, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1;
          if (!ptx::mbar_wait(&empty_bar[s], ph ^ 1, a.err, ERR_TIMEOUT_PRODUCER)) {
            ok = false;
            break;
          }
          uint8_t* sa = stage_base + s * STAGE_BYTES;
          uint8_t* sb = sa + A_STAGE_BYTES;
          const int xa = kb * EPS, xb = kb * EPS;
          if (PAIR) {
            if (rank == 0) ptx::mbar_arrive_expect_tx(&full_bar[s], 2 * STAGE_BYTES);
            const uint32_t fb = full0 + (uint32_t)s * 8u;
            ptx::tma_load_2d_pair(sa, &mapA, fb, xa, (int)v.q0 + (int)rank * BM);
            ptx::tma_load_2d_pair(sb, &mapB, fb, xb, (int)v.c0 + (int)rank * Stg<PAIR>::B_ROWS);
          } else {
            ptx::mbar_arrive_expect_tx(&full_bar[s], STAGE_BYTES);
            ptx::tma_load_2d(sa, &mapA, &full_bar[s], xa, (int)v.q0);
            ptx::tma_load_2d(sb, &mapB, &full_bar[s], xb, (int)v.c0);
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0 && rank == 0) {
      constexpr uint32_t idesc = FP8 ? ptx::idesc_e4m3_f32(QROWS, BN) : ptx::idesc_bf16_f32(QROWS, BN);
      // the main K-steps' operand type: FP16 in the FP16 form (both operands, as
      // every kind::f16 MMA needs), else the form's own; the fold step is BF16
      const uint32_t idesc_main = (!FP8 && a.f16) ? ptx::idesc_f16_f32(QROWS, BN) : idesc;
      uint32_t it = 0;
      int tcount = 0;
      bool ok = true;
      for (int64_t st = 0; st < it1 - it0 && ok; ++st, ++tcount) {
        const int buf = tcount & 1;
        const uint32_t tph = (tcount >> 1) & 1;
        const bool freed = PAIR ? ptx::mbar_wait_cluster(&tempty_bar[buf], tph ^ 1, a.err, ERR_TIMEOUT_MMA)
                                : ptx::mbar_wait(&tempty_bar[buf], tph ^ 1, a.err, ERR_TIMEOUT_MMA);
        if (!freed) break;
        ptx::tc_fence_after();
        const uint32_t dcol = tmem_base + (uint32_t)(buf * BN);
        for (int kb = 0; kb < a.nkb; ++kb, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1;
          if (!ptx::mbar_wait(&full_bar[s], ph, a.err, ERR_TIMEOUT_MMA)) {
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          const uint32_t sa = ptx::smem_u32(stage_base + s * STAGE_BYTES);
          const uint32_t sb = sa + A_STAGE_BYTES;
          const int rem = a.dp - kb * EPS;  // main (zero-padded) columns left
          const int ksteps = rem >= EPS ? 4 : (rem > 0 ? (rem + EPK - 1) / EPK : 0);
          for (int kk = 0; kk < ksteps; ++kk) {  // each MMA covers 32 bytes of K
            const uint64_t ad = ptx::sw128_desc(sa + kk * 32);
            const uint64_t bd = ptx::sw128_desc(sb + kk * 32);
            if (PAIR)
              ptx::mma_f16_pair(dcol, ad, bd, idesc_main, (kb > 0 || kk > 0) ? 1u : 0u);
            else if (FP8)
              ptx::mma_f8(dcol, ad, bd, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
            else
              ptx::mma_f16(dcol, ad, bd, idesc_main, (kb > 0 || kk > 0) ? 1u : 0u);
          }
          if (!FP8 && a.augx > 0 && kb == a.augx / EPS) {
            // the norm-fold K-step: the query block at its first column, the
            // point block eight columns (16 bytes) later -- inside the same
            // 128-byte swizzled row (fold columns start at 0, 16 or 32 of the stage)
            const int ka = (a.augx % EPS) / 16;
            const uint64_t ad = ptx::sw128_desc(sa + ka * 32);
            const uint64_t bd = ptx::sw128_desc(sb + ka * 32 + 16);
            if (PAIR)
              ptx::mma_f16_pair(dcol, ad, bd, idesc, 1u);
            else
              ptx::mma_f16(dcol, ad, bd, idesc, 1u);
          }
          // frees the stage (in both CTAs of a pair) when these MMAs finish
          if (PAIR)
            ptx::mma_commit_pair_mc(&empty_bar[s], 0x3);
          else
            ptx::mma_commit(&empty_bar[s]);
        }
        if (ok) {
          if (PAIR)
            ptx::mma_commit_pair_mc(&tfull_bar[buf], 0x3);
          else
            ptx::mma_commit(&tfull_bar[buf]);
        }
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int ew = warp - 2;          // 0 .. NEPI-1
    const int set = ew >> 2;          // which column half this warp drains (two sets)
    const int quad = warp & 3;        // TMEM lane quadrant this warp may access
    const int row = quad * 32 + lane; // this lane's row of the 128-query tile
    constexpr int CPS = (BN / 32) / NSETS;  // 32-column chunks per set and tile
    const int cbeg = set * CPS, cend = cbeg + CPS;
    uint64_t* setlists = lists + (size_t)set * CAP * BM;      // entry e of row r at setlists[e * BM + r]
    uint64_t* mylist = setlists + row;
    const float INF = __int_as_float(0x7F800000);
    uint64_t seed_key = KEY_NONE;
    uint64_t thr_key = KEY_NONE;
    float thr_est = INF;
    int lslot = 0, nfill = 0;
    uint64_t dq[ADMIT_Q];  // candidates waiting for the end of the tile (dn of them)
    int dn = 0;
    uint64_t gmax[LGROUPS];  // the list's group maxima and their slots (list_admit)
    int gidx[LGROUPS];
#pragma unroll
    for (int g = 0; g < LGROUPS; ++g) {
      gmax[g] = 0;
      gidx[g] = 8 * g;
    }
    uint64_t top[SEED_DEPTH];
#pragma unroll
    for (int i = 0; i < SEED_DEPTH; ++i) top[i] = KEY_NONE;
    int tcount = 0;
    int64_t cur_run = -1, cur_q0 = 0, cur_qend = 0;
    int seg_slot = 0;
    bool alive = true;

    for (int e = 0; e < CAP; ++e) mylist[e * BM] = KEY_NONE;

    // write the warp's 32 row lists of a finished segment, each sorted across the lanes
    const int64_t row0 = (int64_t)rank * BM;  // this CTA's rows inside a work unit's query block
    const uint32_t tempty0 = PAIR ? ptx::mapa(ptx::smem_u32(&tempty_bar[0]), 0) : 0u;
    auto flush = [&](int64_t q0_, int64_t qend_, int slot_) {
      if (a.seedmode) {
        const int64_t gq = q0_ + row0 + row;
        if (gq < qend_) {
          uint64_t* dst = a.partial + (gq * a.smax + slot_) * LIST;
#pragma unroll
          for (int i = 0; i < SEED_DEPTH; ++i) dst[i] = top[i];
        }
#pragma unroll
        for (int i = 0; i < SEED_DEPTH; ++i) top[i] = KEY_NONE;
        return;
      }
      __syncwarp();
      const uint64_t* wl = setlists + quad * 32;
      for (int r = 0; r < 32; ++r) {
        uint64_t v = lane < CAP ? wl[lane * BM + r] : KEY_NONE;
        v = warp_sort32(v, lane);
        const int64_t gq = q0_ + row0 + quad * 32 + r;
        if (gq < qend_ && lane < CAP) a.partial[(gq * a.smax + slot_) * LIST + lane] = v;
      }
      __syncwarp();
    };

    // point norms, lane j holding column 32 i + j of the tile in nbc[i]: the
    // current tile's in nbc, the next tile's fetched into nbn one tile ahead
    float nbn[BN / 32], nbc[BN / 32];
    float csn[FP8 ? BN / 32 : 1], csc[FP8 ? BN / 32 : 1];  // FP8: -2 (1/f) of the columns
    float rs = 1.0f;                                        // FP8: 1/f of this lane's row
    // (the BF16 form folds the norms into the MMA and needs none of these)
    auto fetch_norms = [&](int64_t st_) {
      if constexpr (FP8) {
        const ItemView v_ = view_item(a, walk_item(it0, it1, a.w, st_), QROWS);
#pragma unroll
        for (int i = 0; i < BN / 32; ++i) {
          const int64_t col = v_.c0 + lane + 32 * i;
          nbn[i] = col < v_.cend ? __ldg(&a.bnorm[col * a.bstride]) : INF;
          csn[i] = col < v_.cend ? -2.0f * __ldg(&a.bscale[col * a.bstride]) : 0.0f;
        }
      }
    };
    if (it1 > it0) fetch_norms(0);
    for (int64_t st = 0; st < it1 - it0; ++st, ++tcount) {
      const ItemView v = view_item(a, walk_item(it0, it1, a.w, st), QROWS);
      if (v.run_first != cur_run) {
        if (cur_run >= 0) {
          // flush the finished segment's lists (every set, even one that saw no candidate)
          flush(cur_q0, cur_qend, seg_slot);
          for (int e = 0; e < CAP; ++e) mylist[e * BM] = KEY_NONE;
        }
        cur_run = v.run_first;
        cur_q0 = v.q0;
        cur_qend = v.qend;
        seg_slot = (v.slot_base + (cta - cta_of(v.run_first, a.w.work, a.w.grid))) * NSETS + set;
        const int64_t gq = v.q0 + row0 + row;
        seed_key = (a.seed != nullptr && gq < v.qend) ? make_key(a.seed[gq], 0u) : KEY_NONE;
        if constexpr (FP8) rs = gq < v.qend ? __ldg(&a.qscale[gq]) : 0.0f;
        thr_key = seed_key;
        thr_est = thr_key == KEY_NONE ? INF : key_dist(thr_key);
        lslot = 0;
        nfill = 0;
      }
      const int buf = tcount & 1;
      const int64_t col0 = v.c0;
      if constexpr (FP8) {
#pragma unroll
        for (int i = 0; i < BN / 32; ++i) {
          nbc[i] = nbn[i];
          csc[i] = csn[i];
        }
      }
      if (st + 1 < it1 - it0) fetch_norms(st + 1);
      const uint32_t tph = (tcount >> 1) & 1;
      if (alive && !ptx::mbar_wait(&tfull_bar[buf], tph, a.err, ERR_TIMEOUT_EPI)) alive = false;
      alive = __all_sync(FULL, alive);  // the warp leaves together
      if (!alive) break;
      ptx::tc_fence_after();
      const uint32_t taddr = tmem_base + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * BN);
      uint32_t va[32], vb[32];
      float ma[2] = {0.0f, 0.0f}, mb[2] = {0.0f, 0.0f};  // the halves' largest values (LD_RED)
      auto ld_chunk = [&](int ch_, uint32_t (&v_)[32], float (&m_)[2]) {
        if constexpr (!FP8 && LD_RED) {
          ptx::tmem_ld16_max(taddr + ch_ * 32, *reinterpret_cast<uint32_t(*)[16]>(&v_[0]), m_[0]);
          ptx::tmem_ld16_max(taddr + ch_ * 32 + 16, *reinterpret_cast<uint32_t(*)[16]>(&v_[16]), m_[1]);
        } else {
          ptx::tmem_ld16(taddr + ch_ * 32, *reinterpret_cast<uint32_t(*)[16]>(&v_[0]));
          ptx::tmem_ld16(taddr + ch_ * 32 + 16, *reinterpret_cast<uint32_t(*)[16]>(&v_[16]));
        }
      };
      ld_chunk(cbeg, va, ma);
      ptx::tmem_ld_wait();
#pragma unroll 1
      for (int ch = cbeg; ch < cend; ch += 2) {
        // chunk ch is in va; fetch ch+1 into vb while va is processed, and so on
        ld_chunk(ch + 1, vb, mb);
        if constexpr (FP8) {
          const float cs_a = pick(csc, ch);
          if (a.seedmode)
            seed_chunk<FP8>(va, pick(nbc, ch), cs_a, rs, top, (uint32_t)(col0 + ch * 32));
          else
            epi_chunk<FP8, GROUPED>(va, pick(nbc, ch), cs_a, rs, mylist, thr_key, thr_est, lslot, nfill,
                           (uint32_t)(col0 + ch * 32), a.depth, gmax, gidx);
        } else {
          const int nva = (int)min((int64_t)32, v.cend - (col0 + ch * 32));
          if (a.seedmode)
            seed_chunk_fold(va, nva, fmaxf(ma[0], ma[1]), top, (uint32_t)(col0 + ch * 32));
          else
            epi_chunk_fold<GROUPED>(va, nva, fmaxf(ma[0], ma[1]), mylist, thr_key, thr_est, lslot, nfill,
                                    (uint32_t)(col0 + ch * 32), a.depth, gmax, gidx, dq, dn);
        }
        ptx::tmem_ld_wait();
        if (ch + 2 < cend) {
          ld_chunk(ch + 2, va, ma);
        } else {
          // every TMEM read of this tile is done: hand the buffer back before the last chunk
          ptx::tc_fence_before();
          if (PAIR) {
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive_cluster(tempty0 + (uint32_t)buf * 8u);
          } else {
            ptx::mbar_arrive(&tempty_bar[buf]);
          }
        }
        if constexpr (FP8) {
          const float cs_b = pick(csc, ch + 1);
          if (a.seedmode)
            seed_chunk<FP8>(vb, pick(nbc, ch + 1), cs_b, rs, top, (uint32_t)(col0 + (ch + 1) * 32));
          else
            epi_chunk<FP8, GROUPED>(vb, pick(nbc, ch + 1), cs_b, rs, mylist, thr_key, thr_est, lslot, nfill,
                           (uint32_t)(col0 + (ch + 1) * 32), a.depth, gmax, gidx);
        } else {
          const int nvb = (int)min((int64_t)32, v.cend - (col0 + (ch + 1) * 32));
          if (a.seedmode)
            seed_chunk_fold(vb, nvb, fmaxf(mb[0], mb[1]), top, (uint32_t)(col0 + (ch + 1) * 32));
          else
            epi_chunk_fold<GROUPED>(vb, nvb, fmaxf(mb[0], mb[1]), mylist, thr_key, thr_est, lslot, nfill,
                                    (uint32_t)(col0 + (ch + 1) * 32), a.depth, gmax, gidx, dq, dn);
        }
        ptx::tmem_ld_wait();
      }
      // the tile's queued candidates, every lane of the warp at once
      if constexpr (!FP8 && !GROUPED)
        admit_drain<GROUPED>(dq, dn, mylist, thr_key, thr_est, lslot, nfill, a.depth, gmax, gidx);
    }
    if (alive && cur_run >= 0) flush(cur_q0, cur_qend, seg_slot);
  }

  ptx::tc_fence_before();
  __syncthreads();
  if (PAIR) ptx::cluster_sync();  // no CTA leaves while the pair's MMAs may touch its memory
  if (warp == 1) {
    ptx::tc_fence_after();
    if (PAIR)
      ptx::tmem_dealloc_pair(tmem_base, TMEM_COLS);
    else
      ptx::tmem_dealloc(tmem_base, TMEM_COLS);
  }
}

// ---------------------------------------------------------------- merge

// The `depth` smallest keys over the CTA segments of each query (warp per
// query); only the first `depth` entries of every segment list take part.
// Segment g of a query enumerates its slots band by band: the CTAs of the
// (band, query block) run in order, each with its nsets lists.
__global__ void k2_merge(const uint64_t* __restrict__ partial, int64_t nq, int smax, Walk w, int depth,
                         int nsets, uint64_t* __restrict__ out, const RunInfo* __restrict__ runs,
                         const int32_t* __restrict__ row_run) {
  constexpr int L = LIST;
  const int lane = threadIdx.x & 31;
  const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (q >= nq) return;
  // slots of this query, at most 64 bands x span x nsets (checked on the host)
  int nseg = 0;
  int band_first_slot[64], band_nslots[64];
  if (runs) {
    // segmented pass: the row's block run, slots 0 .. (CTAs of the run) x nsets
    const RunInfo ri = runs[row_run[q]];
    const int c0 = cta_of(ri.first, w.work, w.grid);
    const int c1 = cta_of(ri.first + ri.len - 1, w.work, w.grid);
    band_first_slot[0] = 0;
    band_nslots[0] = (c1 - c0 + 1) * nsets;
    nseg = band_nslots[0];
  } else {
    const int qb = (int)(q / w.qrows);
    for (int b = 0; b < w.nbands; ++b) {
      const int64_t r0 = run_begin(w, b, qb);
      const int c0 = cta_of(r0, w.work, w.grid);
      const int c1 = cta_of(r0 + band_len(w, b) - 1, w.work, w.grid);
      band_first_slot[b] = b * w.span * nsets;
      band_nslots[b] = (c1 - c0 + 1) * nsets;
      nseg += band_nslots[b];
    }
  }
  auto slot_of = [&](int g) {
    int b = 0;
    while (g >= band_nslots[b]) {
      g -= band_nslots[b];
      ++b;
    }
    return band_first_slot[b] + g;
  };
  static_assert(LIST == 32, "one list entry per lane");
  uint64_t Lr = lane < depth ? partial[(q * smax + slot_of(0)) * L + lane] : KEY_NONE;
  uint64_t pre[4];  // the next lists, one coalesced load each, issued together
#pragma unroll
  for (int u = 0; u < 4; ++u)
    pre[u] = (1 + u < nseg && lane < depth) ? partial[(q * smax + slot_of(1 + u)) * L + lane] : KEY_NONE;
  for (int g = 1; g < nseg; ++g) {
    uint64_t b;
    if (g <= 4) {
      b = pre[0];
#pragma unroll
      for (int u = 1; u < 4; ++u)
        if (g == 1 + u) b = pre[u];
    } else {
      b = lane < depth ? partial[(q * smax + slot_of(g)) * L + lane] : KEY_NONE;
    }
    // bitonic merge of two ascending lists: against the other list reversed,
    // the lane-wise minima are the 32 smallest keys of both (a bitonic
    // sequence), which five half-cleaner steps sort
    const uint64_t br = __shfl_sync(FULL, (unsigned long long)b, 31 - lane);
    uint64_t m = br < Lr ? br : Lr;
#pragma unroll
    for (int j = 16; j > 0; j >>= 1) {
      const uint64_t o = __shfl_xor_sync(FULL, (unsigned long long)m, j);
      m = (lane & j) ? (o > m ? o : m) : (o < m ? o : m);
    }
    Lr = m;
  }
  out[q * L + lane] = lane < depth ? Lr : KEY_NONE;
}

// ---------------------------------------------------------------- certify + rerank

struct RerankArgs {
  const float* base;
  const float* qs;
  int64_t nq, n;
  int d, L, kreq, metric, depth;
  const float* seed;   // per query admission seed of the main pass (NULL = none)
  const float* scale;  // the est values are in units of scale^2 * distance
  unsigned long long* depth_hist;  // [LIST + 2]: rows by the list depth their certificate needed
  const RowInfo* qinfo;
  const BaseMax* bmax;
  const uint64_t* lists;  // [nq][L] sorted by est
  uint64_t* cand;         // [nq][L] sorted (fp32 distance, id)
  int* cand_count;        // [nq]
  float* floor_val;       // [nq] lower bound of FP32 distances of non-candidates
  int* fb_rows;           // rows that need the FP32 scan
  int* fb_count;
  unsigned long long* cand_total;
  // cosine: the tensor-core pass ran on unit-normalised rows; the candidates
  // are reranked with the FP32 form's cosine on the original rows
  const float* cos_qn;  // [nq] squared norms of the original queries (FP32 form order)
  const float* cos_bn;  // [n]  squared norms of the original points
  float eps_c;          // |FP32 cosine - ||q^ - p^||^2 / 2| bound (rounded up)
  int kdim;             // columns of the tensor-core dot (dp, or 3 dp in the split form; + the fold step)
  int full_est;         // list keys hold est (norm-folded BF16 form), not est' = est - ||q~||^2
  int coop;             // d % 4 == 0 and 16-byte aligned rows: warp-cooperative row loads
};

constexpr int RR_WARPS = 2;   // warps (queries) per rerank block
constexpr int RR_CH = 64;     // dimensions per staged chunk
constexpr int RR_STR = 68;    // staged row stride (floats): 16-byte aligned rows

// sequential difference-form sum over dimensions 0..d-1 (the FP32 form's order)
__device__ __forceinline__ float fp32_dist_row(const float* __restrict__ x,
                                               const float* __restrict__ y, int d, int metric) {
  float s = 0.0f;
  int c = 0;
  if ((d & 3) == 0 && ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) == 0) {
    const float4* x4 = reinterpret_cast<const float4*>(x);
    const float4* y4 = reinterpret_cast<const float4*>(y);
    // two float4 per step: each lane reads whole 32-byte sectors of its row
#pragma unroll 2
    for (; c < (d >> 2); ++c) {
      const float4 a = __ldg(x4 + c), b = __ldg(y4 + c);
      float t = __fsub_rn(a.x, b.x);
      s = __fmaf_rn(t, t, s);
      t = __fsub_rn(a.y, b.y);
      s = __fmaf_rn(t, t, s);
      t = __fsub_rn(a.z, b.z);
      s = __fmaf_rn(t, t, s);
      t = __fsub_rn(a.w, b.w);
      s = __fmaf_rn(t, t, s);
    }
    c = d;
  }
  for (; c < d; ++c) {
    const float t = __fsub_rn(x[c], y[c]);
    s = __fmaf_rn(t, t, s);
  }
  return metric == MANN_METRIC_EUCLIDEAN ? __fsqrt_rn(s) : s;
}

// the FP32 form's cosine: sequential dot, then 1 - dot / (sqrt(|q|^2) sqrt(|p|^2)), clamped at 0
__device__ __forceinline__ float fp32_cos_row(const float* __restrict__ x, const float* __restrict__ y, int d,
                                              float xn, float yn) {
  float s = 0.0f;
  for (int c = 0; c < d; ++c) s = __fmaf_rn(__ldg(x + c), __ldg(y + c), s);
  const float den = __fmul_rn(__fsqrt_rn(xn), __fsqrt_rn(yn));
  float v = __fsub_rn(1.0f, __fdiv_rn(s, den));
  if (v < 0.0f) v = 0.0f;
  return v;
}

// Certificate of one query row (lane 0 computes it, the warp shares it): the
// threshold T (every point of the exact top-k has est <= T), the floor of
// non-candidates' exact distances, and whether the row is certified; the
// row's certificate depth goes to the warp's histogram and an uncertified row
// is queued for the FP32 form.
struct RowCert {
  float T, d_floor, qn;
  bool certified, all_in;
};

__device__ __forceinline__ RowCert rerank_certify(const RerankArgs& a, int64_t q, int lane, int* hist_w) {
  const uint64_t* lst = a.lists + q * a.L;
  const uint64_t ek_key = lst[a.kreq - 1];
  const uint64_t last_key = lst[a.depth - 1];
  // threshold: computed by lane 0, then broadcast.  FP32 with directed
  // rounding (FP64 is slow on this part): upper bounds round up, lower bounds
  // round down, and est' + ||q~||^2 is rounded down where it is compared with
  // T, so the candidate set only grows and the certificate stays rigorous.
  const bool cosine = a.metric == MANN_METRIC_COSINE;
  // list keys hold est' = est - ||q~||^2, or est itself in the norm-folded form
  const float qn = a.full_est ? 0.0f : a.qinfo[q].nrm;
  float T = 0.0f, d_floor = 0.0f;
  int cert_i = 0, all_in_i = 0;
  if (lane == 0) {
    const RowInfo qi = a.qinfo[q];
    const float bxn = __uint_as_float(a.bmax->xn_bits);
    const float br = __uint_as_float(a.bmax->r_bits);
    const float u = 5.9604644775390625e-08f;
    // one FP32 rounding (or truncation) per 16-term MMA step, x2 margin
    const float gam = (float)((a.kdim + 15) / 16 + 2) * 2.384185791015625e-07f;  // exact
    // + the relative error of the FP32-accumulated row norms (two of them)
    const int dpad = (a.d + 7) & ~7;
    const float nerr = (float)((dpad + 31) / 32 + 2 + 5) * u;  // exact
    const float c1 = __fadd_ru(__fadd_ru(4.0f * u, 2.0f * gam), 2.0f * nerr);
    // split form: the MMA adds |hi| |lo| cross terms to the magnitudes it sums
    // (<= (1 + 2^-7) |x~| per side, squared 1.01568) and leaves out 2 lo_q.lo_p
    // of the estimate
    const float blo = __uint_as_float(a.bmax->lo_bits);
    const float inflate = blo > 0.0f ? 1.0161f : 1.0f;
    const float xs = __fadd_ru(qi.xn_up, bxn);
    const float A = __fadd_ru(__fmul_ru(__fmul_ru(xs, xs), inflate), __fdiv_ru(__fmul_ru(2.0f * qi.lo_up, blo), c1));
    const float Rs = __fadd_ru(qi.r_up, br);
    const float c1A = __fmul_ru(c1, A);
    const float ek = ek_key == KEY_NONE ? 0.0f : fmaxf(__fadd_ru(key_dist(ek_key), qn), 0.0f);
    const float sc = *a.scale;
    const float sc2_up = __fmul_ru(sc, sc);
    float sU = __fadd_ru(__fsqrt_ru(__fadd_ru(ek, c1A)), Rs);
    // cosine: every point of the FP32-form top-k has ||q^ - p^||^2 <= U / s^2 + 4 eps_c
    if (cosine) sU = __fsqrt_ru(__fadd_ru(__fmul_ru(sU, sU), __fmul_ru(4.0f * a.eps_c, sc2_up)));
    const float U = __fmul_ru(sU, sU);
    const float rel3 = __fmul_ru((float)(3 * (a.d + 2)), u);
    const float slack = __fadd_ru(__fadd_ru(__fmul_ru(rel3, U), __fmul_ru(1e-6f, U)), 1e-30f);
    const float w = __fadd_ru(sU, Rs);
    T = __fadd_ru(__fadd_ru(__fmul_ru(w, w), c1A), slack);
    // lower bound on the exact distance of any point outside the list's est <= T set
    const float e_floor = fmaxf(__fsub_rd(T, c1A), 0.0f);
    const float s_floor = fmaxf(__fsub_rd(__fsqrt_rd(e_floor), Rs), 0.0f);
    const float s_floor2 = __fmul_rd(s_floor, s_floor);
    d_floor = cosine ? __fsub_rd(__fdiv_rd(0.5f * s_floor2, sc2_up), a.eps_c)
                     : __fdiv_rd(__fmul_rd(s_floor2, __fsub_rd(1.0f, rel3)), sc2_up);
    // Every point outside the merged list has est' >= its depth-th entry, or >=
    // the seed when the list is not full; with neither, the list holds every point.
    const float sd = a.seed ? a.seed[q] : __int_as_float(0x7F800000);
    const bool all_in = (last_key == KEY_NONE) && !(sd < 3.0e38f);
    const float beyond = last_key != KEY_NONE ? key_dist(last_key) : sd;
    // without the row's k-th estimate (fewer than k points admitted below the
    // seed) the threshold is unknown: the row is not certified
    bool certified = all_in || (ek_key != KEY_NONE && __fadd_rd(beyond, qn) > T);
    // a zero-norm (or non-finite) query has no unit direction: the FP32 form answers it
    if (cosine && !(a.cos_qn[q] > 0.0f && a.cos_qn[q] < 3.0e38f)) certified = false;
    cert_i = certified ? 1 : 0;
    all_in_i = all_in ? 1 : 0;
  }
  T = __shfl_sync(FULL, T, 0);
  d_floor = __shfl_sync(FULL, d_floor, 0);
  const bool certified = __shfl_sync(FULL, cert_i, 0) != 0;
  const bool all_in = __shfl_sync(FULL, all_in_i, 0) != 0;
  {
    // depth this row's certificate needs: one past its last est <= T entry
    const uint64_t kl = lst[lane];
    const int le = __popc(__ballot_sync(FULL, kl != KEY_NONE && __fadd_rd(key_dist(kl), qn) <= T));
    if (lane == 0) ++hist_w[certified ? min(le + 1, LIST) : LIST + 1];
  }
  if (!certified) {
    if (lane == 0) {
      const int slot = atomicAdd(a.fb_count, 1);
      a.fb_rows[slot] = (int)q;
      a.cand_count[q] = -1;
    }
    return RowCert{T, d_floor, qn, false, all_in};
  }
  if (all_in) d_floor = 3.0e38f;
  return RowCert{T, d_floor, qn, true, all_in};
}

// The row's candidates, one key per lane in key[] (KEY_NONE elsewhere), go to
// its candidate table sorted by (distance, id), with its count and floor.
__device__ __forceinline__ void rerank_finish(const RerankArgs& a, int64_t q, int lane, const uint64_t (&key)[2],
                                              const RowCert& cr, unsigned long long& cand_sum) {
  const bool cosine = a.metric == MANN_METRIC_COSINE;
  const bool all_in = cr.all_in;
  const float d_floor = cr.d_floor;
  const int ncand = __popc(__ballot_sync(FULL, key[0] != KEY_NONE)) + __popc(__ballot_sync(FULL, key[1] != KEY_NONE));
  if (cosine && !all_in) {
    // a zero-norm point has a NaN cosine and no bound from the unit-norm
    // pass: a row that needs such points (fewer than k finite candidates)
    // goes to the FP32 form
    const bool f0 = key[0] != KEY_NONE && key_dist(key[0]) == key_dist(key[0]);
    const bool f1 = key[1] != KEY_NONE && key_dist(key[1]) == key_dist(key[1]);
    const int nfin = __popc(__ballot_sync(FULL, f0)) + __popc(__ballot_sync(FULL, f1));
    if (nfin < a.kreq) {
      if (lane == 0) {
        const int slot = atomicAdd(a.fb_count, 1);
        a.fb_rows[slot] = (int)q;
        a.cand_count[q] = -1;
      }
      return;
    }
  }
  // rank sort by (distance, id)
  int rank[2] = {0, 0};
  for (int src = 0; src < 32; ++src) {
    const uint64_t b0 = __shfl_sync(FULL, key[0], src);
    const uint64_t b1 = __shfl_sync(FULL, key[1], src);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      rank[s] += (b0 < key[s]) + (b1 < key[s]);
    }
  }
  uint64_t* out = a.cand + q * a.L;
#pragma unroll
  for (int s = 0; s < 2; ++s)
    if (key[s] != KEY_NONE) out[rank[s]] = key[s];
  for (int e = ncand + lane; e < a.L; e += 32) out[e] = KEY_NONE;
  if (lane == 0) {
    a.cand_count[q] = ncand;
    float fl = d_floor;
    if (a.metric == MANN_METRIC_EUCLIDEAN) fl = __fmul_rd(__fsqrt_rd(fmaxf(d_floor, 0.0f)), 1.0f - 1e-6f);
    a.floor_val[q] = fl;
    cand_sum += (unsigned long long)ncand;
  }
}


// Exact FP32 distances of the candidates (list entries with est <= T) of one
// or two certified rows, one lane per candidate: row 0's candidates take lanes
// [0, nc0) and row 1's the next ones (the caller keeps the total <= 32).  The
// warp streams the candidates' rows through shared memory in chunks of RR_CH
// dimensions (cp.async, 16 bytes a lane, two chunks in flight), with each
// row's query chunk beside them; lane i then adds candidate i's chunk to its
// sequential FP32 sum, in the same order as the one-lane-per-row form.
// Two rows per warp fill the lanes that one row's ~11 candidates leave idle.
// Returns this lane's key (KEY_NONE past the candidates).
__device__ __forceinline__ uint64_t rerank_coop(const RerankArgs& a, int ng, const int64_t (&qv)[2],
                                                const RowCert (&cr)[2], int lane, int& nc0) {
  __shared__ __align__(16) float rr_rows[RR_WARPS][2][32 * RR_STR];
  __shared__ __align__(16) float rr_q[RR_WARPS][2][2][RR_CH];
  __shared__ int rr_id[RR_WARPS][32];
  const bool cosine = a.metric == MANN_METRIC_COSINE;
  const int w = threadIdx.x >> 5;
  int nc = 0;
  nc0 = 0;
  for (int g = 0; g < ng; ++g) {
    const uint64_t k0 = a.lists[qv[g] * a.L + lane];
    const bool isc = k0 != KEY_NONE && __fadd_rd(key_dist(k0), cr[g].qn) <= cr[g].T;
    const unsigned cm = __ballot_sync(FULL, isc);
    if (isc) rr_id[w][nc + __popc(cm & ((1u << lane) - 1u))] = key_id(k0);
    if (g == 0) nc0 = __popc(cm);
    nc += __popc(cm);
  }
  __syncwarp();
  const int gl = lane < nc0 ? 0 : 1;  // this lane's row
  const float* qrow0 = a.qs + qv[0] * a.d;
  const float* qrow1 = a.qs + qv[ng > 1 ? 1 : 0] * a.d;
  const int nch = (a.d + RR_CH - 1) / RR_CH;
  auto issue = [&](int chunk, int b) {
    const int c0 = chunk * RR_CH;
    const int cw = min(RR_CH, a.d - c0);
    const int c4 = lane & 15;
    if (c4 * 4 < cw) {
      for (int r = lane >> 4; r < nc; r += 2)
        ptx::cp_async16(&rr_rows[w][b][r * RR_STR + c4 * 4], a.base + (int64_t)rr_id[w][r] * a.d + c0 + c4 * 4);
      if (lane < 16)
        ptx::cp_async16(&rr_q[w][b][0][c4 * 4], qrow0 + c0 + c4 * 4);
      else if (ng > 1)
        ptx::cp_async16(&rr_q[w][b][1][c4 * 4], qrow1 + c0 + c4 * 4);
    }
    ptx::cp_async_commit();
  };
  float acc = 0.0f;
  issue(0, 0);
  for (int chunk = 0; chunk < nch; ++chunk) {
    const int b = chunk & 1;
    if (chunk + 1 < nch) {
      issue(chunk + 1, b ^ 1);
      ptx::cp_async_wait<1>();
    } else {
      ptx::cp_async_wait<0>();
    }
    __syncwarp();
    if (lane < nc) {
      // float4 reads: a quarter-warp's rows start 272 bytes apart, so its
      // 16-byte reads fall in distinct banks; a row's query chunk is a broadcast
      const float4* row = reinterpret_cast<const float4*>(&rr_rows[w][b][lane * RR_STR]);
      const float4* qq = reinterpret_cast<const float4*>(rr_q[w][b][gl]);
      const int cw4 = min(RR_CH, a.d - chunk * RR_CH) >> 2;  // d % 4 == 0 here
      if (cosine) {
#pragma unroll 4
        for (int c = 0; c < cw4; ++c) {
          const float4 x = qq[c], y = row[c];
          acc = __fmaf_rn(x.x, y.x, acc);
          acc = __fmaf_rn(x.y, y.y, acc);
          acc = __fmaf_rn(x.z, y.z, acc);
          acc = __fmaf_rn(x.w, y.w, acc);
        }
      } else {
#pragma unroll 4
        for (int c = 0; c < cw4; ++c) {
          const float4 x = qq[c], y = row[c];
          float t = __fsub_rn(x.x, y.x);
          acc = __fmaf_rn(t, t, acc);
          t = __fsub_rn(x.y, y.y);
          acc = __fmaf_rn(t, t, acc);
          t = __fsub_rn(x.z, y.z);
          acc = __fmaf_rn(t, t, acc);
          t = __fsub_rn(x.w, y.w);
          acc = __fmaf_rn(t, t, acc);
        }
      }
    }
    __syncwarp();  // the buffer is refilled two chunks on
  }
  if (lane >= nc) return KEY_NONE;
  const int id = rr_id[w][lane];
  float dist;
  if (cosine) {
    const float den = __fmul_rn(__fsqrt_rn(a.cos_qn[qv[gl]]), __fsqrt_rn(a.cos_bn[id]));
    dist = __fsub_rn(1.0f, __fdiv_rn(acc, den));
    if (dist < 0.0f) dist = 0.0f;
  } else {
    dist = a.metric == MANN_METRIC_EUCLIDEAN ? __fsqrt_rn(acc) : acc;
  }
  return make_key(dist, (uint32_t)id);
}

// One query row (one warp): certify, then rerank the candidates.  The row's
// certificate depth goes to the warp's histogram hist_w and its candidate
// count to cand_sum (lane 0), flushed to global memory once per warp.
__device__ __forceinline__ void rerank_row(const RerankArgs& a, int64_t q, int lane, int* hist_w,
                                           unsigned long long& cand_sum) {
  const RowCert cr = rerank_certify(a, q, lane, hist_w);
  if (!cr.certified) return;
  uint64_t key[2] = {KEY_NONE, KEY_NONE};
  if (a.coop && a.L == 32) {
    const int64_t qv[2] = {q, q};
    const RowCert crs[2] = {cr, cr};
    int nc0 = 0;
    key[0] = rerank_coop(a, 1, qv, crs, lane, nc0);
  } else {
    const bool cosine = a.metric == MANN_METRIC_COSINE;
    const uint64_t* lst = a.lists + q * a.L;
    const float* qrow = a.qs + q * a.d;
    const float qn = cr.qn, T = cr.T;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int e = s * 32 + lane;
      if (e < a.L) {
        const uint64_t k = lst[e];
        if (k != KEY_NONE && __fadd_rd(key_dist(k), qn) <= T) {
          const int id = key_id(k);
          const float dist = cosine ? fp32_cos_row(qrow, a.base + (int64_t)id * a.d, a.d, a.cos_qn[q], a.cos_bn[id])
                                    : fp32_dist_row(qrow, a.base + (int64_t)id * a.d, a.d, a.metric);
          key[s] = make_key(dist, (uint32_t)id);
        }
      }
    }
  }
  rerank_finish(a, q, lane, key, cr, cand_sum);
}

// Two query rows in one warp (the shared-memory path): both certified and
// together at most 32 candidates -> one pass over both rows' candidates.
__device__ __forceinline__ void rerank_pair(const RerankArgs& a, int64_t qa, int64_t qb, int lane, int* hist_w,
                                            unsigned long long& cand_sum) {
  const RowCert ca = rerank_certify(a, qa, lane, hist_w);
  const RowCert cb = rerank_certify(a, qb, lane, hist_w);
  auto count = [&](int64_t q, const RowCert& c) {
    const uint64_t k0 = a.lists[q * a.L + lane];
    return __popc(__ballot_sync(FULL, c.certified && k0 != KEY_NONE && __fadd_rd(key_dist(k0), c.qn) <= c.T));
  };
  const int na = count(qa, ca), nb = count(qb, cb);
  const int64_t qv[2] = {qa, qb};
  const RowCert crs[2] = {ca, cb};
  if (ca.certified && cb.certified && na + nb <= 32) {
    int nc0 = 0;
    const uint64_t k = rerank_coop(a, 2, qv, crs, lane, nc0);
    const uint64_t ka[2] = {lane < nc0 ? k : KEY_NONE, KEY_NONE};
    const uint64_t kb[2] = {lane >= nc0 ? k : KEY_NONE, KEY_NONE};
    rerank_finish(a, qa, lane, ka, ca, cand_sum);
    rerank_finish(a, qb, lane, kb, cb, cand_sum);
    return;
  }
  for (int g = 0; g < 2; ++g) {
    if (!crs[g].certified) continue;
    const int64_t qs1[2] = {qv[g], qv[g]};
    const RowCert cs1[2] = {crs[g], crs[g]};
    int nc0 = 0;
    const uint64_t key[2] = {rerank_coop(a, 1, qs1, cs1, lane, nc0), KEY_NONE};
    rerank_finish(a, qv[g], lane, key, crs[g], cand_sum);
  }
}

// Warps stride over the query rows; per-warp histogram and candidate count
// reach global memory with one set of atomics per warp, not per row.
__global__ void __launch_bounds__(32 * RR_WARPS) k2_rerank(RerankArgs a) {
  __shared__ int hist[RR_WARPS][LIST + 2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = lane; i < LIST + 2; i += 32) hist[w][i] = 0;
  __syncwarp();
  unsigned long long csum = 0;
  const int64_t nw = (int64_t)gridDim.x * RR_WARPS;
  if (a.coop && a.L == 32) {
    // the shared-memory path takes rows two at a time
    for (int64_t q = 2 * ((int64_t)blockIdx.x * RR_WARPS + w); q < a.nq; q += 2 * nw) {
      if (q + 1 < a.nq)
        rerank_pair(a, q, q + 1, lane, hist[w], csum);
      else
        rerank_row(a, q, lane, hist[w], csum);
    }
  } else {
    for (int64_t q = (int64_t)blockIdx.x * RR_WARPS + w; q < a.nq; q += nw) rerank_row(a, q, lane, hist[w], csum);
  }
  __syncwarp();
  for (int i = lane; i < LIST + 2; i += 32)
    if (hist[w][i]) atomicAdd(&a.depth_hist[i], (unsigned long long)hist[w][i]);
  if (lane == 0 && csum) atomicAdd(a.cand_total, csum);
}

// rows re-run by the FP32 scan: copy their sorted keys into the candidate table
__global__ void k2_scatter_fallback(const uint64_t* __restrict__ keys, const int* __restrict__ rows,
                                    const int* __restrict__ count, int kk, int L,
                                    uint64_t* __restrict__ cand, int* __restrict__ cand_count,
                                    float* __restrict__ floor_val) {
  const int cnt = *count;
  for (int i = blockIdx.x; i < cnt; i += gridDim.x) {
  const int q = rows[i];
  for (int e = threadIdx.x; e < L; e += blockDim.x) cand[(int64_t)q * L + e] = e < kk ? keys[(int64_t)i * kk + e] : KEY_NONE;
  if (threadIdx.x == 0) {
    int c = 0;
    while (c < kk && keys[(int64_t)i * kk + c] != KEY_NONE) ++c;
    cand_count[q] = c;
    // the kk-th FP32 distance bounds every point outside the list from below
    floor_val[q] = (c == kk) ? key_dist(keys[(int64_t)i * kk + kk - 1]) : 3.0e38f;
  }
  }
}

// Work items of the segmented fallback: item i * nsplit + c is row
// r = fb_rows[i] against points [c * chunk, (c + 1) * chunk) of the set
// holding it (empty past the set's end); its exact FP32 list goes to split
// slot c of compact row i.
__global__ void fb_items_kernel(const int* __restrict__ fb_rows, int cnt, const int64_t* __restrict__ offs,
                                int nsets, int nsplit, int64_t chunk, SegItem* __restrict__ items) {
  const int64_t total = (int64_t)cnt * nsplit;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / nsplit), c = (int)(t % nsplit);
    const int64_t r = fb_rows[i];
    int lo = 0, hi = nsets - 1;
    while (lo < hi) {  // last set whose offset <= r
      const int mid = (lo + hi + 1) >> 1;
      if (offs[mid] <= r) lo = mid;
      else hi = mid - 1;
    }
    SegItem it{};
    it.q0 = i;
    it.qend = i + 1;
    it.nb1 = offs[lo + 1];
    it.nb0 = min(it.nb1, offs[lo] + c * chunk);
    it.nb1 = min(it.nb1, it.nb0 + chunk);
    it.split = c;
    items[t] = it;
  }
}

// The fallback rows' exact FP32 top-LIST lists (compact row i) go to their
// candidate slots, with their counts and floors (the LIST-th distance bounds
// every other point).
__global__ void fb_finish_kernel(const int* __restrict__ fb_rows, int cnt, const uint64_t* __restrict__ keys,
                                 uint64_t* __restrict__ cand, int* __restrict__ cand_count,
                                 float* __restrict__ floor_val) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    const int64_t r = fb_rows[i];
    const uint64_t* src = keys + (int64_t)i * LIST;
    uint64_t* row = cand + r * LIST;
    int c = 0;
    for (int e = 0; e < LIST; ++e) {
      row[e] = src[e];
      c += src[e] != KEY_NONE ? 1 : 0;
    }
    cand_count[r] = c;
    floor_val[r] = (c == LIST) ? key_dist(src[LIST - 1]) : 3.0e38f;
  }
}

}  // namespace

// ---------------------------------------------------------------- FP64 resolve (shared)

namespace {

__device__ __forceinline__ double fp64_dist_row(const float* __restrict__ x,
                                                const float* __restrict__ y, int d, int metric) {
  if (metric == MANN_METRIC_COSINE) {
    double ab = 0.0, aa = 0.0, bb = 0.0;
    for (int c = 0; c < d; ++c) {
      const double xv = (double)x[c], yv = (double)y[c];
      ab = fma(xv, yv, ab);
      aa = fma(xv, xv, aa);
      bb = fma(yv, yv, bb);
    }
    const double r = 1.0 - ab / (sqrt(aa) * sqrt(bb));
    return r < 0.0 ? 0.0 : r;
  }
  double s = 0.0;
  for (int c = 0; c < d; ++c) {
    const double t = (double)x[c] - (double)y[c];
    s = fma(t, t, s);
  }
  return metric == MANN_METRIC_EUCLIDEAN ? sqrt(s) : s;
}

// Clusters of adjacent candidates whose FP32 distances lie within the FP32
// rounding bound of each other: cl[p] = first position of p's cluster.
__device__ __forceinline__ void tie_clusters(const uint64_t* key, int cm, int d, int metric, int* cl) {
  const double eps = (double)(d + 2) * 5.9604644775390625e-08 * 1.01 + 1.2e-7;
  int start = 0;
  cl[0] = 0;
  for (int p = 1; p < cm; ++p) {
    const double a = (double)key_dist(key[p - 1]);
    const double b = (double)key_dist(key[p]);
    // FP32 cosine distances carry an absolute error of order (d+4)u
    const bool link = metric == MANN_METRIC_COSINE ? (b - a) <= 2.0 * eps + 4.8e-7
                                                   : (b - a) <= eps * (fabs(a) + fabs(b));
    if (!link) start = p;
    cl[p] = start;
  }
}

struct TieTask {  // one FP64 distance to compute: candidate row i, position p, point id
  int64_t i;
  int32_t p, id;
};

// Pass 1 of the FP64 near-tie order (one warp per candidate row i; the row
// belongs to query / output row q = rows[i], or i).  cand[i][0..count) is
// sorted by (fp32, id).  Writes the first kreq keys to keys_out[q] in FP32
// order; when `fp64` and the cluster holding position kreq-1 is a real tie,
// the row is marked (state[i] = 1) and every member of the clusters up to
// that one becomes a task of the compacted list (task_count[0] entries), so
// pass 2 runs 32 FP64 sums per warp.  A row whose boundary cluster may reach
// past its candidates is counted in n_unresolved and, with unres_rows, listed.
__global__ void resolve_mark_kernel(int d, int metric, int64_t nq, int L, int kreq, int fp64,
                                    const uint64_t* __restrict__ cand, const int* __restrict__ cand_count,
                                    const float* __restrict__ floor_val, uint64_t* __restrict__ keys_out,
                                    unsigned long long* __restrict__ n_fp64_rows,
                                    unsigned long long* __restrict__ n_unresolved,
                                    unsigned long long* __restrict__ task_count, TieTask* __restrict__ tasks,
                                    int8_t* __restrict__ state, const int32_t* __restrict__ rows,
                                    int32_t* __restrict__ unres_rows) {
  __shared__ uint64_t s_key[4][256];
  __shared__ int s_cl[4][256];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * 4 + w;
  if (i >= nq) return;
  const int64_t q = rows ? (int64_t)rows[i] : i;
  const uint64_t* cq = cand + i * L;
  const int c = min(cand_count[i], L);
  uint64_t* out = keys_out + q * kreq;
  for (int e = lane; e < kreq; e += 32) out[e] = e < c ? cq[e] : KEY_NONE;
  if (state && lane == 0) state[i] = 0;
  if (!fp64 || c <= 1) return;
  const int cm = min(c, 256);
  for (int e = lane; e < cm; e += 32) s_key[w][e] = cq[e];
  __syncwarp();
  if (lane == 0) tie_clusters(s_key[w], cm, d, metric, s_cl[w]);
  __syncwarp();
  // the cluster holding position kreq-1 must end inside the candidate list
  const int kl = kreq - 1 < cm ? kreq - 1 : cm - 1;
  int end = kl;
  while (end + 1 < cm && s_cl[w][end + 1] == s_cl[w][kl]) ++end;
  bool resolvable = true;
  if (end == cm - 1) {
    const double eps = (double)(d + 2) * 5.9604644775390625e-08 * 1.01 + 1.2e-7;
    const double lastv = (double)key_dist(s_key[w][cm - 1]);
    const double fl = (double)floor_val[i];
    const bool clear = metric == MANN_METRIC_COSINE ? lastv + 2.0 * eps + 4.8e-7 < fl
                                                    : lastv * (1.0 + eps) < fl * (1.0 - eps);
    resolvable = clear || fl >= 3.0e38;
  }
  bool any_tie = false;
  for (int p = 1; p <= end; ++p)
    if (s_cl[w][p] != p) {
      any_tie = true;
      break;
    }
  if (!resolvable) {
    if (lane == 0) {
      const unsigned long long slot = atomicAdd(n_unresolved, 1ull);
      if (unres_rows) unres_rows[slot] = (int32_t)q;
    }
    return;
  }
  if (!any_tie) return;
  // members: positions <= end inside a cluster of two or more
  unsigned long long base_slot = 0;
  for (int p0 = 0; p0 <= end; p0 += 32) {
    const int p = p0 + lane;
    const bool member = p <= end && ((s_cl[w][p] != p) || (p + 1 <= end && s_cl[w][p + 1] == p));
    const unsigned m = __ballot_sync(FULL, member);
    if (lane == 0) base_slot = atomicAdd(task_count, (unsigned long long)__popc(m));
    base_slot = __shfl_sync(FULL, base_slot, 0);
    if (member) {
      const unsigned long long slot = base_slot + __popc(m & ((1u << lane) - 1u));
      tasks[slot] = TieTask{i, p, key_id(s_key[w][p])};
    }
  }
  if (lane == 0) {
    state[i] = 1;
    atomicAdd(n_fp64_rows, 1ull);
  }
}

// Pass 2: the FP64 distance of every task (one thread each), the sequential
// sum of the FP64 oracle; vals[i][p].
__global__ void resolve_fp64_kernel(const float* __restrict__ base, const float* __restrict__ qs, int d, int metric,
                                    int L, const unsigned long long* __restrict__ task_count,
                                    const TieTask* __restrict__ tasks, const int32_t* __restrict__ rows,
                                    double* __restrict__ vals) {
  const unsigned long long cnt = *task_count;
  for (unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; t < cnt;
       t += (unsigned long long)gridDim.x * blockDim.x) {
    const TieTask tk = tasks[t];
    const int64_t q = rows ? (int64_t)rows[tk.i] : tk.i;
    vals[tk.i * L + tk.p] = fp64_dist_row(qs + q * d, base + (int64_t)tk.id * d, d, metric);
  }
}

// Pass 3 (one warp per marked row): insertion sort of each cluster up to the
// boundary one by (FP64 distance, id); the first kreq keys go out.
__global__ void resolve_sort_kernel(int d, int metric, int64_t nq, int L, int kreq,
                                    const uint64_t* __restrict__ cand, const int* __restrict__ cand_count,
                                    const int8_t* __restrict__ state, const double* __restrict__ vals,
                                    uint64_t* __restrict__ keys_out, const int32_t* __restrict__ rows) {
  __shared__ uint64_t s_key[4][256];
  __shared__ double s_val[4][256];
  __shared__ int s_cl[4][256];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * 4 + w;
  if (i >= nq || state[i] == 0) return;
  const int64_t q = rows ? (int64_t)rows[i] : i;
  const uint64_t* cq = cand + i * L;
  const int cm = min(min(cand_count[i], L), 256);
  for (int e = lane; e < cm; e += 32) {
    s_key[w][e] = cq[e];
    s_val[w][e] = vals[i * L + e];
  }
  __syncwarp();
  if (lane == 0) {
    tie_clusters(s_key[w], cm, d, metric, s_cl[w]);
    const int kl = kreq - 1 < cm ? kreq - 1 : cm - 1;
    int end = kl;
    while (end + 1 < cm && s_cl[w][end + 1] == s_cl[w][kl]) ++end;
    int p = 0;
    while (p <= end) {
      int e = p;
      while (e + 1 <= end && s_cl[w][e + 1] == p) ++e;
      for (int a = p + 1; a <= e; ++a) {
        const uint64_t kk = s_key[w][a];
        const double vv = s_val[w][a];
        int j = a - 1;
        while (j >= p && (s_val[w][j] > vv || (s_val[w][j] == vv && key_id(s_key[w][j]) > key_id(kk)))) {
          s_key[w][j + 1] = s_key[w][j];
          s_val[w][j + 1] = s_val[w][j];
          --j;
        }
        s_key[w][j + 1] = kk;
        s_val[w][j + 1] = vv;
      }
      p = e + 1;
    }
  }
  __syncwarp();
  uint64_t* out = keys_out + q * kreq;
  for (int e = lane; e < kreq; e += 32) out[e] = e < cm ? s_key[w][e] : KEY_NONE;
}

// ---- (Sq)Euclidean near-tie order without bulk FP64 arithmetic
//
// FP64 runs at a small fraction of the FP32 rate on this GPU, so the members
// of a tie cluster are ordered by a double-float value instead: V ~ S, the
// exact sum over c of (q_c - p_c)^2, with a rigorous bound |V - S| <= E.
// Where two neighbours of a cluster (sorted by V) are separated by more than
// E_a + E_b + R_a + R_b, with R the error bound of the FP64 sequential sum
// (and of its square root), their FP64 values order the same way; only the
// rare groups that stay inside that window get the FP64 sequential sums.
//
// hp_sqdist: one warp per distance, lane l takes dimensions l, l + 32, ...
//   t = th + tl exactly (TwoSum of q_c and -p_c), th^2 = p + e exactly
//   (TwoProd), cc = fl(e + 2 th tl) (tl^2 <= u^2 th^2 is dropped);
//   (sh, r) = Fast2Sum(sh, p) exactly, sl += fl(r + cc); then a butterfly of
//   the lanes' (sh, sl) pairs in the same form.  With u = 2^-24 and n the
//   dimensions per lane, |sl| stays below u S (n + 9) and the roundings sum to
//   at most u^2 S (4 + (n + 3.01)(n + 1)(1.001) + 10 (n + 8.1)); E doubles the
//   leading terms, adds the double rounding of sh + sl and, for gradual
//   underflow, 4 d 2^-149 per distance.
__device__ __forceinline__ void hp_step(float a, float b, float& sh, float& sl) {
  const float th = __fsub_rn(a, b);
  const float bb = __fsub_rn(th, a);
  const float tl = __fadd_rn(__fsub_rn(a, __fsub_rn(th, bb)), __fsub_rn(-b, bb));
  const float p = __fmul_rn(th, th);
  const float e = __fmaf_rn(th, th, -p);
  const float cc = __fmaf_rn(__fmul_rn(2.0f, th), tl, e);
  const float hi = fmaxf(sh, p), lo = fminf(sh, p);
  const float s2 = __fadd_rn(hi, lo);
  const float r = __fsub_rn(lo, __fsub_rn(s2, hi));
  sh = s2;
  sl = __fadd_rn(sl, __fadd_rn(r, cc));
}

// The loads of U strides are issued before their arithmetic (the lane's
// dimensions are still added in order).
template <int U>
__device__ __forceinline__ void hp_sqdist(const float* __restrict__ qr, const float* __restrict__ pr, int d,
                                          int lane, double& V, double& E) {
  float sh = 0.0f, sl = 0.0f;
  int c = lane;
  for (; c + 32 * (U - 1) < d; c += 32 * U) {
    float a[U], b[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      a[u] = __ldg(qr + c + 32 * u);
      b[u] = __ldg(pr + c + 32 * u);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) hp_step(a[u], b[u], sh, sl);
  }
  for (; c < d; c += 32) hp_step(__ldg(qr + c), __ldg(pr + c), sh, sl);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(FULL, sh, o), ol = __shfl_xor_sync(FULL, sl, o);
    const float hi = fmaxf(sh, oh), lo = fminf(sh, oh);
    const float s2 = __fadd_rn(hi, lo);
    const float r = __fsub_rn(lo, __fsub_rn(s2, hi));
    sh = s2;
    sl = __fadd_rn(__fadd_rn(sl, ol), r);
  }
  V = (double)sh + (double)sl;
  const double n = (double)((d + 31) / 32);
  const double u2 = 3.5527136788005009e-15;  // 2^-48
  E = u2 * V * (8.0 + 1.01 * (n + 4.0) * (n + 1.0) + 11.0 * (n + 9.0)) + 2.3e-16 * V + (double)d * 2.9e-44;
  if (!(V < 1e30) || !(sh == sh)) E = __longlong_as_double(0x7FF0000000000000ll);  // +inf: FP64 decides
}

// error bound of the oracle's FP64 sequential FMA sum (t = q - p in FP64, s =
// fma(t, t, s)) around S, plus four ulps for square-root collisions
__device__ __forceinline__ double fp64_seq_bound(double V, int d) {
  return V * ((double)(d + 3) * 1.1102230246251565e-16 * 1.01 + 8.9e-16) + 1e-300;
}

// Conservative FP32 link of adjacent sorted candidates: never false where the
// FP64 test (b - a) <= eps (|a| + |b|) holds.
__device__ __forceinline__ bool link_l2(float a, float b, float eps_up) {
  return __fsub_rd(b, a) <= __fmul_ru(eps_up, __fadd_ru(fabsf(a), fabsf(b)));
}

__device__ __forceinline__ bool hp_less(double va, uint64_t ka, double vb, uint64_t kb) {
  const unsigned long long ba = (unsigned long long)__double_as_longlong(va);
  const unsigned long long bb = (unsigned long long)__double_as_longlong(vb);
  return ba < bb || (ba == bb && key_id(ka) < key_id(kb));
}

// insertion sort of positions [p, e] by (value bits, id); values >= 0
__device__ void sort_range(uint64_t* K, double* Vv, double* Ee, int p, int e) {
  for (int a = p + 1; a <= e; ++a) {
    const uint64_t kk = K[a];
    const double vv = Vv[a], ee = Ee[a];
    int j = a - 1;
    while (j >= p && hp_less(vv, kk, Vv[j], K[j])) {
      K[j + 1] = K[j];
      Vv[j + 1] = Vv[j];
      Ee[j + 1] = Ee[j];
      --j;
    }
    K[j + 1] = kk;
    Vv[j + 1] = vv;
    Ee[j + 1] = ee;
  }
}

// One warp per candidate row i (query / output row q = rows[i], or i), for
// Euclidean and SqEuclidean with the FP64 near-tie order.  cand[i][0..count)
// is sorted by (fp32, id).  The row's clusters (adjacent candidates whose FP32
// distances lie within the FP32 rounding bound of each other) up to the one
// holding position kreq-1 are ordered as the FP64 oracle orders them, and the
// first kreq keys are written to keys_out[q].  When that cluster runs to the
// end of the candidate list and the FP32 floor test cannot clear it, the row
// is still settled when the double-float bound of its kreq-th member lies
// below the floor; otherwise it keeps the FP32 order, is counted in
// n_unresolved and (with unres_rows) listed for a wider list.
// counters: [0] rows with a tie, [1] unresolved rows, [2] rows that needed
// FP64 sequential sums.
__global__ void __launch_bounds__(128, 10) resolve_l2_kernel(const float* __restrict__ base,
                                                         const float* __restrict__ qs, int d, int metric,
                                                         int64_t nq, int L, int kreq, float eps_up, double eps,
                                                         const uint64_t* __restrict__ cand,
                                                         const int* __restrict__ cand_count,
                                                         const float* __restrict__ floor_val,
                                                         uint64_t* __restrict__ keys_out,
                                                         unsigned long long* __restrict__ counters,
                                                         const int32_t* __restrict__ rows,
                                                         int32_t* __restrict__ unres_rows) {
  // per warp, lc = min(L, 256) entries each: keys, values, bounds (8 bytes),
  // cluster and group starts (2 bytes) -- sized by the call, so that short
  // lists leave room for more blocks per SM
  extern __shared__ __align__(16) uint8_t rs_smem[];
  const int lc = min(L, 256);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t* K = reinterpret_cast<uint64_t*>(rs_smem) + w * lc;
  double* Vv = reinterpret_cast<double*>(rs_smem + (size_t)4 * lc * 8) + w * lc;
  double* Ee = reinterpret_cast<double*>(rs_smem + (size_t)8 * lc * 8) + w * lc;
  short* cl = reinterpret_cast<short*>(rs_smem + (size_t)12 * lc * 8) + w * lc;
  short* gr = reinterpret_cast<short*>(rs_smem + (size_t)12 * lc * 8 + (size_t)4 * lc * 2) + w * lc;
  const int64_t i = (int64_t)blockIdx.x * 4 + w;
  if (i >= nq) return;
  const int64_t q = rows ? (int64_t)rows[i] : i;
  const uint64_t* cq = cand + i * L;
  const int c = min(cand_count[i], L);
  uint64_t* out = keys_out + q * kreq;
  for (int e = lane; e < kreq; e += 32) out[e] = e < c ? cq[e] : KEY_NONE;
  if (c <= 1) return;
  const int cm = min(c, lc);
  for (int e = lane; e < cm; e += 32) K[e] = cq[e];
  __syncwarp();
  // cluster starts by ballot: cl[p] = the last start at or before p
  int carry = 0;
  for (int b = 0; b < cm; b += 32) {
    const int p = b + lane;
    bool start = true;
    if (p > 0 && p < cm) start = !link_l2(key_dist(K[p - 1]), key_dist(K[p]), eps_up);
    const unsigned sm = __ballot_sync(FULL, p < cm && start);
    const unsigned mine = sm & (0xFFFFFFFFu >> (31 - lane));
    if (p < cm) cl[p] = (short)(mine ? b + 31 - __clz(mine) : carry);
    if (sm) carry = b + 31 - __clz(sm);
  }
  __syncwarp();
  const int kl = kreq - 1 < cm ? kreq - 1 : cm - 1;
  int end = cm - 1;
  bool any_tie = false;
  for (int b = 0; b < cm; b += 32) {
    const int p = b + lane;
    const unsigned nx = __ballot_sync(FULL, p < cm && p > kl && cl[p] == p);
    if (nx) {
      end = b + __ffs(nx) - 2;
      break;
    }
  }
  for (int b = 0; b <= end; b += 32) {
    const int p = b + lane;
    if (__any_sync(FULL, p >= 1 && p <= end && cl[p] != p)) any_tie = true;
  }
  bool clear = true;
  double fl_exact = 0.0;  // lower bound of every non-candidate's exact S
  if (end == cm - 1) {
    const double lastv = (double)key_dist(K[cm - 1]);
    const double fl = (double)floor_val[i];
    clear = lastv * (1.0 + eps) < fl * (1.0 - eps) || fl >= 3.0e38;
    const double f1 = fl * (1.0 - eps);
    fl_exact = f1 <= 0.0 ? 0.0 : (metric == MANN_METRIC_EUCLIDEAN ? f1 * f1 * (1.0 - 1e-15) : f1);
  }
  if (clear && !any_tie) return;
  // double-float values of the cluster members (every position when the
  // boundary cluster has to be settled against the floor)
  const float* qr = qs + q * d;
  for (int p = 0; p <= end; ++p) {
    const bool need = !clear || cl[p] != p || (p + 1 <= end && cl[p + 1] == p);
    if (!need) continue;  // warp-uniform
    double V, E;
    // (four positions side by side measured slower: 0.31 vs 0.22 ms per headline step)
    hp_sqdist<8>(qr, base + (int64_t)key_id(K[p]) * d, d, lane, V, E);
    if (lane == 0) {
      Vv[p] = V;
      Ee[p] = E;
    }
  }
  __syncwarp();
  int flag64 = 0, settled = 1;
  if (lane == 0) {
    int p = 0;
    while (p <= end) {
      int e = p;
      while (e + 1 <= end && cl[e + 1] == p) ++e;
      gr[p] = (short)p;
      if (e > p) {
        sort_range(K, Vv, Ee, p, e);
        for (int a = p + 1; a <= e; ++a) {
          const double thr = Ee[a - 1] + Ee[a] + fp64_seq_bound(Vv[a - 1], d) + fp64_seq_bound(Vv[a], d);
          const bool lk = !(Vv[a] - Vv[a - 1] > thr);
          gr[a] = lk ? gr[a - 1] : (short)a;
          flag64 |= lk ? 1 : 0;
        }
      }
      p = e + 1;
    }
    if (!clear) {
      // every member of the group holding position kl lies at or below ub
      int ge = kl;
      while (ge + 1 <= end && gr[ge + 1] == gr[kl]) ++ge;
      double ub = 0.0;
      for (int a = 0; a <= ge; ++a) ub = fmax(ub, Vv[a] + Ee[a]);
      const double m = ((double)d + 8.0) * 4.4408920985006262e-16;  // FP64 sums and roundings
      settled = ub * (1.0 + m) < fl_exact * (1.0 - m) ? 1 : 0;
    }
  }
  settled = __shfl_sync(FULL, settled, 0);
  if (!settled) {
    if (lane == 0) {
      const unsigned long long slot = atomicAdd(&counters[1], 1ull);
      if (unres_rows) unres_rows[slot] = (int32_t)q;
    }
    return;
  }
  flag64 = __shfl_sync(FULL, flag64, 0);
  if (flag64) {
    // groups still inside the window: the oracle's FP64 values and ids decide
    for (int p = lane; p <= end; p += 32) {
      const bool in_group = gr[p] != p || (p + 1 <= end && gr[p + 1] == p);
      if (in_group) Vv[p] = fp64_dist_row(qr, base + (int64_t)key_id(K[p]) * d, d, metric);
    }
    __syncwarp();
    if (lane == 0) {
      int p = 0;
      while (p <= end) {
        int e = p;
        while (e + 1 <= end && gr[e + 1] == p) ++e;
        if (e > p) sort_range(K, Vv, Ee, p, e);
        p = e + 1;
      }
      atomicAdd(&counters[2], 1ull);
    }
  }
  if (lane == 0 && any_tie) atomicAdd(&counters[0], 1ull);
  __syncwarp();
  for (int e = lane; e < kreq; e += 32) out[e] = e < cm ? K[e] : KEY_NONE;
}

}  // namespace

namespace {

// |returned FP32 distance - FP64 distance| of every returned neighbour; the
// maximum as the bits of a non-negative double (which order as integers)
__global__ void fp64_err_kernel(const float* __restrict__ base, const float* __restrict__ qs, int d, int metric,
                                int64_t nq, int kout, const int32_t* __restrict__ ids,
                                const float* __restrict__ dists, unsigned long long* __restrict__ max_bits) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nq * kout) return;
  const int32_t id = ids[e];
  if (id < 0) return;
  const double ref = fp64_dist_row(qs + (e / kout) * d, base + (int64_t)id * d, d, metric);
  const double err = fabs((double)dists[e] - ref);
  if (err == err) atomicMax(max_bits, (unsigned long long)__double_as_longlong(err));
}

}  // namespace

mann_status fp64_max_error(Context* ctx, cudaStream_t s, const float* base, const float* qs, int d, int metric,
                           int64_t nq, int kout, const int32_t* ids, const float* dists, double* out) {
  unsigned long long* bits = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_FP64_ERR, 1, &bits));
  MANN_CUDA_TRY(cudaMemsetAsync(bits, 0, sizeof(unsigned long long), s));
  if (nq > 0 && kout > 0) {
    fp64_err_kernel<<<(unsigned)ceil_div(nq * kout, 256), 256, 0, s>>>(base, qs, d, metric, nq, kout, ids, dists,
                                                                      bits);
    MANN_CHECK_LAUNCH();
  }
  unsigned long long h = 0;
  MANN_CUDA_TRY(cudaMemcpyAsync(&h, bits, sizeof(h), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  double v;
  std::memcpy(&v, &h, sizeof(v));
  *out = v;
  return MANN_OK;
}

mann_status launch_resolve(Context* ctx, const float* base, const float* qs, int d, int metric, int64_t nq, int L,
                           int kreq, int fp64, const uint64_t* cand, const int* cand_count,
                           const float* floor_val, uint64_t* keys_out, unsigned long long* counters,
                           cudaStream_t s, const int32_t* rows, int32_t* unres_rows) {
  if (nq <= 0) return MANN_OK;
  if (fp64 && metric != MANN_METRIC_COSINE) {
    // (Sq)Euclidean: one pass, double-float order with FP64 only where it must decide
    const double eps = (double)(d + 2) * 5.9604644775390625e-08 * 1.01 + 1.2e-7;
    const float eps_up = std::nextafter((float)eps, 1.0f);
    const size_t smem = (size_t)4 * std::min(L, 256) * (8 + 8 + 8 + 2 + 2);  // <= 28 KB
    resolve_l2_kernel<<<(unsigned)ceil_div(nq, 4), 128, smem, s>>>(base, qs, d, metric, nq, L, kreq, eps_up, eps,
                                                                   cand, cand_count, floor_val, keys_out, counters,
                                                                   rows, unres_rows);
    MANN_CHECK_LAUNCH();
    return MANN_OK;
  }
  TieTask* tasks = nullptr;
  double* vals = nullptr;
  int8_t* state = nullptr;
  if (fp64) {
    MANN_TRY(ctx->scratch_t(SLOT_TIES_TASKS, (size_t)nq * L, &tasks));
    MANN_TRY(ctx->scratch_t(SLOT_TIES_VALS, (size_t)nq * L, &vals));
    MANN_TRY(ctx->scratch_t(SLOT_TIES_STATE, (size_t)nq, &state));
    // the task cursor starts at zero on every call (callers may share counters)
    MANN_CUDA_TRY(cudaMemsetAsync(counters + 2, 0, sizeof(unsigned long long), s));
  }
  const unsigned grid = (unsigned)ceil_div(nq, 4);
  resolve_mark_kernel<<<grid, 128, 0, s>>>(d, metric, nq, L, kreq, fp64, cand, cand_count, floor_val, keys_out,
                                           counters, counters + 1, counters + 2, tasks, state, rows, unres_rows);
  MANN_CHECK_LAUNCH();
  if (fp64) {
    resolve_fp64_kernel<<<(unsigned)ctx->num_sms * 8, 256, 0, s>>>(base, qs, d, metric, L, counters + 2, tasks,
                                                                   rows, vals);
    MANN_CHECK_LAUNCH();
    resolve_sort_kernel<<<grid, 128, 0, s>>>(d, metric, nq, L, kreq, cand, cand_count, state, vals, keys_out,
                                             rows);
    MANN_CHECK_LAUNCH();
  }
  return MANN_OK;
}

namespace {

// candidate table from an exact FP32 top-kk list: counts and the floor (the
// kk-th distance bounds every point outside the list from below)
__global__ void fp32_lists_to_cand_kernel(const uint64_t* __restrict__ keys, int64_t nq, int kk,
                                          int* __restrict__ cand_count, float* __restrict__ floor_val) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint64_t* r = keys + q * kk;
  int c = 0;
  while (c < kk && r[c] != KEY_NONE) ++c;
  cand_count[q] = c;
  floor_val[q] = (c == kk) ? key_dist(r[kk - 1]) : 3.0e38f;
}

}  // namespace

// Rows whose boundary tie cluster reached past their candidates (listed in
// unres_rows, h_unres of them): their exact FP32 top-64, then the FP64
// near-tie order again, written over those rows of keys_out; rows whose
// cluster is longer still get their exact top-min(n, KMAX_FUSED).  Rows left
// unsettled after that (a tie cluster longer than the list) are returned in
// *still_unresolved; they keep the FP32 (distance, id) order.
mann_status widen_unresolved(Context* ctx, cudaStream_t s, const float* base, const float* qs,
                             int64_t n, int d, int metric, int kreq, const float* qn,
                             const float* bn, const int32_t* unres_rows, int64_t h_unres,
                             uint64_t* keys_out, int64_t* still_unresolved) {
  *still_unresolved = 0;
  const int32_t* rows = unres_rows;
  for (int stage = 0; stage < 2 && h_unres > 0; ++stage) {
    const int kk = (int)std::min<int64_t>(n, stage == 0 ? 64 : KMAX_FUSED);
    if (kk <= kreq || (stage == 1 && kk <= 64)) {  // every point is already a candidate
      *still_unresolved = 0;
      return MANN_OK;
    }
    int* cand_count = nullptr;
    float* floor_val = nullptr;
    unsigned long long* counters = nullptr;
    int32_t* next_rows = nullptr;
    MANN_TRY(ctx->scratch_t(SLOT_TIES_CNT, (size_t)h_unres, &cand_count));
    MANN_TRY(ctx->scratch_t(SLOT_TIES_FLOOR, (size_t)h_unres, &floor_val));
    MANN_TRY(ctx->scratch_t(SLOT_TIES_COUNTERS, 4, &counters));
    MANN_TRY(ctx->scratch_t(stage == 0 ? SLOT_TIES_ROWS2 : SLOT_TIES_ROWS3, (size_t)h_unres, &next_rows));
    MANN_CUDA_TRY(cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned long long), s));
    // batches of at most 32 rows take the few-row scan (one point per thread
    // across the GPU) when the list fits it; a wider list scans all rows at once
    const int64_t chunk = kk <= 64 ? 32 : h_unres;
    for (int64_t r0 = 0; r0 < h_unres; r0 += chunk) {
      const int64_t nr = std::min<int64_t>(chunk, h_unres - r0);
      uint64_t* fkeys = nullptr;
      MANN_TRY(knn_fp32_keys(ctx, s, base, n, qs, nr, d, metric, kk, rows + r0, qn, bn, &fkeys,
                             SLOT_TIES_PARTIAL, SLOT_TIES_KEYS));
      fp32_lists_to_cand_kernel<<<(unsigned)ceil_div(nr, 128), 128, 0, s>>>(fkeys, nr, kk, cand_count + r0,
                                                                           floor_val + r0);
      MANN_CHECK_LAUNCH();
      MANN_TRY(launch_resolve(ctx, base, qs, d, metric, nr, kk, kreq, 1, fkeys, cand_count + r0, floor_val + r0,
                              keys_out, counters, s, rows + r0, next_rows));
    }
    unsigned long long h[2] = {0, 0};
    MANN_CUDA_TRY(cudaMemcpyAsync(h, counters, sizeof(h), cudaMemcpyDeviceToHost, s));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));
    h_unres = (int64_t)h[1];
    rows = next_rows;
    *still_unresolved = h_unres;
  }
  return MANN_OK;
}

mann_status fp32_then_resolve(Context* ctx, cudaStream_t s, const float* base, const float* qs,
                              int64_t n, int64_t nq, int d, int metric, int kk, int kreq,
                              const uint64_t* fkeys, const float* qn, const float* bn,
                              uint64_t** out_keys, mann_knn_report* rep) {
  int* cand_count = nullptr;
  float* floor_val = nullptr;
  unsigned long long* counters = nullptr;
  uint64_t* keys = nullptr;
  int32_t* unres = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_MISC0, (size_t)nq, &cand_count));
  MANN_TRY(ctx->scratch_t(SLOT_MISC1, (size_t)nq, &floor_val));
  MANN_TRY(ctx->scratch_t(SLOT_COUNTERS, 64, &counters));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_KEYS_BF16, (size_t)nq * kreq, &keys));
  MANN_TRY(ctx->scratch_t(SLOT_TIES_ROWS, (size_t)nq, &unres));
  MANN_CUDA_TRY(cudaMemsetAsync(counters, 0, 64 * sizeof(unsigned long long), s));
  fp32_lists_to_cand_kernel<<<(unsigned)ceil_div(nq, 128), 128, 0, s>>>(fkeys, nq, kk, cand_count,
                                                                       floor_val);
  MANN_CHECK_LAUNCH();
  MANN_TRY(launch_resolve(ctx, base, qs, d, metric, nq, kk, kreq, 1, fkeys, cand_count, floor_val, keys,
                          counters + 4, s, nullptr, unres));
  unsigned long long h[2] = {0, 0};
  MANN_CUDA_TRY(cudaMemcpyAsync(h, counters + 4, sizeof(h), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  int64_t left = 0;
  MANN_TRY(widen_unresolved(ctx, s, base, qs, n, d, metric, kreq, qn, bn, unres, (int64_t)h[1], keys, &left));
  if (rep) {
    rep->rows_fp64_ties = (int64_t)h[0];
    rep->rows_ties_widened = (int64_t)h[1];
    rep->rows_unresolved = left;
  }
  *out_keys = keys;
  return MANN_OK;
}

// ---------------------------------------------------------------- host side

namespace {

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
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &qr) == cudaSuccess &&
        qr == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// rows of dp BF16 values (E4M3 bytes with fp8); row r of the map is row
// r * row_step of the buffer; boxes of 128 bytes x box_rows
mann_status make_map(CUtensorMap* m, const void* ptr, int64_t rows, int dp, int box_rows,
                     int64_t row_step = 1, bool fp8 = false) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return fail(MANN_ECUDA, "cuTensorMapEncodeTiled unavailable");
  const int es_bytes = fp8 ? 1 : 2;
  cuuint64_t dims[2] = {(cuuint64_t)dp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)dp * es_bytes * (cuuint64_t)row_step};
  cuuint32_t box[2] = {(cuuint32_t)(128 / es_bytes), (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(m, fp8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                   const_cast<void*>(ptr), dims, strides, box,
                   es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(MANN_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return MANN_OK;
}

int64_t h_chunk(int c, int64_t work, int grid) { return (int64_t)((__int128)c * work / grid); }
int h_cta_of(int64_t i, int64_t work, int grid) {
  int c = (int)((__int128)i * grid / work);
  while (c + 1 < grid && h_chunk(c + 1, work, grid) <= i) ++c;
  while (c > 0 && h_chunk(c, work, grid) > i) --c;
  return c;
}

// Launch of one k2_main instance: `units` CTAs, or `units` clusters of two CTAs (PAIR).
template <int CAP, int NSETS, bool PAIR, bool FP8 = false, bool GROUPED = false, int NST = 0>
mann_status launch_k2(const CUtensorMap& mapA, const CUtensorMap& mapB, const MainArgs& ma, int units, size_t smem,
                      cudaStream_t s) {
  auto fn = k2_main<CAP, NSETS, PAIR, FP8, GROUPED, NST>;
  MANN_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(PAIR ? 2 * units : units));
  cfg.blockDim = dim3(64 + 128 * NSETS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  if (PAIR) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  MANN_CUDA_TRY(cudaLaunchKernelEx(&cfg, fn, mapA, mapB, ma));
  return MANN_OK;
}

// Clusters of two k2_main CTAs (one per SM) that can be resident at once on
// this device (0 when pairs cannot run); asked once per context and instance.
template <int CAP, int NSETS>
int k2_pair_capacity(Context* ctx) {
  const uint64_t key = 0xC2A1F00000000000ull | ((uint64_t)CAP << 8) | (uint64_t)NSETS;
  auto it = ctx->tune.find(key);
  if (it != ctx->tune.end()) return (int)it->second;
  int n = 0;
  auto fn = k2_main<CAP, NSETS, true, false>;
  const size_t smem = k2_smem_bytes<true>(CAP, NSETS);
  if (smem <= ctx->smem_optin &&
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(2 * ctx->num_sms));
    cfg.blockDim = dim3(64 + 128 * NSETS);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) n = 0;
  }
  (void)cudaGetLastError();
  ctx->tune[key] = (uint64_t)std::max(n, 0);
  return std::max(n, 0);
}

// One tensor-core pass (k2_main + k2_merge): the `depth` smallest est' of
// every query over n points (binfo row p * bstride), as sorted lists [nq][LIST].
// mapA: the queries' operand (128-row boxes); binfo_map: the points' operand
// (pass its buffer, rows and row step; the box height follows the form).
// Segmented pass: the items (in run order), the runs and each row's run
// (device), the runs on the host (for the slot span) and their count.
struct SegPass {
  const TileItem* items = nullptr;
  int64_t nitems = 0;
  const RunInfo* runs = nullptr;
  const int32_t* row_run = nullptr;
  const RunInfo* runs_host = nullptr;
  int64_t nruns = 0;
};

mann_status run_main_pass(Context* ctx, cudaStream_t s, const CUtensorMap& mapA, const void* bxb, int64_t bstride,
                          const RowInfo* qinfo, const RowInfo* binfo, const float* bnorm, int64_t n, int64_t nq,
                          int d, int dp, int mainw, int augx, int depth, const float* seed, int* err, int slot_partial, int slot_lists,
                          bool timed, uint64_t** lists_out, int seedmode = 0, const SegPass* seg = nullptr,
                          const float* qscale = nullptr, const float* bscale = nullptr, int f16 = 0) {
  const bool fp8 = qscale != nullptr;
  const int nkb = (int)(augx > 0 ? ceil_div(augx + AUG, BK) : ceil_div(mainw, fp8 ? 128 : BK));
  // passes with few K-stages per tile (the many-set pass at small d, FP16
  // rows of moderate d): three pipeline stages leave shared memory for two
  // epilogue sets of 24- or 32-entry lists, so eight warps admit candidates
  // instead of four
  const bool seg3 = !seedmode && !fp8 && depth > 16 &&
                    ((seg && depth <= 24 && nkb <= 3) || (!seg && nkb <= SHORT_K_STAGES));
  const int cap3 = depth <= 24 ? 24 : 32;
  // two epilogue sets with 16-entry lists when the depth allows it, for the
  // many-set and seed passes (each set writes its own slot); single-matrix
  // main passes keep one set, whose one list admits about half as many
  // candidates (held-out query pass 0.795 -> 0.789 ms)
  const int nsets = ((depth <= 16 && (seg || seedmode)) || seg3) ? 2 : 1;
  // CTA pairs (cta_group::2) when there are at least two 128-row query blocks
  const int pairs = (K2_USE_PAIRS && nq > BM && !seg && !fp8)
                        ? (nsets == 2 ? k2_pair_capacity<16, 2>(ctx) : k2_pair_capacity<32, 1>(ctx))
                        : 0;
  const bool pair = pairs >= 1;
  const int qrows = pair ? 2 * BM : BM;
  const int64_t qblocks = ceil_div(nq, qrows);
  const int tiles = (int)ceil_div(n, BN);
  Walk w;
  if (seg) {
    // one band over the item list in run order; a run is one block's items
    w.tiles = 1;
    w.qblocks = (int)seg->nruns;
    w.qrows = BM;
    w.work = seg->nitems;
    w.grid = (int)std::min<int64_t>(ctx->num_sms, w.work);
    w.band_tiles = 1;
    w.nbands = 1;
    w.span = 1;
    for (int64_t r = 0; r < seg->nruns; ++r) {
      const int c0 = h_cta_of(seg->runs_host[r].first, w.work, w.grid);
      const int c1 = h_cta_of(seg->runs_host[r].first + seg->runs_host[r].len - 1, w.work, w.grid);
      w.span = std::max(w.span, c1 - c0 + 1);
    }
  } else {
    w.tiles = tiles;
    w.qblocks = (int)qblocks;
    w.qrows = qrows;
    w.work = qblocks * tiles;
    w.grid = (int)std::min<int64_t>(pair ? pairs : ctx->num_sms, w.work);
    // bands: a point operand above BAND_MIN_BYTES is walked in bands of about
    // BAND_BYTES so each band stays in L2 while every query block passes over it
    const double tile_bytes = (double)BN * dp * 2.0;
    w.band_tiles = tiles;
    if (bstride == 1 && (double)n * dp * 2.0 > BAND_MIN_BYTES && ceil_div(nq, BM) >= 8)
      w.band_tiles = std::max(1, std::min(tiles, (int)(BAND_BYTES / tile_bytes)));
    w.nbands = (int)ceil_div(tiles, w.band_tiles);
    if (w.nbands > 64) {  // the merge enumerates at most 64 bands
      w.band_tiles = (int)ceil_div(tiles, 64);
      w.nbands = (int)ceil_div(tiles, w.band_tiles);
    }
    w.span = 1;
    for (int b = 0; b < w.nbands; ++b)
      for (int64_t qb = 0; qb < qblocks; ++qb) {
        const int64_t r0 = run_begin(w, b, (int)qb);
        const int c0 = h_cta_of(r0, w.work, w.grid);
        const int c1 = h_cta_of(r0 + band_len(w, b) - 1, w.work, w.grid);
        w.span = std::max(w.span, c1 - c0 + 1);
      }
  }
  const int smax = w.nbands * w.span * nsets;
  uint64_t* partial = nullptr;
  MANN_TRY(ctx->scratch_t(slot_partial, (size_t)nq * smax * LIST, &partial));
  CUtensorMap mapB;
  MANN_TRY(make_map(&mapB, bxb, n, dp, pair ? Stg<true>::B_ROWS : Stg<false>::B_ROWS, bstride, fp8));
  MainArgs ma;
  ma.nq = nq;
  ma.n = n;
  ma.d = d;
  ma.dp = mainw;
  ma.nkb = nkb;
  ma.augx = augx;
  ma.w = w;
  ma.titems = seg ? seg->items : nullptr;
  ma.qscale = qscale;
  ma.bscale = bscale;
  ma.smax = smax;
  ma.L = LIST;
  ma.depth = depth;
  ma.qinfo = qinfo;
  ma.binfo = binfo;
  ma.bnorm = bnorm;
  ma.bstride = bstride;
  ma.seed = seed;
  ma.partial = partial;
  ma.err = err;
  ma.seedmode = seedmode;
  ma.f16 = f16;
  const size_t smem = pair   ? k2_smem_bytes<true>(nsets == 2 ? 16 : 32, nsets)
                     : seg3 ? k2_smem_bytes<false>(cap3, 2, 3)
                            : k2_smem_bytes<false>(nsets == 2 ? 16 : 32, nsets);
  if (smem > ctx->smem_optin) return fail(MANN_ECUDA, "shared memory budget exceeded");
  if (timed) ctx->time_begin(s);
  if (pair) {
    if (nsets == 2)
      MANN_TRY((launch_k2<16, 2, true>(mapA, mapB, ma, w.grid, smem, s)));
    else
      MANN_TRY((launch_k2<32, 1, true>(mapA, mapB, ma, w.grid, smem, s)));
  } else if (fp8) {
    if (nsets == 2)
      MANN_TRY((launch_k2<16, 2, false, true>(mapA, mapB, ma, w.grid, smem, s)));
    else
      MANN_TRY((launch_k2<32, 1, false, true>(mapA, mapB, ma, w.grid, smem, s)));
  } else if (seg3) {
    if (cap3 == 24)
      MANN_TRY((launch_k2<24, 2, false, false, true, 3>(mapA, mapB, ma, w.grid, smem, s)));
    else
      MANN_TRY((launch_k2<32, 2, false, false, true, 3>(mapA, mapB, ma, w.grid, smem, s)));
  } else if (!seedmode && (seg || depth >= GROUPED_MIN_DEPTH)) {
    // grouped list maxima where rows admit many candidates: the many-set pass
    // (short per-set scans) and deep lists
    if (nsets == 2)
      MANN_TRY((launch_k2<16, 2, false, false, true>(mapA, mapB, ma, w.grid, smem, s)));
    else
      MANN_TRY((launch_k2<32, 1, false, false, true>(mapA, mapB, ma, w.grid, smem, s)));
  } else {
    if (nsets == 2)
      MANN_TRY((launch_k2<16, 2, false>(mapA, mapB, ma, w.grid, smem, s)));
    else
      MANN_TRY((launch_k2<32, 1, false>(mapA, mapB, ma, w.grid, smem, s)));
  }
  if (timed) ctx->time_end(s);
  MANN_CHECK_LAUNCH();
  uint64_t* lists = nullptr;
  MANN_TRY(ctx->scratch_t(slot_lists, (size_t)nq * LIST, &lists));
  k2_merge<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(partial, nq, smax, w, depth, nsets, lists,
                                                     seg ? seg->runs : nullptr, seg ? seg->row_run : nullptr);
  MANN_CHECK_LAUNCH();
  *lists_out = lists;
  return MANN_OK;
}

__global__ void seed_from_lists_kernel(const uint64_t* __restrict__ lists, int64_t nq, int e,
                                       float* __restrict__ seed) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint64_t k = lists[q * LIST + e];
  seed[q] = k == KEY_NONE ? __int_as_float(0x7F800000) : key_dist(k);
}

}  // namespace

// Prepared BF16 operand of one matrix (points or queries).
struct Bf16Operand {
  __nv_bfloat16* xb = nullptr;  // BF16 rows, or E4M3 bytes in the FP8 form
  RowInfo* info = nullptr;
  float* norms = nullptr;   // contiguous ||x~||^2 (points only)
  float* rscale = nullptr;  // FP8 form: 1/f per row
};

// Operands of one BF16 search: unit-normalised rows for cosine, the centre
// and scale chosen on a row sample, the split decision (read back: the one
// host synchronisation of the preparation), the converted rows and their
// bound terms, and the zeroed counters [2] candidates, [4..5] resolve,
// [8] error word + fallback count (as ints), [16..49] depth histogram.
struct Bf16Prep {
  Bf16Operand B, Q;
  int split = 0, dp = 0, dpe = 0;
  int f16 = 0;    // FP16 main columns (the FP16 form)
  int width = 0;  // operand row length: mainw + AUG (BF16), dp (FP8)
  int mainw = 0;  // main columns: dpe zero-padded to a multiple of 16 (BF16), dp (FP8)
  int augx = 0;   // first augmented column (BF16: mainw), 0 without the norm fold
  float* scale = nullptr;
  BaseMax* bmax = nullptr;
  float *cos_bn = nullptr, *cos_qn = nullptr;
  unsigned long long* counters = nullptr;
  int* err = nullptr;
  int* fb_count = nullptr;
};

// Fills P's query-side operand (converting the queries unless they are the
// points themselves in an unsplit form), the zeroed counters and the fields.
static mann_status prep_finish(Context* ctx, cudaStream_t s, const float* mqs, int64_t nq, int d, bool self,
                               const float* rn_q, const float* mu, float* scale, BaseMax* bmax, int split, bool f16,
                               int dp, int dpe, int mainw, int augx, int width, const Bf16Operand& B,
                               float* cos_bn, float* cos_qn, Bf16Prep* P) {
  Bf16Operand Q;
  if (self && !split) {
    Q = B;
  } else {
    MANN_TRY(ctx->scratch_t(SLOT_BF16_Q, (size_t)nq * width, &Q.xb));
    MANN_TRY(ctx->scratch_t(SLOT_ROWINFO_Q, (size_t)nq, &Q.info));
    convert_rows_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(mqs, nq, d, dp, augx, width, mu, scale, Q.xb,
                                                                  Q.info, nullptr, nullptr, split, 0, f16 ? 1 : 0,
                                                                  rn_q);
    MANN_CHECK_LAUNCH();
  }
  unsigned long long* counters = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_COUNTERS, 64, &counters));
  MANN_CUDA_TRY(cudaMemsetAsync(counters, 0, 64 * sizeof(unsigned long long), s));
  P->B = B;
  P->Q = Q;
  P->split = split;
  P->f16 = f16 ? 1 : 0;
  P->dp = dp;
  P->dpe = dpe;
  P->width = width;
  P->mainw = mainw;
  P->augx = augx;
  P->scale = scale;
  P->bmax = bmax;
  P->cos_bn = cos_bn;
  P->cos_qn = cos_qn;
  P->counters = counters;
  P->err = reinterpret_cast<int*>(counters + 8);
  P->fb_count = P->err + 1;
  return MANN_OK;
}

// misc buffer of the prepared points: mu (d, padded to 32) | BaseMax | scale |
// inexact | FP16 scale, 64 floats past mu; then the cosine row norms (n)
static inline size_t misc_floats(int d, int64_t n, bool cosine) {
  return (size_t)((d + 31) & ~31) + 64 + (cosine ? (size_t)n : 0);
}

// grows one cached device buffer (the old one is freed: cudaFree waits for the device)
static bool cache_reserve(void** buf, size_t* have, size_t want) {
  if (*buf && *have >= want) return true;
  if (*buf) (void)cudaFree(*buf);
  *buf = nullptr;
  *have = 0;
  if (cudaMalloc(buf, want) != cudaSuccess) {
    (void)cudaGetLastError();
    *buf = nullptr;
    return false;
  }
  *have = want;
  return true;
}

mann_status bf16_prepare(Context* ctx, cudaStream_t s, const float* base, int64_t n, const float* qs, int64_t nq,
                         int d, int metric, Bf16Prep* P, int form = FORM_BF16) {
  const bool fp8 = form == FORM_FP8;
  bool f16 = form == FORM_FP16;  // FORM_AUTO16 decides below, from the row sample
  // operand rows: 16-byte multiples (8 BF16 / FP16 or 16 E4M3 values)
  const int dp = fp8 ? (d + 15) & ~15 : (d + 7) & ~7;
  const bool self = (qs == base);
  const bool cosine = metric == MANN_METRIC_COSINE;
  const size_t mu_pad = (size_t)((d + 31) & ~31);

  // ---- a dataset handle's points prepared by an earlier call with the same
  // upload, metric and form: only the queries are prepared (no probe, no
  // host synchronisation, no conversion of the points)
  PointsOperand* pc = nullptr;
  uint64_t pkey = 0;
  if (!fp8 && ctx->points_owner && base == ctx->points_base) {
    pc = &ctx->points_cache[ctx->points_owner];
    // the upload's name (handle serial, generation), metric and form; never 0
    pkey = (ctx->points_generation << 8) | ((uint64_t)metric << 4) | (uint64_t)form | (1ull << 63);
  }
  if (pc && pc->key == pkey && pc->n == n && pc->d == d) {
    float* mu = pc->misc;
    BaseMax* bmax = reinterpret_cast<BaseMax*>(mu + mu_pad);
    float* scale = reinterpret_cast<float*>(bmax + 1);
    float* f16_scale = reinterpret_cast<float*>(reinterpret_cast<int*>(scale + 1) + 1);
    float *cos_bn = nullptr, *cos_qn = nullptr;
    const float* rn_q = nullptr;
    if (cosine) {
      cos_bn = mu + mu_pad + 64;
      if (self) {
        cos_qn = cos_bn;
      } else {
        MANN_TRY(ctx->scratch_t(SLOT_COS_NQ, (size_t)nq, &cos_qn));
        MANN_TRY(launch_row_sqnorm(qs, nq, d, cos_qn, s));
      }
      rn_q = cos_qn;
    }
    Bf16Operand B;
    B.xb = static_cast<__nv_bfloat16*>(pc->rows);
    const size_t off_info = ((size_t)n * pc->width * 2 + 255) & ~(size_t)255;
    B.info = reinterpret_cast<RowInfo*>(static_cast<char*>(pc->rows) + off_info);
    B.norms = reinterpret_cast<float*>(static_cast<char*>(pc->rows) + off_info +
                                       (((size_t)n * sizeof(RowInfo) + 255) & ~(size_t)255));
    return prep_finish(ctx, s, qs, nq, d, self, rn_q, mu, pc->f16 ? f16_scale : scale, bmax, pc->split,
                       pc->f16 != 0, pc->dp, pc->dpe, pc->mainw, pc->augx, pc->width, B, cos_bn, cos_qn, P);
  }
  if (pc) {
    pc->key = 0;  // (re)prepared below
    if (!cache_reserve(reinterpret_cast<void**>(&pc->misc), &pc->misc_bytes,
                       sizeof(float) * misc_floats(d, n, cosine)))
      pc = nullptr;  // no room to keep them: this call prepares into scratch
  }

  // ---- cosine: the tensor-core passes run on unit-normalised rows
  // (1 - cos = ||q^ - p^||^2 / 2); the rerank uses the original rows.  The
  // BF16 and FP16 forms normalise on the fly (rn_b / rn_q: the row norms the
  // prep kernels divide by); the FP8 conversion reads a normalised copy.
  const float* mbase = base;
  const float* mqs = qs;
  float *cos_bn = nullptr, *cos_qn = nullptr;
  const float *rn_b = nullptr, *rn_q = nullptr;
  if (cosine) {
    if (pc)
      cos_bn = pc->misc + mu_pad + 64;
    else
      MANN_TRY(ctx->scratch_t(SLOT_COS_NB, (size_t)n, &cos_bn));
    MANN_TRY(launch_row_sqnorm(base, n, d, cos_bn, s));
    if (self) {
      cos_qn = cos_bn;
    } else {
      MANN_TRY(ctx->scratch_t(SLOT_COS_NQ, (size_t)nq, &cos_qn));
      MANN_TRY(launch_row_sqnorm(qs, nq, d, cos_qn, s));
    }
    if (fp8) {
      float *xb = nullptr, *xq = nullptr;
      MANN_TRY(ctx->scratch_t(SLOT_COS_B, (size_t)n * d, &xb));
      scale_rows_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(base, n, d, cos_bn, xb);
      MANN_CHECK_LAUNCH();
      mbase = xb;
      if (self) {
        mqs = xb;
      } else {
        MANN_TRY(ctx->scratch_t(SLOT_COS_Q, (size_t)nq * d, &xq));
        scale_rows_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(qs, nq, d, cos_qn, xq);
        MANN_CHECK_LAUNCH();
        mqs = xq;
      }
    } else {
      rn_b = cos_bn;
      rn_q = cos_qn;
    }
  }

  // ---- prep
  double* cpart = nullptr;
  float* mu = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_CENTRE, 64, &cpart));
  if (pc)
    mu = pc->misc;
  else
    MANN_TRY(ctx->scratch_t(SLOT_MISC3, (size_t)d + 64, &mu));  // mu | BaseMax | scale
  BaseMax* bmax = reinterpret_cast<BaseMax*>(mu + mu_pad);
  {
    const int64_t rows = std::min<int64_t>(n, CENTRE_ROWS);
    const int64_t stride = n / rows;
    centre_sample_kernel<<<(unsigned)ceil_div(d, 32), 1024, 0, s>>>(mbase, n, d, stride, rows, mu, rn_b);
    MANN_CHECK_LAUNCH();
  }
  // pick the centre / scale with the smallest BF16 residual on a row sample
  double* score = cpart;  // probe scores
  MANN_CUDA_TRY(cudaMemsetAsync(score, 0, (NUM_SCALES + 1) * sizeof(double), s));  // scores | sampled max
  const int64_t sample_rows = std::min<int64_t>(n, 1024);
  const int64_t stride = std::max<int64_t>(1, n / sample_rows);
  dim3 pg((unsigned)ceil_div(ceil_div(n, stride), 8), NUM_SCALES);
  scale_probe_kernel<<<pg, 256, 0, s>>>(mbase, n, d, mu, stride, score, rn_b);
  MANN_CHECK_LAUNCH();
  float* scale = reinterpret_cast<float*>(bmax + 1);
  int* inexact = reinterpret_cast<int*>(scale + 1);
  float* f16_scale = reinterpret_cast<float*>(inexact + 1);
  choose_scale_kernel<<<1, 128, 0, s>>>(score, mu, d, scale, inexact, ceil_div(n, stride), f16_scale);
  MANN_CHECK_LAUNCH();
  MANN_CUDA_TRY(cudaMemsetAsync(bmax, 0, sizeof(BaseMax), s));
  // Data that BF16 cannot hold exactly (after the best centre and scale) runs
  // in the split form: x~ = hi + lo, three BF16 products per term, bounds ~2^8
  // tighter, so the certificate holds for close neighbours too.
  int h_inexact = 0;
  MANN_CUDA_TRY(cudaMemcpyAsync(&h_inexact, inexact, sizeof(int), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  if (form == FORM_AUTO16 && h_inexact) f16 = true;
  const int split = (h_inexact && form == FORM_BF16) ? 1 : 0;  // the FP8 and FP16 forms have no split
  if (f16) scale = f16_scale;  // the conversion and the certificate use the FP16 form's scale
  const int dpe = split ? 3 * dp : dp;  // columns of the tensor-core operands
  Bf16Operand B;
  if (fp8) {
    // E4M3 rows with per-row power-of-two scales (dp bytes per row), no norm fold
    Bf16Operand Q;
    P->width = dp;
    P->mainw = dp;
    P->augx = 0;
    MANN_TRY(ctx->scratch_t(SLOT_BF16_B, (size_t)n * dp / 2 + 1, &B.xb));
    MANN_TRY(ctx->scratch_t(SLOT_ROWINFO_B, (size_t)n, &B.info));
    MANN_TRY(ctx->scratch_t(SLOT_NORMS_B, (size_t)n, &B.norms));
    MANN_TRY(ctx->scratch_t(SLOT_FP8_SCALE_B, (size_t)n, &B.rscale));
    convert_rows_fp8_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(mbase, n, d, dp, mu, scale,
                                                                    reinterpret_cast<uint8_t*>(B.xb), B.rscale,
                                                                    B.info, B.norms, bmax);
    MANN_CHECK_LAUNCH();
    if (self) {
      Q = B;
    } else {
      MANN_TRY(ctx->scratch_t(SLOT_BF16_Q, (size_t)nq * dp / 2 + 1, &Q.xb));
      MANN_TRY(ctx->scratch_t(SLOT_ROWINFO_Q, (size_t)nq, &Q.info));
      MANN_TRY(ctx->scratch_t(SLOT_FP8_SCALE_Q, (size_t)nq, &Q.rscale));
      convert_rows_fp8_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(mqs, nq, d, dp, mu, scale,
                                                                       reinterpret_cast<uint8_t*>(Q.xb), Q.rscale,
                                                                       Q.info, nullptr, nullptr);
      MANN_CHECK_LAUNCH();
    }
    unsigned long long* counters = nullptr;
    MANN_TRY(ctx->scratch_t(SLOT_COUNTERS, 64, &counters));
    MANN_CUDA_TRY(cudaMemsetAsync(counters, 0, 64 * sizeof(unsigned long long), s));
    P->B = B;
    P->Q = Q;
    P->split = 0;
    P->f16 = 0;
    P->dp = dp;
    P->dpe = dpe;
    P->scale = scale;
    P->bmax = bmax;
    P->cos_bn = cos_bn;
    P->cos_qn = cos_qn;
    P->counters = counters;
    P->err = reinterpret_cast<int*>(counters + 8);
    P->fb_count = P->err + 1;
    return MANN_OK;
  }
  // rows: [main (dpe) | zeros up to augx | the first 16 norm-fold columns];
  // the fold's last 8 columns (zeros) lie past the row, where TMA fills zeros.
  // augx is mainw (dpe rounded up to 16) when the fold's 24 columns fit in
  // that stage, else the next stage.  Rows are 32-byte multiples (rows that
  // straddle 32-byte sectors slowed k2_main 1.6x).
  const int mainw = (dpe + 15) & ~15;
  const int augx = (mainw % BK) + AUG <= BK ? mainw : (mainw + BK - 1) / BK * BK;  // fold inside one stage
  const int width = augx + 16;
  const size_t off_info = ((size_t)n * width * 2 + 255) & ~(size_t)255;
  const size_t off_norms = off_info + (((size_t)n * sizeof(RowInfo) + 255) & ~(size_t)255);
  if (pc && !cache_reserve(&pc->rows, &pc->rows_bytes, off_norms + (size_t)n * sizeof(float))) pc = nullptr;
  if (pc) {
    B.xb = static_cast<__nv_bfloat16*>(pc->rows);
    B.info = reinterpret_cast<RowInfo*>(static_cast<char*>(pc->rows) + off_info);
    B.norms = reinterpret_cast<float*>(static_cast<char*>(pc->rows) + off_norms);
  } else {
    MANN_TRY(ctx->scratch_t(SLOT_BF16_B, (size_t)n * width, &B.xb));
    MANN_TRY(ctx->scratch_t(SLOT_ROWINFO_B, (size_t)n, &B.info));
    MANN_TRY(ctx->scratch_t(SLOT_NORMS_B, (size_t)n, &B.norms));
  }
  convert_rows_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(mbase, n, d, dp, augx, width, mu, scale, B.xb,
                                                              B.info, B.norms, bmax, split, 1, f16 ? 1 : 0, rn_b);
  MANN_CHECK_LAUNCH();
  if (pc) {
    // the handle's points are prepared: later calls with this upload, metric and form reuse them
    pc->n = n;
    pc->d = d;
    pc->split = split;
    pc->f16 = f16 ? 1 : 0;
    pc->dp = dp;
    pc->dpe = dpe;
    pc->width = width;
    pc->mainw = mainw;
    pc->augx = augx;
    pc->key = pkey;
  }
  return prep_finish(ctx, s, mqs, nq, d, self, rn_q, mu, scale, bmax, split, f16, dp, dpe, mainw, augx, width, B,
                     cos_bn, cos_qn, P);
}

// The autotuned admission depth (list entries a certificate may need) from
// the depth histogram of a rerank: the 99.9th percentile + 1, 16 when that
// is <= 16 (the two-set kernel), the full list when > 0.1 % of rows fell back.
int tuned_depth(const unsigned long long* hist, int kreq) {
  const int L = LIST;
  unsigned long long total = 0, acc = 0;
  for (int j = 0; j <= L + 1; ++j) total += hist[j];
  if (hist[L + 1] * 1000 > total) return L;
  for (int j = 0; j <= L; ++j) {
    acc += hist[j];
    if (acc * 1000 >= total * 999) {
      int want = std::min(L, std::max(kreq + 2, j + 1));
      if (want <= 16) want = 16;
      return want;
    }
  }
  return L;
}

mann_status knn_bf16_keys(Context* ctx, cudaStream_t s, const float* base, int64_t n,
                          const float* qs, int64_t nq, int d, int metric, int kreq, int margin,
                          bool fp64, uint64_t** out_keys, mann_knn_report* rep, int form) {
  if (nq <= 0) return MANN_OK;
  const int L = LIST;
  const bool fp8 = form == FORM_FP8;
  // admission depth = k + margin.  margin > 0: as given.  margin == 0: the
  // autotuner's choice for this shape class -- the full list on first sight,
  // then the depth 99.9% of rows needed plus one (refreshed after every call).
  const uint64_t tkey = ((uint64_t)kreq << 56) ^ ((uint64_t)d << 36) ^ ((uint64_t)metric << 32) ^
                        (uint64_t)(n >> 10) ^ ((uint64_t)(qs == base) << 63) ^ ((uint64_t)form << 60);
  int depth = L;
  if (kreq > KREQ_MAX_BF16)
    return fail(MANN_EINVAL_ARG, "the BF16 form supports k <= " + std::to_string(KREQ_MAX_BF16) +
                                     " (k+1 for graphs)");
  const bool cosine = metric == MANN_METRIC_COSINE;
  Bf16Prep P;
  MANN_TRY(bf16_prepare(ctx, s, base, n, qs, nq, d, metric, &P, form));
  const int split = P.split, dpe = P.dpe;
  if (margin > 0) {
    depth = std::min(L, kreq + margin);
  } else {
    auto it = ctx->tune.find(tkey ^ ((uint64_t)split << 62) ^ ((uint64_t)P.f16 << 59));
    depth = it != ctx->tune.end() ? (int)it->second : L;
  }
  Bf16Operand B = P.B, Q = P.Q;
  float* scale = P.scale;
  BaseMax* bmax = P.bmax;
  float *cos_bn = P.cos_bn, *cos_qn = P.cos_qn;
  unsigned long long* counters = P.counters;
  int* err = P.err;
  int* fb_count = P.fb_count;

  CUtensorMap mapA;
  MANN_TRY(make_map(&mapA, Q.xb, nq, P.width, BM, 1, fp8));

  // ---- seed pass: over an evenly spaced sample of SEED_SAMPLE points, the
  // SEED_DEPTH-th smallest 32-column chunk minimum of each query (an upper
  // bound of its SEED_DEPTH-th smallest est' there, roughly its
  // 5n/SEED_SAMPLE-th neighbour) becomes its admission seed in the main pass,
  // which spares most insertions.  A seed below the row's k-th estimate
  // leaves the row uncertified.
  float* seed = nullptr;
  if (n >= 16 * SEED_SAMPLE) {
    const int64_t bstride = n / SEED_SAMPLE;
    uint64_t* slists = nullptr;
    MANN_TRY(run_main_pass(ctx, s, mapA, B.xb, bstride, Q.info, B.info, B.norms, SEED_SAMPLE, nq, d, P.width, P.mainw, P.augx,
                           SEED_DEPTH, nullptr, err, SLOT_SEED_PARTIAL, SLOT_SEED_LISTS, false, &slists, 1,
                           nullptr, Q.rscale, B.rscale, P.f16));
    MANN_TRY(ctx->scratch_t(SLOT_SEED, (size_t)nq, &seed));
    seed_from_lists_kernel<<<(unsigned)ceil_div(nq, 256), 256, 0, s>>>(slists, nq, SEED_DEPTH - 1, seed);
    MANN_CHECK_LAUNCH();
  }

  // ---- main pass over every point
  uint64_t* lists = nullptr;
  MANN_TRY(run_main_pass(ctx, s, mapA, B.xb, 1, Q.info, B.info, B.norms, n, nq, d, P.width, P.mainw, P.augx, depth, seed, err,
                         SLOT_PARTIAL, SLOT_KEYS, true, &lists, 0, nullptr, Q.rscale, B.rscale, P.f16));

  // ---- certify + rerank
  uint64_t* cand = nullptr;
  int* cand_count = nullptr;
  float* floor_val = nullptr;
  int* fb_rows = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_CAND, (size_t)nq * L, &cand));
  MANN_TRY(ctx->scratch_t(SLOT_MISC0, (size_t)nq, &cand_count));
  MANN_TRY(ctx->scratch_t(SLOT_MISC1, (size_t)nq, &floor_val));
  MANN_TRY(ctx->scratch_t(SLOT_FALLBACK, (size_t)nq, &fb_rows));
  RerankArgs ra;
  ra.base = base;
  ra.qs = qs;
  ra.nq = nq;
  ra.n = n;
  ra.d = d;
  ra.L = L;
  ra.kreq = kreq;
  ra.metric = metric;
  ra.scale = scale;
  ra.depth = depth;
  ra.seed = seed;
  ra.depth_hist = counters + 16;
  ra.qinfo = Q.info;
  ra.bmax = bmax;
  ra.lists = lists;
  ra.cand = cand;
  ra.cand_count = cand_count;
  ra.floor_val = floor_val;
  ra.fb_rows = fb_rows;
  ra.fb_count = fb_count;
  ra.cand_total = counters + 2;
  // the norm fold adds one 16-term K-step to the accumulation
  ra.kdim = P.augx > 0 ? P.mainw + 16 : dpe;
  ra.full_est = P.augx > 0 ? 1 : 0;
  ra.cos_qn = cos_qn;
  ra.cos_bn = cos_bn;
  {
    const double u = 5.9604644775390625e-08;
    const double gd = (double)d * u / (1.0 - (double)d * u);
    ra.eps_c = std::nextafter((float)(1.25 * (4.0 * gd + 16.0 * u)), 1.0f);
  }
  ra.coop = (d % 4 == 0 && ((reinterpret_cast<uintptr_t>(base) | reinterpret_cast<uintptr_t>(qs)) & 15) == 0) ? 1 : 0;
  k2_rerank<<<(unsigned)std::min<int64_t>(ceil_div(nq, RR_WARPS), (int64_t)ctx->num_sms * 6), 32 * RR_WARPS, 0,
              s>>>(ra);
  MANN_CHECK_LAUNCH();

  // ---- exact FP32 scan of uncertified rows (count known only on the device:
  // read it back; the common case is zero rows)
  unsigned long long hc[64];
  MANN_CUDA_TRY(cudaMemcpyAsync(hc, counters, sizeof(hc), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  const int h_err = reinterpret_cast<const int*>(hc + 8)[0];
  const int h_fb = reinterpret_cast<const int*>(hc + 8)[1];
  if (margin <= 0 && h_err == 0) {
    // autotune the admission depth (the k-margin) from the depths the certificates needed
    ctx->tune[tkey ^ ((uint64_t)split << 62) ^ ((uint64_t)P.f16 << 59)] = (uint64_t)tuned_depth(hc + 16, kreq);
  }
  if (h_err != 0)
    return fail(MANN_ETIMEOUT, "tensor-core kernel: a bounded wait ran out (role " + std::to_string(h_err) + ")");
  if (h_fb > 0) {
    const int kk = (int)std::min<int64_t>(std::min<int64_t>(n, KMAX_FUSED), std::min(L, kreq + 32));
    uint64_t* fkeys = nullptr;
    const float* no_norm = nullptr;
    MANN_TRY(knn_fp32_keys(ctx, s, base, n, qs, h_fb, d, metric, kk, fb_rows, cosine ? cos_qn : no_norm,
                           cosine ? cos_bn : no_norm, &fkeys, SLOT_FALLBACK_KEYS, SLOT_MISC2));
    k2_scatter_fallback<<<h_fb, 64, 0, s>>>(fkeys, fb_rows, fb_count, kk, L, cand, cand_count, floor_val);
    MANN_CHECK_LAUNCH();
  }

  // ---- resolve + truncate
  uint64_t* keys = nullptr;
  int32_t* unres = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_OUT_KEYS_BF16, (size_t)nq * kreq, &keys));
  if (fp64) MANN_TRY(ctx->scratch_t(SLOT_TIES_ROWS, (size_t)nq, &unres));
  MANN_TRY(launch_resolve(ctx, base, qs, d, metric, nq, L, kreq, fp64 ? 1 : 0, cand, cand_count, floor_val,
                          keys, counters + 4, s, nullptr, unres));
  if (rep || fp64) {
    unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
    MANN_CUDA_TRY(cudaMemcpyAsync(h, counters, sizeof(h), cudaMemcpyDeviceToHost, s));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));
    int64_t left = 0;
    if (fp64)
      MANN_TRY(widen_unresolved(ctx, s, base, qs, n, d, metric, kreq, cosine ? cos_qn : nullptr,
                                cosine ? cos_bn : nullptr, unres, (int64_t)h[5], keys, &left));
    if (rep) {
      rep->rows_fallback = h_fb;
      rep->candidates = (int64_t)h[2];
      rep->rows_fp64_ties = (int64_t)h[4];
      rep->rows_ties_widened = fp64 ? (int64_t)h[5] : 0;
      rep->rows_unresolved = left;
      rep->precision_used = fp8 ? MANN_PREC_FP8 : (P.f16 ? MANN_PREC_FP16 : MANN_PREC_BF16);
      rep->margin_used = depth - kreq;
    }
  }
  *out_keys = keys;
  return MANN_OK;
}


// ---------------------------------------------------------------- many point sets (segmented)

namespace {

// Items, runs and row -> run table of one set layout, kept on the host and
// uploaded once per layout.
struct SegTables {
  uint64_t hash = 0;
  std::vector<TileItem> items;
  std::vector<RunInfo> runs;
  std::vector<int32_t> row_run;
  // seed pass: each block against its own set's every SEG_SEED_STRIDE-th point
  // (rows of a strided map over the same operand)
  std::vector<TileItem> sitems;
  std::vector<RunInfo> sruns;
  std::vector<int32_t> srow_run;
  const void* uploaded = nullptr;  // device items buffer the tables were copied to
  const void* suploaded = nullptr;  // device seed-items buffer
  uint64_t uploaded_hash = 0;
};
std::mutex g_seg_mu;
std::map<Context*, SegTables*> g_seg;

SegTables& seg_tables(Context* ctx) {
  std::lock_guard<std::mutex> lk(g_seg_mu);
  SegTables*& t = g_seg[ctx];
  if (!t) t = new SegTables();
  return *t;
}

void build_seg_tables(const int64_t* offs, int nsets, SegTables* T) {
  uint64_t h = 1469598103934665603ull;
  for (int c = 0; c <= nsets; ++c) {
    h ^= (uint64_t)offs[c];
    h *= 1099511628211ull;
  }
  if (T->hash == h && !T->items.empty()) return;
  T->items.clear();
  T->runs.clear();
  T->row_run.assign((size_t)offs[nsets], 0);
  T->sitems.clear();
  T->sruns.clear();
  T->srow_run.assign((size_t)offs[nsets], 0);
  for (int c = 0; c < nsets; ++c) {
    const int64_t o = offs[c], nc = offs[c + 1] - offs[c];
    // the set's sampled points: map rows i with i * stride in [o, o + nc)
    const int64_t s0 = (o + SEG_SEED_STRIDE - 1) / SEG_SEED_STRIDE;
    const int64_t s1 = (o + nc + SEG_SEED_STRIDE - 1) / SEG_SEED_STRIDE;
    for (int64_t q = 0; q < nc; q += BM) {
      const int64_t first = (int64_t)T->items.size();
      for (int64_t t = 0; t < nc; t += BN) T->items.push_back(TileItem{o + q, o + nc, o + t, o + nc, first});
      const int32_t r = (int32_t)T->runs.size();
      T->runs.push_back(RunInfo{first, (int64_t)T->items.size() - first});
      for (int64_t row = o + q; row < std::min(o + q + BM, o + nc); ++row) T->row_run[(size_t)row] = r;
      const int64_t sfirst = (int64_t)T->sitems.size();
      for (int64_t t = s0; t < s1; t += BN) T->sitems.push_back(TileItem{o + q, o + nc, t, s1, sfirst});
      if (s1 == s0) T->sitems.push_back(TileItem{o + q, o + nc, s0, s0, sfirst});  // no sample: an empty item
      const int32_t sr = (int32_t)T->sruns.size();
      T->sruns.push_back(RunInfo{sfirst, (int64_t)T->sitems.size() - sfirst});
      for (int64_t row = o + q; row < std::min(o + q + BM, o + nc); ++row) T->srow_run[(size_t)row] = sr;
    }
  }
  T->hash = h;
}

}  // namespace

// Self-kNN keys of many independent point sets stored back to back (set c is
// rows [offs[c], offs[c+1])), each searched against its own points only, in
// the BF16 form: one operand preparation over all rows, one segmented k2_main
// pass over every (set, 128-row block, 256-point tile) item, the certificate
// and exact FP32 rerank per row, uncertified rows re-scanned exactly over
// their own set on the device (work queue published by a kernel, so the host
// never waits for their count), and the (distance, id) truncation to kreq.
// Result: keys [N][kreq] with global ids (the row itself included).
mann_status knn_bf16_batched_keys(Context* ctx, cudaStream_t s, const float* data, const int64_t* offs_host,
                                  const int64_t* offs_dev, int nsets, int d, int metric, int kreq, int margin,
                                  uint64_t** out_keys, mann_knn_report* rep, int form) {
  const int L = LIST;
  if (kreq > KREQ_MAX_BF16)
    return fail(MANN_EINVAL_ARG, "the BF16 form supports k <= " + std::to_string(KREQ_MAX_BF16) +
                                     " (k+1 for graphs)");
  if (metric != MANN_METRIC_EUCLIDEAN && metric != MANN_METRIC_SQEUCLIDEAN)
    return fail(MANN_EINVAL_ARG, "batched graphs: Euclidean or SqEuclidean");
  const int64_t N = offs_host[nsets];
  SegTables& T = seg_tables(ctx);
  build_seg_tables(offs_host, nsets, &T);
  TileItem* d_items = nullptr;
  RunInfo* d_runs = nullptr;
  int32_t* d_row_run = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_SEG_ITEMS, T.items.size(), &d_items));
  MANN_TRY(ctx->scratch_t(SLOT_SEG_RUNS, T.runs.size(), &d_runs));
  MANN_TRY(ctx->scratch_t(SLOT_SEG_ROWRUN, (size_t)N, &d_row_run));
  TileItem* d_sitems = nullptr;
  RunInfo* d_sruns = nullptr;
  int32_t* d_srow_run = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_SEG_SITEMS, T.sitems.size(), &d_sitems));
  MANN_TRY(ctx->scratch_t(SLOT_SEG_SRUNS, T.sruns.size(), &d_sruns));
  MANN_TRY(ctx->scratch_t(SLOT_SEG_SROWRUN, (size_t)N, &d_srow_run));
  if (T.uploaded != d_items || T.suploaded != d_sitems || T.uploaded_hash != T.hash) {
    MANN_CUDA_TRY(cudaMemcpyAsync(d_items, T.items.data(), sizeof(TileItem) * T.items.size(), cudaMemcpyHostToDevice, s));
    MANN_CUDA_TRY(cudaMemcpyAsync(d_runs, T.runs.data(), sizeof(RunInfo) * T.runs.size(), cudaMemcpyHostToDevice, s));
    MANN_CUDA_TRY(cudaMemcpyAsync(d_row_run, T.row_run.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice, s));
    MANN_CUDA_TRY(cudaMemcpyAsync(d_sitems, T.sitems.data(), sizeof(TileItem) * T.sitems.size(),
                                  cudaMemcpyHostToDevice, s));
    MANN_CUDA_TRY(cudaMemcpyAsync(d_sruns, T.sruns.data(), sizeof(RunInfo) * T.sruns.size(), cudaMemcpyHostToDevice, s));
    MANN_CUDA_TRY(cudaMemcpyAsync(d_srow_run, T.srow_run.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice, s));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));  // the copies read pageable host memory
    T.uploaded = d_items;
    T.suploaded = d_sitems;
    T.uploaded_hash = T.hash;
  }
  Bf16Prep P;
  MANN_TRY(bf16_prepare(ctx, s, data, N, data, N, d, metric, &P, form));
  // the admission depth (k-margin): tuned per (layout, k, d, metric, form)
  const uint64_t tkey = 0x5E6B000000000000ull ^ (T.hash >> 8) ^ ((uint64_t)kreq << 40) ^ ((uint64_t)d << 24) ^
                        ((uint64_t)metric << 20) ^ ((uint64_t)P.split << 19) ^ ((uint64_t)P.f16 << 18);
  int depth = L;
  if (margin > 0) {
    depth = std::min(L, kreq + margin);
  } else {
    auto it = ctx->tune.find(tkey);
    if (it != ctx->tune.end()) depth = (int)it->second;
  }
  CUtensorMap mapA;
  MANN_TRY(make_map(&mapA, P.Q.xb, N, P.width, BM));
  SegPass sp;
  sp.items = d_items;
  sp.nitems = (int64_t)T.items.size();
  sp.runs = d_runs;
  sp.row_run = d_row_run;
  sp.runs_host = T.runs.data();
  sp.nruns = (int64_t)T.runs.size();
  // ---- seed pass: each row's SEED_DEPTH-th smallest chunk minimum over
  // every SEG_SEED_STRIDE-th point of its own set bounds its estimates from
  // above (a set with no sampled point gets no seed), so the main pass admits
  // ~3x fewer candidates
  SegPass ssp;
  ssp.items = d_sitems;
  ssp.nitems = (int64_t)T.sitems.size();
  ssp.runs = d_sruns;
  ssp.row_run = d_srow_run;
  ssp.runs_host = T.sruns.data();
  ssp.nruns = (int64_t)T.sruns.size();
  uint64_t* slists = nullptr;
  const int64_t nsample = (N + SEG_SEED_STRIDE - 1) / SEG_SEED_STRIDE;
  MANN_TRY(run_main_pass(ctx, s, mapA, P.B.xb, SEG_SEED_STRIDE, P.Q.info, P.B.info, P.B.norms, nsample, N, d, P.width,
                         P.mainw, P.augx, SEED_DEPTH, nullptr, P.err, SLOT_SEED_PARTIAL, SLOT_SEED_LISTS, false, &slists,
                         1, &ssp, nullptr, nullptr, P.f16));
  float* seed = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_SEED, (size_t)N, &seed));
  seed_from_lists_kernel<<<(unsigned)ceil_div(N, 256), 256, 0, s>>>(slists, N, SEED_DEPTH - 1, seed);
  MANN_CHECK_LAUNCH();
  uint64_t* lists = nullptr;
  MANN_TRY(run_main_pass(ctx, s, mapA, P.B.xb, 1, P.Q.info, P.B.info, P.B.norms, N, N, d, P.width, P.mainw, P.augx, depth, seed,
                         P.err, SLOT_PARTIAL, SLOT_KEYS, true, &lists, 0, &sp, nullptr, nullptr, P.f16));
  // ---- certify + rerank (per row; the bounds are global, so valid for every set)
  uint64_t* cand = nullptr;
  int* cand_count = nullptr;
  float* floor_val = nullptr;
  int* fb_rows = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_CAND, (size_t)N * L, &cand));
  MANN_TRY(ctx->scratch_t(SLOT_MISC0, (size_t)N, &cand_count));
  MANN_TRY(ctx->scratch_t(SLOT_MISC1, (size_t)N, &floor_val));
  MANN_TRY(ctx->scratch_t(SLOT_FALLBACK, (size_t)N, &fb_rows));
  RerankArgs ra;
  ra.base = data;
  ra.qs = data;
  ra.nq = N;
  ra.n = N;
  ra.d = d;
  ra.L = L;
  ra.kreq = kreq;
  ra.metric = metric;
  ra.scale = P.scale;
  ra.depth = depth;
  ra.seed = seed;
  ra.depth_hist = P.counters + 16;
  ra.qinfo = P.Q.info;
  ra.bmax = P.bmax;
  ra.lists = lists;
  ra.cand = cand;
  ra.cand_count = cand_count;
  ra.floor_val = floor_val;
  ra.fb_rows = fb_rows;
  ra.fb_count = P.fb_count;
  ra.cand_total = P.counters + 2;
  ra.kdim = P.augx > 0 ? P.mainw + 16 : P.dpe;
  ra.full_est = P.augx > 0 ? 1 : 0;
  ra.cos_qn = nullptr;
  ra.cos_bn = nullptr;
  ra.eps_c = 0.0f;
  ra.coop = (d % 4 == 0 && (reinterpret_cast<uintptr_t>(data) & 15) == 0) ? 1 : 0;
  k2_rerank<<<(unsigned)std::min<int64_t>(ceil_div(N, RR_WARPS), (int64_t)ctx->num_sms * 6), 32 * RR_WARPS, 0,
              s>>>(ra);
  MANN_CHECK_LAUNCH();
  // ---- uncertified rows: exact FP32 scan of their own set, on the device;
  // each row's set is cut into FB_CHUNK-point items so that a few rows of the
  // largest sets spread over the GPU (one item per row: 1.8 ms for 124 rows)
  int h_fbc = 0;
  MANN_CUDA_TRY(cudaMemcpyAsync(&h_fbc, P.fb_count, sizeof(int), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  SegQueue* fq = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_SEG_QUEUE, 1, &fq));
  if (h_fbc > 0) {
    int64_t max_set = 1;
    for (int i = 0; i < nsets; ++i) max_set = std::max(max_set, offs_host[i + 1] - offs_host[i]);
    int64_t chunk = std::max<int64_t>(FB_CHUNK, ceil_div(max_set, 128));  // the merge takes <= 128 lists
    const int nsplit = (int)ceil_div(max_set, chunk);
    const int64_t nitems = (int64_t)h_fbc * nsplit;
    if (nitems > INT32_MAX) return fail(MANN_EINVAL_ARG, "batched graphs: too many fallback items");
    SegItem* fitems = nullptr;
    uint64_t* fpart = nullptr;
    uint64_t* fkeys = nullptr;
    MANN_TRY(ctx->scratch_t(SLOT_FALLBACK_KEYS, (size_t)nitems, &fitems));
    MANN_TRY(ctx->scratch_t(SLOT_PARTIAL, (size_t)nitems * L, &fpart));  // the main pass's slots are merged
    MANN_TRY(ctx->scratch_t(SLOT_SEED_PARTIAL, (size_t)h_fbc * L, &fkeys));
    const int gfb = ctx->num_sms * 8;
    fb_items_kernel<<<gfb, 256, 0, s>>>(fb_rows, h_fbc, offs_dev, nsets, nsplit, chunk, fitems);
    MANN_CHECK_LAUNCH();
    static unsigned fb_epoch = 0x40000000u;
    const unsigned ep = ++fb_epoch;
    MANN_TRY(launch_publish_queue(fq, (int)nitems, nullptr, ep, s));
    MANN_TRY(launch_k1_persistent(ctx->num_sms, data, fitems, fq, ep, 1ll << 31, d, metric, 32, L, nsplit,
                                  nsplit > 1 ? fpart : fkeys, s, fb_rows));
    if (nsplit > 1) MANN_TRY(launch_merge_lists(fpart, h_fbc, nsplit, L, fkeys, s));
    fb_finish_kernel<<<gfb, 256, 0, s>>>(fb_rows, h_fbc, fkeys, cand, cand_count, floor_val);
    MANN_CHECK_LAUNCH();
  }
  // ---- truncate to kreq (ties at the k-th distance keep the FP32 (distance, id) order)
  uint64_t* keys = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_OUT_KEYS_BF16, (size_t)N * kreq, &keys));
  MANN_TRY(launch_resolve(ctx, data, data, d, metric, N, L, kreq, 0, cand, cand_count, floor_val, keys,
                          P.counters + 4, s));
  // ---- status, report, and the depth for the next call of this layout
  unsigned long long hc[64];
  MANN_CUDA_TRY(cudaMemcpyAsync(hc, P.counters, sizeof(hc), cudaMemcpyDeviceToHost, s));
  int qstatus = 0;  // (the queue is published only when some row fell back)
  if (h_fbc > 0) MANN_CUDA_TRY(cudaMemcpyAsync(&qstatus, &fq->status, sizeof(int), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  const int h_err = reinterpret_cast<const int*>(hc + 8)[0];
  const int h_fb = reinterpret_cast<const int*>(hc + 8)[1];
  if (h_err != 0)
    return fail(MANN_ETIMEOUT, "tensor-core kernel: a bounded wait ran out (role " + std::to_string(h_err) + ")");
  if (qstatus != 0) return fail(MANN_ETIMEOUT, "batched graphs: the fallback work queue was not published in time");
  if (margin <= 0) ctx->tune[tkey] = (uint64_t)tuned_depth(hc + 16, kreq);
  if (rep) {
    rep->rows_fallback = h_fb;
    rep->candidates = (int64_t)hc[2];
    rep->precision_used = P.f16 ? MANN_PREC_FP16 : MANN_PREC_BF16;
    rep->margin_used = depth - kreq;
  }
  *out_keys = keys;
  return MANN_OK;
}

}  // namespace mann
