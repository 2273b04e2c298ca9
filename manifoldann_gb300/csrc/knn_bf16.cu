// knn_bf16.cu -- exact kNN through BF16 tensor-core tiles (tcgen05 / TMEM),
// a certified top-(k+m) candidate set, exact FP32 rerank and FP64 near-tie
// resolution.  Metrics: SqEuclidean and Euclidean.
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

#include <algorithm>
#include <mutex>

#include "kernels.cuh"
#include "ptx.cuh"

namespace mann {

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr int BM = 128;          // queries per CTA tile (TMEM lanes)
constexpr int BN = 256;          // points per tile (TMEM columns per accumulator)
constexpr int BK = 64;           // BF16 elements per stage row (128 bytes, one swizzle span)
constexpr int STAGES = 3;
constexpr int A_STAGE_BYTES = BM * BK * 2;  // 16 KB
constexpr int B_STAGE_BYTES = BN * BK * 2;  // 32 KB
constexpr int STAGE_BYTES = A_STAGE_BYTES + B_STAGE_BYTES;
constexpr int NUM_EPI_WARPS = 4;
constexpr int K2_THREADS = 64 + NUM_EPI_WARPS * 32;  // producer, MMA, 4 epilogue warps
constexpr int STAGE_CAP = 16;                        // staged candidates per row per 16-column chunk
constexpr uint32_t TMEM_COLS = 2 * BN;               // double-buffered accumulator

enum : int { ERR_TIMEOUT_PRODUCER = 1, ERR_TIMEOUT_MMA = 2, ERR_TIMEOUT_EPI = 3 };

struct RowInfo {
  float nrm;    // ||x~||^2 (FP64 sum rounded to nearest)
  float xn_up;  // ||x~|| rounded up
  float r_up;   // bound on ||(x - mu) - x~|| (includes the FP32 rounding of x - mu)
  float pad;
};

struct BaseMax {
  unsigned xn_bits;  // max over points of xn_up (positive float bits, integer max)
  unsigned r_bits;   // max over points of r_up
};

// ---------------------------------------------------------------- prep kernels

// partial column sums over a chunk of rows (deterministic order)
__global__ void centre_partial_kernel(const float* __restrict__ x, int64_t n, int d, int64_t rows_per,
                                      double* __restrict__ partial) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d) return;
  const int64_t r0 = (int64_t)blockIdx.y * rows_per;
  const int64_t r1 = min(n, r0 + rows_per);
  double s = 0.0;
  for (int64_t r = r0; r < r1; ++r) s += (double)x[r * d + c];
  partial[(int64_t)blockIdx.y * d + c] = s;
}

__global__ void centre_final_kernel(const double* __restrict__ partial, int chunks, int d, int64_t n,
                                    float* __restrict__ mu) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d) return;
  double s = 0.0;
  for (int i = 0; i < chunks; ++i) s += partial[(int64_t)i * d + c];
  mu[c] = (float)(s / (double)n);
}

__device__ __forceinline__ float round_up_f(double v) {
  float f = __double2float_ru(v);
  return f;
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

// per candidate: sum over sampled rows of ||cv - bf16(cv)||^2 / ||cv||^2
__global__ void scale_probe_kernel(const float* __restrict__ x, int64_t n, int d,
                                   const float* __restrict__ mu, int64_t stride,
                                   double* __restrict__ score) {
  const int lane = threadIdx.x & 31;
  const int64_t row = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * stride;
  const int cand = blockIdx.y;
  if (row >= n) return;
  double rr = 0.0, cc = 0.0;
  for (int c = lane; c < d; c += 32) {
    float sc, mc;
    scale_candidate(cand, mu[c], &sc, &mc);
    const float cv = __fmul_rn(sc, __fsub_rn(x[row * d + c], mc));
    const float bv = __bfloat162float(__float2bfloat16_rn(cv));
    rr += (double)(cv - bv) * (double)(cv - bv);
    cc += (double)cv * (double)cv;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    rr += __shfl_xor_sync(FULL, rr, o);
    cc += __shfl_xor_sync(FULL, cc, o);
  }
  if (lane == 0) atomicAdd(&score[cand], cc > 0.0 ? rr / cc : 0.0);
}

// replace mu by the chosen candidate's centre
__global__ void apply_centre_kernel(float* __restrict__ mu, int d, int cand) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d) return;
  float sc, mc;
  scale_candidate(cand, mu[c], &sc, &mc);
  mu[c] = mc;
}

// One warp per row: BF16 copy of scale*(x - mu) padded to dp, and the row's bound terms.
__global__ void convert_rows_kernel(const float* __restrict__ x, int64_t n, int d, int dp,
                                    const float* __restrict__ mu, float scale,
                                    __nv_bfloat16* __restrict__ xb, RowInfo* __restrict__ info,
                                    BaseMax* __restrict__ bmax) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= n) return;
  const float* xr = x + row * d;
  __nv_bfloat16* br = xb + row * dp;
  double s_b = 0.0, s_r = 0.0, s_c = 0.0;
  for (int c = lane; c < dp; c += 32) {
    float cv = 0.0f;
    if (c < d) cv = __fmul_rn(scale, __fsub_rn(xr[c], mu[c]));
    const __nv_bfloat16 b = __float2bfloat16_rn(cv);
    br[c] = b;
    const float bv = __bfloat162float(b);
    const float rv = cv - bv;  // exact: the rounding residual of a float fits in a float
    s_b += (double)bv * (double)bv;
    s_r += (double)rv * (double)rv;
    s_c += (double)cv * (double)cv;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s_b += __shfl_xor_sync(FULL, s_b, o);
    s_r += __shfl_xor_sync(FULL, s_r, o);
    s_c += __shfl_xor_sync(FULL, s_c, o);
  }
  if (lane == 0) {
    RowInfo ri;
    ri.nrm = __double2float_rn(s_b);
    ri.xn_up = round_up_f(sqrt(s_b) * (1.0 + 1e-12));
    // ||s(x-mu)_exact - x~|| <= ||cv - x~|| + 2u ||cv|| (1+u), cv = fl(s fl(x-mu))
    ri.r_up = round_up_f((sqrt(s_r) + 2.0 * 5.9604645e-08 * 1.0000002 * sqrt(s_c)) * (1.0 + 1e-9));
    ri.pad = 0.0f;
    info[row] = ri;
    if (bmax) {
      atomicMax(&bmax->xn_bits, __float_as_uint(ri.xn_up));
      atomicMax(&bmax->r_bits, __float_as_uint(ri.r_up));
    }
  }
}

// ---------------------------------------------------------------- main kernel

struct MainArgs {
  int64_t nq, n;
  int d, dp, nkb;
  int tiles;          // point tiles of BN
  int64_t work;       // qblocks * tiles
  int grid;           // CTAs
  int smax;           // partial-list slots per query
  int L;              // list length (k + margin), 32 or 64
  const RowInfo* qinfo;
  const RowInfo* binfo;
  uint64_t* partial;  // [nq][smax][L]
  int* err;
};

__device__ __forceinline__ int64_t chunk_begin(int c, int64_t work, int grid) {
  return (int64_t)((__int128)c * work / grid);
}

// the CTA whose work range contains item i
__device__ __forceinline__ int cta_of(int64_t i, int64_t work, int grid) {
  int c = (int)((__int128)i * grid / work);
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

template <int KW>
__global__ void __launch_bounds__(K2_THREADS, 1)
    k2_main(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
            MainArgs a) {
  constexpr int L = KW * 32;
  extern __shared__ __align__(1024) uint8_t k2_smem_raw[];
  // 1024-byte alignment for the swizzled stages
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(k2_smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* stage_base = smem;                                            // STAGES * 48 KB
  uint64_t* lists = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);  // [BM][L]
  uint64_t* staging = lists + BM * L;                                   // [STAGE_CAP][BM]
  uint64_t* bars = staging + STAGE_CAP * BM;                            // full[S], empty[S], tfull[2], tempty[2]
  uint64_t* full_bar = bars;
  uint64_t* empty_bar = bars + STAGES;
  uint64_t* tfull_bar = bars + 2 * STAGES;
  uint64_t* tempty_bar = bars + 2 * STAGES + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 4);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cta = blockIdx.x;
  const int64_t it0 = chunk_begin(cta, a.work, a.grid);
  const int64_t it1 = chunk_begin(cta + 1, a.work, a.grid);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      ptx::mbar_init(&full_bar[s], 1);
      ptx::mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(&tfull_bar[b], 1);
      ptx::mbar_init(&tempty_bar[b], NUM_EPI_WARPS * 32);
    }
    ptx::fence_mbar_init();
    ptx::prefetch_tensormap(&mapA);
    ptx::prefetch_tensormap(&mapB);
  }
  if (warp == 1) {
    ptx::tmem_alloc(tmem_slot, TMEM_COLS);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int64_t item = it0; item < it1 && ok; ++item) {
        const int qb = (int)(item / a.tiles);
        const int t = (int)(item % a.tiles);
        for (int kb = 0; kb < a.nkb; ++kb, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1;
          if (!ptx::mbar_wait(&empty_bar[s], ph ^ 1, a.err, ERR_TIMEOUT_PRODUCER)) {
            ok = false;
            break;
          }
          uint8_t* sa = stage_base + s * STAGE_BYTES;
          uint8_t* sb = sa + A_STAGE_BYTES;
          ptx::mbar_arrive_expect_tx(&full_bar[s], STAGE_BYTES);
          ptx::tma_load_2d(sa, &mapA, &full_bar[s], kb * BK, qb * BM);
          ptx::tma_load_2d(sb, &mapB, &full_bar[s], kb * BK, t * BN);
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = ptx::idesc_bf16_f32(BM, BN);
      uint32_t it = 0;
      int tcount = 0;
      bool ok = true;
      for (int64_t item = it0; item < it1 && ok; ++item, ++tcount) {
        const int buf = tcount & 1;
        const uint32_t tph = (tcount >> 1) & 1;
        if (!ptx::mbar_wait(&tempty_bar[buf], tph ^ 1, a.err, ERR_TIMEOUT_MMA)) break;
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
          const int rem = a.dp - kb * BK;  // valid (zero-padded) columns left
          const int ksteps = rem >= BK ? BK / 16 : (rem + 15) / 16;
          for (int kk = 0; kk < ksteps; ++kk) {
            const uint64_t ad = ptx::sw128_desc(sa + kk * 32);
            const uint64_t bd = ptx::sw128_desc(sb + kk * 32);
            ptx::mma_f16(dcol, ad, bd, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
          }
          ptx::mma_commit(&empty_bar[s]);  // frees the stage when these MMAs finish
        }
        if (ok) ptx::mma_commit(&tfull_bar[buf]);
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int ew = warp - 2;           // 0..3
    const int quad = warp & 3;         // TMEM lane quadrant this warp may access
    const int row = quad * 32 + lane;  // row of the 128-query tile
    uint64_t* my_list_base = lists;    // list of row r: lists[r * L + e]
    float thr = __int_as_float(0x7F800000);
    int cnt = 0;
    int tcount = 0;
    int cur_qb = -1;
    int seg_first_cta = 0;
    float qn = 0.0f;
    bool alive = true;
    (void)ew;

    // reset the 32 lists owned by this warp
    for (int r = 0; r < 32; ++r)
      for (int e = lane; e < L; e += 32) my_list_base[(quad * 32 + r) * L + e] = KEY_NONE;
    __syncwarp();

    auto flush = [&](int qb) {
      // write this warp's 32 lists into the partial buffer and reset them
      const int slot = cta - seg_first_cta;
      for (int r = 0; r < 32; ++r) {
        const int64_t gq = (int64_t)qb * BM + quad * 32 + r;
        uint64_t* lr = my_list_base + (quad * 32 + r) * L;
        for (int e = lane; e < L; e += 32) {
          if (gq < a.nq) a.partial[(gq * a.smax + slot) * L + e] = lr[e];
          lr[e] = KEY_NONE;
        }
      }
      __syncwarp();
      thr = __int_as_float(0x7F800000);
    };

    for (int64_t item = it0; item < it1; ++item, ++tcount) {
      const int qb = (int)(item / a.tiles);
      const int t = (int)(item % a.tiles);
      if (qb != cur_qb) {
        if (cur_qb >= 0) flush(cur_qb);
        cur_qb = qb;
        seg_first_cta = cta_of((int64_t)qb * a.tiles, a.work, a.grid);
        const int64_t gq = (int64_t)qb * BM + row;
        qn = gq < a.nq ? a.qinfo[gq].nrm : 0.0f;
      }
      const int buf = tcount & 1;
      const uint32_t tph = (tcount >> 1) & 1;
      if (alive && !ptx::mbar_wait(&tfull_bar[buf], tph, a.err, ERR_TIMEOUT_EPI)) alive = false;
      if (!alive) break;
      ptx::tc_fence_after();
      const int64_t col0 = (int64_t)t * BN;
      const uint32_t taddr = tmem_base + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * BN);
      for (int ch = 0; ch < BN / 16; ++ch) {
        uint32_t v[16];
        ptx::tmem_ld16(taddr + ch * 16, v);
        ptx::tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int64_t col = col0 + ch * 16 + j;
          if (col < a.n) {
            const float nb = __ldg(&a.binfo[col].nrm);
            const float est = __fmaf_rn(-2.0f, __uint_as_float(v[j]), __fadd_rn(qn, nb));
            if (est < thr) {
              staging[cnt * BM + row] = make_key(est, (uint32_t)col);
              ++cnt;
            }
          }
        }
        // fold staged candidates into the lists, one row at a time (warp-cooperative)
        unsigned pending = __ballot_sync(FULL, cnt > 0);
        while (pending) {
          const int r = __ffs(pending) - 1;
          pending &= pending - 1;
          const int rrow = quad * 32 + r;
          const int rc = __shfl_sync(FULL, cnt, r);
          uint64_t* lr = my_list_base + rrow * L;
          uint64_t Lr[KW];
#pragma unroll
          for (int s = 0; s < KW; ++s) Lr[s] = lr[s * 32 + lane];
          uint64_t tk = __shfl_sync(FULL, Lr[KW - 1], 31);
          for (int e = 0; e < rc; ++e) {
            const uint64_t c = staging[e * BM + rrow];
            if (c < tk) {
              wl_insert<KW>(Lr, c, lane);
              tk = __shfl_sync(FULL, Lr[KW - 1], 31);
            }
          }
#pragma unroll
          for (int s = 0; s < KW; ++s) lr[s * 32 + lane] = Lr[s];
          if (lane == r) {
            cnt = 0;
            thr = (tk == KEY_NONE) ? __int_as_float(0x7F800000) : key_dist(tk);
          }
        }
        __syncwarp();
      }
      ptx::tc_fence_before();
      ptx::mbar_arrive(&tempty_bar[buf]);
    }
    if (alive && cur_qb >= 0) flush(cur_qb);
  }

  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem_base, TMEM_COLS);
  }
}

// ---------------------------------------------------------------- merge

// L smallest keys over the CTA segments of each query (warp per query).
template <int KW>
__global__ void k2_merge(const uint64_t* __restrict__ partial, int64_t nq, int smax, int tiles,
                         int64_t work, int grid, uint64_t* __restrict__ out) {
  constexpr int L = KW * 32;
  const int lane = threadIdx.x & 31;
  const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (q >= nq) return;
  const int64_t qb = q / BM;
  const int c0 = cta_of(qb * tiles, work, grid);
  const int c1 = cta_of(qb * tiles + tiles - 1, work, grid);
  const int nseg = c1 - c0 + 1;
  uint64_t Lr[KW];
#pragma unroll
  for (int s = 0; s < KW; ++s) Lr[s] = partial[(q * smax + 0) * L + s * 32 + lane];
  for (int g = 1; g < nseg; ++g) {
    const uint64_t* src = partial + (q * smax + g) * L;
    uint64_t tk = __shfl_sync(FULL, Lr[KW - 1], 31);
    for (int e = 0; e < L; ++e) {
      const uint64_t c = src[e];  // sorted: stop at the first that cannot enter
      if (!(c < tk)) break;
      wl_insert<KW>(Lr, c, lane);
      tk = __shfl_sync(FULL, Lr[KW - 1], 31);
    }
  }
#pragma unroll
  for (int s = 0; s < KW; ++s) out[q * L + s * 32 + lane] = Lr[s];
}

// ---------------------------------------------------------------- certify + rerank

struct RerankArgs {
  const float* base;
  const float* qs;
  int64_t nq, n;
  int d, L, kreq, metric;
  float scale;  // the est values are in units of scale^2 * distance
  const RowInfo* qinfo;
  const BaseMax* bmax;
  const uint64_t* lists;  // [nq][L] sorted by est
  uint64_t* cand;         // [nq][L] sorted (fp32 distance, id)
  int* cand_count;        // [nq]
  float* floor_val;       // [nq] lower bound of FP32 distances of non-candidates
  int* fb_rows;           // rows that need the FP32 scan
  int* fb_count;
  unsigned long long* cand_total;
};

__device__ __forceinline__ float fp32_dist_row(const float* __restrict__ x,
                                               const float* __restrict__ y, int d, int metric) {
  float s = 0.0f;
  for (int c = 0; c < d; ++c) {
    const float t = __fsub_rn(x[c], y[c]);
    s = __fmaf_rn(t, t, s);
  }
  return metric == MANN_METRIC_EUCLIDEAN ? __fsqrt_rn(s) : s;
}

__global__ void k2_rerank(RerankArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (q >= a.nq) return;
  const uint64_t* lst = a.lists + q * a.L;
  const uint64_t ek_key = lst[a.kreq - 1];
  const uint64_t last_key = lst[a.L - 1];
  // threshold (identical on every lane)
  const RowInfo qi = a.qinfo[q];
  const double bxn = (double)__uint_as_float(a.bmax->xn_bits);
  const double br = (double)__uint_as_float(a.bmax->r_bits);
  const double u = 5.9604644775390625e-08;
  // one FP32 rounding (or truncation) per 16-term MMA step, x2 margin
  const double gam = (double)((a.d + 15) / 16 + 2) * 2.384185791015625e-07;
  const double c1 = 4.0 * u + 2.0 * gam;
  const double A = ((double)qi.xn_up + bxn) * ((double)qi.xn_up + bxn);
  const double Rs = (double)qi.r_up + br;
  const double ek = ek_key == KEY_NONE ? 0.0 : fmax((double)key_dist(ek_key), 0.0);
  const double sU = sqrt(ek + c1 * A) + Rs;
  const double U = sU * sU;
  const double slack = 3.0 * (double)(a.d + 2) * u * U + 1e-6 * U + 1e-30;
  const double T = ((sU + Rs) * (sU + Rs) + c1 * A + slack) * (1.0 + 1e-9);
  // lower bound on the exact distance of any point outside the list's est <= T set
  const double e_floor = fmax(T - c1 * A, 0.0);
  const double s_floor = fmax(sqrt(e_floor) - Rs, 0.0);
  double d_floor = s_floor * s_floor * (1.0 - 3.0 * (double)(a.d + 2) * u) / ((double)a.scale * a.scale);
  const bool all_in = (last_key == KEY_NONE);  // the list holds every point
  const bool certified = all_in || (double)key_dist(last_key) > T;
  if (!certified) {
    if (lane == 0) {
      const int slot = atomicAdd(a.fb_count, 1);
      a.fb_rows[slot] = (int)q;
      a.cand_count[q] = -1;
    }
    return;
  }
  if (all_in) d_floor = 3.0e38;
  const float* qrow = a.qs + q * a.d;
  // candidates: entries with est <= T (the list is sorted by est)
  uint64_t key[2] = {KEY_NONE, KEY_NONE};
  int ncand = 0;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int e = s * 32 + lane;
    if (e < a.L) {
      const uint64_t k = lst[e];
      if (k != KEY_NONE && (double)key_dist(k) <= T) {
        const int id = key_id(k);
        const float dist = fp32_dist_row(qrow, a.base + (int64_t)id * a.d, a.d, a.metric);
        key[s] = make_key(dist, (uint32_t)id);
      }
    }
  }
  ncand = __popc(__ballot_sync(FULL, key[0] != KEY_NONE)) + __popc(__ballot_sync(FULL, key[1] != KEY_NONE));
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
    float fl = (float)d_floor;
    if (a.metric == MANN_METRIC_EUCLIDEAN) fl = (float)sqrt(fmax(d_floor, 0.0)) * (1.0f - 1e-6f);
    a.floor_val[q] = fl;
    atomicAdd(a.cand_total, (unsigned long long)ncand);
  }
}

// rows re-run by the FP32 scan: copy their sorted keys into the candidate table
__global__ void k2_scatter_fallback(const uint64_t* __restrict__ keys, const int* __restrict__ rows,
                                    const int* __restrict__ count, int kk, int L,
                                    uint64_t* __restrict__ cand, int* __restrict__ cand_count,
                                    float* __restrict__ floor_val) {
  const int i = blockIdx.x;
  if (i >= *count) return;
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

// One warp per query.  cand[q][0..count) sorted by (fp32, id).  Writes the
// first kreq keys to keys_out, ordering near-tie clusters by FP64 when asked.
__global__ void resolve_kernel(const float* __restrict__ base, const float* __restrict__ qs,
                               int d, int metric, int64_t nq, int L, int kreq, int fp64,
                               const uint64_t* __restrict__ cand, const int* __restrict__ cand_count,
                               const float* __restrict__ floor_val, uint64_t* __restrict__ keys_out,
                               unsigned long long* __restrict__ n_fp64_rows,
                               unsigned long long* __restrict__ n_unresolved) {
  __shared__ uint64_t s_key[4][256];
  __shared__ double s_val[4][256];
  __shared__ int s_cl[4][256];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t q = (int64_t)blockIdx.x * 4 + w;
  if (q >= nq) return;
  const uint64_t* cq = cand + q * L;
  const int c = min(cand_count[q], L);
  uint64_t* out = keys_out + q * kreq;
  if (!fp64 || c <= 1) {
    for (int e = lane; e < kreq; e += 32) out[e] = e < c ? cq[e] : KEY_NONE;
    return;
  }
  const int cm = min(c, 256);
  for (int e = lane; e < cm; e += 32) s_key[w][e] = cq[e];
  __syncwarp();
  const double eps = (double)(d + 2) * 5.9604644775390625e-08 * 1.01 + 1.2e-7;
  if (lane == 0) {
    // clusters of adjacent positions whose FP32 distances are within the rounding bound
    int start = 0;
    s_cl[w][0] = 0;
    for (int p = 1; p < cm; ++p) {
      const double a = (double)key_dist(s_key[w][p - 1]);
      const double b = (double)key_dist(s_key[w][p]);
      // FP32 cosine distances carry an absolute error of order (d+4)u
      const bool link = metric == MANN_METRIC_COSINE ? (b - a) <= 2.0 * eps + 4.8e-7
                                                     : (b - a) <= eps * (fabs(a) + fabs(b));
      if (!link) start = p;
      s_cl[w][p] = start;
    }
  }
  __syncwarp();
  // the cluster holding position kreq-1 must end inside the candidate list
  int end = kreq - 1;
  if (end >= cm) end = cm - 1;
  while (end + 1 < cm && s_cl[w][end + 1] == s_cl[w][kreq - 1 < cm ? kreq - 1 : cm - 1]) ++end;
  bool resolvable = true;
  if (end == cm - 1) {
    const double lastv = (double)key_dist(s_key[w][cm - 1]);
    const double fl = (double)floor_val[q];
    const bool clear = metric == MANN_METRIC_COSINE ? lastv + 2.0 * eps + 4.8e-7 < fl
                                                    : lastv * (1.0 + eps) < fl * (1.0 - eps);
    resolvable = clear || fl >= 3.0e38;
  }
  bool any_tie = false;
  for (int p = 1; p <= end; ++p)
    if (s_cl[w][p] != p) { any_tie = true; break; }
  if (!resolvable) {
    if (lane == 0) atomicAdd(n_unresolved, 1ull);
  } else if (any_tie) {
    const float* qrow = qs + q * d;
    for (int p = lane; p <= end; p += 32) {
      const bool member = (s_cl[w][p] != p) || (p + 1 <= end && s_cl[w][p + 1] == p);
      s_val[w][p] = member ? fp64_dist_row(qrow, base + (int64_t)key_id(s_key[w][p]) * d, d, metric) : 0.0;
    }
    __syncwarp();
    if (lane == 0) {
      atomicAdd(n_fp64_rows, 1ull);
      // insertion sort inside each cluster by (fp64 distance, id)
      int p = 0;
      while (p <= end) {
        int e = p;
        while (e + 1 <= end && s_cl[w][e + 1] == p) ++e;
        for (int i = p + 1; i <= e; ++i) {
          const uint64_t kk = s_key[w][i];
          const double vv = s_val[w][i];
          int j = i - 1;
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
  }
  __syncwarp();
  for (int e = lane; e < kreq; e += 32) out[e] = e < cm ? s_key[w][e] : KEY_NONE;
}

}  // namespace

mann_status launch_resolve(const float* base, const float* qs, int d, int metric, int64_t nq, int L,
                           int kreq, int fp64, const uint64_t* cand, const int* cand_count,
                           const float* floor_val, uint64_t* keys_out, unsigned long long* counters,
                           cudaStream_t s) {
  if (nq <= 0) return MANN_OK;
  resolve_kernel<<<(unsigned)ceil_div(nq, 4), 128, 0, s>>>(base, qs, d, metric, nq, L, kreq, fp64,
                                                            cand, cand_count, floor_val, keys_out,
                                                            counters, counters + 1);
  MANN_CHECK_LAUNCH();
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

mann_status fp32_then_resolve(Context* ctx, cudaStream_t s, const float* base, const float* qs,
                              int64_t n, int64_t nq, int d, int metric, int kk, int kreq,
                              const uint64_t* fkeys, uint64_t** out_keys, mann_knn_report* rep) {
  (void)n;
  int* cand_count = nullptr;
  float* floor_val = nullptr;
  unsigned long long* counters = nullptr;
  uint64_t* keys = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_MISC0, (size_t)nq, &cand_count));
  MANN_TRY(ctx->scratch_t(SLOT_MISC1, (size_t)nq, &floor_val));
  MANN_TRY(ctx->scratch_t(SLOT_COUNTERS, 64, &counters));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_KEYS_BF16, (size_t)nq * kreq, &keys));
  MANN_CUDA_TRY(cudaMemsetAsync(counters, 0, 64 * sizeof(unsigned long long), s));
  fp32_lists_to_cand_kernel<<<(unsigned)ceil_div(nq, 128), 128, 0, s>>>(fkeys, nq, kk, cand_count,
                                                                       floor_val);
  MANN_CHECK_LAUNCH();
  MANN_TRY(launch_resolve(base, qs, d, metric, nq, kk, kreq, 1, fkeys, cand_count, floor_val, keys,
                          counters + 4, s));
  if (rep) {
    unsigned long long h[2] = {0, 0};
    MANN_CUDA_TRY(cudaMemcpyAsync(h, counters + 4, sizeof(h), cudaMemcpyDeviceToHost, s));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));
    rep->rows_fp64_ties = (int64_t)h[0];
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

mann_status make_map(CUtensorMap* m, const void* ptr, int64_t rows, int dp, int box_rows) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return fail(MANN_ECUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[2] = {(cuuint64_t)dp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)dp * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box,
                   es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(MANN_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return MANN_OK;
}

size_t main_smem_bytes(int L) {
  return 1024 /* alignment */ + (size_t)STAGES * STAGE_BYTES + (size_t)BM * L * 8 +
         (size_t)STAGE_CAP * BM * 8 + (2 * STAGES + 4) * 8 + 16;
}

int64_t h_chunk(int c, int64_t work, int grid) { return (int64_t)((__int128)c * work / grid); }
int h_cta_of(int64_t i, int64_t work, int grid) {
  int c = (int)((__int128)i * grid / work);
  while (c + 1 < grid && h_chunk(c + 1, work, grid) <= i) ++c;
  while (c > 0 && h_chunk(c, work, grid) > i) --c;
  return c;
}

}  // namespace

// Prepared BF16 operand of one matrix (points or queries).
struct Bf16Operand {
  __nv_bfloat16* xb = nullptr;
  RowInfo* info = nullptr;
};

mann_status knn_bf16_keys(Context* ctx, cudaStream_t s, const float* base, int64_t n,
                          const float* qs, int64_t nq, int d, int metric, int kreq, int margin,
                          bool fp64, uint64_t** out_keys, mann_knn_report* rep) {
  if (metric == MANN_METRIC_COSINE) return fail(MANN_EINVAL_ARG, "BF16 form: L2 metrics only");
  if (nq <= 0) return MANN_OK;
  const int L = (kreq + std::max(margin, 0) <= 32 && margin > 0) ? 32 : 64;
  if (kreq > L) return fail(MANN_EINVAL_ARG, "BF16 form supports k <= 64");
  const int dp = (d + 7) & ~7;
  const bool self = (qs == base);

  // ---- prep
  const int chunks = (int)std::min<int64_t>(256, std::max<int64_t>(1, n / 512));
  const int64_t rows_per = ceil_div(n, chunks);
  double* cpart = nullptr;
  float* mu = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_CENTRE, (size_t)chunks * d + (size_t)d + 8, &cpart));
  MANN_TRY(ctx->scratch_t(SLOT_MISC3, (size_t)d + 64, &mu));
  BaseMax* bmax = reinterpret_cast<BaseMax*>(mu + ((d + 31) & ~31));
  dim3 cg((unsigned)ceil_div(d, 128), (unsigned)chunks);
  centre_partial_kernel<<<cg, 128, 0, s>>>(base, n, d, rows_per, cpart);
  MANN_CHECK_LAUNCH();
  centre_final_kernel<<<(unsigned)ceil_div(d, 128), 128, 0, s>>>(cpart, chunks, d, n, mu);
  MANN_CHECK_LAUNCH();
  // pick the centre / scale with the smallest BF16 residual on a row sample
  double* score = cpart;  // reuse: the partial sums are consumed
  MANN_CUDA_TRY(cudaMemsetAsync(score, 0, NUM_SCALES * sizeof(double), s));
  const int64_t sample_rows = std::min<int64_t>(n, 2048);
  const int64_t stride = std::max<int64_t>(1, n / sample_rows);
  dim3 pg((unsigned)ceil_div(ceil_div(n, stride), 8), NUM_SCALES);
  scale_probe_kernel<<<pg, 256, 0, s>>>(base, n, d, mu, stride, score);
  MANN_CHECK_LAUNCH();
  double h_score[NUM_SCALES];
  MANN_CUDA_TRY(cudaMemcpyAsync(h_score, score, sizeof(h_score), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  int best = 0;
  for (int i = 1; i < NUM_SCALES; ++i)
    if (h_score[i] < 0.25 * h_score[best]) best = i;  // move off the plain mean only for a clear win
  const float scale = best == 1 ? 255.0f : 1.0f;
  if (best != 0) {
    apply_centre_kernel<<<(unsigned)ceil_div(d, 128), 128, 0, s>>>(mu, d, best);
    MANN_CHECK_LAUNCH();
  }
  MANN_CUDA_TRY(cudaMemsetAsync(bmax, 0, sizeof(BaseMax), s));
  Bf16Operand B, Q;
  MANN_TRY(ctx->scratch_t(SLOT_BF16_B, (size_t)n * dp, &B.xb));
  MANN_TRY(ctx->scratch_t(SLOT_ROWINFO_B, (size_t)n, &B.info));
  convert_rows_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(base, n, d, dp, mu, scale, B.xb, B.info, bmax);
  MANN_CHECK_LAUNCH();
  if (self) {
    Q = B;
  } else {
    MANN_TRY(ctx->scratch_t(SLOT_BF16_Q, (size_t)nq * dp, &Q.xb));
    MANN_TRY(ctx->scratch_t(SLOT_ROWINFO_Q, (size_t)nq, &Q.info));
    convert_rows_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(qs, nq, d, dp, mu, scale, Q.xb, Q.info, nullptr);
    MANN_CHECK_LAUNCH();
  }

  // ---- main
  CUtensorMap mapA, mapB;
  MANN_TRY(make_map(&mapA, Q.xb, nq, dp, BM));
  MANN_TRY(make_map(&mapB, B.xb, n, dp, BN));
  const int64_t qblocks = ceil_div(nq, BM);
  const int tiles = (int)ceil_div(n, BN);
  const int64_t work = qblocks * tiles;
  const int grid = (int)std::min<int64_t>(ctx->num_sms, work);
  int smax = 1;
  for (int64_t qb = 0; qb < qblocks; ++qb) {
    const int c0 = h_cta_of(qb * tiles, work, grid);
    const int c1 = h_cta_of(qb * tiles + tiles - 1, work, grid);
    smax = std::max(smax, c1 - c0 + 1);
  }
  uint64_t* partial = nullptr;
  int* err = nullptr;
  unsigned long long* counters = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_PARTIAL, (size_t)nq * smax * L, &partial));
  MANN_TRY(ctx->scratch_t(SLOT_COUNTERS, 64, &counters));
  err = reinterpret_cast<int*>(counters + 8);
  int* fb_count = err + 1;
  MANN_CUDA_TRY(cudaMemsetAsync(counters, 0, 64 * sizeof(unsigned long long), s));
  MainArgs ma;
  ma.nq = nq;
  ma.n = n;
  ma.d = d;
  ma.dp = dp;
  ma.nkb = (int)ceil_div(dp, BK);
  ma.tiles = tiles;
  ma.work = work;
  ma.grid = grid;
  ma.smax = smax;
  ma.L = L;
  ma.qinfo = Q.info;
  ma.binfo = B.info;
  ma.partial = partial;
  ma.err = err;
  const size_t smem = main_smem_bytes(L);
  if (smem > ctx->smem_optin) return fail(MANN_ECUDA, "shared memory budget exceeded");
  if (L == 32) {
    MANN_CUDA_TRY(cudaFuncSetAttribute(k2_main<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ctx->time_begin(s);
    k2_main<1><<<grid, K2_THREADS, smem, s>>>(mapA, mapB, ma);
  } else {
    MANN_CUDA_TRY(cudaFuncSetAttribute(k2_main<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ctx->time_begin(s);
    k2_main<2><<<grid, K2_THREADS, smem, s>>>(mapA, mapB, ma);
  }
  ctx->time_end(s);
  MANN_CHECK_LAUNCH();
  uint64_t* lists = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_KEYS, (size_t)nq * L, &lists));
  if (L == 32)
    k2_merge<1><<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(partial, nq, smax, tiles, work, grid, lists);
  else
    k2_merge<2><<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(partial, nq, smax, tiles, work, grid, lists);
  MANN_CHECK_LAUNCH();

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
  ra.qinfo = Q.info;
  ra.bmax = bmax;
  ra.lists = lists;
  ra.cand = cand;
  ra.cand_count = cand_count;
  ra.floor_val = floor_val;
  ra.fb_rows = fb_rows;
  ra.fb_count = fb_count;
  ra.cand_total = counters + 2;
  k2_rerank<<<(unsigned)ceil_div(nq, 4), 128, 0, s>>>(ra);
  MANN_CHECK_LAUNCH();

  // ---- exact FP32 scan of uncertified rows (count known only on the device:
  // read it back; the common case is zero rows)
  int h_fb = 0, h_err = 0;
  MANN_CUDA_TRY(cudaMemcpyAsync(&h_fb, fb_count, sizeof(int), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  if (h_err != 0)
    return fail(MANN_ETIMEOUT, "tensor-core kernel: a bounded wait ran out (role " + std::to_string(h_err) + ")");
  if (h_fb > 0) {
    const int kk = (int)std::min<int64_t>(std::min<int64_t>(n, KMAX_FUSED), std::min(L, kreq + 32));
    uint64_t* fkeys = nullptr;
    const float* no_norm = nullptr;
    MANN_TRY(knn_fp32_keys(ctx, s, base, n, qs, h_fb, d, metric, kk, fb_rows, no_norm, no_norm,
                           &fkeys, SLOT_FALLBACK_KEYS, SLOT_MISC2));
    k2_scatter_fallback<<<h_fb, 64, 0, s>>>(fkeys, fb_rows, fb_count, kk, L, cand, cand_count, floor_val);
    MANN_CHECK_LAUNCH();
  }

  // ---- resolve + truncate
  uint64_t* keys = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_OUT_KEYS_BF16, (size_t)nq * kreq, &keys));
  MANN_TRY(launch_resolve(base, qs, d, metric, nq, L, kreq, fp64 ? 1 : 0, cand, cand_count, floor_val,
                          keys, counters + 4, s));
  if (rep) {
    unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
    MANN_CUDA_TRY(cudaMemcpyAsync(h, counters, sizeof(h), cudaMemcpyDeviceToHost, s));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));
    rep->rows_fallback = h_fb;
    rep->candidates = (int64_t)h[2];
    rep->rows_fp64_ties = (int64_t)h[4];
    rep->precision_used = MANN_PREC_BF16;
    rep->margin_used = L - kreq;
  }
  *out_keys = keys;
  return MANN_OK;
}

}  // namespace mann
