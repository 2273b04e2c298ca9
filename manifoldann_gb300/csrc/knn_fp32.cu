// knn_fp32.cu -- exact FP32 kNN with fused per-row top-k (the plain form).
//
// Replaces the per-query scan of src/indices/bruteforce.jl:59-65 (one
// Distances.jl evaluation per point, then partialsortperm) and the batch loop
// of src/ann_index.jl:91-98.  One CTA owns BQ queries and a contiguous split
// of the points; it walks the split in tiles of 128 points, computes the
// BQ x 128 distance tile in registers (difference form, one fused
// multiply-add per dimension in order 0..d-1 -- bit-identical to the oracle's
// sequential sum), stages it in shared memory and folds it into per-row
// sorted top-k lists that live in the registers of the warp owning the row.
// Splits are merged by a second kernel.  Order: (distance, id) as
// partialsortperm (bruteforce.jl:65).
#include <algorithm>

#include "kernels.cuh"
#include "f32x2.cuh"
#include "warp_list.cuh"

namespace mann {

namespace {

constexpr int K1_THREADS = 256;
constexpr int K1_BN = 128;  // points per tile
constexpr int K1_DK = 16;   // dimensions per shared-memory stage
constexpr unsigned FULL = 0xFFFFFFFFu;
using wl::list_get;
using wl::list_insert;

// Squared row norms as the FP32 form's sequential sum (dimension order, one
// fmaf per term).  One warp per 32 rows: 32 x 32 tiles come in through
// shared memory with coalesced loads (a row's 32 columns per load
// instruction), then lane l adds row l's squares in order; the next tile's
// loads are issued before the current tile's sums.
__global__ void __launch_bounds__(256) row_sqnorm_kernel(const float* __restrict__ x, int64_t n, int d,
                                                         float* __restrict__ out) {
  __shared__ float tile[8][32][33];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t r0 = ((int64_t)blockIdx.x * 8 + w) * 32;
  if (r0 >= n) return;
  const int nr = (int)min((int64_t)32, n - r0);
  float nxt[32];
  auto fetch = [&](int c0) {
#pragma unroll
    for (int i = 0; i < 32; ++i)
      nxt[i] = (i < nr && c0 + lane < d) ? __ldg(&x[(r0 + i) * d + c0 + lane]) : 0.0f;
  };
  fetch(0);
  float s = 0.0f;
  for (int c0 = 0; c0 < d; c0 += 32) {
    const int cw = min(32, d - c0);
#pragma unroll
    for (int i = 0; i < 32; ++i) tile[w][i][lane] = nxt[i];
    __syncwarp();
    if (c0 + 32 < d) fetch(c0 + 32);
    if (lane < nr)
      for (int c = 0; c < cw; ++c) s = __fmaf_rn(tile[w][lane][c], tile[w][lane][c], s);
    __syncwarp();
  }
  if (lane < nr) out[r0 + lane] = s;
}

// Thread-tile row/column maps.  TQ rows per thread: 8 -> {ty*4+i, 64+ty*4+i},
// 4 -> ty*4+i, 2 -> ty*2+i.  Eight columns per thread: {tx*4+j, 64+tx*4+j}.
template <int TQ>
__device__ __forceinline__ int tile_row(int ty, int i) {
  if constexpr (TQ == 8) return (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
  else if constexpr (TQ == 4) return ty * 4 + i;
  else return ty * 2 + i;
}
__device__ __forceinline__ int tile_col(int tx, int j) {
  return (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
}

template <int TQ>
__device__ __forceinline__ void load_q_frag(const float* p, int ty, float (&v)[TQ]) {
  if constexpr (TQ == 8) {
    float4 a = *reinterpret_cast<const float4*>(p + ty * 4);
    float4 b = *reinterpret_cast<const float4*>(p + 64 + ty * 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  } else if constexpr (TQ == 4) {
    float4 a = *reinterpret_cast<const float4*>(p + ty * 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  } else {
    float2 a = *reinterpret_cast<const float2*>(p + ty * 2);
    v[0] = a.x; v[1] = a.y;
  }
}

__device__ __forceinline__ void load_b_frag(const float* p, int tx, float (&v)[8]) {
  float4 a = *reinterpret_cast<const float4*>(p + tx * 4);
  float4 b = *reinterpret_cast<const float4*>(p + 64 + tx * 4);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

// Stage loader: rows [r0, r0+R) x dims [c0, c0+16) of a row-major [*][d]
// matrix into registers (VEC: float4 per thread-slot, else scalars).
template <int R, bool VEC>
struct StageLoader {
  static constexpr int NV = VEC ? (R * 4 + K1_THREADS - 1) / K1_THREADS
                                : (R * 16 + K1_THREADS - 1) / K1_THREADS;
  float4 v4[VEC ? NV : 1];
  float v1[VEC ? 1 : NV];

  __device__ __forceinline__ void load(const float* __restrict__ src, const int32_t* rows,
                                       int64_t r0, int64_t rend, int d, int c0, int tid) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if constexpr (VEC) {
        const int e = tid + i * K1_THREADS;
        float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
        if (e < R * 4) {
          const int r = e >> 2, c = c0 + (e & 3) * 4;
          const int64_t gr = r0 + r;
          if (gr < rend && c < d) {
            const int64_t row = rows ? (int64_t)rows[gr] : gr;
            val = __ldg(reinterpret_cast<const float4*>(src + row * (int64_t)d + c));
          }
        }
        v4[i] = val;
      } else {
        const int e = tid + i * K1_THREADS;
        float val = 0.f;
        if (e < R * 16) {
          const int r = e >> 4, c = c0 + (e & 15);
          const int64_t gr = r0 + r;
          if (gr < rend && c < d) {
            const int64_t row = rows ? (int64_t)rows[gr] : gr;
            val = __ldg(src + row * (int64_t)d + c);
          }
        }
        v1[i] = val;
      }
    }
  }

  // transpose into dst[dim][row] (row stride `str`)
  __device__ __forceinline__ void store(float* dst, int str, int tid) const {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if constexpr (VEC) {
        const int e = tid + i * K1_THREADS;
        if (e < R * 4) {
          const int r = e >> 2, c = (e & 3) * 4;
          dst[(c + 0) * str + r] = v4[i].x;
          dst[(c + 1) * str + r] = v4[i].y;
          dst[(c + 2) * str + r] = v4[i].z;
          dst[(c + 3) * str + r] = v4[i].w;
        }
      } else {
        const int e = tid + i * K1_THREADS;
        if (e < R * 16) dst[(e & 15) * str + (e >> 4)] = v1[i];
      }
    }
  }
};

// One CTA's work: queries [q0, min(q0 + BQ, nq)) against points [nb0, nb1);
// the sorted list of query row gq goes to dst + gq * dst_stride.
template <int METRIC, int BQ, int KW, bool VEC>
__device__ __forceinline__ void k1_body(const float* __restrict__ base, int64_t nb0, int64_t nb1,
                                        const float* __restrict__ qs, const int32_t* __restrict__ qrows,
                                        int64_t q0, int64_t nq, int d, const float* __restrict__ qnorm,
                                        const float* __restrict__ bnorm, int k, uint64_t* __restrict__ dst0,
                                        int64_t dst_stride, float* smem) {
  constexpr int TQ = BQ / 16;
  constexpr int TN = 8;
  constexpr int RPW = BQ / 8;
  constexpr int QSTR = BQ + 4;
  constexpr int BSTR = K1_BN + 4;
  float* Qs = smem;                   // [2][DK][QSTR]
  float* Bs = Qs + 2 * K1_DK * QSTR;  // [2][DK][BSTR]
  float* Dt = Bs + 2 * K1_DK * BSTR;  // [BQ][BSTR]

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ty = tid >> 4, tx = tid & 15;
  const int nchunks = (d + K1_DK - 1) / K1_DK;

  uint64_t L[RPW][KW];
#pragma unroll
  for (int r = 0; r < RPW; ++r)
#pragma unroll
    for (int s = 0; s < KW; ++s) L[r][s] = KEY_NONE;

  StageLoader<BQ, VEC> qload;
  StageLoader<K1_BN, VEC> bload;

  for (int64_t t0 = nb0; t0 < nb1; t0 += K1_BN) {
    const int64_t tend = min(nb1, t0 + K1_BN);
    // accumulators of columns 2j, 2j+1 packed in one f32x2 pair
    uint64_t acc2[TQ][TN / 2];
#pragma unroll
    for (int i = 0; i < TQ; ++i)
#pragma unroll
      for (int j = 0; j < TN / 2; ++j) acc2[i][j] = 0ull;

    qload.load(qs, qrows, q0, nq, d, 0, tid);
    bload.load(base, nullptr, t0, tend, d, 0, tid);
    qload.store(Qs, QSTR, tid);
    bload.store(Bs, BSTR, tid);
    __syncthreads();

    for (int c = 0; c < nchunks; ++c) {
      const int buf = c & 1;
      const bool more = (c + 1) < nchunks;
      if (more) {
        qload.load(qs, qrows, q0, nq, d, (c + 1) * K1_DK, tid);
        bload.load(base, nullptr, t0, tend, d, (c + 1) * K1_DK, tid);
      }
      const float* qsb = Qs + buf * K1_DK * QSTR;
      const float* bsb = Bs + buf * K1_DK * BSTR;
#pragma unroll
      for (int kk = 0; kk < K1_DK; ++kk) {
        float qv[TQ], bv[TN];
        load_q_frag<TQ>(qsb + kk * QSTR, ty, qv);
        load_b_frag(bsb + kk * BSTR, tx, bv);
        uint64_t b2[TN / 2];
#pragma unroll
        for (int j = 0; j < TN / 2; ++j) b2[j] = f2::pack(bv[2 * j], bv[2 * j + 1]);
#pragma unroll
        for (int i = 0; i < TQ; ++i) {
          const uint64_t q2 = f2::pack(qv[i], qv[i]);
#pragma unroll
          for (int j = 0; j < TN / 2; ++j) {
            if constexpr (METRIC == MANN_METRIC_COSINE) {
              acc2[i][j] = f2::fma(q2, b2[j], acc2[i][j]);
            } else {
              const uint64_t t = f2::sub(q2, b2[j]);
              acc2[i][j] = f2::fma(t, t, acc2[i][j]);
            }
          }
        }
      }
      if (more) {
        qload.store(Qs + (buf ^ 1) * K1_DK * QSTR, QSTR, tid);
        bload.store(Bs + (buf ^ 1) * K1_DK * BSTR, BSTR, tid);
      }
      __syncthreads();
    }

    float acc[TQ][TN];
#pragma unroll
    for (int i = 0; i < TQ; ++i)
#pragma unroll
      for (int j = 0; j < TN / 2; ++j) f2::unpack(acc2[i][j], acc[i][2 * j], acc[i][2 * j + 1]);
    // finish the metric and stage the tile
#pragma unroll
    for (int i = 0; i < TQ; ++i) {
      const int r = tile_row<TQ>(ty, i);
      float qn = 0.f;
      if constexpr (METRIC == MANN_METRIC_COSINE) {
        const int64_t gq = q0 + r;
        qn = (gq < nq) ? qnorm[qrows ? qrows[gq] : gq] : 1.0f;
      }
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        float v = acc[i][j];
        if constexpr (METRIC == MANN_METRIC_EUCLIDEAN) {
          v = __fsqrt_rn(v);
        } else if constexpr (METRIC == MANN_METRIC_COSINE) {
          const int64_t gb = t0 + tile_col(tx, j);
          const float bn = (gb < tend) ? bnorm[gb] : 1.0f;
          const float den = __fmul_rn(__fsqrt_rn(qn), __fsqrt_rn(bn));
          v = __fsub_rn(1.0f, __fdiv_rn(v, den));
          if (v < 0.0f) v = 0.0f;
        }
        acc[i][j] = v;
      }
      float* drow = Dt + r * BSTR;
      *reinterpret_cast<float4*>(drow + tx * 4) =
          make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
      *reinterpret_cast<float4*>(drow + 64 + tx * 4) =
          make_float4(acc[i][4], acc[i][5], acc[i][6], acc[i][7]);
    }
    __syncthreads();

    // fold the tile into the per-row lists (warp `warp` owns RPW rows)
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const int row = warp * RPW + r;
      const float* drow = Dt + row * BSTR;
      uint64_t thr = list_get<KW>(L[r], k - 1);
      // keys are built only for distances at or below the threshold's (the
      // exact key order decides); a list that is not full, or whose threshold
      // is NaN, takes every key through the exact comparison
      const float thr_f = thr == KEY_NONE ? 0.0f : key_dist(thr);
      const bool exact = thr == KEY_NONE || !(thr_f == thr_f);
      uint64_t key[4];
      unsigned pend = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int col = lane + 32 * j;
        const int64_t gid = t0 + col;
        const float dv = drow[col];
        key[j] = KEY_NONE;
        if (gid < tend && (exact || dv <= thr_f)) {
          key[j] = make_key(dv, (uint32_t)gid);
          if (key[j] < thr) pend |= 1u << j;
        }
      }
      for (;;) {
        const unsigned any = __ballot_sync(FULL, pend != 0);
        if (!any) break;
        const int src = __ffs(any) - 1;
        uint64_t mine = KEY_NONE;
        if (pend) {
          const int j = __ffs(pend) - 1;
          mine = (j == 0) ? key[0] : (j == 1) ? key[1] : (j == 2) ? key[2] : key[3];
        }
        const uint64_t cnd = __shfl_sync(FULL, mine, src);
        if (lane == src) pend &= pend - 1;
        if (cnd < thr) {
          list_insert<KW>(L[r], cnd, lane);
          thr = list_get<KW>(L[r], k - 1);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (!(key[j] < thr)) pend &= ~(1u << j);
      }
    }
    __syncthreads();
  }

  // write this split's lists
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
    const int64_t gq = q0 + warp * RPW + r;
    if (gq >= nq) continue;
    uint64_t* dst = dst0 + gq * dst_stride;
#pragma unroll
    for (int s = 0; s < KW; ++s) {
      const int e = s * 32 + lane;
      if (e < k) dst[e] = L[r][s];
    }
  }
}

template <int METRIC, int BQ, int KW, bool VEC>
__global__ void __launch_bounds__(K1_THREADS, 1)
    k1_tile_topk(const float* __restrict__ base, int64_t n, const float* __restrict__ qs,
                 const int32_t* __restrict__ qrows, int64_t nq, int d,
                 const float* __restrict__ qnorm, const float* __restrict__ bnorm, int k,
                 int64_t split_len, int nsplit, uint64_t* __restrict__ partial) {
  extern __shared__ float4 k1_smem[];
  const int split = blockIdx.y;
  const int64_t nb0 = (int64_t)split * split_len;
  const int64_t nb1 = min(n, nb0 + split_len);
  k1_body<METRIC, BQ, KW, VEC>(base, nb0, nb1, qs, qrows, (int64_t)blockIdx.x * BQ, nq, d, qnorm, bnorm, k,
                               partial + (int64_t)split * k, (int64_t)nsplit * k,
                               reinterpret_cast<float*>(k1_smem));
}

// Segmented persistent form over a device work queue: the work items of many
// independent point sets stored back to back -- item i covers queries
// [q0, qend) of one set against that set's points [nb0, nb1) (global rows,
// so the keys carry global ids) and writes split slot `split` of each
// query's lists.  A grid of resident CTAs takes the items (largest first) from the queue
// by an atomic counter until the queue is exhausted.  Before taking work a
// CTA waits until the queue of this call is published (q->epoch == epoch,
// written with the plan ahead of the kernel in stream order); the wait is
// bounded by `wait_cycles`, after which the CTA records MANN_ETIMEOUT in
// q->status and returns without touching any list.
template <int METRIC, int BQ, int KW, bool VEC>
__global__ void __launch_bounds__(K1_THREADS, 2)
    k1_persistent(const float* __restrict__ data, const SegItem* __restrict__ items, SegQueue* q, unsigned epoch,
                  long long wait_cycles, int d, int k, int nsplit, uint64_t* __restrict__ partial,
                  const int32_t* __restrict__ qrows) {
  extern __shared__ float4 k1_smem[];
  __shared__ int s_item;
  __shared__ int s_count;
  if (threadIdx.x == 0) {
    volatile SegQueue* vq = q;
    const long long t0 = clock64();
    int ok = 1;
    while (vq->epoch != epoch) {
      if (clock64() - t0 > wait_cycles) {
        atomicCAS(&q->status, 0, (int)MANN_ETIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    s_count = ok ? vq->count : 0;
  }
  __syncthreads();
  const int count = s_count;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned long long i = atomicAdd(&q->head, 1ull);
      s_item = i < (unsigned long long)count ? (int)i : -1;
    }
    __syncthreads();
    const int idx = s_item;
    if (idx < 0) break;
    const SegItem it = items[idx];
    k1_body<METRIC, BQ, KW, VEC>(data, it.nb0, it.nb1, data, qrows, it.q0, it.qend, d, nullptr, nullptr, k,
                                 partial + (int64_t)it.split * k, (int64_t)nsplit * k,
                                 reinterpret_cast<float*>(k1_smem));
    __syncthreads();  // s_item is rewritten only after every thread read it
  }
}

// Exact FP32 scan for a handful of query rows (nq <= 32, e.g. the rows the
// BF16 form could not certify): one point per thread, blocks striding over
// 256-point chunks, every distance the FP32 form's sequential sum in
// dimension order (queries staged 32 dimensions at a time in shared memory,
// the point's slice in registers); warp w keeps the lists of rows w, w+8,
// w+16, w+24; one list per (row, block), merged afterwards.
constexpr int FEW_Q = 32;
constexpr int FEW_T = 256;
constexpr int FEW_DC = 32;
// up to FEW_QS rows with d <= FEW_STAGED_D: the rows are staged whole in shared
// memory once, and each thread streams its point with no barrier per chunk
constexpr int FEW_QS = 4;
constexpr int FEW_STAGED_D = 2048;

// the FP32 form's distance from the sequential sum `acc` (row qrow, point pi)
template <int METRIC>
__device__ __forceinline__ float few_distance(float acc, const float* __restrict__ qnorm, int64_t qrow,
                                              const float* __restrict__ bnorm, int64_t pi, bool valid) {
  float v = acc;
  if constexpr (METRIC == MANN_METRIC_EUCLIDEAN) {
    v = __fsqrt_rn(v);
  } else if constexpr (METRIC == MANN_METRIC_COSINE) {
    const float qnv = qnorm[qrow];
    const float bnv = valid ? bnorm[pi] : 1.0f;
    const float den = __fmul_rn(__fsqrt_rn(qnv), __fsqrt_rn(bnv));
    v = __fsub_rn(1.0f, __fdiv_rn(v, den));
    if (v < 0.0f) v = 0.0f;
  }
  return v;
}

// the block's distances dsm[j][0, np) (points p0 ...) into the lists of rows
// j = warp + 8 m, held by that warp
template <int KW, int M>
__device__ __forceinline__ void few_fold(const float (*dsm)[FEW_T + 1], uint64_t (&L)[M][KW], int nq, int warp,
                                         int lane, int64_t p0, int np, int k) {
#pragma unroll
  for (int m = 0; m < M; ++m) {
    const int j = warp + 8 * m;
    if (j >= nq) continue;  // warp-uniform
    uint64_t thr = list_get<KW>(L[m], k - 1);
    for (int c8 = 0; c8 < FEW_T; c8 += 32) {
      const int col = c8 + lane;
      const uint64_t key = col < np ? make_key(dsm[j][col], (uint32_t)(p0 + col)) : KEY_NONE;
      unsigned pend = __ballot_sync(FULL, key < thr);
      while (pend) {
        const int src = __ffs(pend) - 1;
        pend &= pend - 1;
        const uint64_t cnd = __shfl_sync(FULL, key, src);
        if (cnd < thr) {
          list_insert<KW>(L[m], cnd, lane);
          thr = list_get<KW>(L[m], k - 1);
        }
      }
    }
  }
}

template <int METRIC, int KW, bool VEC>
__global__ void __launch_bounds__(FEW_T, 2)
    few_rows_kernel(const float* __restrict__ base, int64_t n, const float* __restrict__ qs,
                    const int32_t* __restrict__ qrows, int nq, int d, const float* __restrict__ qnorm,
                    const float* __restrict__ bnorm, int k, uint64_t* __restrict__ partial) {
  __shared__ __align__(16) float qsm[FEW_Q][FEW_DC];
  __shared__ float dsm[FEW_Q][FEW_T + 1];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint64_t L[4][KW];
#pragma unroll
  for (int m = 0; m < 4; ++m)
#pragma unroll
    for (int s = 0; s < KW; ++s) L[m][s] = KEY_NONE;
  for (int64_t p0 = (int64_t)blockIdx.x * FEW_T; p0 < n; p0 += (int64_t)gridDim.x * FEW_T) {
    const int64_t pi = p0 + t;
    const bool valid = pi < n;
    const float* prow = base + (valid ? pi : 0) * d;
    float acc[FEW_Q];
#pragma unroll
    for (int j = 0; j < FEW_Q; ++j) acc[j] = 0.0f;
    for (int c0 = 0; c0 < d; c0 += FEW_DC) {
      const int dc = min(FEW_DC, d - c0);
      __syncthreads();
      for (int e = t; e < FEW_Q * FEW_DC; e += FEW_T) {
        const int r = e / FEW_DC, c = e % FEW_DC;
        float v = 0.0f;
        if (r < nq && c < dc) v = __ldg(&qs[(int64_t)(qrows ? qrows[r] : r) * d + c0 + c]);
        qsm[r][c] = v;
      }
      float pv[FEW_DC];
      if (VEC && dc == FEW_DC) {
#pragma unroll
        for (int c = 0; c < FEW_DC; c += 4) {
          const float4 v = valid ? __ldg(reinterpret_cast<const float4*>(prow + c0 + c)) : make_float4(0, 0, 0, 0);
          pv[c] = v.x;
          pv[c + 1] = v.y;
          pv[c + 2] = v.z;
          pv[c + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int c = 0; c < FEW_DC; ++c) pv[c] = (valid && c < dc) ? __ldg(prow + c0 + c) : 0.0f;
      }
      __syncthreads();
      // dimensions past d are zero on both sides and add nothing
#pragma unroll
      for (int j = 0; j < FEW_Q; ++j) {
        if (j < nq) {
          float a = acc[j];
#pragma unroll
          for (int c = 0; c < FEW_DC; c += 4) {
            const float4 q4 = *reinterpret_cast<const float4*>(&qsm[j][c]);
            if constexpr (METRIC == MANN_METRIC_COSINE) {
              a = __fmaf_rn(q4.x, pv[c], a);
              a = __fmaf_rn(q4.y, pv[c + 1], a);
              a = __fmaf_rn(q4.z, pv[c + 2], a);
              a = __fmaf_rn(q4.w, pv[c + 3], a);
            } else {
              float u = __fsub_rn(q4.x, pv[c]);
              a = __fmaf_rn(u, u, a);
              u = __fsub_rn(q4.y, pv[c + 1]);
              a = __fmaf_rn(u, u, a);
              u = __fsub_rn(q4.z, pv[c + 2]);
              a = __fmaf_rn(u, u, a);
              u = __fsub_rn(q4.w, pv[c + 3]);
              a = __fmaf_rn(u, u, a);
            }
          }
          acc[j] = a;
        }
      }
    }
#pragma unroll
    for (int j = 0; j < FEW_Q; ++j)
      if (j < nq) dsm[j][t] = few_distance<METRIC>(acc[j], qnorm, qrows ? qrows[j] : j, bnorm, pi, valid);
    __syncthreads();
    few_fold<KW, 4>(dsm, L, nq, warp, lane, p0, (int)min((int64_t)FEW_T, n - p0), k);
  }
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int j = warp + 8 * m;
    if (j >= nq) continue;
    uint64_t* dst = partial + ((int64_t)j * gridDim.x + blockIdx.x) * k;
#pragma unroll
    for (int s = 0; s < KW; ++s) {
      const int e = s * 32 + lane;
      if (e < k) dst[e] = L[m][s];
    }
  }
}

// few_rows_kernel for nq <= FEW_QS rows of d <= FEW_STAGED_D: the rows sit in
// shared memory ([FEW_QS][d], staged once), and each thread reads its point
// with eight float4 loads in flight and no barrier per chunk (the chunked
// form waits for its loads 25 times per point at d = 784); the same
// sequential sums in dimension order, the same lists and layout.
template <int METRIC, int KW, bool VEC>
__global__ void __launch_bounds__(FEW_T, 2)
    few_rows_staged_kernel(const float* __restrict__ base, int64_t n, const float* __restrict__ qs,
                           const int32_t* __restrict__ qrows, int nq, int d, const float* __restrict__ qnorm,
                           const float* __restrict__ bnorm, int k, uint64_t* __restrict__ partial) {
  extern __shared__ __align__(16) float fq[];  // [FEW_QS][d]
  __shared__ float dsm[FEW_QS][FEW_T + 1];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  for (int e = t; e < FEW_QS * d; e += FEW_T) {
    const int r = e / d, c = e % d;
    fq[e] = r < nq ? __ldg(&qs[(int64_t)(qrows ? qrows[r] : r) * d + c]) : 0.0f;
  }
  __syncthreads();
  uint64_t L[1][KW];
#pragma unroll
  for (int s = 0; s < KW; ++s) L[0][s] = KEY_NONE;
  for (int64_t p0 = (int64_t)blockIdx.x * FEW_T; p0 < n; p0 += (int64_t)gridDim.x * FEW_T) {
    const int64_t pi = p0 + t;
    const bool valid = pi < n;
    const float* prow = base + (valid ? pi : 0) * d;
    float acc[FEW_QS];
#pragma unroll
    for (int j = 0; j < FEW_QS; ++j) acc[j] = 0.0f;
    if (valid) {
      if (VEC) {  // d % 4 == 0 and 16-byte aligned rows
#pragma unroll 8
        for (int c = 0; c < d; c += 4) {
          const float4 v = __ldg(reinterpret_cast<const float4*>(prow + c));
#pragma unroll
          for (int j = 0; j < FEW_QS; ++j) {
            if (j < nq) {
              const float4 q4 = *reinterpret_cast<const float4*>(&fq[j * d + c]);
              float a = acc[j];
              if constexpr (METRIC == MANN_METRIC_COSINE) {
                a = __fmaf_rn(q4.x, v.x, a);
                a = __fmaf_rn(q4.y, v.y, a);
                a = __fmaf_rn(q4.z, v.z, a);
                a = __fmaf_rn(q4.w, v.w, a);
              } else {
                float u = __fsub_rn(q4.x, v.x);
                a = __fmaf_rn(u, u, a);
                u = __fsub_rn(q4.y, v.y);
                a = __fmaf_rn(u, u, a);
                u = __fsub_rn(q4.z, v.z);
                a = __fmaf_rn(u, u, a);
                u = __fsub_rn(q4.w, v.w);
                a = __fmaf_rn(u, u, a);
              }
              acc[j] = a;
            }
          }
        }
      } else {
#pragma unroll 8
        for (int c = 0; c < d; ++c) {
          const float pv = __ldg(prow + c);
#pragma unroll
          for (int j = 0; j < FEW_QS; ++j) {
            if (j < nq) {
              const float qv = fq[j * d + c];
              if constexpr (METRIC == MANN_METRIC_COSINE) {
                acc[j] = __fmaf_rn(qv, pv, acc[j]);
              } else {
                const float u = __fsub_rn(qv, pv);
                acc[j] = __fmaf_rn(u, u, acc[j]);
              }
            }
          }
        }
      }
    }
    __syncthreads();  // the previous points' fold has read dsm
#pragma unroll
    for (int j = 0; j < FEW_QS; ++j)
      if (j < nq) dsm[j][t] = few_distance<METRIC>(acc[j], qnorm, qrows ? qrows[j] : j, bnorm, pi, valid);
    __syncthreads();
    few_fold<KW, 1>(dsm, L, nq, warp, lane, p0, (int)min((int64_t)FEW_T, n - p0), k);
  }
  if (warp < nq) {
    uint64_t* dst = partial + ((int64_t)warp * gridDim.x + blockIdx.x) * k;
#pragma unroll
    for (int s = 0; s < KW; ++s) {
      const int e = s * 32 + lane;
      if (e < k) dst[e] = L[0][s];
    }
  }
}

template <int METRIC, bool VEC>
mann_status launch_few_m(int grid, const float* base, int64_t n, const float* qs, const int32_t* rows, int nq,
                         int d, const float* qn, const float* bn, int kk, uint64_t* partial, cudaStream_t s) {
  if (nq <= FEW_QS && d <= FEW_STAGED_D) {
    const size_t smem = sizeof(float) * FEW_QS * d;  // <= 32 KB
    if (kk <= 32)
      few_rows_staged_kernel<METRIC, 1, VEC><<<grid, FEW_T, smem, s>>>(base, n, qs, rows, nq, d, qn, bn, kk, partial);
    else
      few_rows_staged_kernel<METRIC, 2, VEC><<<grid, FEW_T, smem, s>>>(base, n, qs, rows, nq, d, qn, bn, kk, partial);
  } else if (kk <= 32) {
    few_rows_kernel<METRIC, 1, VEC><<<grid, FEW_T, 0, s>>>(base, n, qs, rows, nq, d, qn, bn, kk, partial);
  } else {
    few_rows_kernel<METRIC, 2, VEC><<<grid, FEW_T, 0, s>>>(base, n, qs, rows, nq, d, qn, bn, kk, partial);
  }
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

// Merge nsplit sorted lists of k keys per query into one sorted list of k.
// One warp per query; lane s walks list s (and s+32, ...).
__global__ void merge_lists_kernel(const uint64_t* __restrict__ partial, int64_t nq, int nsplit,
                                   int k, uint64_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (q >= nq) return;
  const uint64_t* src = partial + q * (int64_t)nsplit * k;
  constexpr int MAXL = 8;  // lists per lane (nsplit <= 256)
  int head[MAXL];
  uint64_t cur[MAXL];
#pragma unroll
  for (int t = 0; t < MAXL; ++t) {
    const int s = lane + 32 * t;
    head[t] = 0;
    cur[t] = (s < nsplit) ? src[(int64_t)s * k] : KEY_NONE;
  }
  for (int e = 0; e < k; ++e) {
    uint64_t m = cur[0];
#pragma unroll
    for (int t = 1; t < MAXL; ++t) m = min(m, cur[t]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = min(m, (uint64_t)__shfl_xor_sync(FULL, m, o));
    if (lane == 0) out[q * k + e] = m;
    if (m == KEY_NONE) continue;
#pragma unroll
    for (int t = 0; t < MAXL; ++t) {
      if (cur[t] == m) {  // keys are unique (ids differ), so exactly one owner
        const int s = lane + 32 * t;
        ++head[t];
        cur[t] = head[t] < k ? src[(int64_t)s * k + head[t]] : KEY_NONE;
      }
    }
  }
}

__global__ void finish_kernel(const uint64_t* __restrict__ keys, int64_t nq, int kk, int kout,
                              int64_t graph_self, const int32_t* __restrict__ rows,
                              int32_t* __restrict__ ids, float* __restrict__ dists) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint64_t* src = keys + q * (int64_t)kk;
  const int64_t orow = rows ? (int64_t)rows[q] : q;  // output row (and query id)
  int32_t* oid = ids + orow * kout;
  float* odist = dists + orow * kout;
  int m = 0;
  for (int e = 0; e < kk && m < kout; ++e) {
    const uint64_t key = src[e];
    if (key == KEY_NONE) break;
    if (graph_self >= 0 && (int64_t)key_id(key) == graph_self + orow) continue;
    oid[m] = key_id(key);
    odist[m] = key_dist(key);
    ++m;
  }
  for (; m < kout; ++m) {
    oid[m] = -1;
    odist[m] = __int_as_float(0x7F800000);
  }
}

template <int METRIC, int BQ, int KW, bool VEC>
mann_status launch_k1(Context* ctx, const float* base, int64_t n, const float* qs, const int32_t* rows,
                      int64_t nq, int d, const float* qn, const float* bn, int k,
                      int64_t split_len, int nsplit, uint64_t* partial, cudaStream_t s) {
  constexpr int QSTR = BQ + 4, BSTR = K1_BN + 4;
  const size_t smem = sizeof(float) * (2 * K1_DK * QSTR + 2 * K1_DK * BSTR + BQ * BSTR);
  auto kern = k1_tile_topk<METRIC, BQ, KW, VEC>;
  MANN_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((unsigned)ceil_div(nq, BQ), (unsigned)nsplit);
  ctx->time_begin(s);
  kern<<<grid, K1_THREADS, smem, s>>>(base, n, qs, rows, nq, d, qn, bn, k, split_len, nsplit,
                                      partial);
  ctx->time_end(s);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

template <int METRIC, bool VEC>
mann_status dispatch_k1(Context* ctx, int k, const float* base, int64_t n, const float* qs, const int32_t* rows,
                        int64_t nq, int d, const float* qn, const float* bn, int64_t split_len,
                        int nsplit, uint64_t* partial, cudaStream_t s) {
  if (nq <= 32) {  // a handful of queries (e.g. rows re-run by the exact scan): narrow tiles
    if (k <= 32)
      return launch_k1<METRIC, 32, 1, VEC>(ctx, base, n, qs, rows, nq, d, qn, bn, k, split_len,
                                           nsplit, partial, s);
    return launch_k1<METRIC, 32, 8, VEC>(ctx, base, n, qs, rows, nq, d, qn, bn, k, split_len,
                                         nsplit, partial, s);
  }
  if (k <= 32)
    return launch_k1<METRIC, 128, 1, VEC>(ctx, base, n, qs, rows, nq, d, qn, bn, k, split_len, nsplit,
                                          partial, s);
  if (k <= 64)
    return launch_k1<METRIC, 128, 2, VEC>(ctx, base, n, qs, rows, nq, d, qn, bn, k, split_len, nsplit,
                                          partial, s);
  if (k <= 128)
    return launch_k1<METRIC, 64, 4, VEC>(ctx, base, n, qs, rows, nq, d, qn, bn, k, split_len, nsplit,
                                         partial, s);
  return launch_k1<METRIC, 32, 8, VEC>(ctx, base, n, qs, rows, nq, d, qn, bn, k, split_len, nsplit,
                                       partial, s);
}

}  // namespace

template <int METRIC, int BQ, int KW, bool VEC>
static mann_status launch_pers_t(int num_sms, const float* data, const SegItem* items, SegQueue* q, unsigned epoch,
                                 long long wait_cycles, int d, int k, int nsplit, uint64_t* partial,
                                 const int32_t* qrows, cudaStream_t s) {
  constexpr int QSTR = BQ + 4, BSTR = K1_BN + 4;
  const size_t smem = sizeof(float) * (2 * K1_DK * QSTR + 2 * K1_DK * BSTR + BQ * BSTR);
  auto kern = k1_persistent<METRIC, BQ, KW, VEC>;
  MANN_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  MANN_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, K1_THREADS, smem));
  const int grid = std::max(1, per_sm) * num_sms;  // every CTA resident: the queue needs no co-scheduling
  kern<<<(unsigned)grid, K1_THREADS, smem, s>>>(data, items, q, epoch, wait_cycles, d, k, nsplit, partial, qrows);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

mann_status launch_k1_persistent(int num_sms, const float* data, const SegItem* items, SegQueue* q, unsigned epoch,
                                 long long wait_cycles, int d, int metric, int bq, int k, int nsplit,
                                 uint64_t* partial, cudaStream_t s, const int32_t* qrows) {
  if (k < 1 || k > 64) return fail(MANN_EINVAL_ARG, "batched graphs support 1 <= k <= 64 (k+1 with self)");
  const bool vec = (d % 4) == 0;
#define PERS_CASE(M, B, KW)                                                                                      \
  return vec ? launch_pers_t<M, B, KW, true>(num_sms, data, items, q, epoch, wait_cycles, d, k, nsplit, partial, \
                                             qrows, s)                                                          \
             : launch_pers_t<M, B, KW, false>(num_sms, data, items, q, epoch, wait_cycles, d, k, nsplit, partial, \
                                              qrows, s)
  if (metric == MANN_METRIC_EUCLIDEAN) {
    if (k > 32) {
      if (bq == 32) PERS_CASE(MANN_METRIC_EUCLIDEAN, 32, 2);
      PERS_CASE(MANN_METRIC_EUCLIDEAN, 64, 2);
    }
    if (bq == 64) PERS_CASE(MANN_METRIC_EUCLIDEAN, 64, 1);
    if (bq == 32) PERS_CASE(MANN_METRIC_EUCLIDEAN, 32, 1);
    PERS_CASE(MANN_METRIC_EUCLIDEAN, 128, 1);
  }
  if (metric == MANN_METRIC_SQEUCLIDEAN) {
    if (k > 32) {
      if (bq == 32) PERS_CASE(MANN_METRIC_SQEUCLIDEAN, 32, 2);
      PERS_CASE(MANN_METRIC_SQEUCLIDEAN, 64, 2);
    }
    if (bq == 64) PERS_CASE(MANN_METRIC_SQEUCLIDEAN, 64, 1);
    if (bq == 32) PERS_CASE(MANN_METRIC_SQEUCLIDEAN, 32, 1);
    PERS_CASE(MANN_METRIC_SQEUCLIDEAN, 128, 1);
  }
#undef PERS_CASE
  return fail(MANN_EINVAL_ARG, "batched graphs: Euclidean or SqEuclidean");
}

mann_status launch_merge_lists(const uint64_t* partial, int64_t nq, int nsplit, int k, uint64_t* out,
                               cudaStream_t s) {
  if (nq <= 0) return MANN_OK;
  if (nsplit > 128) return fail(MANN_EINVAL_ARG, "at most 128 lists per query can be merged");
  merge_lists_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(partial, nq, nsplit, k, out);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

mann_status launch_row_sqnorm(const float* x, int64_t n, int d, float* out, cudaStream_t s) {
  if (n <= 0) return MANN_OK;
  row_sqnorm_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(x, n, d, out);  // 8 warps x 32 rows
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

mann_status launch_finish(const uint64_t* keys, int64_t nq, int kk, int kout, int64_t graph_self,
                          const int32_t* rows, int32_t* ids, float* dists, cudaStream_t s) {
  if (nq <= 0 || kout <= 0) return MANN_OK;
  finish_kernel<<<(unsigned)ceil_div(nq, 128), 128, 0, s>>>(keys, nq, kk, kout, graph_self, rows,
                                                           ids, dists);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

mann_status knn_fp32_keys(Context* ctx, cudaStream_t s, const float* base, int64_t n,
                          const float* qs, int64_t nq, int d, int metric, int kk,
                          const int32_t* rows, const float* qn, const float* bn,
                          uint64_t** out_keys, int slot_partial, int slot_keys) {
  if (kk < 1 || kk > KMAX_FUSED)
    return fail(MANN_EINVAL_ARG, "fused top-k supports 1 <= k <= " + std::to_string(KMAX_FUSED));
  if (nq <= 0) return MANN_OK;
  if (metric == MANN_METRIC_COSINE && (qn == nullptr || bn == nullptr))
    return fail(MANN_EINVAL_ARG, "cosine search needs row norms");
  if (nq <= FEW_Q && kk <= 64) {
    // a handful of rows: one point per thread across the whole GPU
    const int grid = (int)std::min<int64_t>(256, ceil_div(n, FEW_T));  // one pass for n <= 65536
    uint64_t* partial = nullptr;
    MANN_TRY(ctx->scratch_t(slot_partial, (size_t)nq * grid * kk, &partial));
    const bool vec4 = (d % 4 == 0) && ((reinterpret_cast<uintptr_t>(base) & 15) == 0);
    ctx->time_begin(s);
    switch (metric) {
      case MANN_METRIC_EUCLIDEAN:
        MANN_TRY((vec4 ? launch_few_m<MANN_METRIC_EUCLIDEAN, true>(grid, base, n, qs, rows, (int)nq, d, qn, bn, kk, partial, s)
                       : launch_few_m<MANN_METRIC_EUCLIDEAN, false>(grid, base, n, qs, rows, (int)nq, d, qn, bn, kk, partial, s)));
        break;
      case MANN_METRIC_SQEUCLIDEAN:
        MANN_TRY((vec4 ? launch_few_m<MANN_METRIC_SQEUCLIDEAN, true>(grid, base, n, qs, rows, (int)nq, d, qn, bn, kk, partial, s)
                       : launch_few_m<MANN_METRIC_SQEUCLIDEAN, false>(grid, base, n, qs, rows, (int)nq, d, qn, bn, kk, partial, s)));
        break;
      default:
        MANN_TRY((vec4 ? launch_few_m<MANN_METRIC_COSINE, true>(grid, base, n, qs, rows, (int)nq, d, qn, bn, kk, partial, s)
                       : launch_few_m<MANN_METRIC_COSINE, false>(grid, base, n, qs, rows, (int)nq, d, qn, bn, kk, partial, s)));
        break;
    }
    ctx->time_end(s);
    if (grid == 1) {
      *out_keys = partial;
      return MANN_OK;
    }
    uint64_t* keys = nullptr;
    MANN_TRY(ctx->scratch_t(slot_keys, (size_t)nq * kk, &keys));
    merge_lists_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(partial, nq, grid, kk, keys);
    MANN_CHECK_LAUNCH();
    *out_keys = keys;
    return MANN_OK;
  }
  const int bq = nq <= 32 ? 32 : (kk <= 64 ? 128 : (kk <= 128 ? 64 : 32));
  const int64_t qblocks = ceil_div(nq, bq);
  const int64_t tiles = ceil_div(n, K1_BN);
  // Split the points so that the grid covers the SMs at least once.
  int64_t want = std::max<int64_t>(1, ceil_div(ctx->num_sms, qblocks));
  want = std::min<int64_t>(want, std::min<int64_t>(tiles, 128));
  const int64_t tiles_per = ceil_div(tiles, want);
  const int nsplit = (int)ceil_div(tiles, tiles_per);
  const int64_t split_len = tiles_per * K1_BN;

  uint64_t* partial = nullptr;
  MANN_TRY(ctx->scratch_t(slot_partial, (size_t)nq * nsplit * kk, &partial));
  const bool vec = (d % 4 == 0) && ((reinterpret_cast<uintptr_t>(base) & 15) == 0) &&
                   ((reinterpret_cast<uintptr_t>(qs) & 15) == 0);
  mann_status st;
  switch (metric) {
    case MANN_METRIC_EUCLIDEAN:
      st = vec ? dispatch_k1<MANN_METRIC_EUCLIDEAN, true>(ctx, kk, base, n, qs, rows, nq, d, qn, bn,
                                                          split_len, nsplit, partial, s)
               : dispatch_k1<MANN_METRIC_EUCLIDEAN, false>(ctx, kk, base, n, qs, rows, nq, d, qn, bn,
                                                           split_len, nsplit, partial, s);
      break;
    case MANN_METRIC_SQEUCLIDEAN:
      st = vec ? dispatch_k1<MANN_METRIC_SQEUCLIDEAN, true>(ctx, kk, base, n, qs, rows, nq, d, qn, bn,
                                                            split_len, nsplit, partial, s)
               : dispatch_k1<MANN_METRIC_SQEUCLIDEAN, false>(ctx, kk, base, n, qs, rows, nq, d, qn,
                                                             bn, split_len, nsplit, partial, s);
      break;
    default:
      st = vec ? dispatch_k1<MANN_METRIC_COSINE, true>(ctx, kk, base, n, qs, rows, nq, d, qn, bn,
                                                       split_len, nsplit, partial, s)
               : dispatch_k1<MANN_METRIC_COSINE, false>(ctx, kk, base, n, qs, rows, nq, d, qn, bn,
                                                        split_len, nsplit, partial, s);
      break;
  }
  MANN_TRY(st);
  if (nsplit == 1) {
    *out_keys = partial;
    return MANN_OK;
  }
  uint64_t* keys = nullptr;
  MANN_TRY(ctx->scratch_t(slot_keys, (size_t)nq * kk, &keys));
  merge_lists_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(partial, nq, nsplit, kk, keys);
  MANN_CHECK_LAUNCH();
  *out_keys = keys;
  return MANN_OK;
}

}  // namespace mann

namespace mann {

// Plan of the FP32 form for (n, nq, kk) on a device with num_sms SMs, as
// knn_fp32_keys makes it: a few rows (nq <= FEW_Q, kk <= 64) go to the
// few-row kernel with `*nsplit_out` = its grid of point slices; otherwise the
// tile kernel with `*nsplit_out` point splits.  `*words_out` = the uint64
// words of scratch (per-split lists, then merged lists when there is more
// than one split).
void knn_fp32_plan(int num_sms, int64_t n, int64_t nq, int kk, int* nsplit_out,
                   size_t* words_out) {
  int nsplit = 1;
  if (nq <= FEW_Q && kk <= 64) {
    nsplit = (int)std::min<int64_t>(256, ceil_div(n, FEW_T));
  } else {
    const int bq = nq <= 32 ? 32 : (kk <= 64 ? 128 : (kk <= 128 ? 64 : 32));
    const int64_t qblocks = ceil_div(nq, bq);
    const int64_t tiles = ceil_div(n, K1_BN);
    int64_t want = std::max<int64_t>(1, ceil_div(num_sms, qblocks));
    want = std::min<int64_t>(want, std::min<int64_t>(tiles, 128));
    const int64_t tiles_per = ceil_div(tiles, want);
    nsplit = (int)ceil_div(tiles, tiles_per);
  }
  *nsplit_out = nsplit;
  *words_out = (size_t)nq * nsplit * kk + (nsplit > 1 ? (size_t)nq * kk : 0);
}

// knn_fp32_keys on caller-provided scratch (`words` uint64 at `scratch`,
// laid out as knn_fp32_plan says); no allocation.
mann_status knn_fp32_keys_on(int num_sms, cudaStream_t s, const float* base, int64_t n,
                             const float* qs, int64_t nq, int d, int metric, int kk,
                             const float* qn, const float* bn, uint64_t* scratch, size_t words,
                             uint64_t** out_keys) {
  if (kk < 1 || kk > KMAX_FUSED)
    return fail(MANN_EINVAL_ARG, "fused top-k supports 1 <= k <= " + std::to_string(KMAX_FUSED));
  if (nq <= 0) return MANN_OK;
  if (metric == MANN_METRIC_COSINE && (qn == nullptr || bn == nullptr))
    return fail(MANN_EINVAL_ARG, "cosine search needs row norms");
  int nsplit = 1;
  size_t need = 0;
  knn_fp32_plan(num_sms, n, nq, kk, &nsplit, &need);
  if (need > words) return fail(MANN_EINVAL_ARG, "scratch too small for this search");
  uint64_t* partial = scratch;
  mann_status st;
  if (nq <= FEW_Q && kk <= 64) {
    // the few-row kernel, exactly as knn_fp32_keys runs it (grid = nsplit)
    const bool vec4 = (d % 4 == 0) && ((reinterpret_cast<uintptr_t>(base) & 15) == 0);
    switch (metric) {
      case MANN_METRIC_EUCLIDEAN:
        st = vec4 ? launch_few_m<MANN_METRIC_EUCLIDEAN, true>(nsplit, base, n, qs, nullptr, (int)nq, d, qn, bn, kk, partial, s)
                  : launch_few_m<MANN_METRIC_EUCLIDEAN, false>(nsplit, base, n, qs, nullptr, (int)nq, d, qn, bn, kk, partial, s);
        break;
      case MANN_METRIC_SQEUCLIDEAN:
        st = vec4 ? launch_few_m<MANN_METRIC_SQEUCLIDEAN, true>(nsplit, base, n, qs, nullptr, (int)nq, d, qn, bn, kk, partial, s)
                  : launch_few_m<MANN_METRIC_SQEUCLIDEAN, false>(nsplit, base, n, qs, nullptr, (int)nq, d, qn, bn, kk, partial, s);
        break;
      default:
        st = vec4 ? launch_few_m<MANN_METRIC_COSINE, true>(nsplit, base, n, qs, nullptr, (int)nq, d, qn, bn, kk, partial, s)
                  : launch_few_m<MANN_METRIC_COSINE, false>(nsplit, base, n, qs, nullptr, (int)nq, d, qn, bn, kk, partial, s);
        break;
    }
  } else {
    const int64_t tiles = ceil_div(n, K1_BN);
    const int64_t tiles_per = ceil_div(tiles, nsplit);
    const int64_t split_len = tiles_per * K1_BN;
    Context plain;  // carries the SM count; no timing, no scratch
    plain.num_sms = num_sms;
    const bool vec = (d % 4 == 0) && ((reinterpret_cast<uintptr_t>(base) & 15) == 0) &&
                     ((reinterpret_cast<uintptr_t>(qs) & 15) == 0);
    switch (metric) {
      case MANN_METRIC_EUCLIDEAN:
        st = vec ? dispatch_k1<MANN_METRIC_EUCLIDEAN, true>(&plain, kk, base, n, qs, nullptr, nq, d, qn,
                                                            bn, split_len, nsplit, partial, s)
                 : dispatch_k1<MANN_METRIC_EUCLIDEAN, false>(&plain, kk, base, n, qs, nullptr, nq, d,
                                                             qn, bn, split_len, nsplit, partial, s);
        break;
      case MANN_METRIC_SQEUCLIDEAN:
        st = vec ? dispatch_k1<MANN_METRIC_SQEUCLIDEAN, true>(&plain, kk, base, n, qs, nullptr, nq, d,
                                                              qn, bn, split_len, nsplit, partial, s)
                 : dispatch_k1<MANN_METRIC_SQEUCLIDEAN, false>(&plain, kk, base, n, qs, nullptr, nq, d,
                                                               qn, bn, split_len, nsplit, partial, s);
        break;
      default:
        st = vec ? dispatch_k1<MANN_METRIC_COSINE, true>(&plain, kk, base, n, qs, nullptr, nq, d, qn,
                                                         bn, split_len, nsplit, partial, s)
                 : dispatch_k1<MANN_METRIC_COSINE, false>(&plain, kk, base, n, qs, nullptr, nq, d, qn,
                                                          bn, split_len, nsplit, partial, s);
        break;
    }
  }
  MANN_TRY(st);
  if (nsplit == 1) {
    *out_keys = partial;
    return MANN_OK;
  }
  uint64_t* keys = partial + (size_t)nq * nsplit * kk;
  merge_lists_kernel<<<(unsigned)ceil_div(nq, 8), 256, 0, s>>>(partial, nq, nsplit, kk, keys);
  MANN_CHECK_LAUNCH();
  *out_keys = keys;
  return MANN_OK;
}

}  // namespace mann
