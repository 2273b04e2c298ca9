// ivf.cu -- IVF-Flat on the GPU: build (KMeans + inverted lists) and search
// (route to nprobe lists, scan them, top-k).
//
// Replaces src/indices/ivf_flat.jl: build_index (:30-93), _centroid_distances
// + partialsortperm routing (:103-131, :150) and the list scan into a bounded
// heap (:153-167); the routing hook is select_indices(TopKRouting)
// (src/indices/multilevel/routing.jl:94-118), and mann_ivf_scan takes any
// routing (the learned probe supplies its own).
//
// The scan runs "inverted" like the reference's batched multi-level query
// (src/indices/multilevel/query.jl:363-396): queries are grouped by the list
// they probe, the data is gathered into list order once per call, and one
// CTA scans one list for up to 32 of its queries, every distance in the FP32
// form's sequential arithmetic, keeping each query's top-k.  Order: (distance,
// id); the reference's heap keeps an arbitrary member of an exact tie at the
// k-th place, this keeps the lower id.
#include <algorithm>
#include <vector>

#include "f32x2.cuh"
#include "kernels.cuh"
#include "warp_list.cuh"

namespace mann {

namespace {

constexpr int SCAN_Q = 32;    // queries per CTA (at most)
constexpr int SCAN_T = 256;   // threads = points per pass
constexpr int SCAN_DC = 32;   // dimensions per register batch of a point row

__global__ void ivf_lists_kernel(const int64_t* __restrict__ start, const int64_t* __restrict__ members,
                                 int k, int64_t n, int64_t* __restrict__ offsets,
                                 int32_t* __restrict__ ids) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ids[i] = (int32_t)members[i];
  if (i <= k) offsets[i] = i < k ? start[i] : n;
}

__global__ void probe_count_kernel(const int32_t* __restrict__ probes, int64_t np, int nlist,
                                   unsigned* __restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const int l = probes[i];
  if (l >= 0 && l < nlist) atomicAdd(&cnt[l], 1u);
}

// Exclusive prefix sums of the per-list query counts and of their 32-query
// chunks; one block of 1024 threads, each owning a contiguous run of lists.
__global__ void __launch_bounds__(1024) probe_scan_kernel(const unsigned* __restrict__ cnt, int nlist, int qc,
                                                          int64_t* __restrict__ qoff,
                                                          int64_t* __restrict__ choff) {
  __shared__ int64_t wa[32], wb[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int per = (nlist + 1023) / 1024;
  const int l0 = min(nlist, t * per), l1 = min(nlist, l0 + per);
  int64_t a = 0, b = 0;
  for (int l = l0; l < l1; ++l) {
    a += cnt[l];
    b += (cnt[l] + qc - 1) / qc;
  }
  int64_t ia = a, ib = b;  // inclusive scans within the warp
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t xa = __shfl_up_sync(0xffffffffu, ia, o), xb = __shfl_up_sync(0xffffffffu, ib, o);
    if (lane >= o) {
      ia += xa;
      ib += xb;
    }
  }
  if (lane == 31) {
    wa[w] = ia;
    wb[w] = ib;
  }
  __syncthreads();
  if (w == 0) {
    int64_t va = wa[lane], vb = wb[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t xa = __shfl_up_sync(0xffffffffu, va, o), xb = __shfl_up_sync(0xffffffffu, vb, o);
      if (lane >= o) {
        va += xa;
        vb += xb;
      }
    }
    wa[lane] = va;
    wb[lane] = vb;
  }
  __syncthreads();
  int64_t ea = ia - a + (w ? wa[w - 1] : 0), eb = ib - b + (w ? wb[w - 1] : 0);
  for (int l = l0; l < l1; ++l) {
    qoff[l] = ea;
    choff[l] = eb;
    ea += cnt[l];
    eb += (cnt[l] + qc - 1) / qc;
  }
  if (t == 1023) {
    qoff[nlist] = ea;
    choff[nlist] = eb;
  }
}

__global__ void probe_scatter_kernel(const int32_t* __restrict__ probes, int64_t nq, int nprobe,
                                     int nlist, const int64_t* __restrict__ qoff,
                                     unsigned* __restrict__ cursor, int32_t* __restrict__ pair_q,
                                     int32_t* __restrict__ pair_r) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq * nprobe) return;
  const int l = probes[i];
  if (l < 0 || l >= nlist) return;
  const int64_t pos = qoff[l] + atomicAdd(&cursor[l], 1u);
  pair_q[pos] = (int32_t)(i / nprobe);
  pair_r[pos] = (int32_t)(i % nprobe);
}

// One CTA: list l and up to QC (16 or 32) of its queries.  Each thread takes one point
// of the list per pass (read in place through the list's ids) and computes
// its distance to every query of the CTA -- the point's coordinates in
// registers, the queries' in shared memory, each distance the sequential
// difference-form sum over dimensions 0..d-1 of the FP32 form.  Warp w keeps
// the sorted top-k of queries w, w+8, ... as warp-distributed lists.
template <int METRIC, int KW, bool VEC, int QC>
__global__ void __launch_bounds__(SCAN_T, QC == 16 ? 3 : 2)
    ivf_scan_kernel(const float* __restrict__ data, const int64_t* __restrict__ loff,
                    const int32_t* __restrict__ lids, const float* __restrict__ qs, int d,
                    const int64_t* __restrict__ qoff, const int32_t* __restrict__ pair_q,
                    const int32_t* __restrict__ pair_r, const int64_t* __restrict__ choff, int nlist,
                    int k, int nprobe, uint64_t* __restrict__ partial) {
  // queries staged transposed, [dimension][query] with a padded stride, so one
  // 16-byte broadcast read gives four queries' value at one dimension
  constexpr int SDQ = QC == 16 ? 128 : 64;  // dimensions per stage
  constexpr int QS = QC + 4;                // stride (floats), a multiple of 4
  __shared__ __align__(16) float qsm[SDQ * QS];
  __shared__ float dsm[QC][SCAN_T + 1];
  __shared__ int32_t s_q[QC];

  const int64_t w = blockIdx.x;
  if (w >= choff[nlist]) return;
  int lo = 0, hi = nlist - 1;
  while (lo < hi) {  // last list whose chunk offset <= w
    const int mid = (lo + hi + 1) >> 1;
    if (choff[mid] <= w) lo = mid;
    else hi = mid - 1;
  }
  const int l = lo;
  const int64_t e0 = qoff[l] + (w - choff[l]) * QC;
  const int nqe = (int)min((int64_t)QC, qoff[l + 1] - e0);
  const int64_t p_begin = loff[l], p_end = loff[l + 1];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t < nqe) s_q[t] = pair_q[e0 + t];
  __syncthreads();

  constexpr int MW = QC / 8;  // queries per warp
  uint64_t L[MW][KW];
#pragma unroll
  for (int m = 0; m < MW; ++m)
#pragma unroll
    for (int s = 0; s < KW; ++s) L[m][s] = KEY_NONE;

  for (int64_t p0 = p_begin; p0 < p_end; p0 += SCAN_T) {
    const int64_t pi = p0 + t;
    const bool valid = pi < p_end;
    const float* prow = data + (valid ? (int64_t)lids[pi] : 0) * d;
    // queries 2i and 2i+1 in one f32x2 pair: each lane rounds as the scalar
    // difference form, dimension by dimension in order
    uint64_t acc2[QC / 2];
#pragma unroll
    for (int i = 0; i < QC / 2; ++i) acc2[i] = 0ull;
    const int ng4 = (nqe + 3) >> 2;  // groups of four staged queries in use
    for (int c0 = 0; c0 < d; c0 += SDQ) {
      const int dq = min(SDQ, d - c0);
      __syncthreads();
      for (int e = t; e < QC * SDQ; e += SCAN_T) {
        const int r = e / SDQ, c = e % SDQ;
        qsm[c * QS + r] = (r < nqe && c < dq) ? __ldg(&qs[(int64_t)s_q[r] * d + c0 + c]) : 0.0f;
      }
      __syncthreads();
      for (int cb = 0; cb < dq; cb += SCAN_DC) {
        const int dc = min(SCAN_DC, dq - cb);
        float pv[SCAN_DC];
        if (VEC && dc == SCAN_DC) {
#pragma unroll
          for (int c = 0; c < SCAN_DC; c += 4) {
            const float4 v =
                valid ? __ldg(reinterpret_cast<const float4*>(prow + c0 + cb + c)) : make_float4(0, 0, 0, 0);
            pv[c] = v.x;
            pv[c + 1] = v.y;
            pv[c + 2] = v.z;
            pv[c + 3] = v.w;
          }
        } else {
#pragma unroll
          for (int c = 0; c < SCAN_DC; ++c) pv[c] = (valid && c < dc) ? __ldg(prow + c0 + cb + c) : 0.0f;
        }
        // dimensions past d are zero in both operands: (0 - 0)^2 adds nothing
#pragma unroll
        for (int c = 0; c < SCAN_DC; ++c) {
          const uint64_t x2 = f2::pack(pv[c], pv[c]);
          const float4* qrow4 = reinterpret_cast<const float4*>(&qsm[(cb + c) * QS]);
#pragma unroll
          for (int g = 0; g < QC / 4; ++g) {
            if (g < ng4) {  // block-uniform
              const float4 q4 = qrow4[g];
              uint64_t u = f2::sub(f2::pack(q4.x, q4.y), x2);
              acc2[2 * g] = f2::fma(u, u, acc2[2 * g]);
              u = f2::sub(f2::pack(q4.z, q4.w), x2);
              acc2[2 * g + 1] = f2::fma(u, u, acc2[2 * g + 1]);
            }
          }
        }
      }
    }
    float acc[QC];
#pragma unroll
    for (int i = 0; i < QC / 2; ++i) f2::unpack(acc2[i], acc[2 * i], acc[2 * i + 1]);
#pragma unroll
    for (int j = 0; j < QC; ++j)
      if (j < nqe) dsm[j][t] = METRIC == MANN_METRIC_EUCLIDEAN ? __fsqrt_rn(acc[j]) : acc[j];
    __syncthreads();
    const int np = (int)min((int64_t)SCAN_T, p_end - p0);
#pragma unroll
    for (int m = 0; m < MW; ++m) {
      const int j = warp + 8 * m;
      if (j >= nqe) continue;  // warp-uniform
      uint64_t thr = wl::list_get<KW>(L[m], k - 1);
      for (int c8 = 0; c8 < SCAN_T; c8 += 32) {
        const int col = c8 + lane;
        const uint64_t key = col < np ? make_key(dsm[j][col], (uint32_t)lids[p0 + col]) : KEY_NONE;
        unsigned pend = __ballot_sync(wl::FULL, key < thr);
        while (pend) {
          const int src = __ffs(pend) - 1;
          pend &= pend - 1;
          const uint64_t cnd = __shfl_sync(wl::FULL, key, src);
          if (cnd < thr) {
            wl::list_insert<KW>(L[m], cnd, lane);
            thr = wl::list_get<KW>(L[m], k - 1);
          }
        }
      }
    }
  }
#pragma unroll
  for (int m = 0; m < MW; ++m) {
    const int j = warp + 8 * m;
    if (j >= nqe) continue;
    uint64_t* dst = partial + ((int64_t)s_q[j] * nprobe + pair_r[e0 + j]) * k;
#pragma unroll
    for (int s = 0; s < KW; ++s) {
      const int e = s * 32 + lane;
      if (e < k) dst[e] = L[m][s];
    }
  }
}


template <int METRIC, int KW, bool VEC>
mann_status launch_scan_t(cudaStream_t s, int qc, int64_t grid, const float* data, const int64_t* loff,
                          const int32_t* lids, const float* qs, int d, const int64_t* qoff,
                          const int32_t* pair_q, const int32_t* pair_r, const int64_t* choff, int nlist, int k,
                          int nprobe, uint64_t* partial) {
  if (qc == 16)
    ivf_scan_kernel<METRIC, KW, VEC, 16><<<(unsigned)grid, SCAN_T, 0, s>>>(data, loff, lids, qs, d, qoff, pair_q,
                                                                           pair_r, choff, nlist, k, nprobe, partial);
  else
    ivf_scan_kernel<METRIC, KW, VEC, 32><<<(unsigned)grid, SCAN_T, 0, s>>>(data, loff, lids, qs, d, qoff, pair_q,
                                                                           pair_r, choff, nlist, k, nprobe, partial);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

template <int METRIC>
mann_status launch_scan_m(cudaStream_t s, int qc, int64_t grid, bool vec, const float* data, const int64_t* loff,
                          const int32_t* lids, const float* qs, int d, const int64_t* qoff,
                          const int32_t* pair_q, const int32_t* pair_r, const int64_t* choff, int nlist, int k,
                          int nprobe, uint64_t* partial) {
  if (k <= 32)
    return vec ? launch_scan_t<METRIC, 1, true>(s, qc, grid, data, loff, lids, qs, d, qoff, pair_q, pair_r, choff,
                                                nlist, k, nprobe, partial)
               : launch_scan_t<METRIC, 1, false>(s, qc, grid, data, loff, lids, qs, d, qoff, pair_q, pair_r, choff,
                                                 nlist, k, nprobe, partial);
  return vec ? launch_scan_t<METRIC, 2, true>(s, qc, grid, data, loff, lids, qs, d, qoff, pair_q, pair_r, choff,
                                              nlist, k, nprobe, partial)
             : launch_scan_t<METRIC, 2, false>(s, qc, grid, data, loff, lids, qs, d, qoff, pair_q, pair_r, choff,
                                               nlist, k, nprobe, partial);
}

}  // namespace

// Scan of the given probes [nq][nprobe] (list ids, -1 = none): the points of
// the probed lists are read in place through list_ids; results as ids/dists
// [nq][k] (-1 / +inf padding).
mann_status ivf_scan_device(Context* ctx, cudaStream_t s, const float* data, int64_t n, int d,
                            int metric, const int64_t* loff, const int32_t* lids, int nlist,
                            const float* qs, int64_t nq, const int32_t* probes, int nprobe, int k,
                            int32_t* out_ids, float* out_dists) {
  (void)n;
  if (k < 1 || k > 64) return fail(MANN_EINVAL_ARG, "IVF search supports 1 <= k <= 64");
  if (nprobe < 1 || nprobe > 128) return fail(MANN_EINVAL_ARG, "IVF search supports 1 <= nprobe <= 128");
  if (metric == MANN_METRIC_COSINE) return fail(MANN_EINVAL_ARG, "IVF search: Euclidean / SqEuclidean");
  if (nq <= 0) return MANN_OK;
  unsigned* cnt = nullptr;
  int64_t *qoff = nullptr, *choff = nullptr;
  int32_t *pair_q = nullptr, *pair_r = nullptr;
  uint64_t *partial = nullptr, *keys = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_IVF_CNT, (size_t)2 * nlist + 4, &cnt));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_OFF, (size_t)2 * (nlist + 1), &qoff));
  choff = qoff + (nlist + 1);
  MANN_TRY(ctx->scratch_t(SLOT_IVF_PAIRS, (size_t)2 * nq * nprobe, &pair_q));
  pair_r = pair_q + nq * nprobe;
  MANN_TRY(ctx->scratch_t(SLOT_IVF_PARTIAL, (size_t)nq * nprobe * k, &partial));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_KEYS, (size_t)nq * k, &keys));
  MANN_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(unsigned) * (2 * nlist + 4), s));
  MANN_CUDA_TRY(cudaMemsetAsync(partial, 0xFF, sizeof(uint64_t) * nq * nprobe * k, s));
  probe_count_kernel<<<(unsigned)ceil_div(nq * nprobe, 256), 256, 0, s>>>(probes, nq * nprobe, nlist, cnt);
  MANN_CHECK_LAUNCH();
  // 16-query chunks when lists see few queries (more, lighter CTAs), else 32
  const int qc = nq * nprobe <= (int64_t)12 * nlist ? 16 : SCAN_Q;
  probe_scan_kernel<<<1, 1024, 0, s>>>(cnt, nlist, qc, qoff, choff);
  MANN_CHECK_LAUNCH();
  probe_scatter_kernel<<<(unsigned)ceil_div(nq * nprobe, 256), 256, 0, s>>>(
      probes, nq, nprobe, nlist, qoff, cnt + nlist, pair_q, pair_r);
  MANN_CHECK_LAUNCH();
  // chunks <= pairs/32 + lists; blocks past the real count return at once
  const int64_t max_chunks = ceil_div(nq * nprobe, qc) + nlist;
  const bool vec = (d % 4) == 0 && (reinterpret_cast<uintptr_t>(data) & 15) == 0;
  ctx->time_begin(s);
  if (metric == MANN_METRIC_EUCLIDEAN)
    MANN_TRY(launch_scan_m<MANN_METRIC_EUCLIDEAN>(s, qc, max_chunks, vec, data, loff, lids, qs, d, qoff, pair_q, pair_r,
                                                  choff, nlist, k, nprobe, partial));
  else
    MANN_TRY(launch_scan_m<MANN_METRIC_SQEUCLIDEAN>(s, qc, max_chunks, vec, data, loff, lids, qs, d, qoff, pair_q,
                                                    pair_r, choff, nlist, k, nprobe, partial));
  ctx->time_end(s);
  MANN_TRY(launch_merge_lists(partial, nq, nprobe, k, keys, s));
  MANN_TRY(launch_finish(keys, nq, k, k, -1, nullptr, out_ids, out_dists, s));
  return MANN_OK;
}

// top-nprobe centroids of every query (TopKRouting on exact centroid distances)
mann_status ivf_route_device(Context* ctx, cudaStream_t s, const float* centroids, int nlist, int d,
                             int centroid_metric, const float* qs, int64_t nq, int nprobe,
                             int32_t* probes) {
  mann_knn_params p{};
  p.metric = centroid_metric;
  p.k = nprobe;
  p.precision = MANN_PREC_AUTO;
  float* dd = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_IVF_ROUTE_D, (size_t)nq * nprobe, &dd));
  return exact_search_device(ctx, s, &p, centroids, nlist, qs, nq, d, -1, std::min(nprobe, nlist),
                             nprobe, probes, dd, nullptr);
}

mann_status ivf_build_device(Context* ctx, cudaStream_t s, const float* data, int64_t n, int d,
                             int nlist, int centroid_metric, int max_iters, double tol,
                             int64_t subsample, uint64_t seed, float* centroids, int64_t* offsets,
                             int32_t* ids, int* iters) {
  int32_t* assign = nullptr;
  int64_t *start = nullptr, *members = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_IVF_ASSIGN, (size_t)n, &assign));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_START, (size_t)2 * nlist, &start));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_MEMBERS, (size_t)n, &members));
  MANN_TRY(kmeans_fit_device(ctx, s, data, n, d, nlist, centroid_metric, 1, max_iters, tol, subsample,
                             seed, centroids, assign, iters));
  MANN_TRY(group_by_cluster_device(ctx, s, assign, n, nlist, start, start + nlist, members));
  ivf_lists_kernel<<<(unsigned)ceil_div(std::max<int64_t>(n, nlist + 1), 256), 256, 0, s>>>(
      start, members, nlist, n, offsets, ids);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

}  // namespace mann

using namespace mann;

extern "C" {

mann_status mann_ivf_build(const mann_ivf_build_params* p, const float* data, int64_t n, int32_t d,
                           float* out_centroids, int64_t* out_offsets, int32_t* out_ids,
                           int32_t* out_iters) {
  clear_error();
  if (!p) return fail(MANN_EINVAL_ARG, "params must not be NULL");
  if (d <= 0) return fail(MANN_EINVAL_ARG, "Dataset must have at least one dimension");
  if (n <= 0) return fail(MANN_EINVAL_ARG, "Dataset must contain at least one point");
  if (p->nlist <= 0) return fail(MANN_EINVAL_ARG, "nlist must be positive");
  if (p->nlist > n) return fail(MANN_EINVAL_ARG, "Cannot fit " + std::to_string(p->nlist) +
                                                     " clusters with only " + std::to_string(n) + " points");
  if (p->centroid_metric != MANN_METRIC_EUCLIDEAN && p->centroid_metric != MANN_METRIC_SQEUCLIDEAN)
    return fail(MANN_EINVAL_ARG, "centroid metric: Euclidean or SqEuclidean");
  if (!data || !out_centroids || !out_offsets || !out_ids) return fail(MANN_EINVAL_ARG, "NULL buffer");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  float *dx = nullptr, *dc = nullptr;
  int64_t* doff = nullptr;
  int32_t* dids = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_BASE, (size_t)n * d, &dx));
  MANN_TRY(ctx->scratch_t(SLOT_KM_CENT, (size_t)p->nlist * d, &dc));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_LOFF, (size_t)p->nlist + 1, &doff));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_LIDS, (size_t)n, &dids));
  MANN_CUDA_TRY(cudaMemcpyAsync(dx, data, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  int iters = 0;
  MANN_TRY(ivf_build_device(ctx, s, dx, n, d, p->nlist, p->centroid_metric,
                            p->kmeans_max_iters > 0 ? p->kmeans_max_iters : 25,
                            p->kmeans_tol > 0 ? p->kmeans_tol : 1e-4, p->kmeans_subsample, p->seed,
                            dc, doff, dids, &iters));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_centroids, dc, sizeof(float) * p->nlist * d, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_offsets, doff, sizeof(int64_t) * (p->nlist + 1), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_ids, dids, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  if (out_iters) *out_iters = iters;
  return MANN_OK;
}

static mann_status ivf_check(const mann_knn_params* p, int32_t nprobe, const float* data, int64_t n,
                             int32_t d, int32_t nlist, const int64_t* offs, const int32_t* ids,
                             const float* qs, int64_t q) {
  if (!p) return fail(MANN_EINVAL_ARG, "params must not be NULL");
  if (d <= 0) return fail(MANN_EINVAL_ARG, "Dataset must have at least one dimension");
  if (n <= 0) return fail(MANN_EINVAL_ARG, "Dataset must contain at least one point");
  if (nlist <= 0 || nprobe <= 0) return fail(MANN_EINVAL_ARG, "nlist and nprobe must be positive");
  if (q < 0) return fail(MANN_EINVAL_ARG, "negative query count");
  if (!data || !offs || !ids || (q > 0 && !qs)) return fail(MANN_EINVAL_ARG, "NULL buffer");
  return MANN_OK;
}

mann_status mann_ivf_search_device(const mann_knn_params* p, int32_t nprobe, int32_t centroid_metric,
                                   const float* data, int64_t n, int32_t d, const float* centroids,
                                   int32_t nlist, const int64_t* list_offsets,
                                   const int32_t* list_ids, const float* queries, int64_t q,
                                   int32_t* out_ids, float* out_dists, void* stream) {
  clear_error();
  MANN_TRY(ivf_check(p, nprobe, data, n, d, nlist, list_offsets, list_ids, queries, q));
  if (p->k <= 0 || q == 0) return MANN_OK;
  nprobe = std::min(nprobe, nlist);  // clamp(nprobe, 1, nlist) (ivf_flat.jl:146)
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CallScope scope(ctx, s);
  int32_t* probes = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_IVF_PROBES, (size_t)q * nprobe, &probes));
  MANN_TRY(ivf_route_device(ctx, s, centroids, nlist, d, centroid_metric, queries, q, nprobe, probes));
  return ivf_scan_device(ctx, s, data, n, d, p->metric, list_offsets, list_ids, nlist, queries, q,
                         probes, nprobe, p->k, out_ids, out_dists);
}

mann_status mann_ivf_scan_device(const mann_knn_params* p, const int32_t* probes, int32_t nprobe,
                                 const float* data, int64_t n, int32_t d, int32_t nlist,
                                 const int64_t* list_offsets, const int32_t* list_ids,
                                 const float* queries, int64_t q, int32_t* out_ids,
                                 float* out_dists, void* stream) {
  clear_error();
  MANN_TRY(ivf_check(p, nprobe, data, n, d, nlist, list_offsets, list_ids, queries, q));
  if (!probes && q > 0) return fail(MANN_EINVAL_ARG, "NULL probes");
  if (p->k <= 0 || q == 0) return MANN_OK;
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CallScope scope(ctx, s);
  return ivf_scan_device(ctx, s, data, n, d, p->metric, list_offsets, list_ids, nlist, queries, q,
                         probes, nprobe, p->k, out_ids, out_dists);
}

mann_status mann_ivf_search(const mann_knn_params* p, int32_t nprobe, int32_t centroid_metric,
                            const float* data, int64_t n, int32_t d, const float* centroids,
                            int32_t nlist, const int64_t* list_offsets, const int32_t* list_ids,
                            const float* queries, int64_t q, int32_t* out_ids, float* out_dists) {
  clear_error();
  MANN_TRY(ivf_check(p, nprobe, data, n, d, nlist, list_offsets, list_ids, queries, q));
  if (p->k <= 0 || q == 0) return MANN_OK;
  nprobe = std::min(nprobe, nlist);
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  float *dx = nullptr, *dc = nullptr, *dq = nullptr, *dd = nullptr;
  int64_t* doff = nullptr;
  int32_t *dids = nullptr, *dout = nullptr, *probes = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_BASE, (size_t)n * d, &dx));
  MANN_TRY(ctx->scratch_t(SLOT_KM_CENT, (size_t)nlist * d, &dc));
  MANN_TRY(ctx->scratch_t(SLOT_QUERIES, (size_t)q * d, &dq));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_LOFF, (size_t)nlist + 1, &doff));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_LIDS, (size_t)n, &dids));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_IDS, (size_t)q * p->k, &dout));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_DISTS, (size_t)q * p->k, &dd));
  MANN_TRY(ctx->scratch_t(SLOT_IVF_PROBES, (size_t)q * nprobe, &probes));
  MANN_CUDA_TRY(cudaMemcpyAsync(dx, data, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dc, centroids, sizeof(float) * nlist * d, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dq, queries, sizeof(float) * q * d, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(doff, list_offsets, sizeof(int64_t) * (nlist + 1), cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dids, list_ids, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
  MANN_TRY(ivf_route_device(ctx, s, dc, nlist, d, centroid_metric, dq, q, nprobe, probes));
  MANN_TRY(ivf_scan_device(ctx, s, dx, n, d, p->metric, doff, dids, nlist, dq, q, probes, nprobe,
                           p->k, dout, dd));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_ids, dout, sizeof(int32_t) * q * p->k, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_dists, dd, sizeof(float) * q * p->k, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  return MANN_OK;
}

}  // extern "C"
