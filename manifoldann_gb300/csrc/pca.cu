// pca.cu -- batched local PCA over kNN neighbourhoods (the PCAMethod fit of
// LocalGeometryEstimator), one warp per centre.
//
// Replaces fit_geometry(::PCAMethod, data, center_idx, neighbor_indices) and
// _fit_pca_geometry / _pca_eigen / _determine_dimension
// (src/geometry/pca.jl:101-241), called once per graph node by
// build_weighted_graph (src/graphs/weighted_knn_graph.jl:247-264).
//
// The reference centres the neighbours on the centre point and takes the
// eigen-decomposition of the smaller of C^T C and C C^T; both give the squared
// singular values of C and its right singular vectors.  Here the warp runs a
// one-sided (Hestenes) Jacobi on the k centred neighbour vectors held as
// columns -- lane a owns column a -- rotating k/2 disjoint pairs at a time in
// a round-robin tournament until every pair is orthogonal.  The columns are
// then sigma_a u_a: eigenvalues sigma_a^2, principal directions
// u_a = w_a / sigma_a, ordered by descending eigenvalue.  FP32 throughout, as
// the reference's Float32 LAPACK call.
#include <algorithm>
#include <cmath>

#include "kernels.cuh"

namespace mann {
namespace {

constexpr int PCA_WARPS = 2;  // warps per block
constexpr int PCA_MAX_SWEEPS = 30;
constexpr unsigned FULLM = 0xffffffffu;

// Columns live in shared memory: column a of warp w at cols[(w * 32 + a) * (d + 1)].
__global__ void __launch_bounds__(PCA_WARPS * 32)
    local_pca_kernel(const float* __restrict__ data, int64_t n, int d, const float* __restrict__ qpts,
                     const int32_t* __restrict__ centres, int64_t m, const int32_t* __restrict__ nbrs, int k,
                     int fixed_dim, float min_ratio, int maxd, int32_t* __restrict__ out_dim,
                     float* __restrict__ out_eig, float* __restrict__ out_basis) {
  extern __shared__ float pca_smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t node = (int64_t)blockIdx.x * PCA_WARPS + w;
  if (node >= m) return;  // warp-uniform
  const int ds = d + 1;
  float* cols_w = pca_smem + (size_t)(w * 32) * ds;
  float* col = cols_w + (size_t)lane * ds;

  // the centre: a data row, or the caller's query point (centre id -1)
  const int32_t ci = centres ? centres[node] : -1;
  int32_t* odim0 = out_dim + node;
  if (ci >= n || (ci < 0 && !qpts)) {  // no centre: nothing fitted
    if (lane == 0) *odim0 = 0;
    for (int j = lane; j < maxd; j += 32) out_eig[node * maxd + j] = 0.0f;
    for (int e = lane; e < maxd * d; e += 32) out_basis[node * (int64_t)maxd * d + e] = 0.0f;
    return;
  }
  const float* cp = ci >= 0 ? data + (int64_t)ci * d : qpts + node * d;
  const int32_t nb = lane < k ? nbrs[node * k + lane] : -1;
  const bool have = nb >= 0 && nb < n;
  const unsigned have_mask = __ballot_sync(FULLM, have);
  const int keff = __popc(have_mask);
  const int slot = __popc(have_mask & ((1u << lane) - 1u));  // neighbours keep their order
  int32_t* odim = out_dim + node;
  float* oeig = out_eig + node * maxd;
  float* obas = out_basis + node * (int64_t)maxd * d;

  if (keff < 2) {
    // fewer than 2 neighbours: identity basis and unit eigenvalues (pca.jl:136-148)
    const int dd = min(fixed_dim > 0 ? fixed_dim : 1, min(d, maxd));
    if (lane == 0) *odim = dd;
    for (int j = lane; j < maxd; j += 32) oeig[j] = j < dd ? 1.0f : 0.0f;
    for (int e = lane; e < maxd * d; e += 32) obas[e] = (e / d < dd && e % d == e / d) ? 1.0f : 0.0f;
    return;
  }
  // centred neighbour vectors as columns 0..keff-1, zero columns above
  if (have) {
    float* dst = cols_w + (size_t)slot * ds;
    const float* src = data + (int64_t)nb * d;
    for (int c = 0; c < d; ++c) dst[c] = __fsub_rn(src[c], cp[c]);
  }
  __syncwarp();
  if (lane >= keff)
    for (int c = 0; c < d; ++c) col[c] = 0.0f;
  __syncwarp();

  // one-sided Jacobi, round-robin pairs over keff columns (padded to an even count)
  const int kp = (keff + 1) & ~1;
  const float tol = (float)(2 * (d + kp)) * 5.9604645e-08f;
  for (int sweep = 0; sweep < PCA_MAX_SWEEPS; ++sweep) {
    bool rotated = false;
    for (int r = 0; r < kp - 1; ++r) {
      // tournament round r: player 0 stays, the others rotate round a circle
      int partner = -1;
      if (lane < kp) {
        const int pos = lane == 0 ? 0 : 1 + ((lane - 1 + r) % (kp - 1));
        const int ppos = kp - 1 - pos;
        partner = ppos == 0 ? 0 : 1 + ((ppos - 1 - r + (kp - 1)) % (kp - 1));
      }
      const bool act = lane < keff && partner >= 0 && partner < keff && partner != lane;
      float cth = 1.0f, sth = 0.0f;
      if (act) {
        // both lanes of a pair evaluate the same sums in the same order
        const float* ca = cols_w + (size_t)min(lane, partner) * ds;
        const float* cb = cols_w + (size_t)max(lane, partner) * ds;
        float alpha = 0.0f, beta = 0.0f, gamma = 0.0f;
        for (int c = 0; c < d; ++c) {
          const float x = ca[c], y = cb[c];
          alpha = __fmaf_rn(x, x, alpha);
          beta = __fmaf_rn(y, y, beta);
          gamma = __fmaf_rn(x, y, gamma);
        }
        if (gamma != 0.0f && fabsf(gamma) > tol * sqrtf(alpha) * sqrtf(beta)) {
          const float zeta = (beta - alpha) / (2.0f * gamma);
          const float t = copysignf(1.0f, zeta) / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
          cth = 1.0f / sqrtf(1.0f + t * t);
          sth = cth * t;
          rotated = true;
        }
      }
      // w_a' = c w_a - s w_b, w_b' = s w_a + c w_b (a the lower column); a lane
      // reads its partner's column chunk before anyone writes that chunk
      const bool first = lane < partner;
      const float* pc = cols_w + (size_t)(act ? partner : lane) * ds;
      for (int c0 = 0; c0 < d; c0 += 8) {
        float tmp[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          tmp[c] = 0.0f;
          if (sth != 0.0f && c0 + c < d) {
            const float own = col[c0 + c], oth = pc[c0 + c];
            tmp[c] = first ? __fsub_rn(__fmul_rn(cth, own), __fmul_rn(sth, oth))
                           : __fadd_rn(__fmul_rn(sth, oth), __fmul_rn(cth, own));
          }
        }
        __syncwarp();
        if (sth != 0.0f) {
#pragma unroll
          for (int c = 0; c < 8; ++c)
            if (c0 + c < d) col[c0 + c] = tmp[c];
        }
        __syncwarp();
      }
    }
    if (!__any_sync(FULLM, rotated)) break;
  }
  // eigenvalues: squared column norms, ranked by descending value (ties: lower column)
  float nrm2 = 0.0f;
  if (lane < keff)
    for (int c = 0; c < d; ++c) nrm2 = __fmaf_rn(col[c], col[c], nrm2);
  int rank = 0;
  float lmax = 0.0f;
  for (int o = 0; o < keff; ++o) {
    const float v = __shfl_sync(FULLM, nrm2, o);
    lmax = fmaxf(lmax, v);
    if (v > nrm2 || (v == nrm2 && o < lane)) ++rank;
  }
  const int maxdim = min(d, keff);
  int dsel;
  if (fixed_dim > 0) {
    dsel = min(fixed_dim, maxdim);
  } else {
    // _determine_dimension: the first rank whose cumulative share reaches the
    // ratio, sums in Float32 in descending order as the reference's
    float total = 0.0f, cum = 0.0f;
    float sorted_v[32];
#pragma unroll
    for (int rr = 0; rr < 32; ++rr) {
      const unsigned who = __ballot_sync(FULLM, lane < keff && rank == rr);
      sorted_v[rr] = who ? __shfl_sync(FULLM, nrm2, __ffs(who) - 1) : 0.0f;
    }
    for (int rr = 0; rr < keff; ++rr) total = __fadd_rn(total, sorted_v[rr]);
    dsel = maxdim;
    if (total == 0.0f) {
      dsel = 1;
    } else {
      for (int rr = 0; rr < maxdim; ++rr) {
        cum = __fadd_rn(cum, sorted_v[rr]);
        if (__fdiv_rn(cum, total) >= min_ratio) {
          dsel = rr + 1;
          break;
        }
      }
    }
  }
  dsel = min(dsel, maxd);
  if (lane == 0) *odim = dsel;
  if (lane < keff && rank < maxd) {
    oeig[rank] = rank < dsel ? nrm2 : 0.0f;
    const float sg = sqrtf(nrm2);
    // null-space columns get e_rank (pca.jl:182-194)
    const float tolz = 1.1920929e-07f * fmaxf(lmax, 1.0f) * (float)max(d, keff);
    float* orow = obas + (int64_t)rank * d;
    for (int c = 0; c < d; ++c) {
      float v = 0.0f;
      if (rank < dsel) v = nrm2 > tolz ? __fdiv_rn(col[c], sg) : (c == rank ? 1.0f : 0.0f);
      orow[c] = v;
    }
  }
  for (int rr = keff + lane; rr < maxd; rr += 32) {
    oeig[rr] = 0.0f;
    for (int c = 0; c < d; ++c) obas[(int64_t)rr * d + c] = 0.0f;
  }
}

// Register form for d <= 32: lane a holds column a in registers and fetches
// its partner's column by shuffles; no shared memory, no warp barriers.
__global__ void __launch_bounds__(256)
    local_pca_reg_kernel(const float* __restrict__ data, int64_t n, int d, const float* __restrict__ qpts,
                         const int32_t* __restrict__ centres, int64_t m, const int32_t* __restrict__ nbrs, int k,
                         int fixed_dim, float min_ratio, int maxd, int32_t* __restrict__ out_dim,
                         float* __restrict__ out_eig, float* __restrict__ out_basis) {
  constexpr int D = 32;
  const int lane = threadIdx.x & 31;
  const int64_t node = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (node >= m) return;  // warp-uniform
  const int32_t ci = centres ? centres[node] : -1;
  int32_t* odim = out_dim + node;
  float* oeig = out_eig + node * maxd;
  float* obas = out_basis + node * (int64_t)maxd * d;
  if (ci >= n || (ci < 0 && !qpts)) {
    if (lane == 0) *odim = 0;
    for (int j = lane; j < maxd; j += 32) oeig[j] = 0.0f;
    for (int e = lane; e < maxd * d; e += 32) obas[e] = 0.0f;
    return;
  }
  const float* cp = ci >= 0 ? data + (int64_t)ci * d : qpts + node * d;
  const int32_t nb = lane < k ? nbrs[node * k + lane] : -1;
  const bool have = nb >= 0 && nb < n;
  const unsigned have_mask = __ballot_sync(FULLM, have);
  const int keff = __popc(have_mask);
  if (keff < 2) {
    const int dd = min(fixed_dim > 0 ? fixed_dim : 1, min(d, maxd));
    if (lane == 0) *odim = dd;
    for (int j = lane; j < maxd; j += 32) oeig[j] = j < dd ? 1.0f : 0.0f;
    for (int e = lane; e < maxd * d; e += 32) obas[e] = (e / d < dd && e % d == e / d) ? 1.0f : 0.0f;
    return;
  }
  // own centred neighbour, then compacted: lane a takes the a-th present neighbour
  float v[D];
#pragma unroll
  for (int c = 0; c < D; ++c) v[c] = (have && c < d) ? __fsub_rn(data[(int64_t)nb * d + c], cp[c]) : 0.0f;
  const int src = lane < keff ? (int)__fns(have_mask, 0, lane + 1) : lane;
  float w[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const float x = __shfl_sync(FULLM, v[c], src);
    w[c] = lane < keff ? x : 0.0f;
  }
  const int kp = (keff + 1) & ~1;
  const float tol = (float)(2 * (d + kp)) * 5.9604645e-08f;
  for (int sweep = 0; sweep < PCA_MAX_SWEEPS; ++sweep) {
    bool rotated = false;
    for (int r = 0; r < kp - 1; ++r) {
      int partner = lane;
      if (lane < kp) {
        const int pos = lane == 0 ? 0 : 1 + ((lane - 1 + r) % (kp - 1));
        const int ppos = kp - 1 - pos;
        partner = ppos == 0 ? 0 : 1 + ((ppos - 1 - r + (kp - 1)) % (kp - 1));
      }
      const bool act = lane < keff && partner < keff && partner != lane;
      float p[D];
#pragma unroll
      for (int c = 0; c < D; ++c) p[c] = __shfl_sync(FULLM, w[c], act ? partner : lane);
      if (act) {
        const bool first = lane < partner;
        // both lanes sum (lower column, higher column) in the same order
        float alpha = 0.0f, beta = 0.0f, gamma = 0.0f;
#pragma unroll
        for (int c = 0; c < D; ++c) {
          const float x = first ? w[c] : p[c], y = first ? p[c] : w[c];
          alpha = __fmaf_rn(x, x, alpha);
          beta = __fmaf_rn(y, y, beta);
          gamma = __fmaf_rn(x, y, gamma);
        }
        if (gamma != 0.0f && fabsf(gamma) > tol * sqrtf(alpha) * sqrtf(beta)) {
          const float zeta = (beta - alpha) / (2.0f * gamma);
          const float t = copysignf(1.0f, zeta) / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
          const float cth = 1.0f / sqrtf(1.0f + t * t);
          const float sth = cth * t;
          rotated = true;
#pragma unroll
          for (int c = 0; c < D; ++c)
            w[c] = first ? __fsub_rn(__fmul_rn(cth, w[c]), __fmul_rn(sth, p[c]))
                         : __fadd_rn(__fmul_rn(sth, p[c]), __fmul_rn(cth, w[c]));
        }
      }
    }
    if (!__any_sync(FULLM, rotated)) break;
  }
  float nrm2 = 0.0f;
#pragma unroll
  for (int c = 0; c < D; ++c) nrm2 = __fmaf_rn(w[c], w[c], nrm2);
  if (lane >= keff) nrm2 = 0.0f;
  int rank = 0;
  float lmax = 0.0f;
  for (int o = 0; o < keff; ++o) {
    const float x = __shfl_sync(FULLM, nrm2, o);
    lmax = fmaxf(lmax, x);
    if (x > nrm2 || (x == nrm2 && o < lane)) ++rank;
  }
  const int maxdim = min(d, keff);
  int dsel;
  if (fixed_dim > 0) {
    dsel = min(fixed_dim, maxdim);
  } else {
    float total = 0.0f, cum = 0.0f;
    for (int rr = 0; rr < keff; ++rr) {
      const unsigned who = __ballot_sync(FULLM, lane < keff && rank == rr);
      total = __fadd_rn(total, __shfl_sync(FULLM, nrm2, __ffs(who) - 1));
    }
    dsel = maxdim;
    if (total == 0.0f) {
      dsel = 1;
    } else {
      for (int rr = 0; rr < maxdim; ++rr) {
        const unsigned who = __ballot_sync(FULLM, lane < keff && rank == rr);
        cum = __fadd_rn(cum, __shfl_sync(FULLM, nrm2, __ffs(who) - 1));
        if (__fdiv_rn(cum, total) >= min_ratio) {
          dsel = rr + 1;
          break;
        }
      }
    }
  }
  dsel = min(dsel, maxd);
  if (lane == 0) *odim = dsel;
  if (lane < keff && rank < maxd) {
    oeig[rank] = rank < dsel ? nrm2 : 0.0f;
    const float sg = sqrtf(nrm2);
    const float tolz = 1.1920929e-07f * fmaxf(lmax, 1.0f) * (float)max(d, keff);
    float* orow = obas + (int64_t)rank * d;
#pragma unroll
    for (int c = 0; c < D; ++c) {
      if (c >= d) break;
      float x = 0.0f;
      if (rank < dsel) x = nrm2 > tolz ? __fdiv_rn(w[c], sg) : (c == rank ? 1.0f : 0.0f);
      orow[c] = x;
    }
  }
  for (int rr = keff + lane; rr < maxd; rr += 32) {
    oeig[rr] = 0.0f;
    for (int c = 0; c < d; ++c) obas[(int64_t)rr * d + c] = 0.0f;
  }
}

}  // namespace

mann_status local_pca_device(cudaStream_t s, const float* data, int64_t n, int d, const float* qpts,
                             const int32_t* centres, int64_t m, const int32_t* nbrs, int k, int fixed_dim,
                             double min_ratio, int maxd, int32_t* out_dim, float* out_eig, float* out_basis) {
  if (m <= 0) return MANN_OK;
  if (d <= 32) {
    local_pca_reg_kernel<<<(unsigned)ceil_div(m, 8), 256, 0, s>>>(data, n, d, qpts, centres, m, nbrs, k, fixed_dim,
                                                                   (float)min_ratio, maxd, out_dim, out_eig,
                                                                   out_basis);
    MANN_CHECK_LAUNCH();
    return MANN_OK;
  }
  const size_t smem = sizeof(float) * PCA_WARPS * 32 * (size_t)(d + 1);
  if (smem > 200 * 1024) return fail(MANN_EINVAL_ARG, "local PCA supports d <= 800");
  if (smem > 48 * 1024)
    MANN_CUDA_TRY(cudaFuncSetAttribute(local_pca_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  local_pca_kernel<<<(unsigned)ceil_div(m, PCA_WARPS), PCA_WARPS * 32, smem, s>>>(
      data, n, d, qpts, centres, m, nbrs, k, fixed_dim, (float)min_ratio, maxd, out_dim, out_eig, out_basis);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

}  // namespace mann

using namespace mann;

extern "C" {

static mann_status pca_check(const mann_pca_params* p, int64_t n, int32_t d, int64_t m, int32_t k, int32_t maxd) {
  if (!p) return fail(MANN_EINVAL_ARG, "params must not be NULL");
  if (d <= 0) return fail(MANN_EINVAL_ARG, "Dataset must have at least one dimension");
  if (n <= 0) return fail(MANN_EINVAL_ARG, "Dataset must contain at least one point");
  if (m < 0) return fail(MANN_EINVAL_ARG, "negative centre count");
  if (k < 0 || k > 32) return fail(MANN_EINVAL_ARG, "local PCA takes at most 32 neighbours per centre");
  if (maxd <= 0) return fail(MANN_EINVAL_ARG, "maxd must be positive");
  if (p->intrinsic_dim < 0) return fail(MANN_EINVAL_ARG, "intrinsic_dim must be >= 1, got " + std::to_string(p->intrinsic_dim));
  if (p->intrinsic_dim == 0 && !(p->min_variance_ratio > 0.0 && p->min_variance_ratio <= 1.0))
    return fail(MANN_EINVAL_ARG, "min_variance_ratio must be in (0, 1], got " + std::to_string(p->min_variance_ratio));
  return MANN_OK;
}

mann_status mann_local_pca_device(const mann_pca_params* p, const float* data, int64_t n, int32_t d,
                                  const int32_t* centres, const float* query_points, int64_t m,
                                  const int32_t* neighbors, int32_t k, int32_t maxd, int32_t* out_dim,
                                  float* out_eigvals, float* out_basis, void* stream) {
  clear_error();
  MANN_TRY(pca_check(p, n, d, m, k, maxd));
  if (m == 0) return MANN_OK;
  if (!data || !neighbors || !out_dim || !out_eigvals || !out_basis || (!centres && !query_points))
    return fail(MANN_EINVAL_ARG, "NULL buffer");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CallScope scope(ctx, s);
  return local_pca_device(s, data, n, d, query_points, centres, m, neighbors, k, p->intrinsic_dim,
                          p->min_variance_ratio, maxd, out_dim, out_eigvals, out_basis);
}

mann_status mann_local_pca(const mann_pca_params* p, const float* data, int64_t n, int32_t d,
                           const int32_t* centres, const float* query_points, int64_t m, const int32_t* neighbors,
                           int32_t k, int32_t maxd, int32_t* out_dim, float* out_eigvals, float* out_basis) {
  clear_error();
  MANN_TRY(pca_check(p, n, d, m, k, maxd));
  if (m == 0) return MANN_OK;
  if (!data || !neighbors || !out_dim || !out_eigvals || !out_basis || (!centres && !query_points))
    return fail(MANN_EINVAL_ARG, "NULL buffer");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  float *dx = nullptr, *dq = nullptr, *de = nullptr, *db = nullptr;
  int32_t *dc = nullptr, *dn = nullptr, *dd = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_BASE, (size_t)n * d, &dx));
  MANN_TRY(ctx->scratch_t(SLOT_PCA_IDX, (size_t)m * (k + 2), &dn));
  dc = dn + m * k;
  dd = dc + m;
  MANN_TRY(ctx->scratch_t(SLOT_OUT_DISTS, (size_t)m * maxd, &de));
  MANN_TRY(ctx->scratch_t(SLOT_PCA_BASIS, (size_t)m * maxd * d, &db));
  MANN_CUDA_TRY(cudaMemcpyAsync(dx, data, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dn, neighbors, sizeof(int32_t) * m * k, cudaMemcpyHostToDevice, s));
  if (centres) MANN_CUDA_TRY(cudaMemcpyAsync(dc, centres, sizeof(int32_t) * m, cudaMemcpyHostToDevice, s));
  if (query_points) {
    MANN_TRY(ctx->scratch_t(SLOT_QUERIES, (size_t)m * d, &dq));
    MANN_CUDA_TRY(cudaMemcpyAsync(dq, query_points, sizeof(float) * m * d, cudaMemcpyHostToDevice, s));
  }
  MANN_TRY(local_pca_device(s, dx, n, d, dq, centres ? dc : nullptr, m, dn, k, p->intrinsic_dim,
                            p->min_variance_ratio, maxd, dd, de, db));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_dim, dd, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_eigvals, de, sizeof(float) * m * maxd, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_basis, db, sizeof(float) * m * maxd * d, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  return MANN_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- edge weights
// compute_edge_weight over every edge of a kNN graph
// (src/graphs/edge_weight.jl:163-262 via _compute_edge_weights_and_diagnostics,
// src/graphs/weighted_knn_graph.jl:194-236): warp per node, lane per edge.
// d_E = ||x_j - x_i||; d_T^(c) = ||B_c^T (x_j - x_i)|| with B_c node c's
// principal directions (rows of basis[c], dims[c] of them).
namespace mann {
namespace {

__device__ __forceinline__ float tangent_chord(const float* __restrict__ B, int dim, int d, bool vec,
                                               const float* __restrict__ x, const float* __restrict__ y) {
  // the displacement's coordinates: with the geometry centred on an endpoint
  // this is project(y) - project(x) of the reference
  float s = 0.0f;
  for (int r = 0; r < dim; ++r) {
    const float* b = B + (int64_t)r * d;
    float t = 0.0f;
    if (vec) {
      for (int c = 0; c < d; c += 4) {
        const float4 bv = __ldg(reinterpret_cast<const float4*>(b + c));
        const float4 xv = __ldg(reinterpret_cast<const float4*>(x + c));
        const float4 yv = __ldg(reinterpret_cast<const float4*>(y + c));
        t = __fmaf_rn(bv.x, __fsub_rn(yv.x, xv.x), t);
        t = __fmaf_rn(bv.y, __fsub_rn(yv.y, xv.y), t);
        t = __fmaf_rn(bv.z, __fsub_rn(yv.z, xv.z), t);
        t = __fmaf_rn(bv.w, __fsub_rn(yv.w, xv.w), t);
      }
    } else {
      for (int c = 0; c < d; ++c) t = __fmaf_rn(b[c], __fsub_rn(y[c], x[c]), t);
    }
    s = __fmaf_rn(t, t, s);
  }
  return sqrtf(s);
}

__global__ void edge_weights_kernel(int rule, const float* __restrict__ data, int64_t n, int d,
                                    const int32_t* __restrict__ nbrs, int k, const int32_t* __restrict__ dims,
                                    const float* __restrict__ basis, int maxd, float* __restrict__ out,
                                    unsigned long long* __restrict__ n_neg) {
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  for (int e = lane; e < k; e += 32) {
    const int32_t j = nbrs[i * k + e];
    float wv = __int_as_float(0x7fc00000);
    if (j >= 0 && j < n) {
      const float* x = data + i * d;
      const float* y = data + (int64_t)j * d;
      // rows, basis rows and the base pointers are 16-byte aligned when d % 4 == 0
      const bool vec = (d & 3) == 0 && ((reinterpret_cast<uintptr_t>(data) | reinterpret_cast<uintptr_t>(basis)) & 15) == 0;
      float s = 0.0f;
      if (vec) {
        for (int c = 0; c < d; c += 4) {
          const float4 xv = __ldg(reinterpret_cast<const float4*>(x + c));
          const float4 yv = __ldg(reinterpret_cast<const float4*>(y + c));
          float t = __fsub_rn(yv.x, xv.x);
          s = __fmaf_rn(t, t, s);
          t = __fsub_rn(yv.y, xv.y);
          s = __fmaf_rn(t, t, s);
          t = __fsub_rn(yv.z, xv.z);
          s = __fmaf_rn(t, t, s);
          t = __fsub_rn(yv.w, xv.w);
          s = __fmaf_rn(t, t, s);
        }
      } else {
        for (int c = 0; c < d; ++c) {
          const float t = __fsub_rn(y[c], x[c]);
          s = __fmaf_rn(t, t, s);
        }
      }
      const float dE = sqrtf(s);
      if (rule == MANN_EDGE_EUCLIDEAN_CHORD) {
        wv = dE;
      } else {
        const float dx = tangent_chord(basis + i * (int64_t)maxd * d, dims[i], d, vec, x, y);
        if (rule == MANN_EDGE_TANGENT_SOURCE) {
          wv = dx;
        } else {
          const float dy = tangent_chord(basis + (int64_t)j * maxd * d, dims[j], d, vec, x, y);
          if (rule == MANN_EDGE_TANGENT_MEAN) {
            wv = 0.5f * (dx + dy);
          } else if (rule == MANN_EDGE_TANGENT_MAX) {
            wv = fmaxf(dx, dy);
          } else {  // curvature-free symmetric, Euclidean chord when negative
            const float raw = (8.0f * dE - dx - dy) / 6.0f;
            if (raw < 0.0f) {
              wv = dE;
              atomicAdd(n_neg, 1ull);
            } else {
              wv = raw;
            }
          }
        }
      }
    }
    out[i * k + e] = wv;
  }
}

}  // namespace
}  // namespace mann

extern "C" {

static mann_status edge_check(int32_t rule, const float* data, int64_t n, int32_t d, const int32_t* nbrs, int32_t k,
                              const int32_t* dims, const float* basis, int32_t maxd, const float* out) {
  if (rule < MANN_EDGE_EUCLIDEAN_CHORD || rule > MANN_EDGE_CURVATURE_FREE)
    return fail(MANN_EINVAL_ARG, "unknown edge weight rule");
  if (d <= 0 || n <= 0 || k < 0) return fail(MANN_EINVAL_ARG, "empty graph");
  if (!data || !nbrs || !out) return fail(MANN_EINVAL_ARG, "NULL buffer");
  if (rule != MANN_EDGE_EUCLIDEAN_CHORD && (!dims || !basis || maxd <= 0))
    return fail(MANN_EINVAL_ARG, "tangent-projected weights require per-vertex tangent estimates");
  return MANN_OK;
}

mann_status mann_edge_weights_device(int32_t rule, const float* data, int64_t n, int32_t d, const int32_t* nbrs,
                                     int32_t k, const int32_t* dims, const float* basis, int32_t maxd,
                                     float* out_weights, int64_t* out_negative, void* stream) {
  clear_error();
  MANN_TRY(edge_check(rule, data, n, d, nbrs, k, dims, basis, maxd, out_weights));
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CallScope scope(ctx, s);
  unsigned long long* cnt = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_EDGE_COUNT, 1, &cnt));
  MANN_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
  if (k > 0) {
    edge_weights_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(rule, data, n, d, nbrs, k, dims, basis, maxd,
                                                                out_weights, cnt);
    MANN_CHECK_LAUNCH();
  }
  if (out_negative) {
    unsigned long long h = 0;
    MANN_CUDA_TRY(cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, s));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));
    *out_negative = (int64_t)h;
  }
  return MANN_OK;
}

mann_status mann_edge_weights(int32_t rule, const float* data, int64_t n, int32_t d, const int32_t* nbrs, int32_t k,
                              const int32_t* dims, const float* basis, int32_t maxd, float* out_weights,
                              int64_t* out_negative) {
  clear_error();
  MANN_TRY(edge_check(rule, data, n, d, nbrs, k, dims, basis, maxd, out_weights));
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  const bool tangent = rule != MANN_EDGE_EUCLIDEAN_CHORD;
  float *dx = nullptr, *dw = nullptr, *db = nullptr;
  int32_t* dn = nullptr;
  unsigned long long* cnt = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_BASE, (size_t)n * d, &dx));
  MANN_TRY(ctx->scratch_t(SLOT_PCA_IDX, (size_t)n * (k + 1), &dn));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_DISTS, (size_t)n * k + 1, &dw));
  MANN_TRY(ctx->scratch_t(SLOT_EDGE_COUNT, 1, &cnt));
  MANN_CUDA_TRY(cudaMemcpyAsync(dx, data, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dn, nbrs, sizeof(int32_t) * n * k, cudaMemcpyHostToDevice, s));
  int32_t* ddim = dn + n * k;
  if (tangent) {
    MANN_TRY(ctx->scratch_t(SLOT_PCA_BASIS, (size_t)n * maxd * d, &db));
    MANN_CUDA_TRY(cudaMemcpyAsync(ddim, dims, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    MANN_CUDA_TRY(cudaMemcpyAsync(db, basis, sizeof(float) * n * maxd * d, cudaMemcpyHostToDevice, s));
  }
  MANN_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
  if (k > 0) {
    edge_weights_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(rule, dx, n, d, dn, k, tangent ? ddim : nullptr,
                                                                db, maxd, dw, cnt);
    MANN_CHECK_LAUNCH();
  }
  unsigned long long h = 0;
  MANN_CUDA_TRY(cudaMemcpyAsync(out_weights, dw, sizeof(float) * n * k, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  if (out_negative) *out_negative = (int64_t)h;
  return MANN_OK;
}

}  // extern "C"
