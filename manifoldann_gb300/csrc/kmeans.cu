// kmeans.cu -- KMeansTransform's GPU work: pairwise distances, exact
// assignment, k-means++ seeding and Lloyd iterations.
//
// Replaces src/transforms/kmeans/distance.jl (pairwise_distances! :28-165,
// assign_clusters! :287-310), init.jl (init_random :22-31,
// init_kmeans_plus_plus :56-128), lloyd.jl (lloyd! :36-134, the M-step
// :149-212) and KMeansTransform.jl fit! (:106-161).
//
// Assignment is the exact arg-min (FP64 order of near-ties, lowest centroid id
// on exact ties) through the exact-search path with k = 1.  The M-step sums
// every cluster's points in point order in FP32 -- a stable counting sort
// groups the points first -- so a fit is deterministic and matches the
// oracle's restatement bit for bit from the same initial centroids.
#include <algorithm>
#include <cmath>
#include <vector>

#include "kernels.cuh"

namespace mann {
namespace {

constexpr int PP_CHUNK = 1024;  // k-means++ running-sum block (the oracle uses the same)
constexpr int SORT_CHUNK = 1024;

// ------------------------------------------------------------------ pairwise
// D[i][j] = dist(X[i], C[j]) in the FP32 form's arithmetic (sequential over
// dimensions); 64 x 64 tiles, 256 threads, 4 x 4 per thread.
template <int METRIC>
__global__ void __launch_bounds__(256) pairwise_kernel(const float* __restrict__ X, int64_t n,
                                                       const float* __restrict__ C, int k, int d,
                                                       const float* __restrict__ xn,
                                                       const float* __restrict__ cn,
                                                       float* __restrict__ D) {
  __shared__ float xs[16][65];
  __shared__ float cs[16][65];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t i0 = (int64_t)blockIdx.y * 64;
  const int j0 = blockIdx.x * 64;
  float acc[4][4] = {};
  for (int c0 = 0; c0 < d; c0 += 16) {
    for (int e = threadIdx.x; e < 64 * 16; e += 256) {
      const int r = e >> 4, c = e & 15;
      const int64_t gi = i0 + r;
      const int gj = j0 + r;
      xs[c][r] = (gi < n && c0 + c < d) ? X[gi * d + c0 + c] : 0.0f;
      cs[c][r] = (gj < k && c0 + c < d) ? C[(int64_t)gj * d + c0 + c] : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      float xv[4], cv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        xv[u] = xs[c][ty + 16 * u];
        cv[u] = cs[c][tx + 16 * u];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          if (METRIC == MANN_METRIC_COSINE) {
            acc[a][b] = __fmaf_rn(xv[a], cv[b], acc[a][b]);
          } else {
            const float t = __fsub_rn(xv[a], cv[b]);
            acc[a][b] = __fmaf_rn(t, t, acc[a][b]);
          }
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int64_t gi = i0 + ty + 16 * a;
    if (gi >= n) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int gj = j0 + tx + 16 * b;
      if (gj >= k) continue;
      float v = acc[a][b];
      if (METRIC == MANN_METRIC_EUCLIDEAN) {
        v = __fsqrt_rn(v);
      } else if (METRIC == MANN_METRIC_COSINE) {
        const float den = __fmul_rn(__fsqrt_rn(xn[gi]), __fsqrt_rn(cn[gj]));
        v = __fsub_rn(1.0f, __fdiv_rn(v, den));
        if (v < 0.0f) v = 0.0f;
      }
      D[gi * k + gj] = v;
    }
  }
}

// ------------------------------------------------------------------ gathers
__global__ void gather_rows_kernel(const float* __restrict__ X, int d, const int64_t* __restrict__ idx,
                                   int64_t m, float* __restrict__ out) {
  const int64_t r = blockIdx.x;
  if (r >= m) return;
  const float* src = X + idx[r] * d;
  for (int c = threadIdx.x; c < d; c += blockDim.x) out[r * d + c] = src[c];
}

// ------------------------------------------------------------------ k-means++
__global__ void fill_inf_kernel(float* __restrict__ v, int64_t n) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) v[j] = __int_as_float(0x7F800000);
}

// min D^2 of every point against the centroid X[idx[i-1]] (FP32 difference
// form, dimensions in order).  Block of 128 points staged 32 dims at a time.
__global__ void __launch_bounds__(128) pp_update_kernel(const float* __restrict__ X, int64_t n, int d,
                                                        const int64_t* __restrict__ idx, int i,
                                                        float* __restrict__ mind) {
  __shared__ float xs[32][129];
  __shared__ float cs[32];
  const int64_t j0 = (int64_t)blockIdx.x * 128;
  const int64_t j = j0 + threadIdx.x;
  const float* c = X + idx[i - 1] * d;
  float s = 0.0f;
  for (int c0 = 0; c0 < d; c0 += 32) {
    for (int e = threadIdx.x; e < 128 * 32; e += 128) {
      const int r = e >> 5, cc = e & 31;
      xs[cc][r] = (j0 + r < n && c0 + cc < d) ? X[(j0 + r) * d + c0 + cc] : 0.0f;
    }
    if (threadIdx.x < 32) cs[threadIdx.x] = (c0 + threadIdx.x < d) ? c[c0 + threadIdx.x] : 0.0f;
    __syncthreads();
    const int lim = min(32, d - c0);
    for (int cc = 0; cc < lim; ++cc) {
      const float t = __fsub_rn(xs[cc][threadIdx.x], cs[cc]);
      s = __fmaf_rn(t, t, s);
    }
    __syncthreads();
  }
  if (j < n && s < mind[j]) mind[j] = s;
}

__global__ void pp_block_sums_kernel(const float* __restrict__ mind, int64_t n,
                                     double* __restrict__ bsum) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nb = (n + PP_CHUNK - 1) / PP_CHUNK;
  if (b >= nb) return;
  double s = 0.0;
  const int64_t e = min(n, (b + 1) * PP_CHUNK);
  for (int64_t j = b * PP_CHUNK; j < e; ++j) s += (double)mind[j];
  bsum[b] = s;
}

// searchsortedfirst(cumsum(mind), u * total) with the blocked running sums
__global__ void pp_pick_kernel(const float* __restrict__ mind, int64_t n,
                               const double* __restrict__ bsum, const double* __restrict__ u, int i,
                               int64_t* __restrict__ idx) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int64_t nb = (n + PP_CHUNK - 1) / PP_CHUNK;
  double total = 0.0;
  for (int64_t b = 0; b < nb; ++b) total += bsum[b];
  const double thr = u[i] * total;
  double acc = 0.0;
  int64_t pick = n - 1;
  for (int64_t b = 0; b < nb; ++b) {
    if (acc + bsum[b] >= thr) {
      const int64_t e = min(n, (b + 1) * PP_CHUNK);
      double a2 = acc;
      for (int64_t j = b * PP_CHUNK; j < e; ++j) {
        a2 += (double)mind[j];
        if (a2 >= thr) {
          pick = j;
          break;
        }
      }
      break;
    }
    acc += bsum[b];
  }
  idx[i] = pick;
}

// ------------------------------------------------------------------ M-step
// hist[c * nb + b] = points of chunk b assigned to c
__global__ void sort_hist_kernel(const int32_t* __restrict__ assign, int64_t n, int64_t nb,
                                 unsigned* __restrict__ hist) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  atomicAdd(&hist[(int64_t)assign[j] * nb + j / SORT_CHUNK], 1u);
}

// exclusive scan of m unsigned counts into int64 offsets (single block, serial
// chunks per thread then a block scan) -- m up to a few million
__global__ void scan_kernel(const unsigned* __restrict__ in, int64_t m, int64_t* __restrict__ out) {
  __shared__ int64_t part[1024];
  const int t = threadIdx.x;
  const int64_t per = (m + 1023) / 1024;
  const int64_t b = t * per, e = min(m, b + per);
  int64_t s = 0;
  for (int64_t i = b; i < e; ++i) s += in[i];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    int64_t acc = 0;
    for (int i = 0; i < 1024; ++i) {
      const int64_t v = part[i];
      part[i] = acc;
      acc += v;
    }
  }
  __syncthreads();
  int64_t acc = part[t];
  for (int64_t i = b; i < e; ++i) {
    out[i] = acc;
    acc += in[i];
  }
}

// cluster c's members occupy [start[c], start[c] + count[c])
__global__ void cluster_ranges_kernel(const int64_t* __restrict__ offs, int k, int64_t nb, int64_t n,
                                      int64_t* __restrict__ start, int64_t* __restrict__ count) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  const int64_t s0 = offs[(int64_t)c * nb];
  const int64_t s1 = (c + 1 < k) ? offs[(int64_t)(c + 1) * nb] : n;
  start[c] = s0;
  count[c] = s1 - s0;
}

// stable scatter: one warp per chunk walks its points in order
__global__ void sort_scatter_kernel(const int32_t* __restrict__ assign, int64_t n, int64_t nb,
                                    int64_t* __restrict__ offs, int64_t* __restrict__ members) {
  const int lane = threadIdx.x & 31;
  const int64_t b = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (b >= nb) return;
  const int64_t e = min(n, (b + 1) * SORT_CHUNK);
  for (int64_t g = b * SORT_CHUNK; g < e; g += 32) {
    const int64_t j = g + lane;
    const bool valid = j < e;
    const int c = valid ? assign[j] : -1;
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, c);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    int64_t* slot = valid ? &offs[(int64_t)c * nb + b] : nullptr;
    const int64_t base = valid ? *slot : 0;
    __syncwarp();
    if (valid) {
      members[base + rank] = j;
      if (rank == 0) *slot = base + __popc(peers);
    }
    __syncwarp();
  }
}

// sums[c][r] = sum over c's members (in point order) of X[m][r], FP32
__global__ void msum_kernel(const float* __restrict__ X, int d, int k,
                            const int64_t* __restrict__ start, const int64_t* __restrict__ count,
                            const int64_t* __restrict__ members, float* __restrict__ sums) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)k * d) return;
  const int c = (int)(t / d), r = (int)(t % d);
  float s = 0.0f;
  const int64_t s0 = start[c], cnt = count[c];
  for (int64_t m = 0; m < cnt; ++m) s = __fadd_rn(s, X[members[s0 + m] * d + r]);
  sums[t] = s;
}

__global__ void mdiv_kernel(const float* __restrict__ sums, const int64_t* __restrict__ count, int d,
                            int k, float* __restrict__ newc) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)k * d) return;
  const int64_t cnt = count[t / d];
  if (cnt > 0) newc[t] = __fdiv_rn(sums[t], (float)cnt);
}

// FP64 distance of every point to its assigned centroid (farthest-point repair)
__global__ void assigned_dist64_kernel(const float* __restrict__ X, int64_t n, int d,
                                       const float* __restrict__ C, const int32_t* __restrict__ assign,
                                       int metric, double* __restrict__ out) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const float* x = X + j * d;
  const float* c = C + (int64_t)assign[j] * d;
  double s = 0.0;
  for (int r = 0; r < d; ++r) {
    const double t = (double)x[r] - (double)c[r];
    s = fma(t, t, s);
  }
  out[j] = metric == MANN_METRIC_EUCLIDEAN ? sqrt(s) : s;
}

// first index of the maximum (single block)
__global__ void argmax_first_kernel(const double* __restrict__ v, int64_t n, int64_t* __restrict__ out) {
  __shared__ double bv[1024];
  __shared__ int64_t bi[1024];
  double best = -INFINITY;
  int64_t bj = 0;
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x)
    if (v[j] > best) {
      best = v[j];
      bj = j;
    }
  bv[threadIdx.x] = best;
  bi[threadIdx.x] = bj;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const double ov = bv[threadIdx.x + o];
      const int64_t oi = bi[threadIdx.x + o];
      if (ov > bv[threadIdx.x] || (ov == bv[threadIdx.x] && oi < bi[threadIdx.x])) {
        bv[threadIdx.x] = ov;
        bi[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = bi[0];
}

__global__ void repair_kernel(const float* __restrict__ X, int d, const int64_t* __restrict__ far,
                              int c, float* __restrict__ newc, int64_t* __restrict__ count,
                              double* __restrict__ dist) {
  const int64_t f = *far;
  for (int r = threadIdx.x; r < d; r += blockDim.x) newc[(int64_t)c * d + r] = X[f * d + r];
  __syncthreads();
  if (threadIdx.x == 0) {
    count[c] = 1;
    dist[f] = -INFINITY;
  }
}

// per-cluster movement in the fit's metric (FP32 form), max over clusters
__global__ void movement_kernel(const float* __restrict__ oldc, const float* __restrict__ newc, int k,
                                int d, int metric, double* __restrict__ out_max) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0.0;
  if (c < k) {
    float s = 0.0f;
    for (int r = 0; r < d; ++r) {
      const float t = __fsub_rn(oldc[(int64_t)c * d + r], newc[(int64_t)c * d + r]);
      s = __fmaf_rn(t, t, s);
    }
    m = metric == MANN_METRIC_EUCLIDEAN ? (double)__fsqrt_rn(s) : (double)s;
  }
  // max over the block, then atomically over blocks (non-negative doubles)
  __shared__ double red[256];
  red[threadIdx.x] = m;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0)
    atomicMax(reinterpret_cast<unsigned long long*>(out_max),
              (unsigned long long)__double_as_longlong(red[0]));
}

// ------------------------------------------------------------------ RNG
// splitmix64-seeded xoshiro256** (host)
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    for (int i = 0; i < 4; ++i) {
      seed += 0x9E3779B97F4A7C15ull;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      s[i] = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  uint64_t below(uint64_t m) { return m ? next() % m : 0; }
};

// first m of a seeded Fisher-Yates permutation of 0..n-1
std::vector<int64_t> sample_indices(Rng& rng, int64_t n, int64_t m) {
  std::vector<int64_t> perm(n);
  for (int64_t i = 0; i < n; ++i) perm[i] = i;
  for (int64_t i = 0; i < m; ++i) {
    const int64_t j = i + (int64_t)rng.below((uint64_t)(n - i));
    std::swap(perm[i], perm[j]);
  }
  perm.resize(m);
  return perm;
}

}  // namespace

// ---------------------------------------------------------------- launchers

mann_status pairwise_device(Context* ctx, cudaStream_t s, const float* X, int64_t n, const float* C,
                            int k, int d, int metric, float* D) {
  const float* xn = nullptr;
  const float* cn = nullptr;
  if (metric == MANN_METRIC_COSINE) {
    float *a = nullptr, *b = nullptr;
    MANN_TRY(ctx->scratch_t(SLOT_NORMS_Q, (size_t)n, &a));
    MANN_TRY(ctx->scratch_t(SLOT_NORMS_B, (size_t)k, &b));
    MANN_TRY(launch_row_sqnorm(X, n, d, a, s));
    MANN_TRY(launch_row_sqnorm(C, k, d, b, s));
    xn = a;
    cn = b;
  }
  dim3 grid((unsigned)ceil_div(k, 64), (unsigned)ceil_div(n, 64));
  if (grid.y > 65535) return fail(MANN_EINVAL_ARG, "too many rows for one pairwise call");
  if (metric == MANN_METRIC_EUCLIDEAN)
    pairwise_kernel<MANN_METRIC_EUCLIDEAN><<<grid, 256, 0, s>>>(X, n, C, k, d, xn, cn, D);
  else if (metric == MANN_METRIC_SQEUCLIDEAN)
    pairwise_kernel<MANN_METRIC_SQEUCLIDEAN><<<grid, 256, 0, s>>>(X, n, C, k, d, xn, cn, D);
  else
    pairwise_kernel<MANN_METRIC_COSINE><<<grid, 256, 0, s>>>(X, n, C, k, d, xn, cn, D);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

// Exact assignment of n points to k centroids (arg-min, FP64 order of
// near-ties, lowest id on exact ties); dist = FP32-form distance (may be NULL).
mann_status kmeans_assign_device(Context* ctx, cudaStream_t s, const float* X, int64_t n,
                                 const float* C, int k, int d, int metric, int32_t* assign,
                                 float* dist) {
  mann_knn_params p{};
  p.metric = metric;
  p.k = 1;
  p.precision = MANN_PREC_AUTO;
  p.flags = MANN_FLAG_FP64_TIES;
  float* dd = dist;
  if (!dd) MANN_TRY(ctx->scratch_t(SLOT_KM_DIST, (size_t)n, &dd));
  return exact_search_device(ctx, s, &p, C, k, X, n, d, -1, 1, 1, assign, dd, nullptr);
}

mann_status kmeanspp_device(Context* ctx, cudaStream_t s, const float* X, int64_t n, int d, int k,
                            int64_t first, const double* u_host, int64_t* idx_dev) {
  float* mind = nullptr;
  double* bsum = nullptr;
  double* u = nullptr;
  const int64_t nb = ceil_div(n, PP_CHUNK);
  MANN_TRY(ctx->scratch_t(SLOT_KM_A, (size_t)n, &mind));
  MANN_TRY(ctx->scratch_t(SLOT_KM_B, (size_t)nb, &bsum));
  MANN_TRY(ctx->scratch_t(SLOT_KM_C, (size_t)k, &u));
  MANN_CUDA_TRY(cudaMemcpyAsync(u, u_host, sizeof(double) * k, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(idx_dev, &first, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  fill_inf_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(mind, n);
  MANN_CHECK_LAUNCH();
  for (int i = 1; i < k; ++i) {
    pp_update_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, s>>>(X, n, d, idx_dev, i, mind);
    MANN_CHECK_LAUNCH();
    pp_block_sums_kernel<<<(unsigned)ceil_div(nb, 128), 128, 0, s>>>(mind, n, bsum);
    MANN_CHECK_LAUNCH();
    pp_pick_kernel<<<1, 32, 0, s>>>(mind, n, bsum, u, i, idx_dev);
    MANN_CHECK_LAUNCH();
  }
  return MANN_OK;
}

mann_status gather_rows_device(cudaStream_t s, const float* X, int d, const int64_t* idx_dev,
                               int64_t m, float* out) {
  if (m <= 0) return MANN_OK;
  gather_rows_kernel<<<(unsigned)m, 128, 0, s>>>(X, d, idx_dev, m, out);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

// Group points by cluster: cluster c's members (ascending point index) are
// members[start[c] .. start[c] + count[c]).
mann_status group_by_cluster_device(Context* ctx, cudaStream_t s, const int32_t* assign, int64_t n,
                                    int k, int64_t* start, int64_t* count, int64_t* members) {
  const int64_t nb = ceil_div(n, SORT_CHUNK);
  unsigned* hist = nullptr;
  int64_t* offs = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_KM_A, (size_t)k * nb, &hist));
  MANN_TRY(ctx->scratch_t(SLOT_KM_B, (size_t)k * nb, &offs));
  MANN_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(unsigned) * k * nb, s));
  sort_hist_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(assign, n, nb, hist);
  MANN_CHECK_LAUNCH();
  scan_kernel<<<1, 1024, 0, s>>>(hist, (int64_t)k * nb, offs);
  MANN_CHECK_LAUNCH();
  cluster_ranges_kernel<<<(unsigned)ceil_div(k, 256), 256, 0, s>>>(offs, k, nb, n, start, count);
  MANN_CHECK_LAUNCH();
  sort_scatter_kernel<<<(unsigned)ceil_div(nb, 4), 128, 0, s>>>(assign, n, nb, offs, members);
  MANN_CHECK_LAUNCH();
  return MANN_OK;
}

// Lloyd from the centroids in C (device, updated in place).
mann_status lloyd_device(Context* ctx, cudaStream_t s, const float* X, int64_t n, int d, int k,
                         float* C, int max_iters, double tol, int metric, int32_t* assign,
                         int* iters_out) {
  const int am = metric == MANN_METRIC_EUCLIDEAN ? MANN_METRIC_EUCLIDEAN : MANN_METRIC_SQEUCLIDEAN;
  const int64_t nb = ceil_div(n, SORT_CHUNK);
  unsigned* hist = nullptr;
  int64_t *offs = nullptr, *start = nullptr, *count = nullptr, *members = nullptr;
  float *sums = nullptr, *newc = nullptr;
  double *dist64 = nullptr, *move = nullptr;
  int64_t* far = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_KM_A, (size_t)k * nb, &hist));
  MANN_TRY(ctx->scratch_t(SLOT_KM_B, (size_t)k * nb, &offs));
  MANN_TRY(ctx->scratch_t(SLOT_KM_C, (size_t)2 * k + 8, &start));
  count = start + k;
  move = reinterpret_cast<double*>(start + 2 * k);
  far = start + 2 * k + 1;
  MANN_TRY(ctx->scratch_t(SLOT_KM_D, (size_t)n, &members));
  MANN_TRY(ctx->scratch_t(SLOT_KM_E, (size_t)2 * k * d, &sums));
  newc = sums + (size_t)k * d;
  int it = 0;
  for (int step = 1; step <= max_iters; ++step) {
    it = step;
    MANN_TRY(kmeans_assign_device(ctx, s, X, n, C, k, d, am, assign, nullptr));
    MANN_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(unsigned) * k * nb, s));
    sort_hist_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(assign, n, nb, hist);
    MANN_CHECK_LAUNCH();
    scan_kernel<<<1, 1024, 0, s>>>(hist, (int64_t)k * nb, offs);
    MANN_CHECK_LAUNCH();
    cluster_ranges_kernel<<<(unsigned)ceil_div(k, 256), 256, 0, s>>>(offs, k, nb, n, start, count);
    MANN_CHECK_LAUNCH();
    sort_scatter_kernel<<<(unsigned)ceil_div(nb, 4), 128, 0, s>>>(assign, n, nb, offs, members);
    MANN_CHECK_LAUNCH();
    msum_kernel<<<(unsigned)ceil_div((int64_t)k * d, 256), 256, 0, s>>>(X, d, k, start, count,
                                                                         members, sums);
    MANN_CHECK_LAUNCH();
    MANN_CUDA_TRY(cudaMemcpyAsync(newc, C, sizeof(float) * k * d, cudaMemcpyDeviceToDevice, s));
    mdiv_kernel<<<(unsigned)ceil_div((int64_t)k * d, 256), 256, 0, s>>>(sums, count, d, k, newc);
    MANN_CHECK_LAUNCH();
    // empty clusters: farthest point (first maximum), marked once taken
    std::vector<int64_t> hcount(k);
    MANN_CUDA_TRY(cudaMemcpyAsync(hcount.data(), count, sizeof(int64_t) * k, cudaMemcpyDeviceToHost, s));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));
    bool any_empty = false;
    for (int c = 0; c < k; ++c) any_empty |= hcount[c] == 0;
    if (any_empty) {
      MANN_TRY(ctx->scratch_t(SLOT_KM_F, (size_t)n, &dist64));
      assigned_dist64_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(X, n, d, C, assign, am, dist64);
      MANN_CHECK_LAUNCH();
      for (int c = 0; c < k; ++c) {
        if (hcount[c] != 0) continue;
        argmax_first_kernel<<<1, 1024, 0, s>>>(dist64, n, far);
        MANN_CHECK_LAUNCH();
        repair_kernel<<<1, 128, 0, s>>>(X, d, far, c, newc, count, dist64);
        MANN_CHECK_LAUNCH();
      }
    }
    MANN_CUDA_TRY(cudaMemsetAsync(move, 0, sizeof(double), s));
    movement_kernel<<<(unsigned)ceil_div(k, 256), 256, 0, s>>>(C, newc, k, d, am, move);
    MANN_CHECK_LAUNCH();
    MANN_CUDA_TRY(cudaMemcpyAsync(C, newc, sizeof(float) * k * d, cudaMemcpyDeviceToDevice, s));
    double hmove = 0.0;
    MANN_CUDA_TRY(cudaMemcpyAsync(&hmove, move, sizeof(double), cudaMemcpyDeviceToHost, s));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));
    if (hmove < tol) break;
  }
  MANN_TRY(kmeans_assign_device(ctx, s, X, n, C, k, d, am, assign, nullptr));
  if (iters_out) *iters_out = it;
  return MANN_OK;
}

// KMeansTransform.fit! : optional subsample, random or k-means++ seeding,
// Lloyd, then the full assignment when a subsample was used.
mann_status kmeans_fit_device(Context* ctx, cudaStream_t s, const float* X, int64_t n, int d, int k,
                              int metric, int init, int max_iters, double tol, int64_t subsample,
                              uint64_t seed, float* C, int32_t* assign, int* iters_out) {
  if (k <= 0 || k > n)
    return fail(MANN_EINVAL_ARG, "Cannot fit " + std::to_string(k) + " clusters with only " +
                                     std::to_string(n) + " points");
  Rng rng(seed);
  const bool use_sub = subsample > 0 && subsample < n;
  const float* Xt = X;
  int64_t nt = n;
  if (use_sub) {
    nt = std::max<int64_t>(subsample, k);
    std::vector<int64_t> idx = sample_indices(rng, n, nt);
    int64_t* didx = nullptr;
    float* xs = nullptr;
    MANN_TRY(ctx->scratch_t(SLOT_KM_G, (size_t)nt, &didx));
    MANN_TRY(ctx->scratch_t(SLOT_KM_H, (size_t)nt * d, &xs));
    MANN_CUDA_TRY(cudaMemcpyAsync(didx, idx.data(), sizeof(int64_t) * nt, cudaMemcpyHostToDevice, s));
    MANN_TRY(gather_rows_device(s, X, d, didx, nt, xs));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));  // idx (host) must outlive the copy
    Xt = xs;
  }
  int64_t* cidx = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_KM_I, (size_t)k, &cidx));
  if (init == 0) {
    std::vector<int64_t> idx = sample_indices(rng, nt, k);
    MANN_CUDA_TRY(cudaMemcpyAsync(cidx, idx.data(), sizeof(int64_t) * k, cudaMemcpyHostToDevice, s));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));
  } else {
    const int64_t first = (int64_t)rng.below((uint64_t)nt);
    std::vector<double> u(k);
    for (int i = 0; i < k; ++i) u[i] = rng.uniform();
    MANN_TRY(kmeanspp_device(ctx, s, Xt, nt, d, k, first, u.data(), cidx));
    MANN_CUDA_TRY(cudaStreamSynchronize(s));
  }
  MANN_TRY(gather_rows_device(s, Xt, d, cidx, k, C));
  int32_t* atrain = assign;
  if (use_sub) MANN_TRY(ctx->scratch_t(SLOT_KM_J, (size_t)nt, &atrain));
  MANN_TRY(lloyd_device(ctx, s, Xt, nt, d, k, C, max_iters, tol, metric, atrain, iters_out));
  if (use_sub) {
    const int am = metric == MANN_METRIC_EUCLIDEAN ? MANN_METRIC_EUCLIDEAN : MANN_METRIC_SQEUCLIDEAN;
    MANN_TRY(kmeans_assign_device(ctx, s, X, n, C, k, d, am, assign, nullptr));
  }
  return MANN_OK;
}

// ---------------------------------------------------------------- C ABI

namespace {

mann_status check_points(const float* X, int64_t n, int d) {
  if (d <= 0) return fail(MANN_EINVAL_ARG, "Dataset must have at least one dimension");
  if (n <= 0) return fail(MANN_EINVAL_ARG, "Dataset must contain at least one point");
  if (n > 0x7FFFFFFFll) return fail(MANN_EINVAL_ARG, "at most 2^31-1 points (int32 ids)");
  if (!X) return fail(MANN_EINVAL_ARG, "NULL buffer");
  return MANN_OK;
}

bool l2_metric(int m) { return m == MANN_METRIC_EUCLIDEAN || m == MANN_METRIC_SQEUCLIDEAN; }

}  // namespace
}  // namespace mann

using namespace mann;

extern "C" {

mann_status mann_pairwise_distances(const float* X, int64_t n, const float* C, int32_t k, int32_t d,
                                    int32_t metric, float* D) {
  clear_error();
  MANN_TRY(check_points(X, n, d));
  if (k <= 0 || !C || !D) return fail(MANN_EINVAL_ARG, "need k > 0 centroids and an output");
  if (!l2_metric(metric) && metric != MANN_METRIC_COSINE) return fail(MANN_EINVAL_ARG, "unknown metric code");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  float *dx = nullptr, *dc = nullptr, *dd = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_KM_X, (size_t)n * d, &dx));
  MANN_TRY(ctx->scratch_t(SLOT_KM_CENT, (size_t)k * d, &dc));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_DISTS, (size_t)n * k, &dd));
  MANN_CUDA_TRY(cudaMemcpyAsync(dx, X, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dc, C, sizeof(float) * k * d, cudaMemcpyHostToDevice, s));
  MANN_TRY(pairwise_device(ctx, s, dx, n, dc, k, d, metric, dd));
  MANN_CUDA_TRY(cudaMemcpyAsync(D, dd, sizeof(float) * n * k, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  return MANN_OK;
}

mann_status mann_kmeans_assign(const float* X, int64_t n, const float* C, int32_t k, int32_t d,
                               int32_t metric, int32_t* out_assign, float* out_dist) {
  clear_error();
  MANN_TRY(check_points(X, n, d));
  if (k <= 0 || !C || !out_assign) return fail(MANN_EINVAL_ARG, "need k > 0 centroids and an output");
  if (!l2_metric(metric) && metric != MANN_METRIC_COSINE) return fail(MANN_EINVAL_ARG, "unknown metric code");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  float *dx = nullptr, *dc = nullptr, *dd = nullptr;
  int32_t* da = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_KM_X, (size_t)n * d, &dx));
  MANN_TRY(ctx->scratch_t(SLOT_KM_CENT, (size_t)k * d, &dc));
  MANN_TRY(ctx->scratch_t(SLOT_KM_ASSIGN, (size_t)n, &da));
  MANN_TRY(ctx->scratch_t(SLOT_OUT_DISTS, (size_t)n, &dd));
  MANN_CUDA_TRY(cudaMemcpyAsync(dx, X, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dc, C, sizeof(float) * k * d, cudaMemcpyHostToDevice, s));
  MANN_TRY(kmeans_assign_device(ctx, s, dx, n, dc, k, d, metric, da, dd));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_assign, da, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  if (out_dist) MANN_CUDA_TRY(cudaMemcpyAsync(out_dist, dd, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  return MANN_OK;
}

mann_status mann_kmeanspp(const float* X, int64_t n, int32_t d, int32_t k, int64_t first,
                          const double* u, int64_t* out_idx) {
  clear_error();
  MANN_TRY(check_points(X, n, d));
  if (k <= 0 || k > n) return fail(MANN_EINVAL_ARG, "Cannot initialize " + std::to_string(k) +
                                                        " clusters with only " + std::to_string(n) + " points");
  if (first < 0 || first >= n || !u || !out_idx) return fail(MANN_EINVAL_ARG, "bad first index or buffers");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  float* dx = nullptr;
  int64_t* di = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_KM_X, (size_t)n * d, &dx));
  MANN_TRY(ctx->scratch_t(SLOT_KM_I, (size_t)k, &di));
  MANN_CUDA_TRY(cudaMemcpyAsync(dx, X, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  MANN_TRY(kmeanspp_device(ctx, s, dx, n, d, k, first, u, di));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_idx, di, sizeof(int64_t) * k, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  return MANN_OK;
}

mann_status mann_kmeans_lloyd(const float* X, int64_t n, int32_t d, int32_t k, float* centroids,
                              int32_t max_iters, double tol, int32_t metric, int32_t* out_assign,
                              int32_t* out_iters) {
  clear_error();
  MANN_TRY(check_points(X, n, d));
  if (k <= 0 || !centroids || !out_assign) return fail(MANN_EINVAL_ARG, "need k > 0 centroids and outputs");
  if (max_iters <= 0 || !(tol > 0)) return fail(MANN_EINVAL_ARG, "max_iters and tol must be positive");
  if (!l2_metric(metric)) return fail(MANN_EINVAL_ARG, "Lloyd runs on Euclidean / SqEuclidean");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  float *dx = nullptr, *dc = nullptr;
  int32_t* da = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_KM_X, (size_t)n * d, &dx));
  MANN_TRY(ctx->scratch_t(SLOT_KM_CENT, (size_t)k * d, &dc));
  MANN_TRY(ctx->scratch_t(SLOT_KM_ASSIGN, (size_t)n, &da));
  MANN_CUDA_TRY(cudaMemcpyAsync(dx, X, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(dc, centroids, sizeof(float) * k * d, cudaMemcpyHostToDevice, s));
  int iters = 0;
  MANN_TRY(lloyd_device(ctx, s, dx, n, d, k, dc, max_iters, tol, metric, da, &iters));
  MANN_CUDA_TRY(cudaMemcpyAsync(centroids, dc, sizeof(float) * k * d, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_assign, da, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  if (out_iters) *out_iters = iters;
  return MANN_OK;
}

mann_status mann_kmeans_fit(const mann_kmeans_params* p, const float* X, int64_t n, int32_t d,
                            float* out_centroids, int32_t* out_assign, int32_t* out_iters) {
  clear_error();
  if (!p) return fail(MANN_EINVAL_ARG, "params must not be NULL");
  MANN_TRY(check_points(X, n, d));
  if (p->k <= 0) return fail(MANN_EINVAL_ARG, "Number of clusters must be positive");
  if (p->init != 0 && p->init != 1) return fail(MANN_EINVAL_ARG, "init must be random (0) or k-means++ (1)");
  if (p->max_iters <= 0 || !(p->tol > 0)) return fail(MANN_EINVAL_ARG, "max_iters and tol must be positive");
  if (p->subsample < 0) return fail(MANN_EINVAL_ARG, "subsample_size must be positive or 0 (none)");
  if (!l2_metric(p->metric)) return fail(MANN_EINVAL_ARG, "KMeans runs on Euclidean / SqEuclidean");
  if (!out_centroids || !out_assign) return fail(MANN_EINVAL_ARG, "NULL buffer");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  float *dx = nullptr, *dc = nullptr;
  int32_t* da = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_KM_X, (size_t)n * d, &dx));
  MANN_TRY(ctx->scratch_t(SLOT_KM_CENT, (size_t)p->k * d, &dc));
  MANN_TRY(ctx->scratch_t(SLOT_KM_ASSIGN, (size_t)n, &da));
  MANN_CUDA_TRY(cudaMemcpyAsync(dx, X, sizeof(float) * n * d, cudaMemcpyHostToDevice, s));
  int iters = 0;
  MANN_TRY(kmeans_fit_device(ctx, s, dx, n, d, p->k, p->metric, p->init, p->max_iters, p->tol,
                             p->subsample, p->seed, dc, da, &iters));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_centroids, dc, sizeof(float) * p->k * d, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_assign, da, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  if (out_iters) *out_iters = iters;
  return MANN_OK;
}

}  // extern "C"
