// graph_csr.cu -- the undirected (union) kNN graph as a device-resident CSR
// matrix: _symmetrize_adjacency (src/graphs/knn_graph.jl:196-210) without the
// host Vector{Vector{Int}} / Set round trip.
//
// Row i of the result is out(i) ∪ in(i), sorted ascending, without repeats.
// Steps: in-degree count -> row capacities k + indeg (scan) -> fill (own list,
// then the in-edges at atomic cursors) -> per-row bitonic sort + dedupe (a warp
// per row up to 1024 entries, a block per row up to 16384) -> scan of the
// unique counts -> compaction.  Sorting makes the result independent of the
// atomic order.
#include <algorithm>

#include "kernels.cuh"

namespace mann {
namespace {

constexpr int WARP_ROW_MAX = 1024;
constexpr int BLOCK_ROW_MAX = 16384;

__global__ void indeg_kernel(const int32_t* __restrict__ ids, int64_t n, int k, unsigned* __restrict__ indeg) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * k) return;
  const int32_t j = ids[e];
  if (j >= 0 && j < n) atomicAdd(&indeg[j], 1u);
}

// exclusive scan of per-row counts (one block of 1024 threads; any n)
__global__ void __launch_bounds__(1024) scan_rows_kernel(const unsigned* __restrict__ cnt, int64_t n, int add,
                                                         int64_t* __restrict__ offs) {
  __shared__ int64_t ws[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int64_t per = (n + 1023) / 1024;
  const int64_t r0 = std::min<int64_t>(n, t * per), r1 = std::min<int64_t>(n, r0 + per);
  int64_t a = 0;
  for (int64_t r = r0; r < r1; ++r) a += (int64_t)cnt[r] + add;
  int64_t ia = a;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t x = __shfl_up_sync(0xffffffffu, ia, o);
    if (lane >= o) ia += x;
  }
  if (lane == 31) ws[w] = ia;
  __syncthreads();
  if (w == 0) {
    int64_t v = ws[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t x = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += x;
    }
    ws[lane] = v;
  }
  __syncthreads();
  int64_t ea = ia - a + (w ? ws[w - 1] : 0);
  for (int64_t r = r0; r < r1; ++r) {
    offs[r] = ea;
    ea += (int64_t)cnt[r] + add;
  }
  if (t == 1023) offs[n] = ea;
}

// own list first (missing entries become -1), then the in-edges; a self
// entry (include_self graphs) lands twice and is deduplicated like any other
__global__ void fill_kernel(const int32_t* __restrict__ ids, int64_t n, int k, const int64_t* __restrict__ offs,
                            unsigned* __restrict__ cursor, int32_t* __restrict__ buf) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * k) return;
  const int64_t i = e / k;
  const int32_t j = ids[e];
  const bool ok = j >= 0 && j < n;
  buf[offs[i] + (e % k)] = ok ? j : -1;
  if (ok) buf[offs[j] + k + atomicAdd(&cursor[j], 1u)] = (int32_t)i;
}

// prepares a bitonic sort of len entries in shared memory by `nt` threads:
// pads to a power of two with INT_MAX and maps missing entries (< 0) to
// INT_MAX, so they sort last; returns the padded length
__device__ int sort_dedupe(int32_t* s, int len, int t, int nt) {
  int p2 = 1;
  while (p2 < len) p2 <<= 1;
  for (int e = len + t; e < p2; e += nt) s[e] = 0x7FFFFFFF;
  for (int e = t; e < len; e += nt)
    if (s[e] < 0) s[e] = 0x7FFFFFFF;
  return p2;
}

__global__ void sort_rows_warp_kernel(const int64_t* __restrict__ offs, int64_t n, int32_t* __restrict__ buf,
                                      unsigned* __restrict__ ucnt, unsigned* __restrict__ long_rows,
                                      unsigned* __restrict__ n_long) {
  __shared__ int32_t sm[8][WARP_ROW_MAX];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * 8 + w;
  if (i >= n) return;
  const int64_t o = offs[i];
  const int len = (int)(offs[i + 1] - o);
  if (len > WARP_ROW_MAX) {
    if (lane == 0) long_rows[atomicAdd(n_long, 1u)] = (unsigned)i;
    return;
  }
  int32_t* s = sm[w];
  for (int e = lane; e < len; e += 32) s[e] = buf[o + e];
  __syncwarp();
  const int p2 = sort_dedupe(s, len, lane, 32);
  __syncwarp();
  for (int size = 2; size <= p2; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int e = lane; e < p2; e += 32) {
        const int partner = e ^ stride;
        if (partner > e) {
          const bool up = (e & size) == 0;
          const int32_t a = s[e], b = s[partner];
          if ((a > b) == up) {
            s[e] = b;
            s[partner] = a;
          }
        }
      }
      __syncwarp();
    }
  // dedupe: keep the first of each run of equal ids
  if (lane == 0) {
    int u = 0;
    for (int e = 0; e < len; ++e) {
      const int32_t v = s[e];
      if (v == 0x7FFFFFFF) break;
      if (u == 0 || s[u - 1] != v) s[u++] = v;
    }
    ucnt[i] = (unsigned)u;
  }
  __syncwarp();
  const unsigned u = ucnt[i];
  for (int e = lane; e < (int)u; e += 32) buf[o + e] = s[e];
}

__global__ void __launch_bounds__(1024) sort_rows_block_kernel(const int64_t* __restrict__ offs,
                                                               const unsigned* __restrict__ long_rows,
                                                               const unsigned* __restrict__ n_long,
                                                               int32_t* __restrict__ buf,
                                                               unsigned* __restrict__ ucnt, int* __restrict__ err) {
  extern __shared__ int32_t sb[];
  const int t = threadIdx.x;
  for (unsigned r = blockIdx.x; r < *n_long; r += gridDim.x) {
    const int64_t i = long_rows[r];
    const int64_t o = offs[i];
    const int len = (int)(offs[i + 1] - o);
    if (len > BLOCK_ROW_MAX) {
      if (t == 0) atomicExch(err, 1);
      continue;
    }
    for (int e = t; e < len; e += 1024) sb[e] = buf[o + e];
    __syncthreads();
    const int p2 = sort_dedupe(sb, len, t, 1024);
    __syncthreads();
    for (int size = 2; size <= p2; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int e = t; e < p2; e += 1024) {
          const int partner = e ^ stride;
          if (partner > e) {
            const bool up = (e & size) == 0;
            const int32_t a = sb[e], b = sb[partner];
            if ((a > b) == up) {
              sb[e] = b;
              sb[partner] = a;
            }
          }
        }
        __syncthreads();
      }
    if (t == 0) {
      int u = 0;
      for (int e = 0; e < len; ++e) {
        const int32_t v = sb[e];
        if (v == 0x7FFFFFFF) break;
        if (u == 0 || sb[u - 1] != v) sb[u++] = v;
      }
      ucnt[i] = (unsigned)u;
    }
    __syncthreads();
    const unsigned u = ucnt[i];
    for (int e = t; e < (int)u; e += 1024) buf[o + e] = sb[e];
    __syncthreads();
  }
}

__global__ void compact_kernel(const int64_t* __restrict__ offs, const int64_t* __restrict__ uoffs, int64_t n,
                               const int32_t* __restrict__ buf, int32_t* __restrict__ cols) {
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const int64_t o = offs[i], u0 = uoffs[i], u = uoffs[i + 1] - u0;
  for (int64_t e = lane; e < u; e += 32) cols[u0 + e] = buf[o + e];
}

}  // namespace

// Union graph of ids [n][k] as CSR: row_offsets [n+1], cols (capacity 2nk).
mann_status symmetrize_device(Context* ctx, cudaStream_t s, const int32_t* ids, int64_t n, int k,
                              int64_t* row_offsets, int32_t* cols, int64_t* nnz_out) {
  unsigned *indeg = nullptr, *ucnt = nullptr, *cursor = nullptr, *long_rows = nullptr, *n_long = nullptr;
  int64_t* offs = nullptr;
  int32_t* buf = nullptr;
  int* err = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_CSR_COUNTS, (size_t)4 * n + 8, &indeg));
  ucnt = indeg + n;
  cursor = ucnt + n;
  long_rows = cursor + n;
  n_long = long_rows + n;
  err = reinterpret_cast<int*>(n_long + 1);
  MANN_TRY(ctx->scratch_t(SLOT_CSR_OFFS, (size_t)n + 1, &offs));
  MANN_TRY(ctx->scratch_t(SLOT_CSR_BUF, (size_t)2 * n * k + 1, &buf));
  MANN_CUDA_TRY(cudaMemsetAsync(indeg, 0, sizeof(unsigned) * (4 * n + 8), s));
  const unsigned eg = (unsigned)ceil_div(n * k, 256);
  indeg_kernel<<<eg, 256, 0, s>>>(ids, n, k, indeg);
  MANN_CHECK_LAUNCH();
  scan_rows_kernel<<<1, 1024, 0, s>>>(indeg, n, k, offs);
  MANN_CHECK_LAUNCH();
  fill_kernel<<<eg, 256, 0, s>>>(ids, n, k, offs, cursor, buf);
  MANN_CHECK_LAUNCH();
  sort_rows_warp_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(offs, n, buf, ucnt, long_rows, n_long);
  MANN_CHECK_LAUNCH();
  const size_t bsm = sizeof(int32_t) * BLOCK_ROW_MAX;
  MANN_CUDA_TRY(cudaFuncSetAttribute(sort_rows_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bsm));
  sort_rows_block_kernel<<<ctx->num_sms, 1024, bsm, s>>>(offs, long_rows, n_long, buf, ucnt, err);
  MANN_CHECK_LAUNCH();
  scan_rows_kernel<<<1, 1024, 0, s>>>(ucnt, n, 0, row_offsets);
  MANN_CHECK_LAUNCH();
  compact_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(offs, row_offsets, n, buf, cols);
  MANN_CHECK_LAUNCH();
  int h_err = 0;
  MANN_CUDA_TRY(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(nnz_out, row_offsets + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  if (h_err) return fail(MANN_EINVAL_ARG, "a vertex has more than 16384 distinct neighbours in the union graph");
  return MANN_OK;
}

}  // namespace mann

using namespace mann;

extern "C" {

mann_status mann_knn_graph_symmetrize_device(const int32_t* ids, int64_t n, int32_t k, int64_t* out_row_offsets,
                                             int32_t* out_cols, int64_t* out_nnz, void* stream) {
  clear_error();
  if (n <= 0 || k <= 0) return fail(MANN_EINVAL_ARG, "empty graph");
  if (n > INT32_MAX) return fail(MANN_EINVAL_ARG, "at most 2^31-1 vertices");
  if (!ids || !out_row_offsets || !out_cols || !out_nnz) return fail(MANN_EINVAL_ARG, "NULL buffer");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CallScope scope(ctx, s);
  return symmetrize_device(ctx, s, ids, n, k, out_row_offsets, out_cols, out_nnz);
}

mann_status mann_knn_graph_symmetrize(const int32_t* ids, int64_t n, int32_t k, int64_t* out_row_offsets,
                                      int32_t* out_cols, int64_t* out_nnz) {
  clear_error();
  if (n <= 0 || k <= 0) return fail(MANN_EINVAL_ARG, "empty graph");
  if (n > INT32_MAX) return fail(MANN_EINVAL_ARG, "at most 2^31-1 vertices");
  if (!ids || !out_row_offsets || !out_cols || !out_nnz) return fail(MANN_EINVAL_ARG, "NULL buffer");
  Context* ctx = nullptr;
  MANN_TRY(get_context(&ctx));
  cudaStream_t s = ctx->stream;
  CallScope scope(ctx, s);
  int32_t *dids = nullptr, *dcols = nullptr;
  int64_t* doffs = nullptr;
  MANN_TRY(ctx->scratch_t(SLOT_OUT_IDS, (size_t)n * k, &dids));
  MANN_TRY(ctx->scratch_t(SLOT_CSR_COLS, (size_t)2 * n * k, &dcols));
  MANN_TRY(ctx->scratch_t(SLOT_CSR_ROWS, (size_t)n + 1, &doffs));
  MANN_CUDA_TRY(cudaMemcpyAsync(dids, ids, sizeof(int32_t) * n * k, cudaMemcpyHostToDevice, s));
  MANN_TRY(symmetrize_device(ctx, s, dids, n, k, doffs, dcols, out_nnz));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_row_offsets, doffs, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaMemcpyAsync(out_cols, dcols, sizeof(int32_t) * *out_nnz, cudaMemcpyDeviceToHost, s));
  MANN_CUDA_TRY(cudaStreamSynchronize(s));
  return MANN_OK;
}

}  // extern "C"
