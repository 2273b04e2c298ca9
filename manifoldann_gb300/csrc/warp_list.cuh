// warp_list.cuh -- a sorted list of uint64 keys distributed over the 32
// lanes of a warp (entry e lives in register slot e/32 of lane e%32), with
// ballot-based insertion.  Used by the fused top-k epilogues of the FP32 tile
// kernel and of the IVF list scan.
#pragma once
#include <stdint.h>

#include "common.cuh"

namespace mann {
namespace wl {

constexpr unsigned FULL = 0xFFFFFFFFu;

template <int KW>
__device__ __forceinline__ void list_insert(uint64_t (&L)[KW], uint64_t c, int lane) {
  int pos = 0;
#pragma unroll
  for (int s = 0; s < KW; ++s) pos += __popc(__ballot_sync(FULL, L[s] < c));
  uint64_t up[KW], last[KW];
#pragma unroll
  for (int s = 0; s < KW; ++s) {
    up[s] = __shfl_up_sync(FULL, L[s], 1);
    last[s] = __shfl_sync(FULL, L[s], 31);
  }
#pragma unroll
  for (int s = 0; s < KW; ++s) {
    const int e = s * 32 + lane;
    uint64_t shifted = up[s];
    if (lane == 0) shifted = (s == 0) ? KEY_NONE : last[s > 0 ? s - 1 : 0];
    if (e > pos) L[s] = shifted;
    else if (e == pos) L[s] = c;
  }
}

template <int KW>
__device__ __forceinline__ uint64_t list_get(const uint64_t (&L)[KW], int e) {
  const int slot = e >> 5, ln = e & 31;
  uint64_t v = L[0];
#pragma unroll
  for (int s = 1; s < KW; ++s)
    if (slot == s) v = L[s];
  return __shfl_sync(FULL, v, ln);
}

}  // namespace wl
}  // namespace mann
