// common.cuh -- shared definitions of libmanngpu (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/mann.h"

namespace mann {

// ---------------------------------------------------------------- status
void set_error(const std::string& msg);
void clear_error();

// kernels launched by the calling thread (reported per call)
void note_launch();
// true once per failure requested through mann_debug_inject(MANN_INJECT_LAUNCH, n)
bool injected_launch_error();
// true once per dropped queue publish requested through mann_debug_inject(MANN_INJECT_QUEUE, n)
bool injected_dropped_publish();
int64_t launch_count();

struct Status {
  mann_status code = MANN_OK;
  bool ok() const { return code == MANN_OK; }
};

#define MANN_CUDA_TRY(expr)                                                              \
  do {                                                                                   \
    cudaError_t _e = (expr);                                                             \
    if (_e != cudaSuccess) {                                                             \
      ::mann::set_error(std::string("CUDA error ") + cudaGetErrorName(_e) + " (" +       \
                        cudaGetErrorString(_e) + ") at " + __FILE__ + ":" +              \
                        std::to_string(__LINE__) + " in " #expr);                        \
      return (_e == cudaErrorMemoryAllocation) ? MANN_ENOMEM : MANN_ECUDA;               \
    }                                                                                    \
  } while (0)

// after every kernel launch: count it and surface launch errors
#define MANN_CHECK_LAUNCH()                                                         \
  do {                                                                              \
    ::mann::note_launch();                                                          \
    MANN_CUDA_TRY(cudaGetLastError());                                              \
    if (::mann::injected_launch_error())                                            \
      return ::mann::fail(MANN_ECUDA, "CUDA error (injected by mann_debug_inject)"); \
  } while (0)

#define MANN_TRY(expr)                 \
  do {                                 \
    mann_status _s = (expr);           \
    if (_s != MANN_OK) return _s;      \
  } while (0)

inline mann_status fail(mann_status code, const std::string& msg) {
  set_error(msg);
  return code;
}

// ---------------------------------------------------------------- ordering keys
// Julia's partialsortperm over Float32 orders by isless (NaN after every
// number, -0.0 before +0.0) and then by index (src/indices/bruteforce.jl:65).
// fkey() maps a float to a uint32 with that order, so a (distance, id) pair is
// one uint64: (fkey(dist) << 32) | id.  Smaller key = nearer neighbour.
constexpr uint64_t KEY_NONE = ~0ull;

__host__ __device__ __forceinline__ uint32_t fkey(float f) {
#ifdef __CUDA_ARCH__
  uint32_t b = __float_as_uint(f);
#else
  uint32_t b;
  std::memcpy(&b, &f, 4);
#endif
  if (f != f) b = 0x7FC00000u;
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__host__ __device__ __forceinline__ float unkey(uint32_t k) {
  uint32_t b = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  std::memcpy(&f, &b, 4);
  return f;
#endif
}

__host__ __device__ __forceinline__ uint64_t make_key(float dist, uint32_t id) {
  return ((uint64_t)fkey(dist) << 32) | (uint64_t)id;
}

__host__ __device__ __forceinline__ float key_dist(uint64_t key) { return unkey((uint32_t)(key >> 32)); }
__host__ __device__ __forceinline__ int32_t key_id(uint64_t key) { return (int32_t)(uint32_t)key; }

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace mann
