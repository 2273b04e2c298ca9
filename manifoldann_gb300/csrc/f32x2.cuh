// f32x2.cuh -- packed pairs of FP32 values for the sm_100+ paired FP32
// instructions (sub.rn.f32x2, fma.rn.f32x2): each lane of the pair is rounded
// exactly as the scalar __fsub_rn / __fmaf_rn, so a kernel that keeps two
// independent accumulators in one pair gets the same bits at half the
// instruction count.
#pragma once
#include <stdint.h>

namespace mann {
namespace f2 {

__device__ __forceinline__ uint64_t pack(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void unpack(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t sub(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
// a * b + c per lane, one rounding
__device__ __forceinline__ uint64_t fma(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

}  // namespace f2
}  // namespace mann
