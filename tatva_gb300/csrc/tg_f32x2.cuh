// Packed FP32 pairs for sm_100+ (f32x2 add / sub / mul / fma, round-to-nearest):
// one instruction operates on two independent lanes.  The Hex8 kernels put two
// elements in the two lanes, so every arithmetic instruction serves two elements.
#pragma once

#include <cuda_runtime.h>

namespace tg {

struct f2 {
  unsigned long long v;
};

__device__ __forceinline__ f2 f2_make(float lo, float hi) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ f2 f2_bcast(float a) { return f2_make(a, a); }
__device__ __forceinline__ void f2_split(f2 x, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(x.v));
}
__device__ __forceinline__ f2 operator+(f2 a, f2 b) {
  f2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 operator-(f2 a, f2 b) {
  f2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 operator*(f2 a, f2 b) {
  f2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
// a * b + c
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}
__device__ __forceinline__ f2 f2_zero() { return f2{0ull}; }

// per-lane reciprocal (the pair has no packed divide)
__device__ __forceinline__ f2 f2_rcp(f2 a) {
  float lo, hi;
  f2_split(a, lo, hi);
  return f2_make(1.0f / lo, 1.0f / hi);
}

}  // namespace tg
