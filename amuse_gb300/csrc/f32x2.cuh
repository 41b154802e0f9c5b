// f32x2.cuh -- packed FP32 pairs for sm_103a: two floats in one 64-bit
// register pair, and the add/sub/mul/fma.rn.f32x2 instructions that apply
// the IEEE round-to-nearest scalar operation to both halves (no
// contraction).  Shared by the force, fixed-step VJP and neighbour kernels.
#ifndef G6_F32X2_CUH
#define G6_F32X2_CUH

#include <cuda_runtime.h>

typedef unsigned long long f2x;

__device__ __forceinline__ f2x f2_add(f2x a, f2x b) {
  f2x d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2x f2_sub(f2x a, f2x b) {
  f2x d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2x f2_mul(f2x a, f2x b) {
  f2x d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2x f2_fma(f2x a, f2x b, f2x c) {
  f2x d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2x f2_pack(float lo, float hi) {
  f2x r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(f2x v, float &lo, float &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ float f2_lo(f2x v) {
  float lo, hi;
  f2_unpack(v, lo, hi);
  return lo;
}
__device__ __forceinline__ float f2_hi(f2x v) {
  float lo, hi;
  f2_unpack(v, lo, hi);
  return hi;
}
__device__ __forceinline__ f2x f2_of(const float2 &v) {
  return *reinterpret_cast<const f2x *>(&v);
}
__device__ __forceinline__ f2x f2_dup(float v) { return f2_pack(v, v); }

#endif
