// Activation storage policies.
//
//  StF32   — one float32 plane, row stride `ld`.
//  StSplit — a float32 value v kept as two bf16 planes hi = bf16(v) and
//            lo = bf16(v - hi) (`plane` elements apart).  hi + lo carries a
//            16-bit significand; both planes are operands of the split-BF16
//            tensor-core GEMMs (hi*hi + hi*lo + lo*hi, FP32 accumulation).
#pragma once
#include "common.cuh"

namespace qmc {

// tanh for the split-BF16 (mixed) form's value-only activations: from
// tanh|x| = (1 - e) / (1 + e), e = 2^(-2 log2(e) |x|), with the hardware
// base-2 exponential (ex2.approx, relative error ~2^-22) and a fast divide.
// Absolute error a few 1e-7, below the ~1e-5 relative error of the form's
// split-BF16 GEMM operands; saturates to +-1 for large |x| and keeps the sign
// of x (tanh(+-0) = +-0).
__device__ __forceinline__ float split_tanh(float x) {
  float e;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(fabsf(x) * -2.8853900817779268f));
  return copysignf(__fdividef(1.f - e, 1.f + e), x);
}

struct StF32 {
  float* p;
  int ld;
  __device__ __forceinline__ float get(size_t r, int c) const { return p[r * ld + c]; }
  __device__ __forceinline__ void put(size_t r, int c, float v) const { p[r * ld + c] = v; }
  __device__ __forceinline__ bool valid() const { return p != nullptr; }
};

struct StSplit {
  __nv_bfloat16* p;
  int ld;
  size_t plane;  // elements between the hi and lo planes
  __device__ __forceinline__ float get(size_t r, int c) const {
    size_t i = r * ld + c;
    return __bfloat162float(p[i]) + __bfloat162float(p[i + plane]);
  }
  __device__ __forceinline__ void put(size_t r, int c, float v) const {
    size_t i = r * ld + c;
    __nv_bfloat16 hi = __float2bfloat16_rn(v);
    p[i] = hi;
    p[i + plane] = __float2bfloat16_rn(v - __bfloat162float(hi));
  }
  __device__ __forceinline__ bool valid() const { return p != nullptr; }
};

}  // namespace qmc
