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
