// Device helpers shared by the index build and the ray march.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fomo {

// Cell coordinate of a coordinate value: floor((v - o) * inv_h), clamped to
// [0, dim-1].  Monotone non-decreasing in v (each FP32 step is monotone), so a
// strict box (lo, hi) maps to the cell range [cell(lo), cell(hi)] that holds
// every point strictly inside it.  NaN maps to cell 0.
__device__ __forceinline__ int cell_coord(float v, float o, float inv_h, int dim) {
  float c = floorf(__fmul_rn(__fsub_rn(v, o), inv_h));
  if (!(c >= 0.0f)) return 0;
  if (c > (float)(dim - 1)) return dim - 1;
  return (int)c;
}

// 2^x on the SFU (PTX ex2.approx.ftz.f32: max rel. error 2^-22, subnormal
// results flushed to zero).
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Kahan-compensated FP32 accumulation.
__device__ __forceinline__ void kahan_add(float& sum, float& comp, float v) {
  const float y = __fsub_rn(v, comp);
  const float t = __fadd_rn(sum, y);
  comp = __fsub_rn(__fsub_rn(t, sum), y);
  sum = t;
}

}  // namespace fomo
