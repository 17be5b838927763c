// Device helpers shared by the index build and the ray march.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fomo {

// ---------------------------------------------------------------------------
// Index checks of the bounds-check build (compiled with FOMO_BOUNDS_CHECK=1;
// `python -m fomo_gb300.build` makes it as libfomo_gpu_checked.so).  Every
// gather and scatter index of the kernels goes through FOMO_IDX(i, n, site):
// in the check build an index outside [0, n) records `site` (the first one
// wins) in this file's device error word and is replaced by 0, so the access
// stays inside its buffer, nothing traps, and no lane leaves the warp's
// collective steps; the runtime reads the words after a synchronising call
// and reports a set one as FOMO_EDEVICE.  In the regular build FOMO_IDX(i, n,
// site) is just i.
// ---------------------------------------------------------------------------
enum CheckSite : unsigned {
  kSiteNone = 0,
  kSitePts = 1,        // sorted points (pts / vel / payloads) of a snapshot
  kSiteCellStart,      // cell_start of the grid
  kSiteKtab,           // per-view LOS table
  kSiteRayXY,          // per-view ray x / y tables
  kSiteNpos,           // neighbour-position buffer
  kSiteNnIdx,          // caller's neighbour-index output
  kSiteCube,           // caller's cube output
  kSiteLam,            // per-line lambda table
  kSiteDeferred,       // deferred-record queue
  kSiteHard,           // hard-sample queue
  kSiteSmem,           // a warp's candidate lists in shared memory
  kSiteTable,          // G(T, n) table
  kSiteIndexBuild,     // index build scatter / scan
  kSiteS2,             // Thomson sin^2 chi per view and point
  kSiteProjection,     // projection scatter
};

static __device__ unsigned int g_check_word;  // one per translation unit (no relocatable device code)

#if defined(FOMO_BOUNDS_CHECK) && FOMO_BOUNDS_CHECK
__device__ __forceinline__ long long checked_index(long long i, long long n, unsigned site) {
  if (i < 0 || i >= n) {
    atomicCAS(&g_check_word, 0u, site);
    return 0;
  }
  return i;
}
#define FOMO_IDX(i, n, site) (::fomo::checked_index((long long)(i), (long long)(n), (site)))
#else
// (sizeof names n without evaluating it: no code, no unused-variable warning)
#define FOMO_IDX(i, n, site) ((void)sizeof(n), (i))
#endif

// Host side: this translation unit's error word, read and cleared (on the
// current device).  Each .cu file defines its reader with this macro.
#define FOMO_DEFINE_CHECK_READER(fn)                                                  \
  cudaError_t fn(unsigned* out) {                                                     \
    *out = 0;                                                                         \
    cudaError_t e = cudaMemcpyFromSymbol(out, g_check_word, sizeof(unsigned));        \
    const unsigned zero = 0;                                                          \
    if (e == cudaSuccess && *out) e = cudaMemcpyToSymbol(g_check_word, &zero, sizeof(unsigned)); \
    return e;                                                                         \
  }

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
