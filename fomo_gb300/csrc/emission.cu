// K1: per-point emissivity, computed once per (snapshot, table, observation
// type) and kept resident next to the sorted points.
//
//  * emission_kernel restates emissionfromdatacube (fomo-c/src/fomo-CHIANTI.cpp:
//    228-322): log10 of n and T (fomo-operations.cpp:63-84, <= 0 -> 0), the
//    G(T, n) lookup of goft (fomo-CHIANTI.cpp:64-121: linear in logT, nearest
//    in logn, index arithmetic in FP32, interpolation in FP64), the thermal
//    FWHM of linefwhm (:220-226) and eps = k * 10^(2 log n) * G / w (:292-293),
//    rounding to FP32 at the same points as the reference's vector operators.
//    log10 is evaluated in FP64 and rounded once (correctly rounded except for
//    double-rounding cases); glibc's log10f is within 1 ulp of that.
//  * thomson_emission_kernel restates thomsonfromdatacube / getThomsonGeomFactor
//    (fomo-thomson.cpp:39-92).
// The G table is staged in shared memory when it fits.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fomo_device.cuh"
#include "fomo_internal.h"

namespace fomo {

namespace {

constexpr int kMaxSmemTableFloats = 40 * 1024;  // 160 KB: covers the 200x200 instrument tables

__device__ __forceinline__ float log10_rn(float v) { return __double2float_rn(log10((double)v)); }

template <bool kSmem>
__global__ void emission_kernel(const float* __restrict__ ne_s, const float* __restrict__ T_s, int64_t n,
                                TableDev t, float2* __restrict__ ew) {
  extern __shared__ float sm[];
  const float* G = t.G;
  const float* logT = t.logT;
  if (kSmem) {
    float* sG = sm;
    float* sT = sm + (size_t)t.nt * t.nrho;
    for (int i = threadIdx.x; i < t.nt * t.nrho; i += blockDim.x) sG[i] = t.G[i];
    for (int i = threadIdx.x; i < t.nt; i += blockDim.x) sT[i] = t.logT[i];
    __syncthreads();
    G = sG;
    logT = sT;
  }
  const float T0 = t.logT[0], T1 = t.logT[1];
  const float r0 = t.logn[0], r1 = t.logn[1];
  const float dT = __fsub_rn(T1, T0), dR = __fsub_rn(r1, r0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float nv = ne_s[i];
    const float Tv = T_s[i];
    const float logrho = nv <= 0.0f ? 0.0f : log10_rn(nv);
    const float lT = Tv <= 0.0f ? 0.0f : log10_rn(Tv);
    // goft (fomo-CHIANTI.cpp:95-116)
    float g = 0.0f;
    const float qT = floorf(__fdiv_rn(__fsub_rn(lT, T0), dT));
    const float qR = roundf(__fdiv_rn(__fsub_rn(logrho, r0), dR));
    if (qT >= 0.0f && qT + 1.0f <= (float)(t.nt - 1) && qR >= 0.0f && qR <= (float)(t.nrho - 1)) {
      const int ft = (int)qT, ct = ft + 1, ri = (int)qR;
      const int gi = ri * t.nt + ct;
      const int ng = t.nt * t.nrho;
      const double x1 = logT[FOMO_IDX(ct, t.nt, kSiteTable)], y1 = G[FOMO_IDX(gi, ng, kSiteTable)];
      const double x2 = logT[FOMO_IDX(ft, t.nt, kSiteTable)], y2 = G[FOMO_IDX(gi - 1, ng, kSiteTable)];
      const double res = __dadd_rn(__ddiv_rn(__dmul_rn(__dsub_rn((double)lT, x1), __dsub_rn(y2, y1)),
                                             __dsub_rn(x2, x1)),
                                   y1);
      g = __double2float_rn(res);
    }
    const float w = t.imaging ? 1.0f : __double2float_rn(__dmul_rn(t.cw, (double)__fsqrt_rn(Tv)));
    const float a = __double2float_rn(__dmul_rn(2.0, (double)logrho));
    const float b = __double2float_rn(pow(10.0, (double)a));
    const float c = __fmul_rn(b, g);
    const float d = __double2float_rn(__dmul_rn(t.k, (double)c));
    ew[i] = make_float2(__fdiv_rn(d, w), w);
  }
}

// getThomsonGeomFactor (fomo-thomson.cpp:39-58), FP32 storage points as there.
__device__ void thomson_geom(float r, float* totterm, float* polterm) {
  const double U = FOMO_LIMB_U;
  const float sinomega = __double2float_rn(__ddiv_rn(FOMO_RSUN, (double)r));
  const float coeff = __double2float_rn(
      __dmul_rn(__dmul_rn(0.5 * FOMO_PI, __dmul_rn(FOMO_ELECTRON_RADIUS, FOMO_ELECTRON_RADIUS)), FOMO_IRRADIANCE));
  const float ss = __fmul_rn(sinomega, sinomega);
  const float cs = __fsub_rn(1.0f, ss);
  const float co = __fsqrt_rn(cs);
  const float lt = __double2float_rn(log(__ddiv_rn(__dadd_rn(1.0, (double)sinomega), (double)co)));
  const float a = __fmul_rn(co, ss);
  const double dss = ss, dcs = cs, dso = sinomega, dlt = lt;
  const float b = __double2float_rn(__dmul_rn(
      -1.0 / 8.0, __dsub_rn(__dsub_rn(1.0, __dmul_rn(3.0, dss)),
                            __dmul_rn(__dmul_rn(dcs, __ddiv_rn(__dadd_rn(1.0, __dmul_rn(3.0, dss)), dso)), dlt))));
  const float c = __double2float_rn(__dsub_rn(__dsub_rn(4.0 / 3.0, (double)co), __ddiv_rn((double)__fmul_rn(co, cs), 3.0)));
  const float d = __double2float_rn(__dmul_rn(
      1.0 / 8.0, __dsub_rn(__dadd_rn(5.0, dss), __dmul_rn(__dmul_rn(dcs, __ddiv_rn(__dsub_rn(5.0, dss), dso)), dlt))));
  const double kk = __dmul_rn((double)coeff, 1. / (1. - U / 3.));
  *polterm = __double2float_rn(__dmul_rn(kk, __dadd_rn((double)a, __dmul_rn(U, (double)__fsub_rn(b, a)))));
  *totterm = __double2float_rn(
      __dmul_rn(kk, __dmul_rn(2.0, __dadd_rn((double)c, __dmul_rn(U, (double)__fsub_rn(d, c))))));
}

__global__ void thomson_emission_kernel(const float4* __restrict__ pts, const float* __restrict__ ne_s, int64_t n,
                                        float2* __restrict__ totpol) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 p = pts[i];
    const double px = p.x, py = p.y, pz = p.z;
    const float r = __double2float_rn(
        __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(px, px), __dmul_rn(py, py)), __dmul_rn(pz, pz))));
    float tt, pt;
    thomson_geom(r, &tt, &pt);
    const float nv = ne_s[i];
    totpol[i] = make_float2(__fmul_rn(nv, tt), __fmul_rn(nv, pt));
  }
}

// Largest line width among points that emit (eps != 0): bounds the lambda
// window the march evaluates.  Non-negative floats order like their bits; NaN
// and inf map to +inf (the host then evaluates every bin).
__global__ void payload_stats_kernel(const float2* __restrict__ ew, int64_t n, unsigned int* wmax_bits) {
  unsigned int m = 0u;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = ew[i];
    if (v.x != 0.0f) {
      float w = fabsf(v.y);
      if (!(w <= 3.0e38f)) w = __int_as_float(0x7f800000);
      m = max(m, __float_as_uint(w));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(wmax_bits, m);
}

// Largest speed |v| of a snapshot: bounds the Doppler shift of every LOS.
__global__ void speed_max_kernel(const float4* __restrict__ vel, int64_t n, unsigned int* vmax_bits) {
  unsigned int m = 0u;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 v = vel[i];
    float s = sqrtf(fmaf(v.z, v.z, fmaf(v.y, v.y, v.x * v.x))) * 1.0001f;
    if (!(s <= 3.0e38f)) s = __int_as_float(0x7f800000);
    m = max(m, __float_as_uint(s));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(vmax_bits, m);
}

// Sorted payload back to the caller's point order: out[orig(i)] = ew[i].
__global__ void unsort_kernel(const float4* __restrict__ pts, const float2* __restrict__ ew, int64_t n,
                              float* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = FOMO_IDX(__float_as_int(pts[i].w), n, kSitePts);
    const float2 v = ew[i];
    a[o] = v.x;
    b[o] = v.y;
  }
}

int blocks_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

FOMO_DEFINE_CHECK_READER(check_word_emission)

cudaError_t launch_emission(const float* ne_s, const float* T_s, int64_t n, TableDev t, float2* ew, cudaStream_t s) {
  const int64_t tab = (int64_t)t.nt * t.nrho + t.nt;
  if (tab <= kMaxSmemTableFloats) {
    const size_t bytes = (size_t)tab * sizeof(float);
    if (bytes > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(emission_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)bytes);
      if (e != cudaSuccess) return e;
    }
    emission_kernel<true><<<blocks_for(n, 256), 256, bytes, s>>>(ne_s, T_s, n, t, ew);
  } else {
    emission_kernel<false><<<blocks_for(n, 256), 256, 0, s>>>(ne_s, T_s, n, t, ew);
  }
  return cudaGetLastError();
}

cudaError_t launch_payload_stats(const float2* ew, int64_t n, unsigned int* wmax_bits, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(wmax_bits, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  payload_stats_kernel<<<blocks_for(n, 256), 256, 0, s>>>(ew, n, wmax_bits);
  return cudaGetLastError();
}

cudaError_t launch_speed_max(const float4* vel, int64_t n, unsigned int* vmax_bits, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(vmax_bits, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  speed_max_kernel<<<blocks_for(n, 256), 256, 0, s>>>(vel, n, vmax_bits);
  return cudaGetLastError();
}

cudaError_t launch_unsort_payload(const float4* pts, const float2* ew, int64_t n, float* a, float* b,
                                  cudaStream_t s) {
  unsort_kernel<<<blocks_for(n, 256), 256, 0, s>>>(pts, ew, n, a, b);
  return cudaGetLastError();
}

cudaError_t launch_thomson_emission(const float4* pts, const float* ne_s, int64_t n, float2* totpol,
                                    cudaStream_t s) {
  thomson_emission_kernel<<<blocks_for(n, 256), 256, 0, s>>>(pts, ne_s, n, totpol);
  return cudaGetLastError();
}

}  // namespace fomo
