// Projection render (fomo-c/src/fomo-projection.cpp:17-193): every data point
// adds its emission to the image pixel nearest its projection -- no line of
// sight is marched.  Per view: j = round((x' - minx)(nx - 1) / (maxx - minx)),
// i = round((y' - miny)(ny - 1) / (maxy - miny)) with x', y' the point rotated
// in FP64 exactly as for the extents (nn:83-85, the same operand order, so the
// pixel of every point is the reference's); a spectroscopic point adds
// eps * 2^(-(2 (lambda - shift) / w)^2) (= eps exp(-4 ln2 (dl / w)^2), :134)
// to the lambda bins of its pixel, an imaging point adds eps.  The view's
// path-length (and DN pixel-area) scale of :161-191 is applied to each
// contribution.  Contributions of points that share a pixel are summed with
// FP32 atomics, so the order of the sum -- like the reference's `omp atomic`
// -- is not fixed.
//
// Work layout: a warp takes 32 consecutive (grid-sorted) points; each lane
// projects one point (FP64) and loads its LOS speed; then for spectroscopy the
// warp walks the 32 points, lane = lambda bin of the line's window, so that
// the 32 atomics of one point hit 32 consecutive floats.  blockIdx.y = view.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fomo_device.cuh"
#include "fomo_internal.h"

namespace fomo {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kProjThreads = 256;

__global__ void __launch_bounds__(kProjThreads) projection_kernel(SnapDev snap, const ViewDesc* __restrict__ views,
                                                                  const LineDesc* __restrict__ lines, int nlines,
                                                                  int imaging) {
  const ViewDesc* V = views + blockIdx.y;
  const LineDesc* LD = lines + (int64_t)blockIdx.y * nlines;
  const double cb = V->rcb, sb = V->rsb, cl = V->cl, sl = V->sl;
  const double minx = V->minx, miny = V->miny;
  const double dxr = __dsub_rn(V->maxx, minx), dyr = __dsub_rn(V->maxy, miny);
  const int nx = V->nx, ny = V->ny, L = V->L;
  const double sx = (double)(nx - 1), sy = (double)(ny - 1);
  const float ux = V->ux, uy = V->uy, uz = V->uz;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (kProjThreads / 32);
  for (int64_t base = ((int64_t)blockIdx.x * (kProjThreads / 32) + (threadIdx.x >> 5)) * 32; base < snap.n;
       base += warps * 32) {
    const int64_t p = base + lane;
    int pix = -1;
    float vlos = 0.0f;
    if (p < snap.n) {
      const float4 q = __ldg(snap.pts + p);
      const double gx = q.x, gy = q.y, gz = q.z;
      const double xa = __dsub_rn(__dsub_rn(__dmul_rn(__dmul_rn(gx, cb), cl), __dmul_rn(__dmul_rn(gy, cb), sl)),
                                  __dmul_rn(gz, sb));
      const double ya = __dadd_rn(__dmul_rn(gx, sl), __dmul_rn(gy, cl));
      // std::round: halves away from zero (:124, :126)
      int j = (int)round(__ddiv_rn(__dmul_rn(__dsub_rn(xa, minx), sx), dxr));
      int i = (int)round(__ddiv_rn(__dmul_rn(__dsub_rn(ya, miny), sy), dyr));
      // x', y' lie within the extents, so i, j are in range; a degenerate
      // extent (max == min) gives NaN in the reference: such points are dropped
      if (j >= 0 && j < nx && i >= 0 && i < ny) pix = i * nx + j;
      if (!imaging) {
        const float4 vv = __ldg(snap.vel + p);
        vlos = fmaf(uz, vv.z, fmaf(uy, vv.y, ux * vv.x));
      }
    }
    if (imaging) {
      for (int l = 0; l < nlines; ++l) {
        const LineDesc& D = LD[l];
        if (!D.ew || pix < 0) continue;
        const float e = __ldg(D.ew + p).x;
        if (e != 0.0f)
          atomicAdd(D.out + FOMO_IDX(pix, (int64_t)nx * ny, kSiteProjection), (float)(D.is_dn ? V->scale_dn : V->scale) * e);
      }
      continue;
    }
    for (int s = 0; s < 32; ++s) {
      const int ps = __shfl_sync(kFull, pix, s);
      const float vs = __shfl_sync(kFull, vlos, s);
      if (ps < 0) continue;  // the same for every lane
      for (int l = 0; l < nlines; ++l) {
        const LineDesc& D = LD[l];
        if (!D.ew) continue;  // views may have fewer lines than the launch
        const float2 pw = __ldg(D.ew + base + s);
        if (pw.x == 0.0f) continue;
        const float sc = __fdividef(2.0f, pw.y);
        const float ns = -(vs * D.shift_k) * sc;
        const float scale = (float)(D.is_dn ? V->scale_dn : V->scale);
        float* out = D.out + FOMO_IDX((int64_t)ps * L, (int64_t)nx * ny * L, kSiteProjection);
        for (int m = 0; m < D.nw; ++m) {
          const int il = D.wstart + 32 * m + lane;
          if (il < L) {
            const float qq = fmaf(__ldg(D.lam + FOMO_IDX(il, L, kSiteLam)), sc, ns);
            const float v = pw.x * ex2_approx(-qq * qq);
            if (v != 0.0f) atomicAdd(out + il, v * scale);
          }
        }
      }
    }
  }
}

}  // namespace

FOMO_DEFINE_CHECK_READER(check_word_projection)

cudaError_t launch_projection(SnapDev snap, const ViewDesc* views, const LineDesc* lines, int nviews, int nlines,
                              bool imaging, int sm_count, cudaStream_t s) {
  if (nviews <= 0 || snap.n <= 0) return cudaSuccess;
  if (nviews > 65535) return cudaErrorInvalidValue;
  const int64_t warps_needed = (snap.n + 31) / 32;
  int64_t blocks = ((warps_needed + kProjThreads / 32 - 1) / (kProjThreads / 32));
  const int64_t cap = (int64_t)sm_count * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  projection_kernel<<<dim3((unsigned)blocks, (unsigned)nviews), kProjThreads, 0, s>>>(snap, views, lines, nlines,
                                                                                     imaging ? 1 : 0);
  return cudaGetLastError();
}

}  // namespace fomo
