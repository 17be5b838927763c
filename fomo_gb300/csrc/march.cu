// K4/K5/K6: the fused ray march (fomo-c/src/fomo-nearestneighbour.cpp:145-229
// and fomo-thomson.cpp:268-343), one warp per ray, persistent over a queue of
// (view, ray) work items so that many views and requests share one launch.
//
// Per ray: the FP64 per-ray terms of the derotation (x cos b cos l + y sin l,
// -x cos b sin l + y cos l, -x sin b) are formed once; lane k of each 32-sample
// chunk adds the per-sample FP64 table entry of its LOS sample, rounds the
// target and the box corners p -+ maxdistance to FP32 exactly as the reference
// does (nn:171,179), and finds the nearest point strictly inside the box.
//
// Neighbour search: rings of grid cells around the target's cell, clipped to
// the box's cell range, x-rows scanned as contiguous point ranges, stopped by
// a conservative ring / row / cell distance bound.  Distances are compared in
// FP32 with the two best kept; when they are within 4e-6 relative (a possible
// tie under the reference's FP64 distance), the candidates are re-ranked with
// the exact FP64 distance in Boost's order (dz^2 + (dy^2 + dx^2)) and the
// lowest original index -- so the chosen neighbour equals the FP64 argmin.
//
// Spectroscopic mode: equal neighbours of consecutive samples are merged into
// runs (warp ballot), and each run adds count * eps * 2^(-(2 (lambda - shift)/w)^2)
// (= eps exp(-4 ln2 (dlambda/w)^2), nn:204) to the lane-owned lambda bins of
// every line with FP32 Kahan sums.  Imaging (L = 1) and Thomson (pB) modes add
// the per-sample value through a warp reduction.  One warp owns one ray: no
// atomics on the output, results are deterministic and independent of what
// else shares the launch.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "fomo_device.cuh"
#include "fomo_internal.h"

namespace fomo {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kThreads = 256;
constexpr float kRelTie = 4e-6f;    // FP32 distance ambiguity band (>> FP32 + FP64 error)
constexpr float kRelPrune = 1e-5f;  // pruning slack on the squared distance
constexpr float kCellMargin = 0.02f;  // cell-boundary slack in cells (binning error < 1e-3 cell)

struct Best {
  float d1, d2;  // two smallest FP32 squared distances
  int pos;       // sorted position of d1
  int orig;      // original index of d1
};

struct BoxQ {
  float tx, ty, tz, lox, loy, loz, hix, hiy, hiz;
};

__device__ __forceinline__ float axis_gap(int c, float t, float o, float h) {
  const float lo = fmaf((float)c - kCellMargin, h, o);
  const float hi = fmaf((float)c + 1.0f + kCellMargin, h, o);
  return fmaxf(fmaxf(lo - t, t - hi), 0.0f);
}

__device__ __forceinline__ double exact_dist2(float px, float py, float pz, const BoxQ& q) {
  const double dx = __dsub_rn((double)px, (double)q.tx);
  const double dy = __dsub_rn((double)py, (double)q.ty);
  const double dz = __dsub_rn((double)pz, (double)q.tz);
  return __dadd_rn(__dmul_rn(dz, dz), __dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dx, dx)));
}

// Scan points [b, e).  EXACT = false: FP32 two-best.  EXACT = true: FP64
// re-rank of the candidates whose FP32 distance is within the tie band.
template <bool EXACT>
__device__ __forceinline__ void scan_range(const float4* __restrict__ pts, int b, int e, const BoxQ& q, Best& B,
                                           float band, double& bestD, int& bestOrig, int& bestPos) {
  for (int p = b; p < e; ++p) {
    const float4 v = __ldg(pts + p);
    if (v.x > q.lox && v.x < q.hix && v.y > q.loy && v.y < q.hiy && v.z > q.loz && v.z < q.hiz) {
      const float dx = v.x - q.tx, dy = v.y - q.ty, dz = v.z - q.tz;
      const float d = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      if (!EXACT) {
        if (d < B.d1) {
          B.d2 = B.d1;
          B.d1 = d;
          B.pos = p;
          B.orig = __float_as_int(v.w);
        } else if (d < B.d2) {
          B.d2 = d;
        }
      } else if (d <= band) {
        const double D = exact_dist2(v.x, v.y, v.z, q);
        const int o = __float_as_int(v.w);
        if (D < bestD || (D == bestD && o < bestOrig)) {
          bestD = D;
          bestOrig = o;
          bestPos = p;
        }
      }
    }
  }
}

// One pass of the ring search.  In the exact pass `bound` is fixed (the first
// pass's best), in the first pass it shrinks as B.d1 improves.
struct CellRange {
  int b0[3], b1[3], c[3];
};

template <bool EXACT>
__device__ __forceinline__ void ring_pass(const SnapDev& S, const BoxQ& q, const CellRange& R, Best& B, float band,
                                          double& bestD, int& bestOrig, int& bestPos) {
  const int* b0 = R.b0;
  const int* b1 = R.b1;
  const int* c = R.c;
  const GridParams& g = S.g;
  const float h = g.h;
  for (int s = 0;; ++s) {
    const float bound = EXACT ? band * (1.0f + kRelPrune) : B.d1 * (1.0f + kRelPrune);
    if (s >= 2) {
      const float lb = ((float)s - 1.0f - 2.0f * kCellMargin) * h;
      if (lb * lb > bound) break;
    }
    if (c[0] - s < b0[0] && c[0] + s > b1[0] && c[1] - s < b0[1] && c[1] + s > b1[1] && c[2] - s < b0[2] &&
        c[2] + s > b1[2])
      break;
    const int z0 = max(c[2] - s, b0[2]), z1 = min(c[2] + s, b1[2]);
    const int y0 = max(c[1] - s, b0[1]), y1 = min(c[1] + s, b1[1]);
    for (int kz = z0; kz <= z1; ++kz) {
      const bool onz = (kz == c[2] - s) || (kz == c[2] + s);
      const float gz = axis_gap(kz, q.tz, g.oz, h);
      const float gz2 = gz * gz;
      if (gz2 > (EXACT ? band * (1.0f + kRelPrune) : B.d1 * (1.0f + kRelPrune))) continue;
      for (int jy = y0; jy <= y1; ++jy) {
        const bool ony = (jy == c[1] - s) || (jy == c[1] + s);
        const float gy = axis_gap(jy, q.ty, g.oy, h);
        const float gyz = fmaf(gy, gy, gz2);
        const float bnd = EXACT ? band * (1.0f + kRelPrune) : B.d1 * (1.0f + kRelPrune);
        if (gyz > bnd) continue;
        const int rowbase = (kz * g.dy + jy) * g.dx;
        if (onz || ony) {
          int x0 = max(c[0] - s, b0[0]), x1 = min(c[0] + s, b1[0]);
          if (bnd < FLT_MAX) {
            // clip the row to cells within sqrt(bnd - gyz) of the target in x
            const float rem = fmaxf(bnd - gyz, 0.0f);
            const float r = (rem > 0.0f ? rem * rsqrtf(rem) * 1.0001f : 0.0f) + kCellMargin * h;
            x0 = max(x0, cell_coord(q.tx - r, g.ox, g.inv_h, g.dx));
            x1 = min(x1, cell_coord(q.tx + r, g.ox, g.inv_h, g.dx));
          }
          if (x0 <= x1) {
            const int pb = __ldg(S.cell_start + rowbase + x0), pe = __ldg(S.cell_start + rowbase + x1 + 1);
            scan_range<EXACT>(S.pts, pb, pe, q, B, band, bestD, bestOrig, bestPos);
          }
        } else {
          const int xl = c[0] - s, xr = c[0] + s;
          if (xl >= b0[0]) {
            const float gx = axis_gap(xl, q.tx, g.ox, h);
            if (fmaf(gx, gx, gyz) <= bnd) {
              const int pb = __ldg(S.cell_start + rowbase + xl), pe = __ldg(S.cell_start + rowbase + xl + 1);
              scan_range<EXACT>(S.pts, pb, pe, q, B, band, bestD, bestOrig, bestPos);
            }
          }
          if (xr <= b1[0]) {
            const float gx = axis_gap(xr, q.tx, g.ox, h);
            const float bnd2 = EXACT ? band * (1.0f + kRelPrune) : B.d1 * (1.0f + kRelPrune);
            if (fmaf(gx, gx, gyz) <= bnd2) {
              const int pb = __ldg(S.cell_start + rowbase + xr), pe = __ldg(S.cell_start + rowbase + xr + 1);
              scan_range<EXACT>(S.pts, pb, pe, q, B, band, bestD, bestOrig, bestPos);
            }
          }
        }
      }
    }
  }
}

// The exact FP64 re-rank runs for a handful of samples per million; keeping it
// out of line keeps the common path free of its register pressure.
__device__ __noinline__ int exact_rerank(const SnapDev& S, const BoxQ& q, const CellRange& R, float d1, int* orig) {
  Best B{d1, d1, -1, -1};
  const float band = d1 * (1.0f + kRelTie);
  double bestD = DBL_MAX;
  int bestOrig = 0x7fffffff, bestPos = -1;
  ring_pass<true>(S, q, R, B, band, bestD, bestOrig, bestPos);
  *orig = bestOrig;
  return bestPos;
}

// Nearest point strictly inside the box; returns the sorted position (-1 if
// none) and the original index in *orig.
__device__ __forceinline__ int nn_search(const SnapDev& S, const BoxQ& q, int* orig) {
  const GridParams& g = S.g;
  *orig = -1;
  if (!(q.lox < g.maxx && q.hix > g.minx && q.loy < g.maxy && q.hiy > g.miny && q.loz < g.maxz &&
        q.hiz > g.minz && q.lox < q.hix && q.loy < q.hiy && q.loz < q.hiz))
    return -1;
  CellRange R;
  R.b0[0] = cell_coord(q.lox, g.ox, g.inv_h, g.dx);
  R.b1[0] = cell_coord(q.hix, g.ox, g.inv_h, g.dx);
  R.b0[1] = cell_coord(q.loy, g.oy, g.inv_h, g.dy);
  R.b1[1] = cell_coord(q.hiy, g.oy, g.inv_h, g.dy);
  R.b0[2] = cell_coord(q.loz, g.oz, g.inv_h, g.dz);
  R.b1[2] = cell_coord(q.hiz, g.oz, g.inv_h, g.dz);
  R.c[0] = cell_coord(q.tx, g.ox, g.inv_h, g.dx);
  R.c[1] = cell_coord(q.ty, g.oy, g.inv_h, g.dy);
  R.c[2] = cell_coord(q.tz, g.oz, g.inv_h, g.dz);
  Best B{FLT_MAX, FLT_MAX, -1, -1};
  double bestD = 0.0;
  int bestOrig = -1, bestPos = -1;
  ring_pass<false>(S, q, R, B, 0.0f, bestD, bestOrig, bestPos);
  if (B.pos >= 0 && B.d2 <= B.d1 * (1.0f + kRelTie)) {
    // possible tie under the FP64 distance: exact re-rank of the contenders
    return exact_rerank(S, q, R, B.d1, orig);
  }
  *orig = B.orig;
  return B.pos;
}

struct RayCtx {
  int v, i, j;
  double A0, A1, A2, md;
  const double3* kt;
};

__device__ __forceinline__ int find_view(const int64_t* off, int nviews, int64_t item) {
  int lo = 0, hi = nviews - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(off + mid) <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Next ray for this warp; false when the queue is drained.
__device__ __forceinline__ bool next_ray(const MarchArgs& a, const double3* ktab, int ktab_stride, RayCtx& r) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long item = 0;
    if (lane == 0) item = atomicAdd(a.counter, 1ull);
    item = __shfl_sync(kFull, item, 0);
    if ((int64_t)item >= a.total_items) return false;
    const int v = find_view(a.ray_offset, a.nviews, (int64_t)item);
    const ViewDesc* V = a.views + v;
    const int nx = V->nx, ny = V->ny, tw = V->ray_tile_w, th = V->ray_tile_h;
    const int local = (int)((int64_t)item - __ldg(a.ray_offset + v));  // < nx*ny < 2^31
    const int tiles_x = (nx + tw - 1) / tw;
    const int tile = local / (tw * th);
    const int within = local - tile * (tw * th);
    const int i = (tile / tiles_x) * th + within / tw;
    const int j = (tile % tiles_x) * tw + within % tw;
    if (i >= ny || j >= nx) continue;
    // ray position in the image plane (nn:152-153, tabulated per view by the
    // finalize kernel) and the per-ray terms of the derotation (nn:165)
    const double x = V->xt[j];
    const double y = V->yt[i];
    const double cb = V->cb, sb = V->sb, cl = V->cl, sl = V->sl;
    r.v = v;
    r.i = i;
    r.j = j;
    r.A0 = __dadd_rn(__dmul_rn(__dmul_rn(x, cb), cl), __dmul_rn(y, sl));
    r.A1 = __dadd_rn(__dmul_rn(__dmul_rn(-x, cb), sl), __dmul_rn(y, cl));
    r.A2 = __dmul_rn(-x, sb);
    r.md = V->md;
    r.kt = ktab + (int64_t)v * ktab_stride;
    return true;
  }
}

// LOS sample k of the ray: exact FP32 target and box (nn:162-179), then NN.
__device__ __forceinline__ int sample_nn(const SnapDev& S, const RayCtx& r, int k, int* orig) {
  const double3 zt = r.kt[k];
  const double p0 = __dadd_rn(r.A0, zt.x);
  const double p1 = __dsub_rn(r.A1, zt.y);
  const double p2 = __dadd_rn(r.A2, zt.z);
  BoxQ q;
  q.tx = __double2float_rn(p0);
  q.ty = __double2float_rn(p1);
  q.tz = __double2float_rn(p2);
  q.lox = __double2float_rn(__dsub_rn(p0, r.md));
  q.loy = __double2float_rn(__dsub_rn(p1, r.md));
  q.loz = __double2float_rn(__dsub_rn(p2, r.md));
  q.hix = __double2float_rn(__dadd_rn(p0, r.md));
  q.hiy = __double2float_rn(__dadd_rn(p1, r.md));
  q.hiz = __double2float_rn(__dadd_rn(p2, r.md));
  return nn_search(S, q, orig);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Spectroscopic march: NL lines x NB bins per lane (bin = m*32 + lane).
// ---------------------------------------------------------------------------
template <int NL, int NB>
__global__ void __launch_bounds__(kThreads) march_spectral(MarchArgs a, const double3* __restrict__ ktab,
                                                           int ktab_stride) {
  const int lane = threadIdx.x & 31;
  RayCtx r;
  while (next_ray(a, ktab, ktab_stride, r)) {
    const ViewDesc* V = a.views + r.v;
    const int nz = V->nz, L = V->L, nx = V->nx;
    const float ux = V->ux, uy = V->uy, uz = V->uz;
    const LineDesc* LD = a.lines + (int64_t)r.v * a.nlines;
    float acc[NL][NB], comp[NL][NB], lam[NL][NB], shk[NL];
    const float2* ew[NL];
    bool lon[NL];
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      const bool on = l < a.nlines && LD[l].ew != nullptr;  // views may have fewer lines than the launch
      lon[l] = on;
      ew[l] = on ? LD[l].ew : nullptr;
      shk[l] = on ? LD[l].shift_k : 0.0f;
#pragma unroll
      for (int m = 0; m < NB; ++m) {
        const int il = m * 32 + lane;
        acc[l][m] = 0.0f;
        comp[l][m] = 0.0f;
        // lambdaval (nn:200), evaluated in FP64 on the host, stored FP32
        lam[l][m] = (on && il < L) ? __ldg(LD[l].lam + il) : 3.0e30f;
      }
    }
    int32_t* nnout = a.nn_idx ? a.nn_idx[r.v] : nullptr;
    const int64_t ray = (int64_t)r.i * nx + r.j;
    for (int k0 = 0; k0 < nz; k0 += 32) {
      const int k = k0 + lane;
      const bool active = k < nz;
      int orig = -1;
      const int pos = active ? sample_nn(a.snap, r, k, &orig) : -1;
      if (nnout && active) nnout[ray * nz + k] = orig;
      const int prev = __shfl_up_sync(kFull, pos, 1);
      const bool start = active && (lane == 0 || pos != prev);
      unsigned starts = __ballot_sync(kFull, start);
      const unsigned act = __ballot_sync(kFull, active);
      const int endlane = 32 - __clz(act);
      while (starts) {
        const int s = __ffs(starts) - 1;
        starts &= starts - 1;
        const int e = starts ? (__ffs(starts) - 1) : endlane;
        const int id = __shfl_sync(kFull, pos, s);
        if (id < 0) continue;
        const float cnt = (float)(e - s);
        const float4 vv = __ldg(a.snap.vel + id);
        const float vlos = fmaf(uz, vv.z, fmaf(uy, vv.y, ux * vv.x));
#pragma unroll
        for (int l = 0; l < NL; ++l) {
          if (lon[l]) {
            const float2 pw = __ldg(ew[l] + id);
            if (pw.x != 0.0f) {
              const float pk = pw.x * cnt;
              const float sc = __fdividef(2.0f, pw.y);  // exp(-4 ln2 (d/w)^2) = 2^(-(2d/w)^2)
              const float sh = vlos * shk[l];
#pragma unroll
              for (int m = 0; m < NB; ++m) {
                const float q = (lam[l][m] - sh) * sc;
                kahan_add(acc[l][m], comp[l][m], pk * ex2_approx(-q * q));
              }
            }
          }
        }
      }
    }
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      if (lon[l]) {
        const double scale = LD[l].is_dn ? V->scale_dn : V->scale;
        float* out = LD[l].out + ray * L;
#pragma unroll
        for (int m = 0; m < NB; ++m) {
          const int il = m * 32 + lane;
          if (il < L) out[il] = __double2float_rn(__dmul_rn(scale, (double)acc[l][m]));
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Imaging (L == 1, broadband channels) and Thomson pB: per-sample values,
// reduced across the warp per 32-sample chunk, Kahan-accumulated per ray.
// ---------------------------------------------------------------------------
template <int NL, bool THOMSON>
__global__ void __launch_bounds__(kThreads) march_imaging(MarchArgs a, const double3* __restrict__ ktab,
                                                          int ktab_stride) {
  const int lane = threadIdx.x & 31;
  RayCtx r;
  while (next_ray(a, ktab, ktab_stride, r)) {
    const ViewDesc* V = a.views + r.v;
    const int nz = V->nz, nx = V->nx;
    const LineDesc* LD = a.lines + (int64_t)r.v * a.nlines;
    float acc[NL], comp[NL];
    bool lon[NL];
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      acc[l] = 0.0f;
      comp[l] = 0.0f;
      lon[l] = l < a.nlines && LD[l].out != nullptr;  // views may have fewer lines than the launch
    }
    const float* s2v = THOMSON ? a.s2 + (int64_t)r.v * a.snap.n : nullptr;
    int32_t* nnout = a.nn_idx ? a.nn_idx[r.v] : nullptr;
    const int64_t ray = (int64_t)r.i * nx + r.j;
    for (int k0 = 0; k0 < nz; k0 += 32) {
      const int k = k0 + lane;
      const bool active = k < nz;
      int orig = -1;
      const int pos = active ? sample_nn(a.snap, r, k, &orig) : -1;
      if (nnout && active) nnout[ray * nz + k] = orig;
#pragma unroll
      for (int l = 0; l < NL; ++l) {
        if (lon[l]) {
          float val = 0.0f;
          if (pos >= 0) {
            if (THOMSON) {
              // pB = pol * sin^2 chi, clamped at 0 (thomson:325-338)
              val = fmaxf(__ldg(a.totpol + pos).y * __ldg(s2v + pos), 0.0f);
            } else {
              val = __ldg(LD[l].ew + pos).x;  // imaging adds the peak (nn:217-225)
            }
          }
          const float cs = warp_sum(val);
          if (lane == 0) kahan_add(acc[l], comp[l], cs);
        }
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int l = 0; l < NL; ++l)
        if (lon[l])
          LD[l].out[ray] = __double2float_rn(__dmul_rn(LD[l].is_dn ? V->scale_dn : V->scale, (double)acc[l]));
    }
  }
}

template <typename K>
cudaError_t launch_persistent(K kernel, const MarchArgs& a, const double3* ktab, int ktab_stride, int sm_count,
                              cudaStream_t s, int blocks_per_sm_hint) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  if (blocks_per_sm_hint > 0 && blocks_per_sm_hint < per_sm) per_sm = blocks_per_sm_hint;
  int64_t warps_needed = a.total_items;
  int64_t blocks = (int64_t)sm_count * per_sm;
  const int64_t cap = (warps_needed + (kThreads / 32) - 1) / (kThreads / 32);
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  kernel<<<(unsigned)blocks, kThreads, 0, s>>>(a, ktab, ktab_stride);
  return cudaGetLastError();
}

}  // namespace

int march_bins_per_lane(int nlines, int L) {
  (void)nlines;
  return (L + 31) / 32;
}

cudaError_t launch_march(const MarchArgs& a, const double3* ktab, int ktab_stride, int max_L, int sm_count,
                         cudaStream_t s, int blocks_per_sm_hint) {
  const bool thomson = a.s2 != nullptr;
  if (thomson) return launch_persistent(march_imaging<1, true>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint);
  if (max_L <= 1) {
    if (a.nlines <= 1) return launch_persistent(march_imaging<1, false>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint);
    if (a.nlines <= 2) return launch_persistent(march_imaging<2, false>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint);
    if (a.nlines <= 4) return launch_persistent(march_imaging<4, false>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint);
    if (a.nlines <= 8) return launch_persistent(march_imaging<8, false>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint);
    return cudaErrorInvalidValue;
  }
  const int nb = (max_L + 31) / 32;
#define FOMO_SPEC(NL_, NB_) \
  if (a.nlines <= NL_ && nb <= NB_) return launch_persistent(march_spectral<NL_, NB_>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint)
  FOMO_SPEC(1, 1);
  FOMO_SPEC(1, 2);
  FOMO_SPEC(1, 4);
  FOMO_SPEC(1, 8);
  FOMO_SPEC(2, 2);
  FOMO_SPEC(2, 4);
  FOMO_SPEC(4, 1);
  FOMO_SPEC(4, 2);
  FOMO_SPEC(4, 4);
#undef FOMO_SPEC
  return cudaErrorInvalidValue;
}

}  // namespace fomo
