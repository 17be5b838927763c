// K3: per-view set-up, entirely on the device (no host round trip).
//
//  * view_extents_kernel: Stage A of the reference (fomo-c/src/fomo-nearest-
//    neighbour.cpp:76-108): the points rotated in FP64 with the reference's
//    operand order, min/max reduced through order-preserving 64-bit atomics
//    (exact, order independent).  An FP32 rotation with a proven error bound
//    screens the points first, so only those near a running extreme are
//    rotated in FP64.  For Thomson every point takes the pole-blended rotation
//    with clamped cos/sin and sin^2(chi) (fomo-thomson.cpp:139-199).
//  * view_finalize_kernel: maxdistance (nn:138 / thomson:249-260), delta z,
//    path length and DN pixel area (nn:235-267), and the per-LOS-sample FP64
//    table z_k*sin(b)*cos(l), z_k*sin(b)*sin(l), z_k*cos(b) that the march
//    adds to the per-ray terms -- the same roundings as the reference's
//    derotation expression (nn:162-165).
// Transcendentals (cos, sin, exp of the blends) are evaluated on the host with
// the host libm and passed in; everything here is +, -, *, /, sqrt in IEEE
// FP64 with explicit round-to-nearest intrinsics (no FMA contraction).
#include <cuda_runtime.h>
#include <float.h>
#include <limits.h>
#include <stdint.h>

#include "fomo_device.cuh"
#include "fomo_internal.h"

namespace fomo {

namespace {

__device__ __forceinline__ unsigned long long d2ord(double d) {
  unsigned long long u = (unsigned long long)__double_as_longlong(d);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord2d(unsigned long long u) {
  u = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
  return __longlong_as_double((long long)u);
}

__global__ void view_init_kernel(ViewDesc* views, int nviews) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nviews) return;
  for (int d = 0; d < 3; ++d) {
    views[v].ext_bits[2 * d] = 0xffffffffffffffffull;  // min
    views[v].ext_bits[2 * d + 1] = 0ull;                // max
    views[v].bnd[2 * d] = INT_MIN;                      // largest lower bound (atomicMax)
    views[v].bnd[2 * d + 1] = INT_MAX;                  // smallest upper bound (atomicMin)
  }
}

// float <-> int with the same order (atomicMax / atomicMin on floats)
__device__ __forceinline__ int ford(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float fdeord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

// The interval of view V's rotated coordinates (x', y', z' of nn:83-85) over
// block b's bounding box, widened by M: lo[a] <= the FP64 rotated coordinate
// a of every point of the block <= hi[a].  False for an empty block.  The
// rotation is evaluated in FP32 (centre . row +- |row| . half-size); M covers
// its rounding (M = 2E, E the FP32 screen's error bound below).
__device__ __forceinline__ bool block_interval(const SnapDev& snap, int64_t b, float cbf, float sbf, float clf,
                                               float slf, float M, float (&lo)[3], float (&hi)[3]) {
  const float* bb = snap.blk + FOMO_IDX(6 * b, 6 * (int64_t)snap.bdx * snap.bdy * snap.bdz, kSitePts);
  const float ax = bb[0], ay = bb[1], az = bb[2], bx = bb[3], by = bb[4], bz = bb[5];
  if (!(ax <= bx)) return false;  // empty
  const float cx = 0.5f * (ax + bx), cy = 0.5f * (ay + by), cz = 0.5f * (az + bz);
  const float hx = 0.5f * (bx - ax), hy = 0.5f * (by - ay), hz = 0.5f * (bz - az);
  // rows of the rotation: x' = (cb cl, -cb sl, -sb), y' = (sl, cl, 0), z' = (sb cl, -sb sl, cb)
  const float r[3][3] = {{cbf * clf, -cbf * slf, -sbf}, {slf, clf, 0.0f}, {sbf * clf, -sbf * slf, cbf}};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float m = r[a][0] * cx + r[a][1] * cy + r[a][2] * cz;
    const float e = fabsf(r[a][0]) * hx + fabsf(r[a][1]) * hy + fabsf(r[a][2]) * hz;
    lo[a] = m - e - M;
    hi[a] = m + e + M;
  }
  return true;
}

__device__ __forceinline__ float screen_bound(const GridParams& g) {
  return ldexpf(fmaxf(fabsf(g.minx), fabsf(g.maxx)) + fmaxf(fabsf(g.miny), fabsf(g.maxy)) +
                    fmaxf(fabsf(g.minz), fabsf(g.maxz)),
                -20);
}

// Phase 1 of the block-bounded extents (views other than Thomson), one thread
// per block: every point's rotated coordinate a lies in its block's interval,
// so the maximum over all points is at least the largest lower bound over the
// blocks, and the minimum at most the smallest upper bound.  grid: (blocks, views)
__global__ void view_bounds_kernel(SnapDev snap, ViewDesc* views) {
  ViewDesc* V = views + blockIdx.y;
  const int64_t nblk = (int64_t)snap.bdx * snap.bdy * snap.bdz;
  const float cbf = (float)V->rcb, sbf = (float)V->rsb, clf = (float)V->cl, slf = (float)V->sl;
  const float M = 2.0f * screen_bound(snap.g);
  float lbm[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX}, ubm[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nblk; b += (int64_t)gridDim.x * blockDim.x) {
    float lo[3], hi[3];
    if (!block_interval(snap, b, cbf, sbf, clf, slf, M, lo, hi)) continue;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      lbm[a] = fmaxf(lbm[a], lo[a]);
      ubm[a] = fminf(ubm[a], hi[a]);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lbm[a] = fmaxf(lbm[a], __shfl_xor_sync(0xffffffffu, lbm[a], o));
      ubm[a] = fminf(ubm[a], __shfl_xor_sync(0xffffffffu, ubm[a], o));
    }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      atomicMax(&V->bnd[2 * a], ford(lbm[a]));
      atomicMin(&V->bnd[2 * a + 1], ford(ubm[a]));
    }
  }
}

__device__ __forceinline__ void warp_minmax(unsigned long long& mn, unsigned long long& mx) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long a = __shfl_xor_sync(0xffffffffu, mn, o);
    unsigned long long b = __shfl_xor_sync(0xffffffffu, mx, o);
    mn = a < mn ? a : mn;
    mx = b > mx ? b : mx;
  }
}

// grid: (blocks over points, views)
__global__ void view_extents_kernel(SnapDev snap, ViewDesc* views, float* s2) {
  ViewDesc* V = views + blockIdx.y;
  const double cb = V->rcb, sb = V->rsb, cl = V->cl, sl = V->sl;
  const bool thomson = V->method == kMethodThomson;
  const double blend = V->blend;
  const double omb = __dsub_rn(1.0, blend);
  unsigned long long mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0ull, 0ull, 0ull};
  float* s2v = s2 ? s2 + (int64_t)blockIdx.y * snap.n : nullptr;
  // LOS unit for sin^2 chi (thomson:194): clamped sin_b/cos_b with cos(l), sin(l)
  const double u0 = __dmul_rn(sb, cl), u1 = __dmul_rn(-sb, sl), u2 = cb;
  if (!thomson) {
    // The FP64 extremes are those of the points whose FP32 rotation comes
    // within 2E of this thread's running FP32 extreme: |x32 - x64| <= E for
    // every point, E = 2^-20 (max|x| + max|y| + max|z|) (the FP32 sum of three
    // products of a coordinate and two trigonometric factors errs by less than
    // 8 * 2^-24 of that), so the point of the FP64 extreme always passes.  Only
    // those points are rotated in FP64.
    const GridParams& g = snap.g;
    const float E = ldexpf(fmaxf(fabsf(g.minx), fabsf(g.maxx)) + fmaxf(fabsf(g.miny), fabsf(g.maxy)) +
                               fmaxf(fabsf(g.minz), fabsf(g.maxz)),
                           -20);
    const float E2 = 2.0f * E;
    const float cbf = (float)cb, sbf = (float)sb, clf = (float)cl, slf = (float)sl;
    float rmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < snap.n;
         i += (int64_t)gridDim.x * blockDim.x) {
      const float4 p = snap.pts[i];
      const float x32 = (p.x * cbf) * clf - (p.y * cbf) * slf - p.z * sbf;
      const float y32 = p.x * slf + p.y * clf;
      const float z32 = (p.x * sbf) * clf - (p.y * sbf) * slf + p.z * cbf;
      const bool near = x32 < rmn[0] + E2 || x32 > rmx[0] - E2 || y32 < rmn[1] + E2 || y32 > rmx[1] - E2 ||
                        z32 < rmn[2] + E2 || z32 > rmx[2] - E2;
      rmn[0] = fminf(rmn[0], x32);
      rmx[0] = fmaxf(rmx[0], x32);
      rmn[1] = fminf(rmn[1], y32);
      rmx[1] = fmaxf(rmx[1], y32);
      rmn[2] = fminf(rmn[2], z32);
      rmx[2] = fmaxf(rmx[2], z32);
      if (near) {
        const double gx = p.x, gy = p.y, gz = p.z;
        // full rotation (nn:83-85)
        const double xa =
            __dsub_rn(__dsub_rn(__dmul_rn(__dmul_rn(gx, cb), cl), __dmul_rn(__dmul_rn(gy, cb), sl)),
                      __dmul_rn(gz, sb));
        const double ya = __dadd_rn(__dmul_rn(gx, sl), __dmul_rn(gy, cl));
        const double za =
            __dadd_rn(__dsub_rn(__dmul_rn(__dmul_rn(gx, sb), cl), __dmul_rn(__dmul_rn(gy, sb), sl)),
                      __dmul_rn(gz, cb));
        const unsigned long long ex = d2ord(xa), ey = d2ord(ya), ez = d2ord(za);
        mn[0] = ex < mn[0] ? ex : mn[0];
        mx[0] = ex > mx[0] ? ex : mx[0];
        mn[1] = ey < mn[1] ? ey : mn[1];
        mx[1] = ey > mx[1] ? ey : mx[1];
        mn[2] = ez < mn[2] ? ez : mn[2];
        mx[2] = ez > mx[2] ? ez : mx[2];
      }
    }
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; thomson && i < snap.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float4 p = snap.pts[i];
    const double gx = p.x, gy = p.y, gz = p.z;
    // full rotation (nn:83-85, thomson:179-181)
    double xa = __dsub_rn(__dsub_rn(__dmul_rn(__dmul_rn(gx, cb), cl), __dmul_rn(__dmul_rn(gy, cb), sl)),
                          __dmul_rn(gz, sb));
    double ya = __dadd_rn(__dmul_rn(gx, sl), __dmul_rn(gy, cl));
    double za = __dadd_rn(__dsub_rn(__dmul_rn(__dmul_rn(gx, sb), cl), __dmul_rn(__dmul_rn(gy, sb), sl)),
                          __dmul_rn(gz, cb));
    if (thomson) {
      // pole rotation and blend (thomson:184-191)
      const double pxr = __dsub_rn(__dmul_rn(gx, cl), __dmul_rn(gy, sl));
      const double pyr = __dadd_rn(__dmul_rn(gx, sl), __dmul_rn(gy, cl));
      const double pzr = gz;
      xa = __dadd_rn(__dmul_rn(xa, omb), __dmul_rn(pxr, blend));
      ya = __dadd_rn(__dmul_rn(ya, omb), __dmul_rn(pyr, blend));
      za = __dadd_rn(__dmul_rn(za, omb), __dmul_rn(pzr, blend));
      // sin^2 chi = 1 - (u.r)^2 / (r.r)  (thomson:194-199)
      double ip = __dmul_rn(u0, xa);
      ip = __dadd_rn(ip, __dmul_rn(u1, ya));
      ip = __dadd_rn(ip, __dmul_rn(u2, za));
      double pp = __dmul_rn(xa, xa);
      pp = __dadd_rn(pp, __dmul_rn(ya, ya));
      pp = __dadd_rn(pp, __dmul_rn(za, za));
      s2v[FOMO_IDX(i, snap.n, kSiteS2)] = __double2float_rn(__dsub_rn(1.0, __ddiv_rn(__dmul_rn(ip, ip), pp)));
    }
    const unsigned long long ex = d2ord(xa), ey = d2ord(ya), ez = d2ord(za);
    mn[0] = ex < mn[0] ? ex : mn[0];
    mx[0] = ex > mx[0] ? ex : mx[0];
    mn[1] = ey < mn[1] ? ey : mn[1];
    mx[1] = ey > mx[1] ? ey : mx[1];
    mn[2] = ez < mn[2] ? ez : mn[2];
    mx[2] = ez > mx[2] ? ez : mx[2];
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) warp_minmax(mn[d], mx[d]);
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      atomicMin(&V->ext_bits[2 * d], mn[d]);
      atomicMax(&V->ext_bits[2 * d + 1], mx[d]);
    }
  }
}

// Phase 2, one warp per block: a block whose interval on some axis reaches the
// bound of phase 1 (above the largest lower bound, or below the smallest upper
// bound) may hold the point of that extreme, and only those blocks' points are
// rotated -- with the same FP32 screen and FP64 rotation as
// view_extents_kernel, so the extremes are the same.  grid: (blocks / 4, views)
__global__ void view_extents_blocks_kernel(SnapDev snap, ViewDesc* views) {
  ViewDesc* V = views + blockIdx.y;
  const int lane = threadIdx.x & 31;
  const int64_t b = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int64_t nblk = (int64_t)snap.bdx * snap.bdy * snap.bdz;
  if (b >= nblk) return;  // the whole warp
  const double cb = V->rcb, sb = V->rsb, cl = V->cl, sl = V->sl;
  const float cbf = (float)cb, sbf = (float)sb, clf = (float)cl, slf = (float)sl;
  const GridParams& g = snap.g;
  const float E = screen_bound(g);
  const float E2 = 2.0f * E;
  float lo[3], hi[3];
  if (!block_interval(snap, b, cbf, sbf, clf, slf, 2.0f * E, lo, hi)) return;
  bool reach = false;
#pragma unroll
  for (int a = 0; a < 3; ++a) reach = reach || hi[a] >= fdeord(V->bnd[2 * a]) || lo[a] <= fdeord(V->bnd[2 * a + 1]);
  if (!reach) return;
  const int bx = (int)(b % snap.bdx), by = (int)((b / snap.bdx) % snap.bdy), bz = (int)(b / ((int64_t)snap.bdx * snap.bdy));
  const int x0 = bx * kBlockCells, x1 = min(x0 + kBlockCells, g.dx) - 1;
  const int64_t entries = (int64_t)g.dx * g.dy * g.dz + 1;
  unsigned long long mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0ull, 0ull, 0ull};
  float rmn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rmx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int r = lane; r < kBlockCells * kBlockCells; r += 32) {
    const int cy = by * kBlockCells + r % kBlockCells, cz = bz * kBlockCells + r / kBlockCells;
    if (cy >= g.dy || cz >= g.dz) continue;
    const int64_t rowbase = ((int64_t)cz * g.dy + cy) * g.dx;
    const int p1 = snap.cell_start[FOMO_IDX(rowbase + x1 + 1, entries, kSiteCellStart)];
    for (int i = snap.cell_start[FOMO_IDX(rowbase + x0, entries, kSiteCellStart)]; i < p1; ++i) {
      const float4 p = snap.pts[FOMO_IDX(i, snap.n, kSitePts)];
      const float x32 = (p.x * cbf) * clf - (p.y * cbf) * slf - p.z * sbf;
      const float y32 = p.x * slf + p.y * clf;
      const float z32 = (p.x * sbf) * clf - (p.y * sbf) * slf + p.z * cbf;
      const bool near = x32 < rmn[0] + E2 || x32 > rmx[0] - E2 || y32 < rmn[1] + E2 || y32 > rmx[1] - E2 ||
                        z32 < rmn[2] + E2 || z32 > rmx[2] - E2;
      rmn[0] = fminf(rmn[0], x32);
      rmx[0] = fmaxf(rmx[0], x32);
      rmn[1] = fminf(rmn[1], y32);
      rmx[1] = fmaxf(rmx[1], y32);
      rmn[2] = fminf(rmn[2], z32);
      rmx[2] = fmaxf(rmx[2], z32);
      if (near) {
        const double gx = p.x, gy = p.y, gz = p.z;
        // full rotation (nn:83-85)
        const double xa =
            __dsub_rn(__dsub_rn(__dmul_rn(__dmul_rn(gx, cb), cl), __dmul_rn(__dmul_rn(gy, cb), sl)),
                      __dmul_rn(gz, sb));
        const double ya = __dadd_rn(__dmul_rn(gx, sl), __dmul_rn(gy, cl));
        const double za =
            __dadd_rn(__dsub_rn(__dmul_rn(__dmul_rn(gx, sb), cl), __dmul_rn(__dmul_rn(gy, sb), sl)),
                      __dmul_rn(gz, cb));
        const unsigned long long ex = d2ord(xa), ey = d2ord(ya), ez = d2ord(za);
        mn[0] = ex < mn[0] ? ex : mn[0];
        mx[0] = ex > mx[0] ? ex : mx[0];
        mn[1] = ey < mn[1] ? ey : mn[1];
        mx[1] = ey > mx[1] ? ey : mx[1];
        mn[2] = ez < mn[2] ? ez : mn[2];
        mx[2] = ez > mx[2] ? ez : mx[2];
      }
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) warp_minmax(mn[d], mx[d]);
  if (lane == 0) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      atomicMin(&V->ext_bits[2 * d], mn[d]);
      atomicMax(&V->ext_bits[2 * d + 1], mx[d]);
    }
  }
}

__device__ __forceinline__ double dmax_ref(double a, double b) { return (a < b) ? b : a; }  // std::max

// One block per view.
__global__ void view_finalize_kernel(ViewDesc* views, double3* ktab, int ktab_stride) {
  ViewDesc* V = views + blockIdx.x;
  __shared__ double s_dz, s_minz;
  if (threadIdx.x == 0) {
    const double minx = ord2d(V->ext_bits[0]), maxx = ord2d(V->ext_bits[1]);
    const double miny = ord2d(V->ext_bits[2]), maxy = ord2d(V->ext_bits[3]);
    const double minz = ord2d(V->ext_bits[4]), maxz = ord2d(V->ext_bits[5]);
    V->minx = minx;
    V->maxx = maxx;
    V->miny = miny;
    V->maxy = maxy;
    V->minz = minz;
    V->maxz = maxz;
    const double dxr = __dsub_rn(maxx, minx), dyr = __dsub_rn(maxy, miny);
    V->dxr = dxr;
    V->dyr = dyr;
    const double px = __ddiv_rn(dxr, (double)(V->nx - 1)), py = __ddiv_rn(dyr, (double)(V->ny - 1));
    double md;
    if (V->method == kMethodThomson) {
      const double eq = dmax_ref(__dmul_rn(0.5, __dsqrt_rn(__dadd_rn(__dmul_rn(px, px), __dmul_rn(py, py)))),
                                 __ddiv_rn(__dmul_rn(0.1, dxr), (double)(V->nx - 1)));
      const double away = __ddiv_rn(dmax_ref(px, py), 0.005);
      md = __dadd_rn(__dmul_rn(eq, __dsub_rn(1.0, V->mdblend)), __dmul_rn(away, V->mdblend));
    } else {
      md = __ddiv_rn(dmax_ref(px, py), .3);
    }
    V->md = md;
    double deltaz = __dsub_rn(maxz, minz);
    if (V->nz != 1) deltaz = __ddiv_rn(deltaz, (double)(V->nz - 1));
    V->deltaz = deltaz;
    double pathlength = __ddiv_rn(__dsub_rn(maxz, minz), (double)(V->nz - 1));
    if (maxz == minz || V->nz == 1) pathlength = 1.0;
    V->pathlength = pathlength;
    double apix = 1.0;
    {
      const float dxf = __double2float_rn(px), dyf = __double2float_rn(py);
      const double as = FOMO_PI / 180. / 3600.;
      apix = __dmul_rn(__dmul_rn(__ddiv_rn((double)dxf, FOMO_MM_PER_ARCSEC), __ddiv_rn((double)dyf, FOMO_MM_PER_ARCSEC)),
                       __dmul_rn(as, as));
    }
    V->apix = apix;
    V->scale = __dmul_rn(__dmul_rn(pathlength, 1e8), 1.0);
    V->scale_dn = __dmul_rn(__dmul_rn(pathlength, 1e8), apix);
    V->lwa = __ddiv_rn(__dmul_rn(V->lambda_width, V->lambda0), FOMO_SPEED_OF_LIGHT);
    V->ux = __double2float_rn(__dmul_rn(V->sb, V->cl));
    V->uy = __double2float_rn(__dmul_rn(-V->sb, V->sl));
    V->uz = __double2float_rn(V->cb);
    s_dz = deltaz;
    s_minz = minz;
  }
  __syncthreads();
  const double cb = V->cb, sb = V->sb, cl = V->cl, sl = V->sl;
  const double dz = s_dz, minz = s_minz;
  // ray positions in the image plane (nn:152-153)
  for (int j = threadIdx.x; j < V->nx; j += blockDim.x)
    V->xt[FOMO_IDX(j, V->nx, kSiteRayXY)] = __dadd_rn(__dmul_rn(__ddiv_rn((double)j, (double)(V->nx - 1)), V->dxr), V->minx);
  for (int i = threadIdx.x; i < V->ny; i += blockDim.x)
    V->yt[FOMO_IDX(i, V->ny, kSiteRayXY)] = __dadd_rn(__dmul_rn(__ddiv_rn((double)i, (double)(V->ny - 1)), V->dyr), V->miny);
  double3* kt = ktab + (int64_t)blockIdx.x * ktab_stride;
  for (int k = threadIdx.x; k < V->nz; k += blockDim.x) {
    const double z = __dadd_rn(__dmul_rn((double)k, dz), minz);  // nn:162
    const double zsb = __dmul_rn(z, sb);
    kt[FOMO_IDX(k, ktab_stride, kSiteKtab)] = make_double3(__dmul_rn(zsb, cl), __dmul_rn(zsb, sl), __dmul_rn(z, cb));
  }
}

}  // namespace

FOMO_DEFINE_CHECK_READER(check_word_view)

cudaError_t launch_view_init(ViewDesc* views, int nviews, cudaStream_t s) {
  view_init_kernel<<<(nviews + 127) / 128, 128, 0, s>>>(views, nviews);
  return cudaGetLastError();
}

cudaError_t launch_view_extents(SnapDev snap, ViewDesc* views, int nviews, float* s2, cudaStream_t s) {
  if (!s2 && snap.blk) {
    // bounded by the per-block boxes: the blocks' intervals, then the points
    // of the blocks that reach the bounds
    const int64_t nblk = (int64_t)snap.bdx * snap.bdy * snap.bdz;
    int64_t b1 = (nblk + 255) / 256;
    if (b1 > 64) b1 = 64;
    view_bounds_kernel<<<dim3((unsigned)b1, (unsigned)nviews), 256, 0, s>>>(snap, views);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    view_extents_blocks_kernel<<<dim3((unsigned)((nblk + 3) / 4), (unsigned)nviews), 128, 0, s>>>(snap, views);
    return cudaGetLastError();
  }
  int64_t blocks = (snap.n + 255) / 256;
  int64_t cap = (152 * 8 + nviews - 1) / nviews;
  if (cap < 8) cap = 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  dim3 grid((unsigned)blocks, (unsigned)nviews);
  view_extents_kernel<<<grid, 256, 0, s>>>(snap, views, s2);
  return cudaGetLastError();
}

cudaError_t launch_view_finalize(ViewDesc* views, int nviews, double3* ktab, int ktab_stride, cudaStream_t s) {
  view_finalize_kernel<<<nviews, 256, 0, s>>>(views, ktab, ktab_stride);
  return cudaGetLastError();
}

}  // namespace fomo
