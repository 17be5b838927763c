// K4/K5/K6: the ray march (fomo-c/src/fomo-nearestneighbour.cpp:145-229 and
// fomo-thomson.cpp:268-343), one warp per ray, persistent over a queue of
// (view, ray) work items so that many views and requests share one launch.
//
// Kernels, in stream order: march_search (stores each sample's neighbour in a
// position buffer), march_split (segments whose capsule overflowed),
// march_far (deferred samples far off the points, searched together),
// march_deferred (the other samples the search could not resolve, one lane
// each), march_hard (deferred samples over
// a lane's budget, one warp each) -- the last four store the neighbours they
// find in the same buffer -- and then the
// emission pass, march_spectral<.., shade> or march_imaging<.., shade>, which
// bins every ray from the buffer.  The no-allocation path has no buffer: its
// first pass (march_spectral / march_imaging, fused) searches and bins, and
// the split, deferred and hard passes add their samples' emission with
// atomics.
//
// Per ray: the FP64 per-ray terms of the derotation (x cos b cos l + y sin l,
// -x cos b sin l + y cos l, -x sin b) are formed once; each LOS sample adds the
// FP64 table entry of its index (z_k sin b cos l, ...) and rounds the target to
// FP32 exactly as the reference does (nn:162-171).
//
// Neighbour search, per 64-sample segment of a ray (warp-cooperative; lane i
// owns samples i and i+32 of the segment):
//  1. gather: the segment's targets lie on one line.  Every x-row of grid
//     cells that can hold a point within R of the segment gets the x-range of
//     cells the segment passes near; the rows' point ranges are prefix-summed
//     across the warp and loaded 32 points per round (balanced), and points
//     within R are compacted into a per-warp shared-memory list with the index
//     of the sample they project onto.  R = min(sqrt(3) * maxdistance, the
//     local point spacing), the spacing estimated from the occupancy of the
//     cells the segment crosses;
//  2. bucket sort: the list is counting-sorted by that sample index;
//  3. scan: each sample tests the candidates of the buckets within R of it:
//     FP32 squared distance, and the Chebyshev distance against maxdistance
//     for the strict box of nn:179 (a candidate within a few ulp of a box face
//     makes the sample "ambiguous");
//  4. accept: a winner is final when it lies within the sample's coverage
//     radius (points farther than R from the segment cannot be nearer) and no
//     candidate was ambiguous; "no neighbour" is final when the box lies outside
//     the points' bounding box or inside the covered ball.  Near-ties (two best
//     FP32 distances within 4e-6) are re-ranked with the exact FP64 distance in
//     Boost's order (dz^2 + (dy^2 + dx^2)) and the lowest original index;
//  5. defer: every other sample (about 1 %) contributes nothing here; its
//     segment is recorded.  A segment whose capsule held more than kSegCap
//     points is first searched again in parts of 32 or 16 samples
//     (march_split); march_deferred then searches each such sample on one
//     lane -- rings of grid cells around the sample's cell, clipped to its box
//     (corners rounded from FP64 as the reference does), nearest ring first,
//     stopped by a distance bound -- or hands it to march_hard, where a whole
//     warp walks the same rings; either adds the sample's emission.
// Either way the chosen neighbour is the FP64 argmin strictly inside the box.
//
// Spectroscopic mode: equal neighbours of consecutive samples are merged into
// runs (warp ballot); the lane starting a run loads its payload and forms, per
// line, count * eps, 2 / w and the Doppler term; every lane then adds
// count * eps * 2^(-(2 (lambda - shift) / w)^2)  (= eps exp(-4 ln2 (dl/w)^2),
// nn:204) to its lambda bins of the line's window (the bins where any point's
// Gaussian can exceed 2^-64 of its peak; the others are written as 0) in a
// per-chunk FP32 partial, folded into the per-ray sum with Kahan compensation.
// Imaging (L = 1) and Thomson (pB) add per-sample values through a warp
// reduction.  One warp owns one ray in the emission pass, which sums its
// samples in order (no atomics), so a cube does not depend on what else
// shares the launch.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "fomo_device.cuh"
#include "fomo_internal.h"

namespace fomo {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kMinCtas = 4;  // resident CTAs per SM: 16 warps of latency hiding at <= 128 registers
constexpr int kMinCtasSearch = 7;   // the search-only pass: 28 warps at <= 72 registers (31 KB shared per CTA)
constexpr int kMinCtasShade = 8;   // the emission-only pass: 32 warps at <= 64 registers
constexpr int kMinCtasImaging = 5; // imaging / Thomson first pass: 20 warps at <= 102 registers
constexpr int kMinCtasDeferred = 8; // one-lane ring walks wait on dependent loads: 32 warps (64 registers, some spill)
constexpr int kMinCtasSplit = 6;    // overflow parts: 24 warps at <= 85 registers (33 KB shared per CTA allows 6)
constexpr float kRelTie = 4e-6f;      // FP32 distance ambiguity band (>> FP32 + FP64 error)
constexpr float kRelPrune = 1e-5f;    // pruning slack on the squared distance
constexpr float kCellMargin = 0.02f;  // cell-boundary slack in cells (binning error < 1e-3 cell)
constexpr int kSeg = 64;              // LOS samples per segment (two per lane)
constexpr int kSegCap = 176;          // candidates per segment (sized so that 7 search CTAs fit an SM)
constexpr int kMaxRows = 4096;        // cell rows of a segment's capsule beyond which it is deferred
constexpr float kRScaleDefault = 0.9f;  // gather radius in local point spacings (MarchArgs::rscale when set)
// Far pass (march_far): samples half a cell or more off the points' bounding box,
// kFarMin or more of them in a half record, searched together by a warp.
constexpr int kFarMin = 4;          // far samples a half needs (fewer: the lane walks of march_deferred)
constexpr float kFarOut2 = 0.25f;   // squared distance, in cells, off the points' bounding box of a far sample
constexpr float kFarBox = 4.0f;     // box half-width, in cells, of the views the far pass takes (narrower: lane walks)
constexpr int kFarIters = 4;        // gathers per half
constexpr int kFarMaxPts = 1024;    // points of a gather beyond which the half is left to march_deferred
// A deferred record is (work item, first sample of its 64-sample segment with
// two flags above it, samples 0-31 of the segment as a bit mask, samples 32-63).
constexpr unsigned kRecS0 = (1u << 30) - 1u;  // the first sample
constexpr unsigned kRecFar0 = 1u << 30;       // samples 0-31 hold kFarMin far samples or more
constexpr unsigned kRecFar1 = 1u << 31;       // samples 32-63 do


struct __align__(16) SegSmem {
  // [0, kSegCap): gathered candidates; [kSegCap, 2 kSegCap): the same sorted by
  // the sample they project onto
  float4 q[2 * kSegCap];
  int pos[2 * kSegCap];
  int bstart[kSeg + 1];
  int cursor[kSeg];
  unsigned char cb[kSegCap];
};

struct BoxQ {
  float tx, ty, tz, lox, loy, loz, hix, hiy, hiz;
};

// Entries of the grid's cell_start array (its cells + 1).
__device__ __forceinline__ int64_t cell_entries(const GridParams& g) { return (int64_t)g.dx * g.dy * g.dz + 1; }

__device__ __forceinline__ float axis_gap(int c, float t, float o, float h) {
  const float lo = fmaf((float)c - kCellMargin, h, o);
  const float hi = fmaf((float)c + 1.0f + kCellMargin, h, o);
  return fmaxf(fmaxf(lo - t, t - hi), 0.0f);
}

__device__ __forceinline__ double exact_dist2(float px, float py, float pz, float tx, float ty, float tz) {
  const double dx = __dsub_rn((double)px, (double)tx);
  const double dy = __dsub_rn((double)py, (double)ty);
  const double dz = __dsub_rn((double)pz, (double)tz);
  return __dadd_rn(__dmul_rn(dz, dz), __dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dx, dx)));
}

// Row rr of a box of rows nyr wide: (rr / nyr, rr % nyr) for 0 <= rr < 2^20 and
// 1 <= nyr < 2^20.  The FP32 estimate of the quotient (inv = the FP32
// reciprocal of nyr) is off by at most one here, and one correction step makes
// it exact (an integer division by a variable costs several times as many
// instructions).
__device__ __forceinline__ int row_div(int rr, int nyr, float inv, int& rem) {
  int q = __float2int_rz((float)rr * inv);
  int r = rr - q * nyr;
  if (r < 0) {
    --q;
    r += nyr;
  } else if (r >= nyr) {
    ++q;
    r -= nyr;
  }
  rem = r;
  return q;
}

// The local point spacing, in cells, at a mean cell occupancy of mocc points:
// mocc^(-1/3), from the SFU's log2 and exp2 (a heuristic for the gather radius;
// a few ulp do not matter).
__device__ __forceinline__ float spacing_cells(float mocc) { return ex2_approx(__log2f(mocc) * (-1.0f / 3.0f)); }

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(kFull, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Lane owning flattened item i: the number of lanes whose inclusive prefix is <= i.
__device__ __forceinline__ int warp_owner(int incl, int i) {
  int own = 0;
#pragma unroll
  for (int step = 16; step >= 1; step >>= 1) {
    const int v = __shfl_sync(kFull, incl, own + step - 1);
    if (v <= i) own += step;
  }
  return own;
}

// ---------------------------------------------------------------------------
// Rays and segments
// ---------------------------------------------------------------------------

struct RayCtx {
  int v, i, j;
  unsigned int item;  // work item of the ray (recorded with its deferred samples)
  double A0, A1, A2, md;
  float mdf;
  int nz;             // LOS samples of the ray's view (the length of its LOS table)
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

// The ray of work item `item` (views' rays in tile order); false for the
// padding items of partial tiles.
__device__ __forceinline__ bool ray_of_item(const MarchArgs& a, const double3* ktab, int ktab_stride,
                                            int64_t item, RayCtx& r) {
  const int v = find_view(a.ray_offset, a.nviews, item);
  const ViewDesc* V = a.views + v;
  const int nx = V->nx, ny = V->ny, tw = V->ray_tile_w, th = V->ray_tile_h;
  const int local = (int)(item - __ldg(a.ray_offset + v));  // < nx*ny < 2^31
  const int tiles_x = (nx + tw - 1) / tw;
  const int tile = local / (tw * th);
  const int within = local - tile * (tw * th);
  const int i = (tile / tiles_x) * th + within / tw;
  const int j = (tile % tiles_x) * tw + within % tw;
  if (i >= ny || j >= nx) return false;
  // ray position in the image plane (nn:152-153, tabulated per view by the
  // finalize kernel) and the per-ray terms of the derotation (nn:165)
  const double x = V->xt[FOMO_IDX(j, nx, kSiteRayXY)];
  const double y = V->yt[FOMO_IDX(i, ny, kSiteRayXY)];
  const double cb = V->cb, sb = V->sb, cl = V->cl, sl = V->sl;
  r.v = v;
  r.i = i;
  r.j = j;
  r.item = (unsigned int)item;
  r.A0 = __dadd_rn(__dmul_rn(__dmul_rn(x, cb), cl), __dmul_rn(y, sl));
  r.A1 = __dadd_rn(__dmul_rn(__dmul_rn(-x, cb), sl), __dmul_rn(y, cl));
  r.A2 = __dmul_rn(-x, sb);
  r.md = V->md;
  r.mdf = __double2float_rn(V->md);
  r.kt = ktab + (int64_t)v * ktab_stride;
  r.nz = V->nz;
  return true;
}

// Warp-collective: the next ray of the work queue (items item_base ..
// total_items - 1, head counter `ctr`), false when the queue is drained.
__device__ __forceinline__ bool next_ray(const MarchArgs& a, const double3* ktab, int ktab_stride, RayCtx& r,
                                         int ctr = kCtrRays) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long item = 0;
    if (lane == 0) {
      item = atomicAdd(a.counter + ctr, 1ull);
      // a stopped batch (every request of it cancelled): the queue counts as
      // drained.  The word only goes from 0 to 1 while a batch runs, so a
      // kernel that starts after one that stopped stops at its first ray too
      // (an emission pass reads no position its search did not write).
      if (a.stop && __ldcv(a.stop) != 0u) item = (unsigned long long)a.total_items;
    }
    item = __shfl_sync(kFull, item, 0) + (unsigned long long)a.item_base;
    if ((int64_t)item >= a.total_items) return false;
    if (ray_of_item(a, ktab, ktab_stride, (int64_t)item, r)) return true;
  }
}

// LOS sample k: derotated position (nn:162-165) in FP64.
__device__ __forceinline__ void sample_pos(const RayCtx& r, int k, double& p0, double& p1, double& p2) {
  const double3 zt = r.kt[FOMO_IDX(k, r.nz, kSiteKtab)];
  p0 = __dadd_rn(r.A0, zt.x);
  p1 = __dsub_rn(r.A1, zt.y);
  p2 = __dadd_rn(r.A2, zt.z);
}

// The reference's FP32 target and box corners of sample k (nn:171-179).
__device__ __forceinline__ BoxQ exact_box(const RayCtx& r, int k) {
  double p0, p1, p2;
  sample_pos(r, k, p0, p1, p2);
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
  return q;
}

// Exact re-rank of a near-tie: among candidates [c0, c1) of the sorted list
// that lie inside the box (Chebyshev distance below md_in) with FP32 distance
// within `band`, the smallest FP64 distance, then the lowest original index.
// Rare (a few samples per million), so kept out of line.
__device__ __noinline__ int exact_rerank_list(const float4* sq, int c0, int c1, float tx, float ty, float tz,
                                              float md_in, float band) {
  double bestD = DBL_MAX;
  int bestOrig = 0x7fffffff, bi = -1;
  for (int c = c0; c < c1; ++c) {
    const float4 q = sq[c];
    const float dx = q.x - tx, dy = q.y - ty, dz = q.z - tz;
    const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    const float cheb = fmaxf(fmaxf(fabsf(dx), fabsf(dy)), fabsf(dz));
    if (cheb < md_in && d2 <= band) {
      const double D = exact_dist2(q.x, q.y, q.z, tx, ty, tz);
      const int o = __float_as_int(q.w);
      if (D < bestD || (D == bestD && o < bestOrig)) {
        bestD = D;
        bestOrig = o;
        bi = c;
      }
    }
  }
  return bi;
}

// s-interval of the segment a + s d, s in [slo, shi], whose coordinate lies in [lo, hi].
__device__ __forceinline__ void clip_interval(float a, float d, float inv_d, float lo, float hi, float& slo,
                                              float& shi) {
  if (fabsf(d) > 1e-30f) {
    const float t1 = (lo - a) * inv_d, t2 = (hi - a) * inv_d;
    slo = fmaxf(slo, fminf(t1, t2) - 1e-4f);
    shi = fminf(shi, fmaxf(t1, t2) + 1e-4f);
  } else if (a < lo || a > hi) {
    slo = 1.0f;
    shi = 0.0f;
  }
}

// The gather radius of a segment: rscale local point spacings, capped where
// no box needs more -- at sqrt(3) times maxdistance widened by the box
// corners' rounding margin (the largest any sample of the segment takes, its
// coordinates at most amax), plus a few ulp of the coordinates.  With that
// margin in the cap, a box smaller than the spacing lies inside the gathered
// ball whole and an empty one is accepted by the search instead of deferred.
__device__ __forceinline__ float gather_radius(const MarchArgs& a, const RayCtx& r, float aloc, float amax) {
  const float md_seg = r.mdf + (amax + r.mdf) * 4.8e-7f + r.mdf * 1.2e-7f;
  const float cap = fmaf(md_seg * 1.7321f, 1.0001f, amax * 4.8e-7f) * 1.0001f;
  return fminf(cap, (a.rscale > 0.0f ? a.rscale : kRScaleDefault) * aloc);
}

struct PartIn {
  float tx[2], ty[2], tz[2];
  bool act[2];
};
struct PartOut {
  int pos[2], orig[2];
  bool need[2];
};

// The samples of a segment whose capsule held too many points, searched as
// parts of `size` samples (32, then 16): each part gathers its own capsule
// (used by march_split, off the first pass).
__device__ __forceinline__ PartOut segment_parts(const MarchArgs& a, const RayCtx& r, int s0, int nz, SegSmem& sm,
                                              const PartIn in, int size) {
  const SnapDev& S = a.snap;
  unsigned long long* const stats = a.stats;
  int st_rows = 0, st_loaded = 0, st_scanned = 0, st_ties = 0, st_samples = 0;
  const int lane = threadIdx.x & 31;
  const GridParams& g = S.g;
  const float tx[2] = {in.tx[0], in.tx[1]}, ty[2] = {in.ty[0], in.ty[1]}, tz[2] = {in.tz[0], in.tz[1]};
  const bool act[2] = {in.act[0], in.act[1]};
  const int nseg = min(s0 + kSeg, nz) - s0;
  int pos[2] = {-1, -1}, orig[2] = {-1, -1};
  bool need0 = false, need1 = false;
  for (int cur = 0; cur < nseg;) {
    const int pn = min(size, nseg - cur);  // this part: samples s0 + cur .. s0 + cur + pn - 1
    // the part's segment through its first and last targets
    const int la = cur & 31, lb = (cur + pn - 1) & 31;
    const bool ha = cur >= 32, hb = cur + pn - 1 >= 32;
    float t0, t1;
    t0 = __shfl_sync(kFull, tx[0], la); t1 = __shfl_sync(kFull, tx[1], la); const float ax = ha ? t1 : t0;
    t0 = __shfl_sync(kFull, ty[0], la); t1 = __shfl_sync(kFull, ty[1], la); const float ay = ha ? t1 : t0;
    t0 = __shfl_sync(kFull, tz[0], la); t1 = __shfl_sync(kFull, tz[1], la); const float az = ha ? t1 : t0;
    t0 = __shfl_sync(kFull, tx[0], lb); t1 = __shfl_sync(kFull, tx[1], lb); const float bx = hb ? t1 : t0;
    t0 = __shfl_sync(kFull, ty[0], lb); t1 = __shfl_sync(kFull, ty[1], lb); const float by = hb ? t1 : t0;
    t0 = __shfl_sync(kFull, tz[0], lb); t1 = __shfl_sync(kFull, tz[1], lb); const float bz = hb ? t1 : t0;
    const float sdx = bx - ax, sdy = by - ay, sdz = bz - az;
    const float len2 = fmaf(sdz, sdz, fmaf(sdy, sdy, sdx * sdx));
    const float inv_len2 = len2 > 0.0f ? 1.0f / len2 : 0.0f;
    const float len = sqrtf(len2);
    // local point spacing from the occupancy of the cells the part crosses
    int occ = 0;
    {
      const float fs = (float)lane * (1.0f / 31.0f);
      const float px = fmaf(fs, sdx, ax), py = fmaf(fs, sdy, ay), pz = fmaf(fs, sdz, az);
      if (px >= g.minx && px <= g.maxx && py >= g.miny && py <= g.maxy && pz >= g.minz && pz <= g.maxz) {
        const int c = (cell_coord(pz, g.oz, g.inv_h, g.dz) * g.dy + cell_coord(py, g.oy, g.inv_h, g.dy)) * g.dx +
                      cell_coord(px, g.ox, g.inv_h, g.dx);
        occ = __ldg(S.cell_start + FOMO_IDX(c + 1, cell_entries(g), kSiteCellStart)) -
              __ldg(S.cell_start + FOMO_IDX(c, cell_entries(g), kSiteCellStart));
      }
    }
    const float mocc = fmaxf((float)__reduce_add_sync(kFull, (unsigned)occ) * (1.0f / 32.0f), 0.125f);
    const float aloc = g.h * spacing_cells(mocc);
    const float amax =
        fmaxf(fmaxf(fmaxf(fabsf(ax), fabsf(bx)), fmaxf(fabsf(ay), fabsf(by))), fmaxf(fabsf(az), fabsf(bz)));
    const float R = gather_radius(a, r, aloc, amax);
    const float Rg = R * 1.0001f + amax * 2.4e-7f;  // + a few ulp of the coordinates
    const float Rg2 = Rg * Rg * (1.0f + kRelPrune);
    // ---- 1. gather
    bool gathered = true;
    int count = 0;
    const float cxl = fmaxf(fminf(ax, bx) - Rg, g.minx), cxh = fminf(fmaxf(ax, bx) + Rg, g.maxx);
    const float cyl = fmaxf(fminf(ay, by) - Rg, g.miny), cyh = fminf(fmaxf(ay, by) + Rg, g.maxy);
    const float czl = fmaxf(fminf(az, bz) - Rg, g.minz), czh = fminf(fmaxf(az, bz) + Rg, g.maxz);
    if (cxl <= cxh && cyl <= cyh && czl <= czh) {
      const int x0 = cell_coord(cxl, g.ox, g.inv_h, g.dx), x1 = cell_coord(cxh, g.ox, g.inv_h, g.dx);
      const int y0 = cell_coord(cyl, g.oy, g.inv_h, g.dy), y1 = cell_coord(cyh, g.oy, g.inv_h, g.dy);
      const int z0 = cell_coord(czl, g.oz, g.inv_h, g.dz), z1 = cell_coord(czh, g.oz, g.inv_h, g.dz);
      const int nyr = y1 - y0 + 1, nzr = z1 - z0 + 1;
      const int nrows = nyr * nzr;
      st_rows += nrows;
      if (nrows > kMaxRows) {
        gathered = false;
      } else {
        const float m = kCellMargin * g.h;
        const float xm = Rg + m + 2e-4f * len;
        const float inv_dy = fabsf(sdy) > 1e-30f ? 1.0f / sdy : 0.0f;
        const float inv_dz = fabsf(sdz) > 1e-30f ? 1.0f / sdz : 0.0f;
        const unsigned lt = (1u << lane) - 1u;
        const float inv_nyr = 1.0f / (float)nyr;
        for (int rb = 0; rb < nrows && count <= kSegCap; rb += 32) {
          const int rr = rb + lane;
          int n = 0, base = 0;
          if (rr < nrows) {
            int ry;
            const int rz = row_div(rr, nyr, inv_nyr, ry);
            const int jy = y0 + ry, kz = z0 + rz;
            float slo = 0.0f, shi = 1.0f;
            clip_interval(ay, sdy, inv_dy, fmaf((float)jy, g.h, g.oy) - m - Rg,
                          fmaf((float)(jy + 1), g.h, g.oy) + m + Rg, slo, shi);
            clip_interval(az, sdz, inv_dz, fmaf((float)kz, g.h, g.oz) - m - Rg,
                          fmaf((float)(kz + 1), g.h, g.oz) + m + Rg, slo, shi);
            slo = fmaxf(slo, 0.0f);
            shi = fminf(shi, 1.0f);
            if (slo <= shi) {
              const float xa = fmaf(slo, sdx, ax), xb = fmaf(shi, sdx, ax);
              const int c0 = max(x0, cell_coord(fminf(xa, xb) - xm, g.ox, g.inv_h, g.dx));
              const int c1 = min(x1, cell_coord(fmaxf(xa, xb) + xm, g.ox, g.inv_h, g.dx));
              if (c0 <= c1) {
                const int rowbase = (kz * g.dy + jy) * g.dx;
                base = __ldg(S.cell_start + FOMO_IDX(rowbase + c0, cell_entries(g), kSiteCellStart));
                n = __ldg(S.cell_start + FOMO_IDX(rowbase + c1 + 1, cell_entries(g), kSiteCellStart)) - base;
              }
            }
          }
          // rows' point ranges, prefix-summed across the warp and loaded 32 at a time
          const int incl = warp_incl_scan(n);
          const int excl = incl - n;
          const int total = __shfl_sync(kFull, incl, 31);
          st_loaded += total;
          for (int ib = 0; ib < total; ib += 32) {
            const int i = ib + lane;
            const int own = warp_owner(incl, i);
            const int ob = __shfl_sync(kFull, base, own);
            const int oe = __shfl_sync(kFull, excl, own);
            bool keep = false;
            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
            int p = 0, bk = 0;
            if (i < total) {
              p = ob + (i - oe);
              q = __ldg(S.pts + FOMO_IDX(p, S.n, kSitePts));
              const float wx = q.x - ax, wy = q.y - ay, wz = q.z - az;
              float s = fmaf(wz, sdz, fmaf(wy, sdy, wx * sdx)) * inv_len2;
              s = fminf(fmaxf(s, 0.0f), 1.0f);
              const float ex = fmaf(-s, sdx, wx), ey = fmaf(-s, sdy, wy), ez = fmaf(-s, sdz, wz);
              keep = fmaf(ez, ez, fmaf(ey, ey, ex * ex)) <= Rg2;
              bk = min(max(__float2int_rn(s * (float)(pn - 1)), 0), pn - 1);
            }
            const unsigned msk = __ballot_sync(kFull, keep);
            if (keep) {
              const int slot = count + __popc(msk & lt);
              if (slot < kSegCap) {
                sm.q[slot] = q;
                sm.pos[slot] = p;
                sm.cb[slot] = (unsigned char)bk;
              }
            }
            count += __popc(msk);
          }
        }
        if (count > kSegCap) gathered = false;
      }
    }
    if (stats && lane == 0) atomicAdd(stats + kStatCandidates, (unsigned long long)count);
    if (!gathered && pn > 16) {
      // too many points for one part: the same samples again as two halves
      if (stats && lane == 0) atomicAdd(stats + kStatNotGathered, 1ull);
      size = pn >> 1;
      continue;
    }
    const int ncand = gathered ? count : 0;
    // ---- 2. counting sort by sample index
    sm.cursor[lane] = 0;
    sm.cursor[lane + 32] = 0;
    __syncwarp();
    for (int c = lane; c < ncand; c += 32) atomicAdd(&sm.cursor[FOMO_IDX(sm.cb[c], kSeg, kSiteSmem)], 1);
    __syncwarp();
    {
      const int h0 = sm.cursor[2 * lane], h1 = sm.cursor[2 * lane + 1];
      const int incl = warp_incl_scan(h0 + h1);
      const int ex = incl - h0 - h1;
      __syncwarp();
      sm.bstart[2 * lane] = ex;
      sm.bstart[2 * lane + 1] = ex + h0;
      if (lane == 31) sm.bstart[kSeg] = incl;
      sm.cursor[2 * lane] = ex;
      sm.cursor[2 * lane + 1] = ex + h0;
    }
    __syncwarp();
    for (int c = lane; c < ncand; c += 32) {
      const int dst = kSegCap + FOMO_IDX(atomicAdd(&sm.cursor[FOMO_IDX(sm.cb[c], kSeg, kSiteSmem)], 1), kSegCap, kSiteSmem);
      sm.q[dst] = sm.q[c];
      sm.pos[dst] = sm.pos[c];
    }
    __syncwarp();
    const float4* sq = sm.q + kSegCap;  // the candidates in sample order
    const int* spos = sm.pos + kSegCap;
    // ---- 3./4. per-sample scan of the buckets within R, acceptance
    const float dlt = (pn > 1) ? len / (float)(pn - 1) : 0.0f;
    const int w = (dlt > 0.0f) ? min((int)(Rg / dlt + 0.51f) + 1, kSeg) : kSeg;
#pragma unroll 1
    for (int i = 0; i < 2; ++i) {
      // one copy of the scan code for both samples of the lane (instruction cache)
      const int j = lane + 32 * i - cur;  // bucket of this lane's sample in the part
      const bool acti = (i ? act[1] : act[0]) && j >= 0 && j < pn;
      if (!acti) continue;
      int pres = -1, ores = -1;
      bool accept = false;
      if (gathered) {
        const int c0 = sm.bstart[max(j - w, 0)], c1 = sm.bstart[min(j + w, pn - 1) + 1];
        st_scanned += c1 - c0;
        const float t_x = i ? tx[1] : tx[0], t_y = i ? ty[1] : ty[0], t_z = i ? tz[1] : tz[0];
        const float tmax = fmaxf(fmaxf(fabsf(t_x), fabsf(t_y)), fabsf(t_z));
        const float delta = (tmax + r.mdf) * 4.8e-7f + r.mdf * 1.2e-7f;  // ~4 ulp of the box corners
        const float md_in = r.mdf - delta, md_out = r.mdf + delta;
        float b1 = FLT_MAX, b2 = FLT_MAX;
        int bi = -1;
        bool amb = false;
        for (int c = c0; c < c1; ++c) {
          const float4 q = sq[c];
          const float dx = q.x - t_x, dy = q.y - t_y, dz = q.z - t_z;
          const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
          const float cheb = fmaxf(fmaxf(fabsf(dx), fabsf(dy)), fabsf(dz));
          if (cheb < md_in) {
            if (d2 < b1) {
              b2 = b1;
              b1 = d2;
              bi = c;
            } else if (d2 < b2) {
              b2 = d2;
            }
          } else if (cheb <= md_out) {
            amb = true;
          }
        }
        // coverage: every point within cov of the target was gathered
        const float wx = t_x - ax, wy = t_y - ay, wz = t_z - az;
        float s = fmaf(wz, sdz, fmaf(wy, sdy, wx * sdx)) * inv_len2;
        s = fminf(fmaxf(s, 0.0f), 1.0f);
        const float ex = fmaf(-s, sdx, wx), ey = fmaf(-s, sdy, wy), ez = fmaf(-s, sdz, wz);
        const float cov = Rg - sqrtf(fmaf(ez, ez, fmaf(ey, ey, ex * ex))) - amax * 2.4e-7f;
        if (!amb && cov > 0.0f) {
          if (bi >= 0)
            accept = b1 < cov * cov * (1.0f - 2.0f * kRelPrune);
          else
            accept = md_out * 1.7321f * 1.0001f < cov;  // the whole box lies inside the gathered ball
        }
        if (!accept && bi < 0 && !amb) {
          // no candidate: the box is empty for sure when it lies outside the
          // points' bounding box (hi <= min or lo >= max on some axis)
          accept = (t_x + md_out <= g.minx) || (t_x - md_out >= g.maxx) || (t_y + md_out <= g.miny) ||
                   (t_y - md_out >= g.maxy) || (t_z + md_out <= g.minz) || (t_z - md_out >= g.maxz);
        }
        if (accept && bi >= 0) {
          if (b2 <= b1 * (1.0f + kRelTie)) {
            // possible FP64 tie: exact re-rank of the in-box contenders
            ++st_ties;
            bi = exact_rerank_list(sq, c0, c1, t_x, t_y, t_z, md_in, b1 * (1.0f + kRelTie));
          }
          pres = spos[FOMO_IDX(bi, kSegCap, kSiteSmem)];
          ores = __float_as_int(sq[FOMO_IDX(bi, kSegCap, kSiteSmem)].w);
        }
        if (stats && !accept)  // rare: counted where it happens
          atomicAdd(stats + (amb ? kStatFbAmb : (bi < 0 ? kStatFbNoCand : kStatFbFar)), 1ull);
      }
      ++st_samples;
      if (i) {
        pos[1] = pres;
        orig[1] = ores;
        need1 = !accept;
      } else {
        pos[0] = pres;
        orig[0] = ores;
        need0 = !accept;
      }
    }
    __syncwarp();  // the candidate lists are rewritten by the next part
    cur += pn;
  }
  if (stats) {
    const unsigned sc = __reduce_add_sync(kFull, (unsigned)st_scanned);
    const unsigned ti = __reduce_add_sync(kFull, (unsigned)st_ties);
    if (lane == 0) {
      atomicAdd(stats + kStatRows, (unsigned long long)st_rows);
      atomicAdd(stats + kStatPointsLoaded, (unsigned long long)st_loaded);
      atomicAdd(stats + kStatScanned, (unsigned long long)sc);
      atomicAdd(stats + kStatTies, (unsigned long long)ti);
    }
  }
  (void)st_samples;
  PartOut o;
  o.pos[0] = pos[0];
  o.pos[1] = pos[1];
  o.orig[0] = orig[0];
  o.orig[1] = orig[1];
  o.need[0] = need0;
  o.need[1] = need1;
  return o;
}

// Warp-collective: nearest neighbours of the segment's samples s0 .. s0+63.
// pos[i]/orig[i] are this lane's results for sample s0 + lane + 32 i.
// Samples it cannot resolve get no neighbour here (-1) and are recorded in
// the deferred queue.
__device__ __forceinline__ void segment_search(const MarchArgs& a, const RayCtx& r, int s0, int nz, SegSmem& sm,
                                               int (&pos)[2], int (&orig)[2]) {
  const SnapDev& S = a.snap;
  unsigned long long* const stats = a.stats;
  int st_rows = 0, st_loaded = 0, st_scanned = 0, st_ties = 0, st_samples = 0;
  const int lane = threadIdx.x & 31;
  const GridParams& g = S.g;
  float tx[2], ty[2], tz[2];
  bool act[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int k = s0 + lane + 32 * i;
    act[i] = k < nz;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0;
    if (act[i]) sample_pos(r, k, p0, p1, p2);
    tx[i] = __double2float_rn(p0);  // the FP32 target (nn:171)
    ty[i] = __double2float_rn(p1);
    tz[i] = __double2float_rn(p2);
  }
  // the segment through the first and last targets
  const int last = min(s0 + kSeg, nz) - 1;
  const int nseg = last - s0 + 1;
  const int li = last - s0, ll = li & 31;
  const float ax = __shfl_sync(kFull, tx[0], 0), ay = __shfl_sync(kFull, ty[0], 0), az = __shfl_sync(kFull, tz[0], 0);
  const float bx0 = __shfl_sync(kFull, tx[0], ll), by0 = __shfl_sync(kFull, ty[0], ll),
              bz0 = __shfl_sync(kFull, tz[0], ll);
  const float bx1 = __shfl_sync(kFull, tx[1], ll), by1 = __shfl_sync(kFull, ty[1], ll),
              bz1 = __shfl_sync(kFull, tz[1], ll);
  const float bx = li >= 32 ? bx1 : bx0, by = li >= 32 ? by1 : by0, bz = li >= 32 ? bz1 : bz0;
  const float sdx = bx - ax, sdy = by - ay, sdz = bz - az;
  const float len2 = fmaf(sdz, sdz, fmaf(sdy, sdy, sdx * sdx));
  const float inv_len2 = len2 > 0.0f ? 1.0f / len2 : 0.0f;
  const float len = sqrtf(len2);
  // local point spacing from the occupancy of the cells the segment crosses
  int occ = 0;
  {
    const float fs = (float)lane * (1.0f / 31.0f);
    const float px = fmaf(fs, sdx, ax), py = fmaf(fs, sdy, ay), pz = fmaf(fs, sdz, az);
    if (px >= g.minx && px <= g.maxx && py >= g.miny && py <= g.maxy && pz >= g.minz && pz <= g.maxz) {
      const int c = (cell_coord(pz, g.oz, g.inv_h, g.dz) * g.dy + cell_coord(py, g.oy, g.inv_h, g.dy)) * g.dx +
                    cell_coord(px, g.ox, g.inv_h, g.dx);
      occ = __ldg(S.cell_start + FOMO_IDX(c + 1, cell_entries(g), kSiteCellStart)) -
            __ldg(S.cell_start + FOMO_IDX(c, cell_entries(g), kSiteCellStart));
    }
  }
  const float mocc = fmaxf((float)__reduce_add_sync(kFull, (unsigned)occ) * (1.0f / 32.0f), 0.125f);
  const float aloc = g.h * spacing_cells(mocc);
  const float amax =
      fmaxf(fmaxf(fmaxf(fabsf(ax), fabsf(bx)), fmaxf(fabsf(ay), fabsf(by))), fmaxf(fabsf(az), fabsf(bz)));
  const float R = gather_radius(a, r, aloc, amax);
  const float Rg = R * 1.0001f + amax * 2.4e-7f;  // + a few ulp of the coordinates
  const float Rg2 = Rg * Rg * (1.0f + kRelPrune);
  // ---- 1. gather
  bool gathered = true;
  int count = 0;
  const float cxl = fmaxf(fminf(ax, bx) - Rg, g.minx), cxh = fminf(fmaxf(ax, bx) + Rg, g.maxx);
  const float cyl = fmaxf(fminf(ay, by) - Rg, g.miny), cyh = fminf(fmaxf(ay, by) + Rg, g.maxy);
  const float czl = fmaxf(fminf(az, bz) - Rg, g.minz), czh = fminf(fmaxf(az, bz) + Rg, g.maxz);
  if (cxl <= cxh && cyl <= cyh && czl <= czh) {
    const int x0 = cell_coord(cxl, g.ox, g.inv_h, g.dx), x1 = cell_coord(cxh, g.ox, g.inv_h, g.dx);
    const int y0 = cell_coord(cyl, g.oy, g.inv_h, g.dy), y1 = cell_coord(cyh, g.oy, g.inv_h, g.dy);
    const int z0 = cell_coord(czl, g.oz, g.inv_h, g.dz), z1 = cell_coord(czh, g.oz, g.inv_h, g.dz);
    const int nyr = y1 - y0 + 1, nzr = z1 - z0 + 1;
    const int nrows = nyr * nzr;
    st_rows = nrows;
    if (nrows > kMaxRows) {
      gathered = false;
    } else {
      const float m = kCellMargin * g.h;
      const float xm = Rg + m + 2e-4f * len;
      const float inv_dy = fabsf(sdy) > 1e-30f ? 1.0f / sdy : 0.0f;
      const float inv_dz = fabsf(sdz) > 1e-30f ? 1.0f / sdz : 0.0f;
      const unsigned lt = (1u << lane) - 1u;
      const float inv_nyr = 1.0f / (float)nyr;
      for (int rb = 0; rb < nrows && count <= kSegCap; rb += 32) {
        const int rr = rb + lane;
        int n = 0, base = 0;
        if (rr < nrows) {
          int ry;
          const int rz = row_div(rr, nyr, inv_nyr, ry);
          const int jy = y0 + ry, kz = z0 + rz;
          float slo = 0.0f, shi = 1.0f;
          clip_interval(ay, sdy, inv_dy, fmaf((float)jy, g.h, g.oy) - m - Rg, fmaf((float)(jy + 1), g.h, g.oy) + m + Rg,
                        slo, shi);
          clip_interval(az, sdz, inv_dz, fmaf((float)kz, g.h, g.oz) - m - Rg, fmaf((float)(kz + 1), g.h, g.oz) + m + Rg,
                        slo, shi);
          slo = fmaxf(slo, 0.0f);
          shi = fminf(shi, 1.0f);
          if (slo <= shi) {
            const float xa = fmaf(slo, sdx, ax), xb = fmaf(shi, sdx, ax);
            const int c0 = max(x0, cell_coord(fminf(xa, xb) - xm, g.ox, g.inv_h, g.dx));
            const int c1 = min(x1, cell_coord(fmaxf(xa, xb) + xm, g.ox, g.inv_h, g.dx));
            if (c0 <= c1) {
              const int rowbase = (kz * g.dy + jy) * g.dx;
              base = __ldg(S.cell_start + FOMO_IDX(rowbase + c0, cell_entries(g), kSiteCellStart));
              n = __ldg(S.cell_start + FOMO_IDX(rowbase + c1 + 1, cell_entries(g), kSiteCellStart)) - base;
            }
          }
        }
        // rows' point ranges, prefix-summed across the warp and loaded 32 at a time
        const int incl = warp_incl_scan(n);
        const int excl = incl - n;
        const int total = __shfl_sync(kFull, incl, 31);
        st_loaded += total;
        for (int ib = 0; ib < total; ib += 32) {
          const int i = ib + lane;
          const int own = warp_owner(incl, i);
          const int ob = __shfl_sync(kFull, base, own);
          const int oe = __shfl_sync(kFull, excl, own);
          bool keep = false;
          float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
          int p = 0, bk = 0;
          if (i < total) {
            p = ob + (i - oe);
            q = __ldg(S.pts + FOMO_IDX(p, S.n, kSitePts));
            const float wx = q.x - ax, wy = q.y - ay, wz = q.z - az;
            float s = fmaf(wz, sdz, fmaf(wy, sdy, wx * sdx)) * inv_len2;
            s = fminf(fmaxf(s, 0.0f), 1.0f);
            const float ex = fmaf(-s, sdx, wx), ey = fmaf(-s, sdy, wy), ez = fmaf(-s, sdz, wz);
            keep = fmaf(ez, ez, fmaf(ey, ey, ex * ex)) <= Rg2;
            bk = min(max(__float2int_rn(s * (float)(nseg - 1)), 0), nseg - 1);
          }
          const unsigned msk = __ballot_sync(kFull, keep);
          if (keep) {
            const int slot = count + __popc(msk & lt);
            if (slot < kSegCap) {
              sm.q[slot] = q;
              sm.pos[slot] = p;
              sm.cb[slot] = (unsigned char)bk;
            }
          }
          count += __popc(msk);
        }
      }
      if (count > kSegCap) gathered = false;
    }
  }
  const int ncand = gathered ? count : 0;
  // ---- 2. counting sort by sample index
  sm.cursor[lane] = 0;
  sm.cursor[lane + 32] = 0;
  __syncwarp();
  for (int c = lane; c < ncand; c += 32) atomicAdd(&sm.cursor[FOMO_IDX(sm.cb[c], kSeg, kSiteSmem)], 1);
  __syncwarp();
  {
    const int h0 = sm.cursor[2 * lane], h1 = sm.cursor[2 * lane + 1];
    const int incl = warp_incl_scan(h0 + h1);
    const int ex = incl - h0 - h1;
    __syncwarp();
    sm.bstart[2 * lane] = ex;
    sm.bstart[2 * lane + 1] = ex + h0;
    if (lane == 31) sm.bstart[kSeg] = incl;
    sm.cursor[2 * lane] = ex;
    sm.cursor[2 * lane + 1] = ex + h0;
  }
  __syncwarp();
  for (int c = lane; c < ncand; c += 32) {
    const int dst = kSegCap + FOMO_IDX(atomicAdd(&sm.cursor[FOMO_IDX(sm.cb[c], kSeg, kSiteSmem)], 1), kSegCap, kSiteSmem);
    sm.q[dst] = sm.q[c];
    sm.pos[dst] = sm.pos[c];
  }
  __syncwarp();
  const float4* sq = sm.q + kSegCap;  // the candidates in sample order
  const int* spos = sm.pos + kSegCap;
  // ---- 3./4. per-sample scan of the buckets within R, acceptance
  const float dlt = (nseg > 1) ? len / (float)(nseg - 1) : 0.0f;
  const int w = (dlt > 0.0f) ? min((int)(Rg / dlt + 0.51f) + 1, kSeg) : kSeg;
  pos[0] = pos[1] = -1;
  orig[0] = orig[1] = -1;
  bool need0 = false, need1 = false;
#pragma unroll 1
  for (int i = 0; i < 2; ++i) {
    // one copy of the scan code for both samples of the lane (instruction cache)
    const bool acti = i ? act[1] : act[0];
    int pres = -1, ores = -1;
    bool accept = false;
    if (gathered && acti) {
      const int j = lane + 32 * i;
      const int c0 = sm.bstart[max(j - w, 0)], c1 = sm.bstart[min(j + w, nseg - 1) + 1];
      st_scanned += c1 - c0;
      const float t_x = i ? tx[1] : tx[0], t_y = i ? ty[1] : ty[0], t_z = i ? tz[1] : tz[0];
      const float tmax = fmaxf(fmaxf(fabsf(t_x), fabsf(t_y)), fabsf(t_z));
      const float delta = (tmax + r.mdf) * 4.8e-7f + r.mdf * 1.2e-7f;  // ~4 ulp of the box corners
      const float md_in = r.mdf - delta, md_out = r.mdf + delta;
      float b1 = FLT_MAX, b2 = FLT_MAX;
      int bi = -1;
      bool amb = false;
      for (int c = c0; c < c1; ++c) {
        const float4 q = sq[c];
        const float dx = q.x - t_x, dy = q.y - t_y, dz = q.z - t_z;
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        const float cheb = fmaxf(fmaxf(fabsf(dx), fabsf(dy)), fabsf(dz));
        if (cheb < md_in) {
          if (d2 < b1) {
            b2 = b1;
            b1 = d2;
            bi = c;
          } else if (d2 < b2) {
            b2 = d2;
          }
        } else if (cheb <= md_out) {
          amb = true;
        }
      }
      // coverage: every point within cov of the target was gathered
      const float wx = t_x - ax, wy = t_y - ay, wz = t_z - az;
      float s = fmaf(wz, sdz, fmaf(wy, sdy, wx * sdx)) * inv_len2;
      s = fminf(fmaxf(s, 0.0f), 1.0f);
      const float ex = fmaf(-s, sdx, wx), ey = fmaf(-s, sdy, wy), ez = fmaf(-s, sdz, wz);
      const float cov = Rg - sqrtf(fmaf(ez, ez, fmaf(ey, ey, ex * ex))) - amax * 2.4e-7f;
      if (!amb && cov > 0.0f) {
        if (bi >= 0)
          accept = b1 < cov * cov * (1.0f - 2.0f * kRelPrune);
        else
          accept = md_out * 1.7321f * 1.0001f < cov;  // the whole box lies inside the gathered ball
      }
      if (!accept && bi < 0 && !amb) {
        // no candidate: the box is empty for sure when it lies outside the
        // points' bounding box (hi <= min or lo >= max on some axis)
        accept = (t_x + md_out <= g.minx) || (t_x - md_out >= g.maxx) || (t_y + md_out <= g.miny) ||
                 (t_y - md_out >= g.maxy) || (t_z + md_out <= g.minz) || (t_z - md_out >= g.maxz);
      }
      if (accept && bi >= 0) {
        if (b2 <= b1 * (1.0f + kRelTie)) {
          // possible FP64 tie: exact re-rank of the in-box contenders
          ++st_ties;
          bi = exact_rerank_list(sq, c0, c1, t_x, t_y, t_z, md_in, b1 * (1.0f + kRelTie));
        }
        pres = spos[FOMO_IDX(bi, kSegCap, kSiteSmem)];
        ores = __float_as_int(sq[FOMO_IDX(bi, kSegCap, kSiteSmem)].w);
      }
      if (stats && !accept)  // rare: counted where it happens
        atomicAdd(stats + (amb ? kStatFbAmb : (bi < 0 ? kStatFbNoCand : kStatFbFar)), 1ull);
    }
    st_samples += acti ? 1 : 0;
    const bool need = acti && !accept;
    if (i) {
      pos[1] = pres;
      orig[1] = ores;
      need1 = need;
    } else {
      pos[0] = pres;
      orig[0] = ores;
      need0 = need;
    }
  }
  __syncwarp();  // the candidate lists are rewritten by the next segment
  // ---- 5. samples this pass could not resolve (about 1 %) are left empty
  // here and deferred to the second kernel: one record per segment
  const unsigned f0 = __ballot_sync(kFull, need0), f1 = __ballot_sync(kFull, need1);
  if ((f0 | f1) && lane == 0) {
    // a segment whose capsule held too many points is queued from the back,
    // for march_split to search in parts; the others from the front
    const bool over = !gathered && nseg > 16;
    const unsigned long long k = atomicAdd(a.counter + (over ? kCtrOverflow : kCtrDeferred), 1ull);
    const int64_t slot = over ? a.deferred_cap - 1 - (int64_t)k : (int64_t)k;
    // the halves the far pass may take, in views whose boxes reach kFarBox
    // cells or more from their target: kFarMin or more deferred samples, the
    // whole half half a cell or more off the points' bounding box (the box of
    // the half's stretch of the segment against the points' box)
    unsigned flags = 0u;
    bool listed = false;
    if (a.far_list && r.mdf >= kFarBox * g.h) {
      const float inv = nseg > 1 ? 1.0f / (float)(nseg - 1) : 0.0f;
      const float off2 = kFarOut2 * g.h * g.h;
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        if (__popc(hh ? f1 : f0) < kFarMin) continue;
        const float t0 = (float)(32 * hh) * inv, t1 = (float)min(32 * hh + 31, nseg - 1) * inv;
        const float xa = fmaf(t0, sdx, ax), xb = fmaf(t1, sdx, ax), ya = fmaf(t0, sdy, ay), yb = fmaf(t1, sdy, ay),
                    za = fmaf(t0, sdz, az), zb = fmaf(t1, sdz, az);
        const float ex = fmaxf(fmaxf(g.minx - fmaxf(xa, xb), fminf(xa, xb) - g.maxx), 0.0f);
        const float ey = fmaxf(fmaxf(g.miny - fmaxf(ya, yb), fminf(ya, yb) - g.maxy), 0.0f);
        const float ez = fmaxf(fmaxf(g.minz - fmaxf(za, zb), fminf(za, zb) - g.maxz), 0.0f);
        if (fmaf(ez, ez, fmaf(ey, ey, ex * ex)) >= off2) flags |= hh ? kRecFar1 : kRecFar0;
      }
      listed = flags != 0u;
    }
    if (slot >= 0 && slot < a.deferred_cap) {  // always: the capacity is one record per segment
      a.deferred[FOMO_IDX(slot, a.deferred_cap, kSiteDeferred)] = make_uint4(r.item, (unsigned)s0 | flags, f0, f1);
      if (listed) {
        const unsigned long long f = atomicAdd(a.counter + kCtrFar, 1ull);
        if ((int64_t)f < a.deferred_cap) a.far_list[FOMO_IDX(f, a.deferred_cap, kSiteDeferred)] = (int32_t)slot;
      }
    }
  }
  if (stats) {
    const unsigned sc = __reduce_add_sync(kFull, (unsigned)st_scanned);
    const unsigned ti = __reduce_add_sync(kFull, (unsigned)st_ties);
    const unsigned sa = __reduce_add_sync(kFull, (unsigned)st_samples);
    if (lane == 0) {
      atomicAdd(stats + kStatSegments, 1ull);
      atomicAdd(stats + kStatCandidates, (unsigned long long)count);
      atomicAdd(stats + kStatRows, (unsigned long long)st_rows);
      atomicAdd(stats + kStatPointsLoaded, (unsigned long long)st_loaded);
      atomicAdd(stats + kStatNotGathered, gathered ? 0ull : 1ull);
      atomicAdd(stats + kStatFallbacks, (unsigned long long)(__popc(f0) + __popc(f1)));
      atomicAdd(stats + kStatDeferredRecs, (f0 | f1) ? 1ull : 0ull);
      atomicAdd(stats + kStatSamples, (unsigned long long)sa);
      atomicAdd(stats + kStatScanned, (unsigned long long)sc);
      atomicAdd(stats + kStatTies, (unsigned long long)ti);
    }
  }
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Search pass of the two-pass spectral march: each sample's neighbour (sorted
// position, -1 for none or deferred) into a.npos, [work item - item_base][k],
// streamed past L2; the NN indices when asked for.  march_spectral<.., true>
// then bins the emission from these positions.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, kMinCtasSearch) march_search(MarchArgs a, const double3* __restrict__ ktab,
                                                               int ktab_stride) {
  __shared__ SegSmem segs[kWarps];
  SegSmem& sm = segs[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  RayCtx r;
  while (next_ray(a, ktab, ktab_stride, r)) {
    const ViewDesc* V = a.views + r.v;
    const int nz = V->nz;
    int32_t* nnout = a.nn_idx ? a.nn_idx[r.v] : nullptr;
    const int64_t ray = (int64_t)r.i * V->nx + r.j;
    int32_t* npos = a.npos + ((int64_t)r.item - a.item_base) * ktab_stride;
    for (int s0 = 0; s0 < nz; s0 += kSeg) {
      int posv[2], origv[2];
      segment_search(a, r, s0, nz, sm, posv, origv);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int k = s0 + 32 * h + lane;
        if (k < nz) {
          __stcs(a.npos + FOMO_IDX(npos - a.npos + k, a.npos_cap, kSiteNpos), h ? posv[1] : posv[0]);
          if (nnout) nnout[FOMO_IDX(ray * nz + k, (int64_t)V->nx * V->ny * nz, kSiteNnIdx)] = h ? origv[1] : origv[0];
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Spectroscopic march: NL lines x up to NB 32-bin windows per line; lane
// `lane` owns bins wstart + 32 m + lane of each line.
// ---------------------------------------------------------------------------
// SHADE: the neighbours come from the position buffer written by
// march_search (a.npos) instead of the search itself; the emission code and
// its arithmetic are the same.
template <int NL, int NB, bool SHADE>
__global__ void __launch_bounds__(kThreads, SHADE ? kMinCtasShade : kMinCtas)
    march_spectral(MarchArgs a, const double3* __restrict__ ktab, int ktab_stride) {
  __shared__ SegSmem segs[SHADE ? 1 : kWarps];
  __shared__ float4 runs[kWarps][32][NL];  // a chunk's runs: (peak x length, 2/w, Doppler term) per line
  const int w = threadIdx.x >> 5;
  SegSmem& sm = segs[SHADE ? 0 : w];
  const int lane = threadIdx.x & 31;
  RayCtx r;
  while (next_ray(a, ktab, ktab_stride, r, SHADE ? kCtrShade : kCtrRays)) {
    const ViewDesc* V = a.views + r.v;
    const int nz = V->nz, L = V->L, nx = V->nx;
    const float ux = V->ux, uy = V->uy, uz = V->uz;
    const LineDesc* LD = a.lines + (int64_t)r.v * a.nlines;
    float acc[NL][NB], comp[NL][NB], part[NL][NB], lam[NL][NB], shk[NL];
    const float2* ew[NL];
    bool lon[NL];
    int nw[NL], ws[NL];
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      const bool on = l < a.nlines && LD[l].ew != nullptr;  // views may have fewer lines than the launch
      lon[l] = on;
      ew[l] = on ? LD[l].ew : nullptr;
      shk[l] = on ? LD[l].shift_k : 0.0f;
      nw[l] = on ? min(LD[l].nw, NB) : 0;
      ws[l] = on ? LD[l].wstart : 0;
#pragma unroll
      for (int m = 0; m < NB; ++m) {
        const int il = ws[l] + m * 32 + lane;
        acc[l][m] = 0.0f;
        comp[l][m] = 0.0f;
        part[l][m] = 0.0f;
        // lambdaval (nn:200), evaluated in FP64 on the host, stored FP32
        lam[l][m] = (m < nw[l] && il < L) ? __ldg(LD[l].lam + FOMO_IDX(il, L, kSiteLam)) : 3.0e30f;
      }
    }
    int32_t* nnout = (!SHADE && a.nn_idx) ? a.nn_idx[r.v] : nullptr;
    const int64_t ray = (int64_t)r.i * nx + r.j;
    const int32_t* npos = SHADE ? a.npos + ((int64_t)r.item - a.item_base) * ktab_stride : nullptr;
    for (int s0 = 0; s0 < nz; s0 += kSeg) {
      int posv[2], origv[2];
      if (SHADE) {
        posv[0] = s0 + lane < nz ? __ldcs(a.npos + FOMO_IDX(npos - a.npos + s0 + lane, a.npos_cap, kSiteNpos)) : -1;
        posv[1] = s0 + 32 + lane < nz ? __ldcs(a.npos + FOMO_IDX(npos - a.npos + s0 + 32 + lane, a.npos_cap, kSiteNpos))
                                      : -1;
      } else {
        segment_search(a, r, s0, nz, sm, posv, origv);
      }
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        const int k = s0 + 32 * h + lane;
        const bool active = k < nz;
        const int pos = h ? posv[1] : posv[0];
        if (nnout && active)
          nnout[FOMO_IDX(ray * nz + k, (int64_t)V->nx * V->ny * nz, kSiteNnIdx)] = h ? origv[1] : origv[0];
        // runs of equal neighbours
        const int prev = __shfl_up_sync(kFull, pos, 1);
        const bool start = active && (lane == 0 || pos != prev);
        const unsigned starts = __ballot_sync(kFull, start);
        const unsigned act = __ballot_sync(kFull, active);
        if (!act) break;
        const int endlane = 32 - __clz(act);
        // the start lane of each run with a neighbour loads its payload and
        // stages the per-line terms (peak x run length, 2/w, Doppler offset)
        // in a compact list; a peak of 0 (intpolpeak ? ... : 0, nn:204) is
        // staged as all zeros and adds nothing
        const bool filled = start && pos >= 0;
        const unsigned fills = __ballot_sync(kFull, filled);
        if (filled) {
          const unsigned later = starts & ~((2u << lane) - 1u);
          const int e = later ? (__ffs(later) - 1) : endlane;
          const float cnt = (float)(e - lane);
          const float4 vv = __ldg(a.snap.vel + FOMO_IDX(pos, a.snap.n, kSitePts));
          const float vlos = fmaf(uz, vv.z, fmaf(uy, vv.y, ux * vv.x));
          float4* dst = runs[w][__popc(fills & ((1u << lane) - 1u))];
#pragma unroll
          for (int l = 0; l < NL; ++l) {
            if (lon[l]) {
              const float2 pw = __ldg(ew[l] + FOMO_IDX(pos, a.snap.n, kSitePts));
              const float sc = __fdividef(2.0f, pw.y);  // exp(-4 ln2 (d/w)^2) = 2^(-(2d/w)^2)
              dst[l] = pw.x != 0.0f ? make_float4(pw.x * cnt, sc, -(vlos * shk[l]) * sc, 0.0f)
                                    : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
          }
        }
        __syncwarp();
        const int nruns = __popc(fills);
        if (a.stats && lane == 0 && nruns > 0) {
          int nwin = 0;
#pragma unroll
          for (int l = 0; l < NL; ++l) nwin += lon[l] ? nw[l] : 0;
          atomicAdd(a.stats + kStatRuns, (unsigned long long)nruns);
          atomicAdd(a.stats + kStatEx2, 32ull * (unsigned long long)(nruns * nwin));
        }
        for (int q0 = 0; q0 < nruns; ++q0) {
#pragma unroll
          for (int l = 0; l < NL; ++l) {
            if (lon[l]) {
              const float4 t = runs[w][q0][l];  // same address in every lane: one broadcast load
#pragma unroll
              for (int m = 0; m < NB; ++m) {
                if (m < nw[l]) {
                  const float q = fmaf(lam[l][m], t.y, t.z);
                  part[l][m] = fmaf(t.x, ex2_approx(-q * q), part[l][m]);
                }
              }
            }
          }
        }
        __syncwarp();  // the run list is rewritten by the next chunk
#pragma unroll
        for (int l = 0; l < NL; ++l)
#pragma unroll
          for (int m = 0; m < NB; ++m) {
            kahan_add(acc[l][m], comp[l][m], part[l][m]);
            part[l][m] = 0.0f;
          }
      }
    }
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      if (lon[l]) {
        const double scale = LD[l].is_dn ? V->scale_dn : V->scale;
        float* out = LD[l].out;
        const int64_t ncube = (int64_t)nx * V->ny * L;
        const int wlo = ws[l], whi = ws[l] + 32 * nw[l];
        for (int il = lane; il < L; il += 32)
          if (il < wlo || il >= whi) out[FOMO_IDX(ray * L + il, ncube, kSiteCube)] = 0.0f;  // below 2^-64 of every peak
#pragma unroll
        for (int m = 0; m < NB; ++m) {
          const int il = wlo + m * 32 + lane;
          if (m < nw[l] && il < L)
            out[FOMO_IDX(ray * L + il, ncube, kSiteCube)] = __double2float_rn(__dmul_rn(scale, (double)acc[l][m]));
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Imaging (L == 1, broadband channels) and Thomson pB: per-sample values,
// reduced across the warp per 32-sample chunk, Kahan-accumulated per ray.
// SHADE: the neighbours come from the position buffer (a.npos), in which the
// search, split, deferred and hard passes have stored every sample's
// neighbour; otherwise (the no-allocation path) the kernel searches itself and
// the deferred samples are added by the later passes.
// ---------------------------------------------------------------------------
template <int NL, bool THOMSON, bool SHADE>
__global__ void __launch_bounds__(kThreads, SHADE ? kMinCtasShade : kMinCtasImaging)
    march_imaging(MarchArgs a, const double3* __restrict__ ktab, int ktab_stride) {
  __shared__ SegSmem segs[SHADE ? 1 : kWarps];
  SegSmem& sm = segs[SHADE ? 0 : (threadIdx.x >> 5)];
  const int lane = threadIdx.x & 31;
  RayCtx r;
  while (next_ray(a, ktab, ktab_stride, r, SHADE ? kCtrShade : kCtrRays)) {
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
    int32_t* nnout = (!SHADE && a.nn_idx) ? a.nn_idx[r.v] : nullptr;
    const int64_t ray = (int64_t)r.i * nx + r.j;
    const int32_t* npos = SHADE ? a.npos + ((int64_t)r.item - a.item_base) * ktab_stride : nullptr;
    for (int s0 = 0; s0 < nz; s0 += kSeg) {
      int posv[2], origv[2];
      if (SHADE) {
        posv[0] = s0 + lane < nz ? __ldcs(a.npos + FOMO_IDX(npos - a.npos + s0 + lane, a.npos_cap, kSiteNpos)) : -1;
        posv[1] = s0 + 32 + lane < nz ? __ldcs(a.npos + FOMO_IDX(npos - a.npos + s0 + 32 + lane, a.npos_cap, kSiteNpos))
                                      : -1;
      } else {
        segment_search(a, r, s0, nz, sm, posv, origv);
      }
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        const int k = s0 + 32 * h + lane;
        const bool active = k < nz;
        const int pos = h ? posv[1] : posv[0];
        if (nnout && active)
          nnout[FOMO_IDX(ray * nz + k, (int64_t)V->nx * V->ny * nz, kSiteNnIdx)] = h ? origv[1] : origv[0];
#pragma unroll
        for (int l = 0; l < NL; ++l) {
          if (lon[l]) {
            float val = 0.0f;
            if (pos >= 0) {
              if (THOMSON) {
                // pB = pol * sin^2 chi, clamped at 0 (thomson:325-338)
                val = fmaxf(__ldg(a.totpol + FOMO_IDX(pos, a.snap.n, kSitePts)).y *
                                __ldg(s2v + FOMO_IDX(pos, a.snap.n, kSiteS2)),
                            0.0f);
              } else {
                val = __ldg(LD[l].ew + FOMO_IDX(pos, a.snap.n, kSitePts)).x;  // imaging adds the peak (nn:217-225)
              }
            }
            const float cs = warp_sum(val);
            if (lane == 0) kahan_add(acc[l], comp[l], cs);
          }
        }
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int l = 0; l < NL; ++l)
        if (lon[l])
          LD[l].out[FOMO_IDX(ray, (int64_t)nx * V->ny, kSiteCube)] =
              __double2float_rn(__dmul_rn(LD[l].is_dn ? V->scale_dn : V->scale, (double)acc[l]));
    }
  }
}

// ---------------------------------------------------------------------------
// Deferred samples: the march's first pass leaves about 1 % of the samples
// (boxes reaching past its gather radius, mostly just outside the point
// cloud, or segments whose capsule holds too many points) empty and records
// them.  This kernel finds their neighbours, writes their NN indices and adds
// their emission to the rays' outputs, which the march has already written
// (same stream, so after it).  A warp takes 32 records at a time, flattens
// their samples and gives every lane one sample to search on its own; the
// contributions are then added per record, lane = lambda bin.
// ---------------------------------------------------------------------------
enum DeferredKind : int { kDeferredSpectral = 0, kDeferredImaging = 1, kDeferredThomson = 2 };
constexpr int kDefBatch = 256;  // deferred samples staged per warp between search and contribution

// Candidate v (sorted position p) against box q: kept when strictly inside;
// the two best FP32 squared distances, or (EXACT) the smallest FP64 distance
// within `band`, lowest original index on exact ties.
// The distance comes first: a point no nearer than the second best (or
// beyond the band) changes nothing whether it lies in the box or not, so the
// box test is made only for the others.
template <bool EXACT>
__device__ __forceinline__ void scan_point(const float4 v, int p, const BoxQ& q, float band, float& best,
                                           float& second, int& bpos, int& borig, double& bD) {
  const float dx = v.x - q.tx, dy = v.y - q.ty, dz = v.z - q.tz;
  const float d = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
  if (!(EXACT ? d <= band : d < second)) return;
  if (!(v.x > q.lox && v.x < q.hix && v.y > q.loy && v.y < q.hiy && v.z > q.loz && v.z < q.hiz)) return;
  const int o = __float_as_int(v.w);
  if (!EXACT) {
    if (d < best) {
      second = best;
      best = d;
      bpos = p;
      borig = o;
    } else {
      second = d;
    }
  } else {
    const double D = exact_dist2(v.x, v.y, v.z, q.tx, q.ty, q.tz);
    if (D < bD || (D == bD && o < borig)) {
      bD = D;
      borig = o;
      bpos = p;
    }
  }
}

// Candidates p in [p0, p1), one after the other.  With BUDGET, `budget` pays
// one unit per row and per point, and a range of more than kLaneDense points
// (dense cells) spends it at once: such samples are searched by a warp.
constexpr int kLaneDense = 48;
template <bool EXACT, bool BUDGET>
__device__ __forceinline__ void lane_scan(const SnapDev& S, const BoxQ& q, int p0, int p1, float band, float& best,
                                          float& second, int& bpos, int& borig, double& bD, int& budget) {
  if (BUDGET) {
    budget -= (p1 - p0 > kLaneDense) ? 0x3fffffff : 1 + (p1 - p0);
    if (budget < 0) return;
  }
  for (int p = p0; p < p1; ++p)
    scan_point<EXACT>(__ldg(S.pts + FOMO_IDX(p, S.n, kSitePts)), p, q, band, best, second, bpos, borig, bD);
}

// Narrow the cell range [lo, hi] of one axis to the cells whose gap from t can
// be within sqrt(rem) (none when rem < 0).  A superset: the reach carries the
// same relative and cell-margin slack as the x-range clip of a row.
__device__ __forceinline__ void clip_reach(float rem, float t, float o, float inv_h, float h, int dim, int& lo,
                                           int& hi) {
  if (rem < 0.0f) {
    hi = lo - 1;
    return;
  }
  const float r = (rem > 0.0f ? rem * rsqrtf(rem) * 1.0001f : 0.0f) + kCellMargin * h;
  lo = max(lo, cell_coord(t - r, o, inv_h, dim));
  hi = min(hi, cell_coord(t + r, o, inv_h, dim));
}

// One lane's walk over the rings of cells around the target's cell c (clamped
// into the grid), nearest first.  A ring, a row or a cell is skipped when its
// lower bound from the target exceeds the bound (the best squared distance so
// far, or `band` in the EXACT pass); every loop is bounded by the box's cells.
template <bool EXACT, bool BUDGET>
__device__ __forceinline__ void lane_rings(const SnapDev& S, const BoxQ& q, const int (&b0)[3], const int (&b1)[3],
                                           const int (&c)[3], const float (&gc)[3], float band, float& best,
                                           float& second, int& bpos, int& borig, double& bD, int& budget) {
  const GridParams& g = S.g;
  const float h = g.h;
  const float to[3] = {q.tx, q.ty, q.tz}, oo[3] = {g.ox, g.oy, g.oz};
  for (int s = 0;; ++s) {
    if (c[0] - s < b0[0] && c[0] + s > b1[0] && c[1] - s < b0[1] && c[1] + s > b1[1] && c[2] - s < b0[2] &&
        c[2] + s > b1[2])
      break;  // no cell of this ring lies in the box
    if (s >= 1) {
      // one axis steps s cells from the centre, the others stay at their nearest slab
      const float bound = EXACT ? band * (1.0f + kRelPrune) : best * (1.0f + kRelPrune);
      float lb2 = FLT_MAX;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        float m = FLT_MAX;
        if (c[j] - s >= b0[j]) m = axis_gap(c[j] - s, to[j], oo[j], h);
        if (c[j] + s <= b1[j]) m = fminf(m, axis_gap(c[j] + s, to[j], oo[j], h));
        if (m < FLT_MAX) lb2 = fminf(lb2, fmaf(m, m, gc[(j + 1) % 3] + gc[(j + 2) % 3]));
      }
      if (lb2 > bound) break;
    }
    const int xl = c[0] - s, xr = c[0] + s;
    const bool has_l = xl >= b0[0], has_r = s > 0 && xr <= b1[0];
    const float gxl = has_l ? axis_gap(xl, q.tx, g.ox, h) : 0.0f;
    const float gxr = has_r ? axis_gap(xr, q.tx, g.ox, h) : 0.0f;
    const int z0 = max(c[2] - s, b0[2]), z1 = min(c[2] + s, b1[2]);
    const int y0 = max(c[1] - s, b0[1]), y1 = min(c[1] + s, b1[1]);
    for (int kz = z0; kz <= z1; ++kz) {
      const float gz = axis_gap(kz, q.tz, g.oz, h);
      const float gz2 = gz * gz;
      const bool zshell = kz == c[2] - s || kz == c[2] + s;
      for (int jy = y0; jy <= y1; ++jy) {
        if (BUDGET && budget < 0) return;  // out of budget: a warp searches this sample
        const float bound = EXACT ? band * (1.0f + kRelPrune) : best * (1.0f + kRelPrune);
        const float gy = axis_gap(jy, q.ty, g.oy, h);
        const float gyz = fmaf(gy, gy, gz2);
        if (gyz + gc[0] > bound) continue;
        const int rowbase = (kz * g.dy + jy) * g.dx;
        if (zshell || jy == c[1] - s || jy == c[1] + s) {
          // a row on the ring's y/z faces: its x-range within the bound
          int x0 = max(xl, b0[0]), x1 = min(xr, b1[0]);
          if (bound < FLT_MAX) {
            const float rem = fmaxf(bound - gyz, 0.0f);
            const float rx = (rem > 0.0f ? rem * rsqrtf(rem) * 1.0001f : 0.0f) + kCellMargin * h;
            x0 = max(x0, cell_coord(q.tx - rx, g.ox, g.inv_h, g.dx));
            x1 = min(x1, cell_coord(q.tx + rx, g.ox, g.inv_h, g.dx));
          }
          if (x0 <= x1)
            lane_scan<EXACT, BUDGET>(S, q, __ldg(S.cell_start + FOMO_IDX(rowbase + x0, cell_entries(g), kSiteCellStart)),
                                     __ldg(S.cell_start + FOMO_IDX(rowbase + x1 + 1, cell_entries(g), kSiteCellStart)),
                                     band, best, second, bpos, borig, bD, budget);
        } else {
          // a row inside the ring's y-z square: only its two end cells are on the ring
          if (has_l && fmaf(gxl, gxl, gyz) <= bound)
            lane_scan<EXACT, BUDGET>(S, q, __ldg(S.cell_start + FOMO_IDX(rowbase + xl, cell_entries(g), kSiteCellStart)),
                                     __ldg(S.cell_start + FOMO_IDX(rowbase + xl + 1, cell_entries(g), kSiteCellStart)),
                                     band, best, second, bpos, borig, bD, budget);
          if (has_r && fmaf(gxr, gxr, gyz) <= (EXACT ? bound : best * (1.0f + kRelPrune)))
            lane_scan<EXACT, BUDGET>(S, q, __ldg(S.cell_start + FOMO_IDX(rowbase + xr, cell_entries(g), kSiteCellStart)),
                                     __ldg(S.cell_start + FOMO_IDX(rowbase + xr + 1, cell_entries(g), kSiteCellStart)),
                                     band, best, second, bpos, borig, bD, budget);
        }
      }
    }
  }
}

// The cells of box q: b0..b1 per axis, the target's cell c (clamped into the
// grid) and the squared gaps from the target to c's faces; false when the box
// misses the grid.
__device__ __forceinline__ bool box_cells(const GridParams& g, const BoxQ& q, int (&b0)[3], int (&b1)[3], int (&c)[3],
                                          float (&gc)[3]) {
  if (!(q.lox < g.maxx && q.hix > g.minx && q.loy < g.maxy && q.hiy > g.miny && q.loz < g.maxz &&
        q.hiz > g.minz && q.lox < q.hix && q.loy < q.hiy && q.loz < q.hiz))
    return false;
  b0[0] = cell_coord(q.lox, g.ox, g.inv_h, g.dx);
  b0[1] = cell_coord(q.loy, g.oy, g.inv_h, g.dy);
  b0[2] = cell_coord(q.loz, g.oz, g.inv_h, g.dz);
  b1[0] = cell_coord(q.hix, g.ox, g.inv_h, g.dx);
  b1[1] = cell_coord(q.hiy, g.oy, g.inv_h, g.dy);
  b1[2] = cell_coord(q.hiz, g.oz, g.inv_h, g.dz);
  c[0] = cell_coord(q.tx, g.ox, g.inv_h, g.dx);
  c[1] = cell_coord(q.ty, g.oy, g.inv_h, g.dy);
  c[2] = cell_coord(q.tz, g.oz, g.inv_h, g.dz);
  const float gx = axis_gap(c[0], q.tx, g.ox, g.h), gy = axis_gap(c[1], q.ty, g.oy, g.h),
              gz = axis_gap(c[2], q.tz, g.oz, g.h);
  gc[0] = gx * gx;
  gc[1] = gy * gy;
  gc[2] = gz * gz;
  return true;
}

constexpr int kLaneBudget = 192;  // rows + points one lane may scan for one sample

// Nearest point strictly inside box q, searched by this lane alone: sorted
// position and original index, or -1 when the box holds no point.  With
// BUDGET, false when the search ran out of kLaneBudget (dense cells, or a
// wide box far from the points): a whole warp then searches the sample
// (warp_search, march_hard).
template <bool BUDGET>
__device__ __forceinline__ bool lane_search(const SnapDev& S, const BoxQ& q, int& pos, int& orig) {
  int budget = kLaneBudget;
  pos = -1;
  orig = -1;
  int b0[3], b1[3], c[3];
  float gc[3];
  if (!box_cells(S.g, q, b0, b1, c, gc)) return true;
  float best = FLT_MAX, second = FLT_MAX;
  int bpos = -1, borig = -1;
  double bD = DBL_MAX;
  lane_rings<false, BUDGET>(S, q, b0, b1, c, gc, 0.0f, best, second, bpos, borig, bD, budget);
  if (BUDGET && budget < 0) return false;
  if (bpos < 0) return true;
  if (second <= best * (1.0f + kRelTie)) {
    // possible FP64 tie (or an exact FP32 tie): re-rank the contenders
    float fb = FLT_MAX, fs = FLT_MAX;
    int p2 = -1, o2 = 0x7fffffff;
    double D2 = DBL_MAX;
    lane_rings<true, BUDGET>(S, q, b0, b1, c, gc, best * (1.0f + kRelTie), fb, fs, p2, o2, D2, budget);
    if (BUDGET && budget < 0) return false;
    bpos = p2;
    borig = o2;
  }
  pos = bpos;
  orig = borig;
  return true;
}

// lane_search without a budget, out of line: for the rare sample that finds
// the hard queue full (a second inlined copy of the ring walks would crowd
// the deferred kernel's instruction cache).
__device__ __noinline__ void lane_search_full(const SnapDev& S, const BoxQ q, int& pos, int& orig) {
  lane_search<false>(S, q, pos, orig);
}

// Warp-collective walk over the same rings as lane_rings for one sample (q
// the same in every lane): the rows of a ring are spread over the lanes, their
// point ranges prefix-summed and loaded 32 per round.  Each lane keeps the
// best of the points it scanned; the pruning bound is the warp's best, taken
// after every ring.
template <bool EXACT>
__device__ __forceinline__ void warp_rings(const SnapDev& S, const BoxQ& q, const int (&b0)[3], const int (&b1)[3],
                                           const int (&c)[3], const float (&gc)[3], float band, float& best,
                                           float& second, int& bpos, int& borig, double& bD) {
  const GridParams& g = S.g;
  const float h = g.h;
  const int lane = threadIdx.x & 31;
  const float to[3] = {q.tx, q.ty, q.tz}, oo[3] = {g.ox, g.oy, g.oz};
  float bound = EXACT ? band * (1.0f + kRelPrune) : FLT_MAX;
  for (int s = 0;; ++s) {
    if (c[0] - s < b0[0] && c[0] + s > b1[0] && c[1] - s < b0[1] && c[1] + s > b1[1] && c[2] - s < b0[2] &&
        c[2] + s > b1[2])
      break;  // no cell of this ring lies in the box
    if (s >= 1) {
      float lb2 = FLT_MAX;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        float m = FLT_MAX;
        if (c[j] - s >= b0[j]) m = axis_gap(c[j] - s, to[j], oo[j], h);
        if (c[j] + s <= b1[j]) m = fminf(m, axis_gap(c[j] + s, to[j], oo[j], h));
        if (m < FLT_MAX) lb2 = fminf(lb2, fmaf(m, m, gc[(j + 1) % 3] + gc[(j + 2) % 3]));
      }
      if (lb2 > bound) break;
    }
    const int xl = c[0] - s, xr = c[0] + s;
    const bool has_l = xl >= b0[0], has_r = s > 0 && xr <= b1[0];
    const float gxl = has_l ? axis_gap(xl, q.tx, g.ox, h) : 0.0f;
    const float gxr = has_r ? axis_gap(xr, q.tx, g.ox, h) : 0.0f;
    int z0 = max(c[2] - s, b0[2]), z1 = min(c[2] + s, b1[2]);
    int y0 = max(c[1] - s, b0[1]), y1 = min(c[1] + s, b1[1]);
    if (bound < FLT_MAX) {  // the ring's y-z square narrowed to the rows within the bound
      clip_reach(bound - gc[0], q.tz, g.oz, g.inv_h, h, g.dz, z0, z1);
      clip_reach(bound - gc[0], q.ty, g.oy, g.inv_h, h, g.dy, y0, y1);
    }
    const int nyr = y1 - y0 + 1, nrows = (nyr > 0 && z1 >= z0) ? nyr * (z1 - z0 + 1) : 0;
    for (int rb = 0; rb < nrows; rb += 32) {
      // this lane's row of the ring: up to two point ranges
      const int rr = rb + lane;
      int a0 = 0, n0 = 0, a1 = 0, n1 = 0;
      if (rr < nrows) {
        const int jy = y0 + rr % nyr, kz = z0 + rr / nyr;
        const float gz = axis_gap(kz, q.tz, g.oz, h);
        const float gy = axis_gap(jy, q.ty, g.oy, h);
        const float gyz = fmaf(gy, gy, gz * gz);
        if (gyz + gc[0] <= bound) {
          const int rowbase = (kz * g.dy + jy) * g.dx;
          if (kz == c[2] - s || kz == c[2] + s || jy == c[1] - s || jy == c[1] + s) {
            int x0 = max(xl, b0[0]), x1 = min(xr, b1[0]);
            if (bound < FLT_MAX) {
              const float rem = fmaxf(bound - gyz, 0.0f);
              const float rx = (rem > 0.0f ? rem * rsqrtf(rem) * 1.0001f : 0.0f) + kCellMargin * h;
              x0 = max(x0, cell_coord(q.tx - rx, g.ox, g.inv_h, g.dx));
              x1 = min(x1, cell_coord(q.tx + rx, g.ox, g.inv_h, g.dx));
            }
            if (x0 <= x1) {
              a0 = __ldg(S.cell_start + FOMO_IDX(rowbase + x0, cell_entries(g), kSiteCellStart));
              n0 = __ldg(S.cell_start + FOMO_IDX(rowbase + x1 + 1, cell_entries(g), kSiteCellStart)) - a0;
            }
          } else {
            if (has_l && fmaf(gxl, gxl, gyz) <= bound) {
              a0 = __ldg(S.cell_start + FOMO_IDX(rowbase + xl, cell_entries(g), kSiteCellStart));
              n0 = __ldg(S.cell_start + FOMO_IDX(rowbase + xl + 1, cell_entries(g), kSiteCellStart)) - a0;
            }
            if (has_r && fmaf(gxr, gxr, gyz) <= bound) {
              a1 = __ldg(S.cell_start + FOMO_IDX(rowbase + xr, cell_entries(g), kSiteCellStart));
              n1 = __ldg(S.cell_start + FOMO_IDX(rowbase + xr + 1, cell_entries(g), kSiteCellStart)) - a1;
            }
          }
        }
      }
      const int n = n0 + n1;
      const int incl = warp_incl_scan(n);
      const int excl = incl - n;
      const int total = __shfl_sync(kFull, incl, 31);
      for (int ib = 0; ib < total; ib += 32) {
        const int i = ib + lane;
        const int own = warp_owner(incl, i) & 31;
        const int oa0 = __shfl_sync(kFull, a0, own), on0 = __shfl_sync(kFull, n0, own);
        const int oa1 = __shfl_sync(kFull, a1, own), oe = __shfl_sync(kFull, excl, own);
        if (i < total) {
          const int k = i - oe;
          const int p = k < on0 ? oa0 + k : oa1 + (k - on0);
          scan_point<EXACT>(__ldg(S.pts + FOMO_IDX(p, S.n, kSitePts)), p, q, band, best, second, bpos, borig, bD);
        }
      }
    }
    if (!EXACT) bound = warp_min(best) * (1.0f + kRelPrune);
  }
}

// Warp-collective: nearest point strictly inside box q (the same q in every
// lane), the same result as lane_search; every lane gets it.
__device__ __noinline__ void warp_search(const SnapDev& S, const BoxQ& q, int& pos, int& orig) {
  const int lane = threadIdx.x & 31;
  pos = -1;
  orig = -1;
  int b0[3], b1[3], c[3];
  float gc[3];
  if (!box_cells(S.g, q, b0, b1, c, gc)) return;
  float best = FLT_MAX, second = FLT_MAX;
  int bpos = -1, borig = -1;
  double bD = DBL_MAX;
  warp_rings<false>(S, q, b0, b1, c, gc, 0.0f, best, second, bpos, borig, bD);
  const float b1v = warp_min(best);
  if (b1v == FLT_MAX) return;  // no point in the box
  // the lowest lane holding the best, and the warp's second best
  const int hl = __ffs(__ballot_sync(kFull, best == b1v)) - 1;
  const float sec = warp_min(lane == hl ? second : best);
  int P = __shfl_sync(kFull, bpos, hl), O = __shfl_sync(kFull, borig, hl);
  if (sec <= b1v * (1.0f + kRelTie)) {
    // possible FP64 tie: the exact re-rank, reduced over the warp by (distance, original index)
    float fb = FLT_MAX, fs = FLT_MAX;
    int p2 = -1, o2 = 0x7fffffff;
    double D2 = DBL_MAX;
    warp_rings<true>(S, q, b0, b1, c, gc, b1v * (1.0f + kRelTie), fb, fs, p2, o2, D2);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double Do = __shfl_xor_sync(kFull, D2, off);
      const int oo = __shfl_xor_sync(kFull, o2, off), po = __shfl_xor_sync(kFull, p2, off);
      if (Do < D2 || (Do == D2 && oo < o2)) {
        D2 = Do;
        o2 = oo;
        p2 = po;
      }
    }
    P = p2;
    O = o2;
  }
  pos = P;
  orig = O;
}

// Ray context of lane `src` (every lane takes part).
__device__ __forceinline__ RayCtx shfl_ray(const RayCtx& r, int src) {
  RayCtx o;
  o.v = __shfl_sync(kFull, r.v, src);
  o.i = __shfl_sync(kFull, r.i, src);
  o.j = __shfl_sync(kFull, r.j, src);
  o.item = __shfl_sync(kFull, r.item, src);
  o.A0 = __shfl_sync(kFull, r.A0, src);
  o.A1 = __shfl_sync(kFull, r.A1, src);
  o.A2 = __shfl_sync(kFull, r.A2, src);
  o.md = __shfl_sync(kFull, r.md, src);
  o.mdf = __shfl_sync(kFull, r.mdf, src);
  o.nz = __shfl_sync(kFull, r.nz, src);
  o.kt = reinterpret_cast<const double3*>(
      __shfl_sync(kFull, (unsigned long long)reinterpret_cast<uintptr_t>(r.kt), src));
  return o;
}

// Bit index of the n-th (from 0) set bit of lo | hi << 32.
__device__ __forceinline__ int nth_set_bit(unsigned lo, unsigned hi, int n) {
  const int nlo = __popc(lo);
  if (n < nlo) return (int)__fns(lo, 0, n + 1);
  return 32 + (int)__fns(hi, 0, n - nlo + 1);
}

// Warp-collective: adds the emission of n samples of ray r, whose neighbours
// (sorted positions, -1 for none) and LOS speeds are sp[0..n) and sv[0..n) in
// shared memory, to the ray's outputs with atomics.  Spectral: lane = lambda
// bin of each line window; imaging and Thomson: a warp sum per line.
__device__ __forceinline__ void add_emission(const MarchArgs& a, const RayCtx& r, int kind, const int* sp,
                                             const float* sv, int n) {
  const int lane = threadIdx.x & 31;
  const ViewDesc* V = a.views + r.v;
  const int64_t ray = (int64_t)r.i * V->nx + r.j;
  const LineDesc* LD = a.lines + (int64_t)r.v * a.nlines;
  if (kind == kDeferredSpectral) {
    const int L = V->L;
    for (int l = 0; l < a.nlines; ++l) {
      const LineDesc& D = LD[l];
      if (!D.ew) continue;  // views may have fewer lines than the launch
      const double scale = D.is_dn ? V->scale_dn : V->scale;
      for (int m = 0; m < D.nw; ++m) {
        const int il = D.wstart + 32 * m + lane;
        const float lamv = il < L ? __ldg(D.lam + FOMO_IDX(il, L, kSiteLam)) : 3.0e30f;
        float part = 0.0f;
        for (int f = 0; f < n; ++f) {
          const int p = sp[f];
          if (p < 0) continue;
          const float2 pw = __ldg(D.ew + FOMO_IDX(p, a.snap.n, kSitePts));
          if (pw.x == 0.0f) continue;  // intpolpeak ? ... : 0 (nn:204)
          const float sc = __fdividef(2.0f, pw.y);
          const float ns = -(sv[f] * D.shift_k) * sc;
          const float q = fmaf(lamv, sc, ns);
          part = fmaf(pw.x, ex2_approx(-q * q), part);
        }
        if (il < L && part != 0.0f)
          atomicAdd(D.out + FOMO_IDX(ray * L + il, (int64_t)V->nx * V->ny * L, kSiteCube),
                    __double2float_rn(__dmul_rn(scale, (double)part)));
      }
    }
  } else {
    const float* s2v = kind == kDeferredThomson ? a.s2 + (int64_t)r.v * a.snap.n : nullptr;
    for (int l = 0; l < a.nlines; ++l) {
      const LineDesc& D = LD[l];
      if (!D.out) continue;
      float val = 0.0f;
      for (int f = lane; f < n; f += 32) {
        const int p = sp[f];
        if (p >= 0) {
          const int64_t pc = FOMO_IDX(p, a.snap.n, kSitePts);
          val += s2v ? fmaxf(__ldg(a.totpol + pc).y * __ldg(s2v + pc), 0.0f) : __ldg(D.ew + pc).x;
        }
      }
      const float sum = warp_sum(val);
      if (lane == 0 && sum != 0.0f)
        atomicAdd(D.out + FOMO_IDX(ray, (int64_t)V->nx * V->ny, kSiteCube),
                  __double2float_rn(__dmul_rn(D.is_dn ? V->scale_dn : V->scale, (double)sum)));
    }
  }
}

// The record at position ri of the deferred queue: the overflow records from
// the back of the buffer first (what their parts left is mostly dense cells,
// the slowest searches: started early, they do not make the kernel's tail),
// then the first pass's records from the front.
__device__ __forceinline__ DeferredRec deferred_at(const MarchArgs& a, int64_t nback, int64_t ri) {
  return ri < nback ? a.deferred[FOMO_IDX(a.deferred_cap - 1 - ri, a.deferred_cap, kSiteDeferred)]
                    : a.deferred[FOMO_IDX(ri - nback, a.deferred_cap, kSiteDeferred)];
}

// Sample k of work item `item` in the position buffer (rows of `stride`
// entries from the launch's first work item).
__device__ __forceinline__ int32_t* npos_at(const MarchArgs& a, unsigned item, int k, int stride) {
  return a.npos + FOMO_IDX(((int64_t)item - a.item_base) * stride + k, a.npos_cap, kSiteNpos);
}

// A deferred sample's result: its NN index, and its neighbour -- into the
// position buffer (POS: the emission pass bins it later, in sample order), or
// staged with its LOS speed for this kernel's own emission step (the
// no-allocation path).
template <bool POS>
__device__ __forceinline__ void store_deferred(const MarchArgs& a, const RayCtx& r, int k, int kind, int p, int o,
                                               int stride, int* sp, float* sv) {
  const ViewDesc* V = a.views + r.v;
  int32_t* nnout = a.nn_idx ? a.nn_idx[r.v] : nullptr;
  if (nnout) nnout[FOMO_IDX(((int64_t)r.i * V->nx + r.j) * V->nz + k, (int64_t)V->nx * V->ny * V->nz, kSiteNnIdx)] = o;
  if (POS) {
    *npos_at(a, r.item, k, stride) = p;
    return;
  }
  float vl = 0.0f;
  if (p >= 0 && kind == kDeferredSpectral) {
    const float4 vv = __ldg(a.snap.vel + FOMO_IDX(p, a.snap.n, kSitePts));
    vl = fmaf(V->uz, vv.z, fmaf(V->uy, vv.y, V->ux * vv.x));
  }
  *sp = p;
  *sv = vl;
}

// ---------------------------------------------------------------------------
// Overflow segments: a segment whose capsule held more than kSegCap points
// (dense clumps, long segments at a coarse LOS step) is queued by the first
// pass at the back of the deferred buffer with all its samples.  This kernel
// searches each such segment again as parts of 32 samples (16 when a part
// overflows too), each part gathering its own, shorter capsule, stores the
// neighbours of the samples it resolves (POS) or adds their emission, and
// rewrites the record with the samples still unresolved, for march_deferred.
// ---------------------------------------------------------------------------
template <bool POS>
__global__ void __launch_bounds__(kThreads, kMinCtasSplit) march_split(MarchArgs a, const double3* __restrict__ ktab,
                                                        int ktab_stride, int kind) {
  __shared__ SegSmem segs[kWarps];
  __shared__ int spos[kWarps][POS ? 1 : kSeg];
  __shared__ float svlos[kWarps][POS ? 1 : kSeg];
  const int w = threadIdx.x >> 5;
  SegSmem& sm = segs[w];
  const int lane = threadIdx.x & 31;
  const int64_t nover = min((int64_t)a.counter[kCtrOverflow], a.deferred_cap);  // written by the march
  for (;;) {
    unsigned long long k = 0;
    if (lane == 0) k = atomicAdd(a.counter + kCtrOverflowHead, 1ull);
    k = __shfl_sync(kFull, k, 0);
    if ((int64_t)k >= nover) return;
    const int64_t slot = a.deferred_cap - 1 - (int64_t)k;
    const DeferredRec rec = a.deferred[FOMO_IDX(slot, a.deferred_cap, kSiteDeferred)];
    RayCtx r;
    if (!ray_of_item(a, ktab, ktab_stride, (int64_t)rec.x, r)) continue;  // records come from real rays only
    const ViewDesc* V = a.views + r.v;
    const int nz = V->nz, s0 = (int)(rec.y & kRecS0);
    PartIn in;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int kk = s0 + lane + 32 * i;
      in.act[i] = kk < nz && (((i ? rec.w : rec.z) >> lane) & 1u);
      double p0 = 0.0, p1 = 0.0, p2 = 0.0;
      if (kk < nz) sample_pos(r, kk, p0, p1, p2);
      in.tx[i] = __double2float_rn(p0);  // the FP32 target (nn:171)
      in.ty[i] = __double2float_rn(p1);
      in.tz[i] = __double2float_rn(p2);
    }
    const PartOut o = segment_parts(a, r, s0, nz, sm, in, 32);
    // resolved samples: NN index, then the emission of those with a neighbour
    int32_t* nnout = a.nn_idx ? a.nn_idx[r.v] : nullptr;
    const int64_t ray = (int64_t)r.i * V->nx + r.j;
    int n = 0;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const bool done = in.act[i] && !o.need[i];
      if (nnout && done) nnout[FOMO_IDX(ray * nz + s0 + lane + 32 * i, (int64_t)V->nx * V->ny * nz, kSiteNnIdx)] = o.orig[i];
      if (POS) {
        if (done) *npos_at(a, rec.x, s0 + lane + 32 * i, ktab_stride) = o.pos[i];
        continue;
      }
      const bool fill = done && o.pos[i] >= 0;
      const unsigned fm = __ballot_sync(kFull, fill);
      if (fill) {
        const int d = n + __popc(fm & ((1u << lane) - 1u));
        float vl = 0.0f;
        if (kind == kDeferredSpectral) {
          const float4 vv = __ldg(a.snap.vel + FOMO_IDX(o.pos[i], a.snap.n, kSitePts));
          vl = fmaf(V->uz, vv.z, fmaf(V->uy, vv.y, V->ux * vv.x));
        }
        spos[w][d] = o.pos[i];
        svlos[w][d] = vl;
      }
      n += __popc(fm);
    }
    if (!POS) {
      __syncwarp();
      if (n > 0) add_emission(a, r, kind, spos[w], svlos[w], n);
      __syncwarp();  // the staging arrays are rewritten by the next record
    }
    const unsigned f0 = __ballot_sync(kFull, in.act[0] && o.need[0]);
    const unsigned f1 = __ballot_sync(kFull, in.act[1] && o.need[1]);
    if (lane == 0) a.deferred[FOMO_IDX(slot, a.deferred_cap, kSiteDeferred)] = make_uint4(rec.x, rec.y, f0, f1);
  }
}

// ---------------------------------------------------------------------------
// Far samples: the deferred samples of one half of a record (up to 32
// consecutive LOS samples of one ray, lane = sample) that lie half a cell or
// more outside the points' bounding box, searched together; the search pass
// flags the halves that hold kFarMin of them or more.  Such samples lie away
// from the points (wide boxes off the cloud, as Thomson's far from the
// equator): each one's own ring walk would scan every cell of the lens where
// the ball of its neighbour's distance cuts into the cloud, and consecutive
// samples scan almost the same lens.  Here each pending sample gets a ball --
// at first its distance to the points' bounding box plus three cells -- and
// each lane marks, in shared memory, the x range its ball covers in every row
// of cells it reaches; the warp then gathers those rows (the union of the
// balls), testing each gathered point against every sample's box as the
// one-lane search does.  A sample whose best point lies
// inside its own ball (gathered whole), without a near-tie, has its neighbour;
// the others take a ball through their best point, or a margin twice as wide
// when they found none, and the warp gathers again.  Samples still open after
// kFarIters gathers, near-ties and gathers beyond the row or point bounds go
// on to march_deferred as before.
// ---------------------------------------------------------------------------
constexpr int kMinCtasFar = 6;   // 24 warps per SM at <= 80 registers
constexpr int kFarRowCap = 256;  // rows of a gather's bounding rectangle (beyond: the half is left)
struct __align__(16) FarSmem {
  float4 pt[32];           // a round of gathered points
  int pp[32];              // their sorted positions
  int xlo[kFarRowCap];     // per row of the rectangle: the union of the balls' chords, as ordered ints
  int xhi[kFarRowCap];
};

// float -> int with the same order (atomicMin / atomicMax on floats)
__device__ __forceinline__ int ford(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float fdeord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// Warp-collective search of the lanes' samples (act: this lane holds one, box
// q).  Returns the lanes whose neighbour was found: pos / orig set, -1 when
// the box holds no point.
__device__ __forceinline__ unsigned far_half(const SnapDev& S, const BoxQ& q, bool act, FarSmem& fs, int& pos,
                                             int& orig) {
  const GridParams& g = S.g;
  const float h = g.h;
  const int lane = threadIdx.x & 31;
  pos = -1;
  orig = -1;
  int b0[3], b1[3], c[3];
  float gc[3];
  const bool in_grid = act && box_cells(g, q, b0, b1, c, gc);
  unsigned solved = __ballot_sync(kFull, act && !in_grid);  // the box misses the points' bounding box
  // squared distance from the target to the points' bounding box: a lower
  // bound of its neighbour's
  const float dxg = fmaxf(fmaxf(g.minx - q.tx, q.tx - g.maxx), 0.0f);
  const float dyg = fmaxf(fmaxf(g.miny - q.ty, q.ty - g.maxy), 0.0f);
  const float dzg = fmaxf(fmaxf(g.minz - q.tz, q.tz - g.maxz), 0.0f);
  const float L2 = fmaf(dzg, dzg, fmaf(dyg, dyg, dxg * dxg));
  float margin2 = 9.0f * h * h;  // the ball's margin beyond that bound, squared: three cells at first
  float r2 = L2 + margin2;
  // far samples only (half a cell or more off the points): near and inside the
  // cloud the balls' union holds too many points for every lane to test
  unsigned pend = __ballot_sync(kFull, in_grid && L2 >= kFarOut2 * h * h);
  if (__popc(pend) < kFarMin) pend = 0;
  for (int it = 0; it < kFarIters && pend; ++it) {
    const bool mine = (pend >> lane) & 1u;
    float best = FLT_MAX, second = FLT_MAX;
    int bpos = -1, borig = -1;
    // the rows this lane's ball reaches, within the box: a point of the grid
    // lies at least the target's distance to the points' bounding box away
    // along each axis, so the ball's y extent there is sqrt(r^2 - dx^2 - dz^2)
    // and its z extent sqrt(r^2 - dx^2 - dy^2), dx, dy, dz those distances
    float ylo = FLT_MAX, yhi = -FLT_MAX, zlo = FLT_MAX, zhi = -FLT_MAX;
    if (mine) {
      const float ry2 = r2 - fmaf(dzg, dzg, dxg * dxg), rz2 = r2 - fmaf(dyg, dyg, dxg * dxg);
      if (ry2 >= 0.0f && rz2 >= 0.0f) {
        const float ry = (ry2 > 0.0f ? ry2 * rsqrtf(ry2) * 1.0001f : 0.0f) + kCellMargin * h;
        const float rz = (rz2 > 0.0f ? rz2 * rsqrtf(rz2) * 1.0001f : 0.0f) + kCellMargin * h;
        ylo = fmaxf(q.ty - ry, q.loy);
        yhi = fminf(q.ty + ry, q.hiy);
        zlo = fmaxf(q.tz - rz, q.loz);
        zhi = fminf(q.tz + rz, q.hiz);
      }
    }
    ylo = warp_min(ylo);
    yhi = warp_max(yhi);
    zlo = warp_min(zlo);
    zhi = warp_max(zhi);
    bool overflow = false;
    int j0 = 0, k0 = 0, nyr = 0, nrows = 0;
    if (ylo <= yhi && zlo <= zhi) {
      j0 = cell_coord(ylo, g.oy, g.inv_h, g.dy);
      const int j1 = cell_coord(yhi, g.oy, g.inv_h, g.dy);
      k0 = cell_coord(zlo, g.oz, g.inv_h, g.dz);
      const int k1 = cell_coord(zhi, g.oz, g.inv_h, g.dz);
      nyr = j1 - j0 + 1;
      nrows = nyr * (k1 - k0 + 1);
      overflow = nrows > kFarRowCap;
      if (!overflow) {
        for (int i = lane; i < nrows; i += 32) {
          fs.xlo[i] = ford(FLT_MAX);
          fs.xhi[i] = ford(-FLT_MAX);
        }
        __syncwarp();
        if (mine) {
          // this lane's rows: where its ball reaches the grid's x range, in the rectangle
          const float rx2 = r2 - dxg * dxg;
          int z0 = k0, z1 = k1;
          clip_reach(rx2 - dyg * dyg, q.tz, g.oz, g.inv_h, h, g.dz, z0, z1);
          for (int kz = z0; kz <= z1; ++kz) {
            const float gz = axis_gap(kz, q.tz, g.oz, h);
            const float gz2 = gz * gz;
            int y0 = j0, y1 = j0 + nyr - 1;
            clip_reach(rx2 - gz2, q.ty, g.oy, g.inv_h, h, g.dy, y0, y1);
            for (int jy = y0; jy <= y1; ++jy) {
              const float gy = axis_gap(jy, q.ty, g.oy, h);
              const float rem = r2 - fmaf(gy, gy, gz2);
              if (rem >= 0.0f) {
                const float rx = (rem > 0.0f ? rem * rsqrtf(rem) * 1.0001f : 0.0f) + kCellMargin * h;
                const float xa = fmaxf(q.tx - rx, q.lox), xb = fminf(q.tx + rx, q.hix);
                if (xa <= xb) {
                  const int row = (kz - k0) * nyr + (jy - j0);
                  atomicMin(&fs.xlo[row], ford(xa));
                  atomicMax(&fs.xhi[row], ford(xb));
                }
              }
            }
          }
        }
        __syncwarp();
      }
      int npts = 0;
      const float inv_nyr = nyr > 0 ? 1.0f / (float)nyr : 0.0f;
      for (int rb = 0; rb < nrows && !overflow; rb += 32) {
        const int rr = rb + lane;
        int base = 0, n = 0;
        if (rr < nrows) {
          int ry;
          const int kz = k0 + row_div(rr, nyr, inv_nyr, ry), jy = j0 + ry;
          const float xa = fdeord(fs.xlo[rr]), xb = fdeord(fs.xhi[rr]);
          if (xa <= xb && xb >= g.minx && xa <= g.maxx) {
            const int c0 = cell_coord(xa, g.ox, g.inv_h, g.dx), c1 = cell_coord(xb, g.ox, g.inv_h, g.dx);
            const int rowbase = (kz * g.dy + jy) * g.dx;
            base = __ldg(S.cell_start + FOMO_IDX(rowbase + c0, cell_entries(g), kSiteCellStart));
            n = __ldg(S.cell_start + FOMO_IDX(rowbase + c1 + 1, cell_entries(g), kSiteCellStart)) - base;
          }
        }
        // the rows' points, 32 per round, each tested by every pending lane
        const int incl = warp_incl_scan(n);
        const int excl = incl - n;
        const int total = __shfl_sync(kFull, incl, 31);
        npts += total;
        if (npts > kFarMaxPts) {
          overflow = true;
          break;
        }
        for (int ib = 0; ib < total; ib += 32) {
          const int i = ib + lane;
          const int own = warp_owner(incl, i) & 31;
          const int ob = __shfl_sync(kFull, base, own), oe = __shfl_sync(kFull, excl, own);
          if (i < total) {
            const int p = ob + (i - oe);
            fs.pt[lane] = __ldg(S.pts + FOMO_IDX(p, S.n, kSitePts));
            fs.pp[lane] = p;
          }
          __syncwarp();
          const int cn = min(32, total - ib);
          if (mine) {
            // every point of the round against this lane's best and box (the
            // same test as scan_point); four at a time, their distances independent
#pragma unroll 4
            for (int k = 0; k < cn; ++k) {
              const float4 v = fs.pt[k];
              const float dx = v.x - q.tx, dy = v.y - q.ty, dz = v.z - q.tz;
              const float d = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
              // rare once the lane has two in-box points: kept a branch around the box test
              if (__builtin_expect(d < second, 0)) {
                if (v.x > q.lox && v.x < q.hix && v.y > q.loy && v.y < q.hiy && v.z > q.loz && v.z < q.hiz) {
                  if (d < best) {
                    second = best;
                    best = d;
                    bpos = fs.pp[k];
                    borig = __float_as_int(v.w);
                  } else {
                    second = d;
                  }
                }
              }
            }
          }
          __syncwarp();  // the round's points are rewritten by the next
        }
      }
    }
    if (overflow) break;
    // found: the best point lies inside the ball, which was gathered whole;
    // a near-tie (FP64 re-rank) is left to the lane walk
    const bool found = mine && best < FLT_MAX && best <= r2 * (1.0f - 2.0f * kRelPrune);
    const bool tie = found && second <= best * (1.0f + kRelTie);
    if (found && !tie) {
      pos = bpos;
      orig = borig;
    }
    solved |= __ballot_sync(kFull, found && !tie);
    margin2 *= 4.0f;
    if (mine && !found) r2 = best < FLT_MAX ? best * (1.0f + 1e-4f) : L2 + margin2;
    pend = __ballot_sync(kFull, mine && !found);
    __syncwarp();  // the lanes' balls are rewritten by the next gather
  }
  return solved;
}

// The far pass over the deferred records the search listed (a.far_list, read
// after march_split), a warp per record: each flagged half with at least
// kFarMin samples left is searched by far_half.  The neighbours go to the
// position buffer and the record keeps the samples still open, for
// march_deferred.
__global__ void __launch_bounds__(kThreads, kMinCtasFar) march_far(MarchArgs a, const double3* __restrict__ ktab,
                                                                   int ktab_stride, int kind) {
  __shared__ FarSmem fsm[kWarps];
  const int w = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  // the records the search flagged, listed by their slots
  const int64_t nlist = min((int64_t)a.counter[kCtrFar], a.deferred_cap);
  if (!a.far_list || nlist == 0) return;
  for (;;) {
    // 32 list entries per grab (one atomic per warp and batch); their records one after the other
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(a.counter + kCtrFarHead, 32ull);
    base = __shfl_sync(kFull, base, 0);
    if ((int64_t)base >= nlist) return;
    const int64_t kk = (int64_t)base + lane;
    long long mslot = -1;
    DeferredRec mrec = make_uint4(0u, 0u, 0u, 0u);
    if (kk < nlist) {
      mslot = a.far_list[FOMO_IDX(kk, a.deferred_cap, kSiteDeferred)];
      mrec = a.deferred[FOMO_IDX(mslot, a.deferred_cap, kSiteDeferred)];
    }
    unsigned todo = __ballot_sync(kFull, mslot >= 0);
    while (todo) {
      const int src = __ffs(todo) - 1;
      todo &= todo - 1u;
      const long long slot = __shfl_sync(kFull, mslot, src);
      DeferredRec rec;
      rec.x = __shfl_sync(kFull, mrec.x, src);
      rec.y = __shfl_sync(kFull, mrec.y, src);
      rec.z = __shfl_sync(kFull, mrec.z, src);
      rec.w = __shfl_sync(kFull, mrec.w, src);
      RayCtx r;
      if (!ray_of_item(a, ktab, ktab_stride, (int64_t)rec.x, r)) continue;  // records come from real rays only
#pragma unroll 1
      for (int hh = 0; hh < 2; ++hh) {
        unsigned mask = hh ? rec.w : rec.z;
        if (!(rec.y & (hh ? kRecFar1 : kRecFar0)) || __popc(mask) < kFarMin) continue;
        const int ks = (int)(rec.y & kRecS0) + 32 * hh + lane;
        const bool act = ((mask >> lane) & 1u) && ks < r.nz;
        BoxQ q = {};
        if (act) q = exact_box(r, ks);
        int pos = -1, orig = -1;
        const unsigned solved = far_half(a.snap, q, act, fsm[w], pos, orig) & mask;
        if (act && ((solved >> lane) & 1u))
          store_deferred<true>(a, r, ks, kind, pos, orig, ktab_stride, nullptr, nullptr);
        if (a.stats && lane == 0) {
          atomicAdd(a.stats + kStatFarGroups, 1ull);
          atomicAdd(a.stats + kStatFar, (unsigned long long)__popc(solved));
        }
        mask &= ~solved;
        if (hh)
          rec.w = mask;
        else
          rec.z = mask;
      }
      if (lane == 0) a.deferred[FOMO_IDX(slot, a.deferred_cap, kSiteDeferred)] = rec;
    }
  }
}

// Phase 1 of march_deferred: samples [0, nsamp) of the staged records, one
// per lane, each searched by its lane; results staged in sp / sv.  With
// BUDGET (a short queue: latency matters), a sample in dense cells or over the
// budget goes to the hard queue (a whole warp searches it in march_hard) and
// adds nothing here.  A long queue has no budget: 32 lanes on 32 samples keep
// more loads in flight than a warp on one, and its walk has no budget checks.
template <bool BUDGET, bool POS>
__device__ __forceinline__ void deferred_search(const MarchArgs& a, int kind, int nsamp, int start, int incl,
                                                int excl, const DeferredRec& rec, const RayCtx& mine, int stride,
                                                int* sp, float* sv) {
  const int lane = threadIdx.x & 31;
  for (int t0 = 0; t0 < nsamp; t0 += 32) {
    const int t = t0 + lane;
    const int own = warp_owner(incl, start + t) & 31;  // the record lane holding flattened sample t
    const unsigned oy = __shfl_sync(kFull, rec.y & kRecS0, own);
    const unsigned oz = __shfl_sync(kFull, rec.z, own), ow = __shfl_sync(kFull, rec.w, own);
    const int oe = __shfl_sync(kFull, excl, own);
    const RayCtx r = shfl_ray(mine, own);
    bool hard = false;
    int k = 0, p = -1, o = -1;
    if (t < nsamp) {
      k = (int)oy + nth_set_bit(oz, ow, start + t - oe);
      hard = !lane_search<BUDGET>(a.snap, exact_box(r, k), p, o);
    }
    if (BUDGET) {
      const unsigned hm = __ballot_sync(kFull, hard);
      unsigned long long hb = 0;
      if (hm && lane == 0) hb = atomicAdd(a.counter + kCtrHard, (unsigned long long)__popc(hm));
      hb = __shfl_sync(kFull, hb, 0);
      if (hard) {
        const int64_t slot = (int64_t)hb + __popc(hm & ((1u << lane) - 1u));
        if (slot < a.hard_cap) {
          a.hard[FOMO_IDX(slot, a.hard_cap, kSiteHard)] = make_uint2(r.item, (unsigned)k);
          p = -1;  // its neighbour and emission come from march_hard
        } else {
          lane_search_full(a.snap, exact_box(r, k), p, o);  // queue full: finish here
          hard = false;
        }
      }
      if (a.stats && hm && lane == 0) atomicAdd(a.stats + kStatHard, (unsigned long long)__popc(hm));
    }
    if (t < nsamp) {
      if (hard) {
        // its neighbour comes from march_hard (the position buffer keeps the
        // search pass's -1 until then)
        if (!POS) {
          sp[t] = -1;
          sv[t] = 0.0f;
        }
      } else {
        store_deferred<POS>(a, r, k, kind, p, o, stride, sp + t, sv + t);
      }
    }
  }
}

// POS: the neighbours go to the position buffer and the emission pass that
// runs after this kernel bins them; otherwise (the no-allocation path) this
// kernel adds their emission to the already written cube with atomics.
template <bool POS>
__global__ void __launch_bounds__(kThreads, kMinCtasDeferred) march_deferred(MarchArgs a, const double3* __restrict__ ktab,
                                                           int ktab_stride, int kind) {
  __shared__ int spos[kWarps][POS ? 1 : kDefBatch];    // neighbour (sorted position) of each staged sample
  __shared__ float svlos[kWarps][POS ? 1 : kDefBatch]; // and its LOS speed (spectral)
  const int w = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  // written by the march and march_split; the two ends of the buffer never meet
  // (at most one record per segment)
  const int64_t nfront = min((int64_t)a.counter[kCtrDeferred], a.deferred_cap);
  const int64_t nback = min((int64_t)a.counter[kCtrOverflow], a.deferred_cap - nfront);
  const int64_t nrec = nfront + nback;
  // records per grab: 32, or fewer when the queue is short, so that every
  // warp of the grid gets a share (a small render has few records)
  const int64_t nwarps = (int64_t)gridDim.x * kWarps;
  const int grab = (int)max((int64_t)1, min((int64_t)32, nrec / nwarps));
  // a short queue (a small render: latency matters) takes the budgeted search
  const bool budgeted = a.hard_cap > 0 && nrec < 256 * nwarps;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(a.counter + kCtrDeferredHead, (unsigned long long)grab);
    base = __shfl_sync(kFull, base, 0);
    if ((int64_t)base >= nrec) return;
    const int64_t ri = (int64_t)base + lane;
    DeferredRec rec = make_uint4(0u, 0u, 0u, 0u);
    if (lane < grab && ri < nrec) rec = deferred_at(a, nback, ri);
    const int cnt = __popc(rec.z) + __popc(rec.w);
    const int incl = warp_incl_scan(cnt);
    const int excl = incl - cnt;
    const int total = __shfl_sync(kFull, incl, 31);  // every lane takes part in the shuffle
    if (a.stats && lane == 0) atomicAdd(a.stats + kStatFbUnion, (unsigned long long)total);
    // each lane decodes its own record's ray once (view, pixel, FP64 ray terms)
    RayCtx mine{};
    if (cnt > 0) ray_of_item(a, ktab, ktab_stride, (int64_t)rec.x, mine);  // records come from real rays only
    for (int r0 = 0; r0 < 32;) {
      // records r0 .. r1-1 whose samples fit the staging arrays (a record has <= 64)
      const int start = __shfl_sync(kFull, excl, r0);
      const unsigned fits = __ballot_sync(kFull, lane >= r0 && incl - start <= kDefBatch);
      const int r1 = r0 + max(__popc(fits), 1);
      const int nsamp = __shfl_sync(kFull, incl, r1 - 1) - start;
      // 1. one sample per lane: its record, ray and box, then its own search
      if (budgeted)
        deferred_search<true, POS>(a, kind, nsamp, start, incl, excl, rec, mine, ktab_stride, spos[w], svlos[w]);
      else
        deferred_search<false, POS>(a, kind, nsamp, start, incl, excl, rec, mine, ktab_stride, spos[w], svlos[w]);
      if (!POS) {
        __syncwarp();
        // 2. their emission, record by record
        for (int rr = r0; rr < r1; ++rr) {
          const int sn = __shfl_sync(kFull, cnt, rr);
          const int so = __shfl_sync(kFull, excl, rr) - start;
          const RayCtx r = shfl_ray(mine, rr);
          if (sn > 0) add_emission(a, r, kind, spos[w] + so, svlos[w] + so, sn);
        }
        __syncwarp();  // the staging arrays are rewritten by the next batch
      }
      r0 = r1;
    }
  }
}

// ---------------------------------------------------------------------------
// Hard samples: deferred samples whose one-lane search ran out of budget
// (dense cells, or a wide box reaching far from the points).  One warp per
// sample, from a queue shared by the whole grid: the rows and points of each
// ring are spread over the lanes (warp_search).  The warp writes the NN index
// and stores the neighbour in the position buffer (POS) or adds the sample's
// emission with atomics.
// ---------------------------------------------------------------------------
template <bool POS>
__global__ void __launch_bounds__(kThreads, kMinCtas) march_hard(MarchArgs a, const double3* __restrict__ ktab,
                                                       int ktab_stride, int kind) {
  __shared__ int sp[kWarps];
  __shared__ float sv[kWarps];
  const int w = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t n = min((int64_t)a.counter[kCtrHard], a.hard_cap);  // written by march_deferred
  for (;;) {
    unsigned long long i = 0;
    if (lane == 0) i = atomicAdd(a.counter + kCtrHardHead, 1ull);
    i = __shfl_sync(kFull, i, 0);
    if ((int64_t)i >= n) return;
    const uint2 hs = a.hard[FOMO_IDX(i, a.hard_cap, kSiteHard)];
    RayCtx r;
    if (!ray_of_item(a, ktab, ktab_stride, (int64_t)hs.x, r)) continue;  // queued from real rays only
    int p, o;
    warp_search(a.snap, exact_box(r, (int)hs.y), p, o);
    if (lane == 0) store_deferred<POS>(a, r, (int)hs.y, kind, p, o, ktab_stride, sp + w, sv + w);
    if (!POS) {
      __syncwarp();
      if (p >= 0) add_emission(a, r, kind, sp + w, sv + w, 1);
      __syncwarp();  // sp / sv are rewritten by the next sample
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
  int64_t blocks = (int64_t)sm_count * per_sm;
  const int64_t cap = (a.total_items - a.item_base + kWarps - 1) / kWarps;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  kernel<<<(unsigned)blocks, kThreads, 0, s>>>(a, ktab, ktab_stride);
  return cudaGetLastError();
}

// A persistent grid over a queue whose length is known on the device only (it
// drains the queue and exits at once when it is empty).
template <typename K>
cudaError_t launch_queue(K kernel, const MarchArgs& a, const double3* ktab, int ktab_stride, int sm_count,
                         cudaStream_t s, int kind) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  kernel<<<(unsigned)(sm_count * per_sm), kThreads, 0, s>>>(a, ktab, ktab_stride, kind);
  return cudaGetLastError();
}

// The kernel that bins the emission from the position buffer (after every
// search pass has stored its neighbours).
cudaError_t launch_emission_pass(const MarchArgs& a, const double3* ktab, int ktab_stride, int max_windows,
                                 int sm_count, cudaStream_t s, bool imaging) {
  if (a.s2) return launch_persistent(march_imaging<1, true, true>, a, ktab, ktab_stride, sm_count, s, 0);
  if (imaging) {
    if (a.nlines <= 1) return launch_persistent(march_imaging<1, false, true>, a, ktab, ktab_stride, sm_count, s, 0);
    if (a.nlines <= 2) return launch_persistent(march_imaging<2, false, true>, a, ktab, ktab_stride, sm_count, s, 0);
    if (a.nlines <= 4) return launch_persistent(march_imaging<4, false, true>, a, ktab, ktab_stride, sm_count, s, 0);
    if (a.nlines <= 8) return launch_persistent(march_imaging<8, false, true>, a, ktab, ktab_stride, sm_count, s, 0);
    return cudaErrorInvalidValue;
  }
  const int nb = max_windows < 1 ? 1 : max_windows;
#define FOMO_SHADE(NL_, NB_) \
  if (a.nlines <= NL_ && nb <= NB_) return launch_persistent(march_spectral<NL_, NB_, true>, a, ktab, ktab_stride, sm_count, s, 0)
  FOMO_SHADE(1, 1);
  FOMO_SHADE(1, 2);
  FOMO_SHADE(1, 4);
  FOMO_SHADE(1, 8);
  FOMO_SHADE(2, 1);
  FOMO_SHADE(2, 2);
  FOMO_SHADE(2, 4);
  FOMO_SHADE(4, 1);
  FOMO_SHADE(4, 2);
  FOMO_SHADE(4, 4);
#undef FOMO_SHADE
  return cudaErrorInvalidValue;
}

// The fused first pass of the no-allocation path: search and emission in one
// kernel (no position buffer).
cudaError_t launch_fused_pass(const MarchArgs& a, const double3* ktab, int ktab_stride, int max_windows,
                              int sm_count, cudaStream_t s, int blocks_per_sm_hint, bool imaging) {
  if (a.s2) return launch_persistent(march_imaging<1, true, false>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint);
  if (imaging) {
    if (a.nlines <= 1) return launch_persistent(march_imaging<1, false, false>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint);
    if (a.nlines <= 2) return launch_persistent(march_imaging<2, false, false>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint);
    if (a.nlines <= 4) return launch_persistent(march_imaging<4, false, false>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint);
    if (a.nlines <= 8) return launch_persistent(march_imaging<8, false, false>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint);
    return cudaErrorInvalidValue;
  }
  const int nb = max_windows < 1 ? 1 : max_windows;
#define FOMO_SPEC(NL_, NB_) \
  if (a.nlines <= NL_ && nb <= NB_) return launch_persistent(march_spectral<NL_, NB_, false>, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint)
  FOMO_SPEC(1, 1);
  FOMO_SPEC(1, 2);
  FOMO_SPEC(1, 4);
  FOMO_SPEC(1, 8);
  FOMO_SPEC(2, 1);
  FOMO_SPEC(2, 2);
  FOMO_SPEC(2, 4);
  FOMO_SPEC(4, 1);
  FOMO_SPEC(4, 2);
  FOMO_SPEC(4, 4);
#undef FOMO_SPEC
  return cudaErrorInvalidValue;
}

}  // namespace

FOMO_DEFINE_CHECK_READER(check_word_march)

int march_bins_per_lane(int nlines, int L) {
  (void)nlines;
  return (L + 31) / 32;
}

// max_windows: largest number of 32-bin lambda windows of any line (1 for imaging).
//
// With a position buffer (a.npos): the search stores every sample's neighbour,
// the split, deferred and hard passes store the neighbours of the samples it
// left, and the emission pass then bins every ray from the buffer in sample
// order.  One warp owns one ray there and nothing is added with atomics, so a
// cube is the same bits whatever else shares the launch.  Without one (the
// no-allocation path): the fused first pass searches and bins, and the later
// passes add the deferred samples' emission with atomics.
cudaError_t launch_march(const MarchArgs& a, const double3* ktab, int ktab_stride, int max_windows, int sm_count,
                         cudaStream_t s, int blocks_per_sm_hint, bool imaging, MarchTimer* timer) {
  if (!a.deferred || a.deferred_cap <= 0 || !a.counter) return cudaErrorInvalidValue;
  const int kind = a.s2 ? kDeferredThomson : (imaging ? kDeferredImaging : kDeferredSpectral);
  auto mark = [&](int k) {
    if (timer) timer->mark(s, k);
  };
  mark(-1);
  cudaError_t e;
  if (a.npos) {
    e = launch_persistent(march_search, a, ktab, ktab_stride, sm_count, s, blocks_per_sm_hint);
    mark(kKSearch);
    if (e == cudaSuccess) e = launch_queue(march_split<true>, a, ktab, ktab_stride, sm_count, s, kind);
    mark(kKSplit);
    if (e == cudaSuccess) e = launch_queue(march_far, a, ktab, ktab_stride, sm_count, s, kind);
    mark(kKFar);
    if (e == cudaSuccess) e = launch_queue(march_deferred<true>, a, ktab, ktab_stride, sm_count, s, kind);
    mark(kKDeferred);
    if (e == cudaSuccess && a.hard_cap > 0) e = launch_queue(march_hard<true>, a, ktab, ktab_stride, sm_count, s, kind);
    mark(kKHard);
    if (e == cudaSuccess) e = launch_emission_pass(a, ktab, ktab_stride, max_windows, sm_count, s, imaging);
    mark(kKEmission);
    return e;
  }
  e = launch_fused_pass(a, ktab, ktab_stride, max_windows, sm_count, s, blocks_per_sm_hint, imaging);
  mark(kKFused);
  if (e == cudaSuccess) e = launch_queue(march_split<false>, a, ktab, ktab_stride, sm_count, s, kind);
  mark(kKSplit);
  if (e == cudaSuccess) e = launch_queue(march_deferred<false>, a, ktab, ktab_stride, sm_count, s, kind);
  mark(kKDeferred);
  if (e == cudaSuccess && a.hard_cap > 0) e = launch_queue(march_hard<false>, a, ktab, ktab_stride, sm_count, s, kind);
  mark(kKHard);
  return e;
}

}  // namespace fomo
