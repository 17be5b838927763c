// Internal structures shared by the CUDA kernels and the host runtime of
// libfomo_gpu.  Nothing here is part of the public C ABI (include/fomo_gpu.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fomo_consts.h"

namespace fomo {

// ---------------------------------------------------------------------------
// Snapshot: the point cloud, sorted into a uniform grid (cell-major, x fastest)
// ---------------------------------------------------------------------------
struct GridParams {
  float ox, oy, oz;     // grid origin = AABB minimum of the points
  float h, inv_h;       // cell edge (Mm) and its FP32 reciprocal used for binning
  int dx, dy, dz;       // cells per axis
  float minx, miny, minz, maxx, maxy, maxz;  // exact AABB of the points (FP32)
};

struct SnapDev {
  int64_t n;
  const float4* pts;    // sorted: x, y, z (FP32 Mm), original index (int bits)
  const float4* vel;    // sorted: vx, vy, vz (m/s), 0
  const int* cell_start;  // dx*dy*dz + 1 slots
  GridParams g;
  const float* blk;     // per block of kBlockCells^3 cells: its points' min x, y, z and max x, y, z
  int bdx, bdy, bdz;    // blocks per axis
};
constexpr int kBlockCells = 8;  // cells per block edge (per-block bounding boxes of a snapshot)

// ---------------------------------------------------------------------------
// One view (l, b) of one snapshot.  Host fills the first block (trig values
// come from the host libm, as in the reference); the device fills the rest.
// ---------------------------------------------------------------------------
enum Method : int { kMethodNN = 0, kMethodThomson = 1, kMethodProjection = 2 };

struct ViewDesc {
  // ---- host-filled
  double cb, sb, cl, sl;     // derotation cos/sin (unclamped)
  double rcb, rsb;           // rotation used for the extents (Thomson clamps)
  double blend;              // Thomson pole blend (fomo-thomson.cpp:176), 0 for NN
  double mdblend;            // Thomson maxdistance blend (fomo-thomson.cpp:249)
  double lambda_width;       // m/s
  double lambda0;            // table lambda0 of the primary line (Angstrom)
  int nx, ny, nz, L;
  int method;
  int is_dn;
  int ray_tile_w, ray_tile_h;  // ray tile shape for the march work order
  // ---- device-filled by the extents + finalize kernels
  unsigned long long ext_bits[6];  // order-preserving encodings for atomic min/max
  int bnd[6];                // per rotated axis: the largest lower bound of a block's values and the smallest
                             // upper bound (order-preserving float encodings), which bound the extremes
  double minx, maxx, miny, maxy, minz, maxz;
  double md;                 // maxdistance
  double deltaz;
  double pathlength;
  double apix;               // DN pixel area (nn:261-262); applied to lines with a DN unit
  double scale;              // pathlength * 1e8            (non-DN lines)
  double scale_dn;           // pathlength * 1e8 * apix     (DN lines)
  double lwa;                // lambda_width in Angstrom (primary line)
  double dxr, dyr;           // (maxx-minx), (maxy-miny) as the reference evaluates them
  double* xt;                // nx ray x positions j/(nx-1)*(maxx-minx)+minx (device, filled by finalize)
  double* yt;                // ny ray y positions
  float ux, uy, uz;          // LOS unit vector in FP32 for the Doppler term
  int pad0;
};

// One spectral line (or broadband channel) rendered with a view.
struct LineDesc {
  const float2* ew;          // sorted per-point (eps, fwhm)
  float* out;                // device cube, (ny*nx*L) floats, L fastest
  const float* lam;          // L relative wavelengths lambdaval (nn:200), FP64 on host -> FP32
  double lambda0;
  double lwa;                // lambda_width * lambda0 / c (Angstrom)
  float shift_k;             // lambda0 / c in FP32 (Doppler shift per m/s)
  int is_dn;                 // unit contains "DN": per-pixel scaling
  int wstart;                // first lambda bin of the evaluated window
  int nw;                    // 32-bin windows evaluated; other bins are below 2^-64 of every peak
};

// Work counters of one march (zeroed before it): the ray queue head, the number
// of deferred-sample records written from the front of the buffer, the
// deferred-record queue head, the number of overflow records written from the
// back (segments whose capsule held too many points), their queue head, the
// number of hard samples queued for a warp each, their queue head, the ray
// queue head of the emission pass of the two-pass spectral march, the number
// of records flagged for the far pass and its queue head.
enum MarchCounter {
  kCtrRays = 0, kCtrDeferred, kCtrDeferredHead, kCtrOverflow, kCtrOverflowHead, kCtrHard, kCtrHardHead, kCtrShade,
  kCtrFar, kCtrFarHead,
  kCtrCount
};

// One segment whose samples the march's first search pass could not resolve:
// x = work item of the ray, y = first LOS sample of the segment (bits 0-29;
// bits 30 and 31 flag the halves the far pass may take), z/w = masks of the
// unresolved samples y + lane and y + 32 + lane.
using DeferredRec = uint4;

struct MarchArgs {
  SnapDev snap;
  ViewDesc* views;           // nviews
  const int64_t* ray_offset; // nviews + 1, prefix sums of work items per view
  const LineDesc* lines;     // nviews * nlines
  int nviews;
  int nlines;
  int64_t item_base;         // first work item of this launch (item ranges of one plan)
  int64_t total_items;       // one past the last work item
  unsigned long long* counter;   // kCtrCount work counters, zeroed before the launch
  DeferredRec* deferred;         // one record per segment at most: capacity deferred_cap
  int64_t deferred_cap;
  int32_t* far_list;             // slots of the records flagged for the far pass (capacity deferred_cap), or null
  uint2* hard;                   // deferred samples (work item, sample) for a whole warp each, or null
  int64_t hard_cap;              // its capacity (0: every deferred sample is searched by one lane)
  int32_t* const* nn_idx;        // per view (nullable array / entries), [ray][nz] original index
  int32_t* npos;                 // neighbour per (work item - item_base, sample), or null (the fused no-allocation march)
  int64_t npos_cap;              // its entries (index checks of the bounds-check build)
  const float* s2;               // Thomson: per-view sin^2(chi) per sorted point (nviews * n), else null
  const float2* totpol;          // Thomson: sorted (n*totterm, n*polterm)
  float rscale;                  // gather radius of the search in local point spacings (0: the default, 0.9)
  unsigned long long* stats;     // optional search counters (profiling), else null
  const unsigned* stop;          // a server batch's stop word (device memory), or null: once it is
                                 // set, the ray-queue kernels take no further rays
};

// Search counters accumulated when MarchArgs::stats is set.
enum MarchStat {
  kStatSegments = 0,   // 64-sample segments searched
  kStatCandidates,     // candidates gathered
  kStatRows,           // cell rows visited by the gather
  kStatPointsLoaded,   // points loaded by the gather
  kStatNotGathered,    // segment parts split in halves (too many rows or candidates for one part)
  kStatFallbacks,      // samples resolved by the per-lane ring search
  kStatSamples,        // LOS samples searched
  kStatScanned,        // candidates scanned by samples
  kStatTies,           // samples re-ranked in FP64
  kStatFbNoCand,       // fallback reason: no in-box candidate within the coverage radius
  kStatFbFar,          // fallback reason: best candidate beyond the coverage radius
  kStatFbAmb,          // fallback reason: a candidate within a few ulp of a box face
  kStatFbUnion,        // samples searched by the deferred pass
  kStatDeferredRecs,   // deferred-sample records (segments with fallback samples)
  kStatHard,           // deferred samples whose one-lane search ran out of budget (searched by a warp)
  kStatRuns,           // runs of equal neighbours binned by the spectral emission pass (with a neighbour)
  kStatEx2,            // ex2 evaluations of the spectral emission pass (32 per run, line and 32-bin window)
  kStatFarGroups,      // record halves searched together by the far pass
  kStatFar,            // deferred samples the far pass resolved
  kStatCount
};

// Kernels of one march, for optional per-kernel timing (direct launches
// only): events recorded on the stream after each kernel, tagged with its kind.
enum MarchKernel : int { kKSearch = 0, kKSplit, kKDeferred, kKHard, kKEmission, kKFused, kKFar, kKCount };
struct MarchTimer {
  cudaEvent_t* ev = nullptr;  // pool of `cap` events
  int* kind = nullptr;        // kind of the kernel that ends at ev[i]; -1 marks a start
  int cap = 0, n = 0;
  // record the next event (false when the pool is full: timing stops there)
  bool mark(cudaStream_t s, int k) {
    if (n >= cap) return false;
    if (cudaEventRecord(ev[n], s) != cudaSuccess) return false;
    kind[n++] = k;
    return true;
  }
};

// ---------------------------------------------------------------------------
// Kernel launchers (defined in the .cu files)
// ---------------------------------------------------------------------------
// index.cu
cudaError_t launch_aabb(const float* x, const float* y, const float* z, int64_t n, unsigned int* bits6,
                        cudaStream_t s);
cudaError_t launch_bin_points(const float* x, const float* y, const float* z, int64_t n, GridParams g,
                              int* cell_of, int* counts, cudaStream_t s);
cudaError_t launch_block_bounds(const float4* pts, const int* cell_start, GridParams g, int bdx, int bdy, int bdz,
                                float* blk, cudaStream_t s);
cudaError_t launch_count_empty(const int* counts, int64_t ncells, unsigned long long* empty, cudaStream_t s);
cudaError_t launch_exclusive_scan(const int* in, int* out, int64_t count, int* scratch, int64_t scratch_ints,
                                  cudaStream_t s);
int64_t exclusive_scan_scratch_ints(int64_t count);
cudaError_t launch_scatter(const float* x, const float* y, const float* z, const float* vx, const float* vy,
                           const float* vz, const float* ne, const float* T, int64_t n, const int* cell_of,
                           const int* cell_start, int* fill, float4* pts, float4* vel, float* ne_s, float* T_s,
                           cudaStream_t s);
cudaError_t launch_sort_cells(const int* cell_start, int64_t ncells, float4* pts, float4* vel, float* ne_s,
                              float* T_s, cudaStream_t s);

// emission.cu
struct TableDev {
  int nt, nrho;
  const float* logT;   // nt
  const float* logn;   // nrho
  const float* G;      // nrho * nt
  double cw;           // linefwhm constant (fomo-CHIANTI.cpp:224)
  double k;            // normaliseconst * abundratio
  int imaging;
};
cudaError_t launch_emission(const float* ne_s, const float* T_s, int64_t n, TableDev t, float2* ew, cudaStream_t s);
cudaError_t launch_thomson_emission(const float4* pts, const float* ne_s, int64_t n, float2* totpol,
                                    cudaStream_t s);
cudaError_t launch_unsort_payload(const float4* pts, const float2* ew, int64_t n, float* a, float* b,
                                  cudaStream_t s);
cudaError_t launch_payload_stats(const float2* ew, int64_t n, unsigned int* wmax_bits, cudaStream_t s);
cudaError_t launch_speed_max(const float4* vel, int64_t n, unsigned int* vmax_bits, cudaStream_t s);

// view.cu
cudaError_t launch_view_init(ViewDesc* views, int nviews, cudaStream_t s);
cudaError_t launch_view_extents(SnapDev snap, ViewDesc* views, int nviews, float* s2, cudaStream_t s);
cudaError_t launch_view_finalize(ViewDesc* views, int nviews, double3* ktab, int ktab_stride, cudaStream_t s);

// projection.cu: the projection render of every view of a group (outputs zeroed beforehand)
cudaError_t launch_projection(SnapDev snap, const ViewDesc* views, const LineDesc* lines, int nviews, int nlines,
                              bool imaging, int sm_count, cudaStream_t s);

// Readers of each file's bounds-check error word (fomo_device.cuh): read and
// clear on the current device; a non-zero word is the site of the first index
// out of range.
cudaError_t check_word_march(unsigned* out);
cudaError_t check_word_index(unsigned* out);
cudaError_t check_word_view(unsigned* out);
cudaError_t check_word_emission(unsigned* out);
cudaError_t check_word_projection(unsigned* out);
cudaError_t check_word_amrvac(unsigned* out);

// march.cu
// The march: the first search pass and the emission sums of every ray, then
// the deferred samples' nearest neighbours and their contributions (a second
// kernel on the same stream).
cudaError_t launch_march(const MarchArgs& a, const double3* ktab, int ktab_stride, int max_windows, int sm_count,
                         cudaStream_t s, int blocks_per_sm_hint, bool imaging, MarchTimer* timer = nullptr);
int march_bins_per_lane(int nlines, int L);
// Capacity of the deferred-record queue for `items` work items of up to nz samples.
inline int64_t deferred_capacity(int64_t items, int nz) { return items * ((nz + 63) / 64); }
// Hard-sample queue of a launch: up to 2^20 entries (8 MB); when it is full a
// lane finishes its search on its own.
inline int64_t hard_capacity(int64_t items, int nz) {
  const int64_t n = items * (int64_t)nz;
  return n < (int64_t(1) << 20) ? n : (int64_t(1) << 20);
}

}  // namespace fomo
