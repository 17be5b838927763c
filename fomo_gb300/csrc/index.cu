// K2: spatial index of a snapshot (replaces the Boost rtree of
// fomo-c/src/fomo-nearestneighbour.cpp:93-100, which the reference rebuilds
// for every view although it indexes the unrotated points).
//
// The points are binned into a uniform grid over their AABB and counting-
// sorted into cell-major order (x fastest), so that a row of cells along x
// is one contiguous range of points.  Each point is stored as a float4
// (x, y, z, original index) -- 16 B, one aligned load per candidate in the
// march -- next to its velocity float4.  Within a cell, points are ordered by
// original index so the layout is deterministic.  The index is built once per
// snapshot and stays resident.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "fomo_device.cuh"
#include "fomo_internal.h"

namespace fomo {

namespace {

__device__ __forceinline__ unsigned int f2ord(float f) {
  unsigned int u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void aabb_kernel(const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ z,
                            int64_t n, unsigned int* bits6) {
  unsigned int mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu};
  unsigned int mx[3] = {0u, 0u, 0u};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    unsigned int v[3] = {f2ord(x[i]), f2ord(y[i]), f2ord(z[i])};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      mn[d] = min(mn[d], v[d]);
      mx[d] = max(mx[d], v[d]);
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn[d] = min(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
      mx[d] = max(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      atomicMin(&bits6[d], mn[d]);
      atomicMax(&bits6[3 + d], mx[d]);
    }
  }
}

__global__ void bin_kernel(const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ z,
                           int64_t n, GridParams g, int* __restrict__ cell_of, int* __restrict__ counts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int cx = cell_coord(x[i], g.ox, g.inv_h, g.dx);
    int cy = cell_coord(y[i], g.oy, g.inv_h, g.dy);
    int cz = cell_coord(z[i], g.oz, g.inv_h, g.dz);
    int c = (cz * g.dy + cy) * g.dx + cx;
    cell_of[i] = c;
    atomicAdd(&counts[FOMO_IDX(c, (int64_t)g.dx * g.dy * g.dz, kSiteIndexBuild)], 1);
  }
}

// ---- three-phase exclusive scan over int32 counts (sum fits in int32: n < 2^31)
constexpr int kScanThreads = 1024;
constexpr int kScanPerThread = 4;
constexpr int kScanTile = kScanThreads * kScanPerThread;

__device__ __forceinline__ int block_exclusive_scan(int v, int* sh, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) sh[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    sh[lane] = wi - w;
    if (lane == 31) sh[32] = wi;
  }
  __syncthreads();
  int res = incl - v + sh[warp];
  *total = sh[32];
  __syncthreads();
  return res;
}

__global__ void scan_tile_sums(const int* __restrict__ in, int64_t count, int* __restrict__ sums) {
  __shared__ int sh[33];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPerThread;
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k)
    if (base + k < count) s += in[base + k];
  int total;
  block_exclusive_scan(s, sh, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void scan_sums_single(int* __restrict__ sums, int64_t nsums) {
  __shared__ int sh[33];
  int64_t per = (nsums + blockDim.x - 1) / blockDim.x;
  int64_t b = threadIdx.x * per;
  int local = 0;
  for (int64_t k = 0; k < per; ++k)
    if (b + k < nsums) local += sums[b + k];
  int total;
  int off = block_exclusive_scan(local, sh, &total);
  for (int64_t k = 0; k < per; ++k) {
    if (b + k < nsums) {
      int v = sums[b + k];
      sums[b + k] = off;
      off += v;
    }
  }
}

__global__ void scan_tiles(const int* __restrict__ in, int64_t count, const int* __restrict__ sums,
                           int* __restrict__ out) {
  __shared__ int sh[33];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPerThread;
  int v[kScanPerThread];
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k) {
    v[k] = (base + k < count) ? in[base + k] : 0;
    s += v[k];
  }
  int total;
  int off = block_exclusive_scan(s, sh, &total) + sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k) {
    if (base + k < count) out[base + k] = off;
    off += v[k];
  }
}

__global__ void scatter_kernel(const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ z,
                               const float* __restrict__ vx, const float* __restrict__ vy,
                               const float* __restrict__ vz, const float* __restrict__ ne,
                               const float* __restrict__ T, int64_t n, const int* __restrict__ cell_of,
                               const int* __restrict__ cell_start, int* __restrict__ fill, float4* __restrict__ pts,
                               float4* __restrict__ vel, float* __restrict__ ne_s, float* __restrict__ T_s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    // cell_of < cells by construction (bin_kernel clamps every coordinate); its
    // capacity is the number of points, which also bounds every position
    int c = cell_of[i];
    int pos = FOMO_IDX(cell_start[c] + atomicAdd(&fill[c], 1), n, kSiteIndexBuild);
    pts[pos] = make_float4(x[i], y[i], z[i], __int_as_float((int)i));
    vel[pos] = make_float4(vx[i], vy[i], vz[i], 0.0f);
    ne_s[pos] = ne[i];
    T_s[pos] = T[i];
  }
}

// Insertion sort of each cell's points by original index (cells are small).
__global__ void sort_cells_kernel(const int* __restrict__ cell_start, int64_t ncells, float4* __restrict__ pts,
                                  float4* __restrict__ vel, float* __restrict__ ne_s, float* __restrict__ T_s) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
    int b = cell_start[c], e = cell_start[c + 1];
    // the cell's points lie in [0, cell_start[ncells]); a range outside it is
    // recorded and skipped in the bounds-check build
    if (e > b && FOMO_IDX(e - 1, cell_start[ncells], kSiteIndexBuild) != e - 1) continue;
    for (int i = b + 1; i < e; ++i) {
      float4 p = pts[i];
      float4 v = vel[i];
      float a = ne_s[i], t = T_s[i];
      int key = __float_as_int(p.w);
      int j = i - 1;
      while (j >= b && __float_as_int(pts[j].w) > key) {
        pts[j + 1] = pts[j];
        vel[j + 1] = vel[j];
        ne_s[j + 1] = ne_s[j];
        T_s[j + 1] = T_s[j];
        --j;
      }
      pts[j + 1] = p;
      vel[j + 1] = v;
      ne_s[j + 1] = a;
      T_s[j + 1] = t;
    }
  }
}

int grid_blocks(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

FOMO_DEFINE_CHECK_READER(check_word_index)

cudaError_t launch_aabb(const float* x, const float* y, const float* z, int64_t n, unsigned int* bits6,
                        cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(bits6, 0xff, 3 * sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(bits6 + 3, 0x00, 3 * sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  aabb_kernel<<<grid_blocks(n, 256), 256, 0, s>>>(x, y, z, n, bits6);
  return cudaGetLastError();
}

cudaError_t launch_bin_points(const float* x, const float* y, const float* z, int64_t n, GridParams g, int* cell_of,
                              int* counts, cudaStream_t s) {
  bin_kernel<<<grid_blocks(n, 256), 256, 0, s>>>(x, y, z, n, g, cell_of, counts);
  return cudaGetLastError();
}

// One warp per block of kBlockCells^3 cells: the bounding box of its points
// (min x, y, z, max x, y, z), from its rows' point ranges; an empty block gets
// min = FLT_MAX, max = -FLT_MAX.  The view set-up bounds each view's extents
// by these boxes (view.cu).
__global__ void block_bounds_kernel(const float4* __restrict__ pts, const int* __restrict__ cell_start, GridParams g,
                                    int bdx, int bdy, int bdz, float* __restrict__ blk) {
  const int64_t nblk = (int64_t)bdx * bdy * bdz;
  const int64_t b = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (b >= nblk) return;  // the whole warp
  const int bx = (int)(b % bdx), by = (int)((b / bdx) % bdy), bz = (int)(b / ((int64_t)bdx * bdy));
  const int x0 = bx * kBlockCells, x1 = min(x0 + kBlockCells, g.dx) - 1;
  const int64_t entries = (int64_t)g.dx * g.dy * g.dz + 1;
  float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int r = lane; r < kBlockCells * kBlockCells; r += 32) {
    const int cy = by * kBlockCells + r % kBlockCells, cz = bz * kBlockCells + r / kBlockCells;
    if (cy >= g.dy || cz >= g.dz) continue;
    const int64_t rowbase = ((int64_t)cz * g.dy + cy) * g.dx;
    const int p1 = cell_start[FOMO_IDX(rowbase + x1 + 1, entries, kSiteIndexBuild)];
    for (int p = cell_start[FOMO_IDX(rowbase + x0, entries, kSiteIndexBuild)]; p < p1; ++p) {
      const float4 v = pts[p];
      mn[0] = fminf(mn[0], v.x);
      mn[1] = fminf(mn[1], v.y);
      mn[2] = fminf(mn[2], v.z);
      mx[0] = fmaxf(mx[0], v.x);
      mx[1] = fmaxf(mx[1], v.y);
      mx[2] = fmaxf(mx[2], v.z);
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
      mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
    }
  if (lane < 6) blk[FOMO_IDX(6 * b + lane, 6 * nblk, kSiteIndexBuild)] = lane < 3 ? mn[lane] : mx[lane - 3];
}

cudaError_t launch_block_bounds(const float4* pts, const int* cell_start, GridParams g, int bdx, int bdy, int bdz,
                                float* blk, cudaStream_t s) {
  const int64_t nblk = (int64_t)bdx * bdy * bdz;
  const int64_t threads = nblk * 32;
  block_bounds_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(pts, cell_start, g, bdx, bdy, bdz, blk);
  return cudaGetLastError();
}

// The number of cells whose count is 0 (added to *empty, zeroed by the caller).
__global__ void count_empty_kernel(const int* __restrict__ counts, int64_t ncells, unsigned long long* empty) {
  unsigned long long k = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncells; i += (int64_t)gridDim.x * blockDim.x)
    k += counts[i] == 0 ? 1ull : 0ull;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
  if ((threadIdx.x & 31) == 0 && k) atomicAdd(empty, k);
}

cudaError_t launch_count_empty(const int* counts, int64_t ncells, unsigned long long* empty, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(empty, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  count_empty_kernel<<<grid_blocks(ncells, 256), 256, 0, s>>>(counts, ncells, empty);
  return cudaGetLastError();
}

int64_t exclusive_scan_scratch_ints(int64_t count) { return (count + kScanTile - 1) / kScanTile + 1; }

cudaError_t launch_exclusive_scan(const int* in, int* out, int64_t count, int* scratch, int64_t scratch_ints,
                                  cudaStream_t s) {
  int64_t tiles = (count + kScanTile - 1) / kScanTile;
  if (tiles < 1 || tiles > scratch_ints) return cudaErrorInvalidValue;
  scan_tile_sums<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, count, scratch);
  scan_sums_single<<<1, kScanThreads, 0, s>>>(scratch, tiles);
  scan_tiles<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, count, scratch, out);
  return cudaGetLastError();
}

cudaError_t launch_scatter(const float* x, const float* y, const float* z, const float* vx, const float* vy,
                           const float* vz, const float* ne, const float* T, int64_t n, const int* cell_of,
                           const int* cell_start, int* fill, float4* pts, float4* vel, float* ne_s, float* T_s,
                           cudaStream_t s) {
  scatter_kernel<<<grid_blocks(n, 256), 256, 0, s>>>(x, y, z, vx, vy, vz, ne, T, n, cell_of, cell_start, fill, pts,
                                                     vel, ne_s, T_s);
  return cudaGetLastError();
}

cudaError_t launch_sort_cells(const int* cell_start, int64_t ncells, float4* pts, float4* vel, float* ne_s,
                              float* T_s, cudaStream_t s) {
  sort_cells_kernel<<<grid_blocks(ncells, 256), 256, 0, s>>>(cell_start, ncells, pts, vel, ne_s, T_s);
  return cudaGetLastError();
}

}  // namespace fomo
