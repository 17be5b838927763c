// Host runtime of libfomo_gpu: the C ABI of include/fomo_gpu.h.
//
// Owns device memory (snapshots with their spatial index, G(T) tables,
// cached emissivity payloads, a grow-only scratch arena for per-render
// descriptors and outputs), orchestrates the kernels of index.cu, emission.cu,
// view.cu and march.cu on one CUDA stream, and maps every failure to a
// negative status with a message (the reference exits instead).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/fomo_gpu.h"
#include "fomo_internal.h"
#include "runtime_internal.h"

using namespace fomo;

namespace fomo {

const char* kVersion = "fomo_gb300 0.1 (sm_103a)";

int set_err(fomo_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_err(fomo_ctx* c, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  cudaGetLastError();  // clear sticky-free errors
  if (e == cudaErrorMemoryAllocation) return set_err(c, FOMO_ENOMEM, m);
  return set_err(c, FOMO_EDEVICE, m);
}

#define FOMO_CUDA(call, what)                           \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_err(ctx, e_, what); \
  } while (0)

// ---------------------------------------------------------------- bounds checks

// The bounds-check build (FOMO_BOUNDS_CHECK=1) records the site of the first
// index out of range per kernel file in a device word and keeps every access
// inside its buffer (fomo_device.cuh).  After each synchronising call the
// words are read and cleared; a set word fails the call with FOMO_EDEVICE.
// The regular build has no such words to read.
int check_device_words(fomo_ctx* ctx) {
#if defined(FOMO_BOUNDS_CHECK) && FOMO_BOUNDS_CHECK
  static const char* const names[] = {"march", "index", "view", "emission", "projection", "amrvac"};
  cudaError_t (*const readers[])(unsigned*) = {check_word_march, check_word_index, check_word_view,
                                               check_word_emission, check_word_projection, check_word_amrvac};
  for (int k = 0; k < 6; ++k) {
    unsigned w = 0;
    const cudaError_t e = readers[k](&w);
    if (e != cudaSuccess) return cuda_err(ctx, e, "bounds-check word");
    if (w)
      return set_err(ctx, FOMO_EDEVICE, std::string("bounds check: index out of range in ") + names[k] +
                                            ".cu (site " + std::to_string(w) + ")");
  }
#else
  (void)ctx;
#endif
  return FOMO_OK;
}

// ---------------------------------------------------------------- memory

int dev_alloc(fomo_ctx* ctx, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  // fault injection for the error paths' tests: the k-th allocation of the
  // context fails as cudaMalloc would (FOMO_INJECT_ALLOC_FAILURE=k)
  if (ctx->fail_alloc_at > 0 && ++ctx->alloc_count == ctx->fail_alloc_at)
    return set_err(ctx, FOMO_ENOMEM, "device allocation failed (injected failure)");
  if (ctx->used + bytes > ctx->budget) {
    std::ostringstream m;
    m << "device allocation of " << bytes << " bytes exceeds the context budget (" << ctx->used << " of "
      << ctx->budget << " used)";
    return set_err(ctx, FOMO_ENOMEM, m.str());
  }
  // a block of this size freed before (a snapshot, table or emissivity made
  // again for the same number of points) is used again as it is
  auto fb = ctx->free_blocks.find(bytes);
  if (fb != ctx->free_blocks.end()) {
    *p = fb->second;
    ctx->free_blocks.erase(fb);
    ctx->cached -= bytes;
  } else {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaErrorMemoryAllocation && !ctx->free_blocks.empty()) {
      cudaGetLastError();  // clear the sticky-free error state, give the kept blocks back and try again
      release_free_blocks(ctx);
      e = cudaMalloc(p, bytes);
    }
    if (e != cudaSuccess) {
      *p = nullptr;
      return cuda_err(ctx, e, "cudaMalloc");
    }
  }
  ctx->used += bytes;
  ctx->sizes[*p] = bytes;
  return FOMO_OK;
}

// Blocks kept by dev_free: at most kKeepBlock bytes each and kKeepTotal in all.
constexpr size_t kKeepBlock = size_t(512) << 20;
constexpr size_t kKeepTotal = size_t(4) << 30;

void release_free_blocks(fomo_ctx* ctx) {
  for (auto& kv : ctx->free_blocks) cudaFree(kv.second);
  ctx->free_blocks.clear();
  ctx->cached = 0;
}

void dev_free(fomo_ctx* ctx, void* p) {
  if (!p) return;
  auto it = ctx->sizes.find(p);
  size_t bytes = 0;
  if (it != ctx->sizes.end()) {
    bytes = it->second;
    ctx->used -= bytes;
    ctx->sizes.erase(it);
  }
  if (bytes > 0 && bytes <= kKeepBlock && ctx->cached + bytes <= kKeepTotal) {
    // kept for the next allocation of the same size instead of unmapped and
    // mapped again; like cudaFree, only once the device is done with it
    cudaDeviceSynchronize();
    ctx->free_blocks.emplace(bytes, p);
    ctx->cached += bytes;
    return;
  }
  cudaFree(p);
}

int Arena::reserve(fomo_ctx* ctx, size_t bytes) {
  if (bytes <= cap) return FOMO_OK;
  size_t want = std::max(bytes, cap * 2);
  want = (want + 4095) & ~size_t(4095);
  if (base) {
    // the previous contents may still be in use by queued work
    cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, base);
    base = nullptr;
    cap = 0;
  }
  void* p = nullptr;
  int rc = dev_alloc(ctx, &p, want);
  if (rc != FOMO_OK) {
    // retry with the exact size
    rc = dev_alloc(ctx, &p, bytes);
    if (rc != FOMO_OK) return rc;
    want = bytes;
  }
  base = static_cast<char*>(p);
  cap = want;
  return FOMO_OK;
}

int Staging::reserve(fomo_ctx* ctx, size_t bytes) {
  if (bytes <= cap) return FOMO_OK;
  if (base) {
    if (copy_done) cudaEventSynchronize(copy_done);
    cudaFreeHost(base);
    base = nullptr;
    cap = 0;
  }
  size_t want = std::max<size_t>(bytes, 1 << 16);
  cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&base), want);
  if (e != cudaSuccess) return cuda_err(ctx, e, "cudaMallocHost (descriptor staging)");
  cap = want;
  return FOMO_OK;
}

// ---------------------------------------------------------------- tables

// readgoftfromchianti (fomo-CHIANTI.cpp:143-218): ion, lambda0, atweight,
// minlevel, maxlevel, rest of line skipped, unit line, version line,
// "nrho nt", nt logT values, then nrho rows of logn followed by nt G values.
// Values parse as double and are stored as float.
int parse_table_text(const std::string& text, TableHost* t, std::string* err) {
  std::istringstream in(text);
  double minlevel = 0, maxlevel = 0;
  in >> t->ion >> t->lambda0 >> t->atweight >> minlevel >> maxlevel;
  in.ignore(1 << 30, '\n');
  std::getline(in, t->unit);
  std::string version;
  std::getline(in, version);
  int nrho = 0, nt = 0;
  in >> nrho >> nt;
  if (!in || nrho <= 0 || nt <= 0) {
    *err = "CHIANTI table not read in properly! (bad header)";
    return FOMO_ETABLE;
  }
  t->nt = nt;
  t->nrho = nrho;
  t->logT.resize(nt);
  for (int i = 0; i < nt; ++i) {
    double v = 0;
    in >> v;
    t->logT[i] = static_cast<float>(v);
  }
  t->logn.clear();
  t->G.clear();
  double row = 0;
  long rows = 0;
  while (in >> row) {
    t->logn.push_back(static_cast<float>(row));
    for (int i = 0; i < nt; ++i) {
      double v = 0;
      if (!(in >> v)) v = 0;
      t->G.push_back(static_cast<float>(v));
    }
    ++rows;
  }
  if (rows != nrho) {
    *err = "CHIANTI table not read in properly! (expected " + std::to_string(nrho) + " density rows, found " +
           std::to_string(rows) + ")";
    return FOMO_ETABLE;
  }
  return FOMO_OK;
}

int upload_table(fomo_ctx* ctx, TableHost&& th, int* id) {
  if (th.nt < 2 || th.nrho < 1 || (long)th.G.size() != (long)th.nt * th.nrho || (long)th.logT.size() != th.nt ||
      (long)th.logn.size() != th.nrho)
    return set_err(ctx, FOMO_ETABLE, "table dimensions inconsistent (need nt >= 2, nrho >= 1)");
  if (th.nrho < 2) {
    // goft uses rhogrid.at(nt) as the second density (fomo-CHIANTI.cpp:97)
    return set_err(ctx, FOMO_ETABLE, "table needs at least two density rows");
  }
  TableRec rec;
  rec.h = std::move(th);
  rec.h.is_dn = rec.h.unit.find("DN") != std::string::npos;
  size_t bytes = sizeof(float) * (rec.h.logT.size() + rec.h.logn.size() + rec.h.G.size());
  void* p = nullptr;
  int rc = dev_alloc(ctx, &p, bytes);
  if (rc) return rc;
  rec.d = static_cast<float*>(p);
  float* d = rec.d;
  FOMO_CUDA(cudaMemcpy(d, rec.h.logT.data(), rec.h.logT.size() * 4, cudaMemcpyHostToDevice), "table upload");
  FOMO_CUDA(cudaMemcpy(d + rec.h.nt, rec.h.logn.data(), rec.h.logn.size() * 4, cudaMemcpyHostToDevice),
            "table upload");
  FOMO_CUDA(cudaMemcpy(d + rec.h.nt + rec.h.nrho, rec.h.G.data(), rec.h.G.size() * 4, cudaMemcpyHostToDevice),
            "table upload");
  int nid = ctx->next_id++;
  ctx->tables[nid] = std::move(rec);
  *id = nid;
  return FOMO_OK;
}

// ---------------------------------------------------------------- snapshots

namespace {
inline float ord2f(unsigned int u) {
  u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
}  // namespace

GridParams choose_grid(const float* mn, const float* mx, int64_t n, double ppc) {
  double ext[3], maxext = 0;
  for (int d = 0; d < 3; ++d) {
    ext[d] = (double)mx[d] - (double)mn[d];
    maxext = std::max(maxext, ext[d]);
  }
  double vol = 1.0;
  int ndim = 0;
  for (int d = 0; d < 3; ++d)
    if (ext[d] > 1e-9 * (maxext > 0 ? maxext : 1.0)) {
      vol *= ext[d];
      ++ndim;
    }
  double h = ndim ? std::pow(vol * ppc / (double)std::max<int64_t>(n, 1), 1.0 / ndim) : 1.0;
  if (!(h > 0) || !std::isfinite(h)) h = 1.0;
  int dims[3];
  for (;;) {
    double cells = 1;
    for (int d = 0; d < 3; ++d) {
      double k = std::ceil(ext[d] / h);
      if (k < 1) k = 1;
      if (k > 4096) k = 4096;
      dims[d] = (int)k;
      cells *= k;
    }
    if (cells <= 4.0 * (double)n + 64.0) break;
    h *= 1.25;
  }
  GridParams g;
  g.ox = mn[0];
  g.oy = mn[1];
  g.oz = mn[2];
  g.h = (float)h;
  g.inv_h = (float)(1.0 / h);
  g.dx = dims[0];
  g.dy = dims[1];
  g.dz = dims[2];
  g.minx = mn[0];
  g.miny = mn[1];
  g.minz = mn[2];
  g.maxx = mx[0];
  g.maxy = mx[1];
  g.maxz = mx[2];
  return g;
}

constexpr double kUniformEmpty = 0.10;  // empty-cell share below which a cloud counts as uniform

int build_snapshot(fomo_ctx* ctx, int64_t n, const float* const host[8], SnapRec* out) {
  NvtxRange range("fomo: snapshot upload and index");
  cudaStream_t s = ctx->stream;
  // staging: 8 arrays of n floats (z may be absent -> zeros, as nn:82 for 2-D data)
  float* stage = nullptr;
  int rc = dev_alloc(ctx, reinterpret_cast<void**>(&stage), sizeof(float) * 8 * (size_t)n);
  if (rc) return rc;
  float* a[8];
  for (int k = 0; k < 8; ++k) a[k] = stage + (size_t)k * n;
  for (int k = 0; k < 8; ++k) {
    if (host[k]) {
      // host or device memory alike (unified addressing: a device array is copied on the device)
      cudaError_t e = cudaMemcpyAsync(a[k], host[k], sizeof(float) * n, cudaMemcpyDefault, s);
      if (e != cudaSuccess) {
        dev_free(ctx, stage);
        return cuda_err(ctx, e, "snapshot upload");
      }
    } else {
      cudaMemsetAsync(a[k], 0, sizeof(float) * n, s);
    }
  }
  unsigned int* bits = nullptr;
  rc = dev_alloc(ctx, reinterpret_cast<void**>(&bits), 64);
  if (rc) {
    dev_free(ctx, stage);
    return rc;
  }
  unsigned int hb[6];
  cudaError_t e = launch_aabb(a[0], a[1], a[2], n, bits, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hb, bits, sizeof(hb), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    dev_free(ctx, stage);
    dev_free(ctx, bits);
    return cuda_err(ctx, e, "snapshot bounds");
  }
  float mn[3], mx[3];
  for (int d = 0; d < 3; ++d) {
    mn[d] = ord2f(hb[d]);
    mx[d] = ord2f(hb[3 + d]);
  }
  if (!(std::isfinite(mn[0]) && std::isfinite(mn[1]) && std::isfinite(mn[2]) && std::isfinite(mx[0]) &&
        std::isfinite(mx[1]) && std::isfinite(mx[2]))) {
    dev_free(ctx, stage);
    dev_free(ctx, bits);
    return set_err(ctx, FOMO_EINVAL, "snapshot coordinates contain NaN or infinity");
  }
  // Grid cell size.  A cloud that is close to uniform at the cell scale (fewer
  // than kUniformEmpty of the cells empty at 2 points per cell) gets cells of 1
  // point: its searches then load fewer points per candidate and its ring
  // walks are shorter (the 2M-point loop's batched render: 4 % faster).  A
  // clustered cloud keeps 2 points per cell: finer cells would leave its sparse
  // regions' walks crossing more empty cells (8M-point flux rope: 17-26 %
  // slower at 1 point per cell).  FOMO_CELL_OCCUPANCY sets the occupancy and
  // skips the choice.
  double ppc = ctx->cell_occupancy;
  if (!ctx->occupancy_set && n >= 1024) {
    const GridParams g2 = choose_grid(mn, mx, n, 2.0);
    const int64_t nc2 = (int64_t)g2.dx * g2.dy * g2.dz;
    int* t2 = nullptr;
    rc = dev_alloc(ctx, reinterpret_cast<void**>(&t2), sizeof(int) * (size_t)(n + nc2));
    if (rc) {
      dev_free(ctx, stage);
      dev_free(ctx, bits);
      return rc;
    }
    unsigned long long hempty = 0;
    unsigned long long* dempty = reinterpret_cast<unsigned long long*>(bits);
    e = cudaMemsetAsync(t2 + n, 0, sizeof(int) * (size_t)nc2, s);
    if (e == cudaSuccess) e = launch_bin_points(a[0], a[1], a[2], n, g2, t2, t2 + n, s);
    if (e == cudaSuccess) e = launch_count_empty(t2 + n, nc2, dempty, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hempty, dempty, sizeof(hempty), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    dev_free(ctx, t2);
    if (e != cudaSuccess) {
      dev_free(ctx, stage);
      dev_free(ctx, bits);
      return cuda_err(ctx, e, "snapshot cell statistics");
    }
    ppc = (double)hempty < kUniformEmpty * (double)nc2 ? 1.0 : 2.0;
  }
  GridParams g = choose_grid(mn, mx, n, ppc);
  const int64_t ncells = (int64_t)g.dx * g.dy * g.dz;
  const int64_t scan_count = ncells + 1;
  const int64_t scr = exclusive_scan_scratch_ints(scan_count);
  // temporaries: cell_of (n), counts (ncells+1), fill (ncells), scan scratch
  int* tmp = nullptr;
  rc = dev_alloc(ctx, reinterpret_cast<void**>(&tmp), sizeof(int) * (size_t)(n + 2 * ncells + 1 + scr));
  if (rc) {
    dev_free(ctx, stage);
    dev_free(ctx, bits);
    return rc;
  }
  int* cell_of = tmp;
  int* counts = tmp + n;
  int* fill = counts + ncells + 1;
  int* scratch = fill + ncells;
  // resident: pts, vel (float4), ne, T, cell_start
  SnapRec R;
  R.n = n;
  R.ncells = ncells;
  R.g = g;
  const int bdx = (g.dx + kBlockCells - 1) / kBlockCells, bdy = (g.dy + kBlockCells - 1) / kBlockCells,
            bdz = (g.dz + kBlockCells - 1) / kBlockCells;
  const int64_t nblk = (int64_t)bdx * bdy * bdz;
  const size_t resident = sizeof(float4) * 2 * (size_t)n + sizeof(float) * 2 * (size_t)n +
                          sizeof(int) * (size_t)(ncells + 1) + sizeof(float) * 6 * (size_t)nblk;
  void* res = nullptr;
  rc = dev_alloc(ctx, &res, resident);
  if (rc) {
    dev_free(ctx, stage);
    dev_free(ctx, bits);
    dev_free(ctx, tmp);
    return rc;
  }
  R.block = res;
  R.bytes = resident;
  char* base = static_cast<char*>(res);
  R.pts = reinterpret_cast<float4*>(base);
  R.vel = R.pts + n;
  R.ne = reinterpret_cast<float*>(R.vel + n);
  R.T = R.ne + n;
  R.cell_start = reinterpret_cast<int*>(R.T + n);
  R.blk = reinterpret_cast<float*>(R.cell_start + ncells + 1);
  R.bdx = bdx;
  R.bdy = bdy;
  R.bdz = bdz;
  e = cudaMemsetAsync(counts, 0, sizeof(int) * (size_t)(2 * ncells + 1), s);
  if (e == cudaSuccess) e = launch_bin_points(a[0], a[1], a[2], n, g, cell_of, counts, s);
  if (e == cudaSuccess) e = launch_exclusive_scan(counts, R.cell_start, scan_count, scratch, scr, s);
  if (e == cudaSuccess)
    e = launch_scatter(a[0], a[1], a[2], a[5], a[6], a[7], a[3], a[4], n, cell_of, R.cell_start, fill, R.pts, R.vel,
                       R.ne, R.T, s);
  if (e == cudaSuccess) e = launch_sort_cells(R.cell_start, ncells, R.pts, R.vel, R.ne, R.T, s);
  if (e == cudaSuccess) e = launch_block_bounds(R.pts, R.cell_start, g, bdx, bdy, bdz, R.blk, s);
  unsigned int vbits = 0x7f800000u;
  if (e == cudaSuccess) e = launch_speed_max(R.vel, n, bits, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&vbits, bits, sizeof(vbits), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  std::memcpy(&R.vmax, &vbits, sizeof(R.vmax));
  dev_free(ctx, stage);
  dev_free(ctx, bits);
  dev_free(ctx, tmp);
  if (e != cudaSuccess) {
    dev_free(ctx, res);
    return cuda_err(ctx, e, "snapshot index build");
  }
  *out = R;
  return FOMO_OK;
}

SnapDev snap_dev(const SnapRec& r) {
  SnapDev s;
  s.n = r.n;
  s.pts = r.pts;
  s.vel = r.vel;
  s.cell_start = r.cell_start;
  s.g = r.g;
  s.blk = r.blk;
  s.bdx = r.bdx;
  s.bdy = r.bdy;
  s.bdz = r.bdz;
  return s;
}

// Emissivity payload for (snapshot, table, observation type, abundance),
// computed once and kept resident (the reference recomputes it on every
// render, fomo-object.cpp:389-400).
int get_payload(fomo_ctx* ctx, int snap, int table, int imaging, double abund, const float2** out) {
  NvtxRange range("fomo: emissivity");
  auto key = std::make_tuple(snap, table, imaging, abund);
  auto it = ctx->payloads.find(key);
  if (it != ctx->payloads.end()) {
    *out = it->second;
    return FOMO_OK;
  }
  auto sit = ctx->snaps.find(snap);
  if (sit == ctx->snaps.end()) return set_err(ctx, FOMO_ENOTFOUND, "unknown snapshot id");
  auto tit = ctx->tables.find(table);
  if (tit == ctx->tables.end()) return set_err(ctx, FOMO_ENOTFOUND, "unknown table id");
  const TableHost& th = tit->second.h;
  if (imaging && std::atoi(th.ion.c_str()) != (int)(th.lambda0 + 0.5))
    return set_err(ctx, FOMO_ETABLE, "GOFT table is not correct! (imaging needs atoi(ion) == int(lambda0+0.5))");
  void* p = nullptr;
  int rc = dev_alloc(ctx, &p, sizeof(float2) * (size_t)sit->second.n);
  if (rc) return rc;
  TableDev td;
  td.nt = th.nt;
  td.nrho = th.nrho;
  td.logT = tit->second.d;
  td.logn = tit->second.d + th.nt;
  td.G = tit->second.d + th.nt + th.nrho;
  // linefwhm constant (fomo-CHIANTI.cpp:224), same expression order
  td.cw = 2 * std::sqrt(2 * std::log(2)) * std::sqrt(FOMO_BOLTZMANN / FOMO_MASS_PROTON / th.atweight) * th.lambda0 /
          FOMO_SPEED_OF_LIGHT;
  const double normaliseconst = imaging ? 1.0 : 1. / FOMO_ALPHA;
  td.k = normaliseconst * (imaging ? 1.0 : abund);
  td.imaging = imaging;
  cudaError_t e = launch_emission(sit->second.ne, sit->second.T, sit->second.n, td, static_cast<float2*>(p),
                                  ctx->stream);
  // largest line width of the emitting points: bounds the evaluated lambda window
  unsigned int* wb = reinterpret_cast<unsigned int*>(ctx->stats_dev);
  unsigned int hw = 0x7f800000u;
  if (e == cudaSuccess) e = launch_payload_stats(static_cast<float2*>(p), sit->second.n, wb, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hw, wb, sizeof(hw), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    dev_free(ctx, p);
    return cuda_err(ctx, e, "emission kernel");
  }
  float wmax;
  std::memcpy(&wmax, &hw, sizeof(wmax));
  ctx->payloads[key] = static_cast<float2*>(p);
  ctx->payload_wmax[key] = imaging ? 1.0f : wmax;
  *out = static_cast<float2*>(p);
  return FOMO_OK;
}

float payload_wmax(fomo_ctx* ctx, int snap, int table, int imaging, double abund) {
  auto it = ctx->payload_wmax.find(std::make_tuple(snap, table, imaging, abund));
  return it == ctx->payload_wmax.end() ? __builtin_inff() : it->second;
}

// lambda window of one line: bins whose Gaussian weight is below 2^-64 of every
// peak (|dlambda| > 4 w_max beyond the largest Doppler shift) are not evaluated.
void line_window(double lwa, int L, double lambda0, float vmax, float wmax, int* wstart, int* nw) {
  const int full = (L + 31) / 32;
  *wstart = 0;
  *nw = full;
  if (L <= 1 || !(lwa > 0) || !std::isfinite(wmax) || !std::isfinite(vmax)) return;
  const double dl = lwa / (L - 1);
  const double S = ((double)vmax * lambda0 / FOMO_SPEED_OF_LIGHT + 4.0 * (double)wmax) * 1.001 + 2.0 * dl;
  const double lo = (lwa / 2. - S) / dl, hi = (lwa / 2. + S) / dl;
  int b0 = (int)std::floor(std::max(lo, 0.0));
  int b1 = (int)std::ceil(std::min(hi, (double)(L - 1)));
  if (b1 < b0) b1 = b0;
  const int n = (b1 - b0 + 1 + 31) / 32;
  if (n >= full) return;
  *wstart = b0;
  *nw = n;
}

int get_thomson_payload(fomo_ctx* ctx, SnapRec& r, const float2** out) {
  if (!r.totpol) {
    void* p = nullptr;
    int rc = dev_alloc(ctx, &p, sizeof(float2) * (size_t)r.n);
    if (rc) return rc;
    cudaError_t e = launch_thomson_emission(r.pts, r.ne, r.n, static_cast<float2*>(p), ctx->stream);
    if (e != cudaSuccess) {
      dev_free(ctx, p);
      return cuda_err(ctx, e, "Thomson emission kernel");
    }
    r.totpol = static_cast<float2*>(p);
  }
  *out = r.totpol;
  return FOMO_OK;
}

// ---------------------------------------------------------------- rendering

// Methods whose emission comes from a G(T, n) table (all but Thomson).
bool uses_table(int method) { return method != FOMO_METHOD_THOMSON; }

// Relative abundance 10^(A_element - A_H) of the element of `ion` ("fe_12" ->
// "fe") in a CHIANTI abundance file: lines "Z  A  symbol" until a negative Z
// (fomo-CHIANTI.cpp:23-62; the symbol compare is case-insensitive and whole).
bool abundance_of(const char* path, const char* ion, double* out, std::string* err) {
  std::ifstream in(path);
  if (!in) {
    *err = std::string("Error: no CHIANTI abundance file exists: ") + path;
    return false;
  }
  std::string name(ion);
  name = name.substr(0, name.find('_'));
  auto same = [](const std::string& p, const std::string& q) {
    if (p.size() != q.size()) return false;
    for (size_t i = 0; i < p.size(); ++i)
      if (std::tolower((unsigned char)p[i]) != std::tolower((unsigned char)q[i])) return false;
    return true;
  };
  double h = 0, el = 0, value = 0;
  int z = 0;
  std::string sym;
  while (in >> z && z >= 0) {
    if (!(in >> value >> sym)) break;
    if (same(sym, "h")) h = value;
    if (same(sym, name)) el = value;
  }
  if (h == 0.0 || el == 0.0) {
    *err = std::string("Error: invalid CHIANTI abundance file (no H or no ") + name + "): " + path;
    return false;
  }
  *out = std::pow(10.0, el - h);
  return true;
}

int validate(fomo_ctx* ctx, const fomo_request& q) {
  if (q.method != FOMO_METHOD_NN && q.method != FOMO_METHOD_THOMSON && q.method != FOMO_METHOD_PROJECTION)
    return set_err(ctx, FOMO_EMETHOD, "Error: unknown rendering method.");
  if (q.nx < 2 || q.ny < 2 || q.nz < 1 || q.nlambda < 1)
    return set_err(ctx, FOMO_EINVAL, "resolution must have nx >= 2, ny >= 2, nz >= 1, nlambda >= 1");
  if ((int64_t)q.nx * q.ny >= (int64_t)1 << 30 || q.nz > (1 << 20) || q.nlambda > 256)
    return set_err(ctx, FOMO_EINVAL, "resolution too large (nx*ny < 2^30, nz <= 2^20, nlambda <= 256)");
  if (!std::isfinite(q.l) || !std::isfinite(q.b)) return set_err(ctx, FOMO_EINVAL, "view angles must be finite");
  if (ctx->snaps.find(q.snapshot) == ctx->snaps.end()) return set_err(ctx, FOMO_ENOTFOUND, "unknown snapshot id");
  if (uses_table(q.method)) {
    if (ctx->tables.find(q.table) == ctx->tables.end()) return set_err(ctx, FOMO_ENOTFOUND, "unknown table id");
    if (!(q.lambda_width > 0) && q.nlambda > 1)
      return set_err(ctx, FOMO_EINVAL, "lambda_width must be > 0 (m/s) for spectroscopic renders");
  }
  return FOMO_OK;
}

size_t cube_elems(const fomo_request& q) {
  return (size_t)q.nx * q.ny * (q.method == FOMO_METHOD_THOMSON ? 1 : q.nlambda);
}

void fill_view_host(const fomo_request& q, double lambda0, int tw, int th, ViewDesc* V) {
  std::memset(V, 0, sizeof(*V));
  V->cb = std::cos(q.b);
  V->sb = std::sin(q.b);
  V->cl = std::cos(q.l);
  V->sl = std::sin(q.l);
  V->rcb = V->cb;
  V->rsb = V->sb;
  V->blend = 0.0;
  V->mdblend = 0.0;
  if (q.method == FOMO_METHOD_THOMSON) {
    // fomo-thomson.cpp:139-152 (clamp), :176 (pole blend), :249 (maxdistance blend)
    const double epsilon = 1e-6;
    double cos_b = std::cos(q.b), sin_b = std::sin(q.b);
    if (std::abs(cos_b) < epsilon) cos_b = epsilon;
    if (std::abs(sin_b) < epsilon) sin_b = epsilon;
    V->rcb = cos_b;
    V->rsb = sin_b;
    const double threshold = 1.309, steepness = 20.0;
    V->blend = 1.0 / (1.0 + std::exp(-steepness * (std::fabs(q.b) - threshold)));
    V->mdblend = 1.0 / (1.0 + std::exp(-10 * (std::fabs(q.b) - 0.1745)));
  }
  V->lambda_width = q.lambda_width;
  V->lambda0 = lambda0;
  V->nx = q.nx;
  V->ny = q.ny;
  V->nz = q.nz;
  V->L = q.method == FOMO_METHOD_THOMSON ? 1 : q.nlambda;
  V->method = q.method == FOMO_METHOD_THOMSON ? kMethodThomson
              : (q.method == FOMO_METHOD_PROJECTION ? kMethodProjection : kMethodNN);
  V->ray_tile_w = tw;
  V->ray_tile_h = th;
}

void view_info_from(const ViewDesc& V, const fomo_request& q, const TableHost* t, fomo_view_info* info) {
  info->minx = V.minx;
  info->maxx = V.maxx;
  info->miny = V.miny;
  info->maxy = V.maxy;
  info->minz = V.minz;
  info->maxz = V.maxz;
  info->maxdistance = V.md;
  info->deltaz = V.deltaz;
  info->pathlength = V.pathlength;
  const bool dn = t && t->is_dn && uses_table(q.method);
  info->apix = dn ? V.apix : 1.0;
  info->scale = dn ? V.scale_dn : V.scale;
  info->lambda0 = q.method == FOMO_METHOD_THOMSON ? 0.0 : (t ? t->lambda0 : 0.0);
  info->lambda_width_A = q.lambda_width * info->lambda0 / FOMO_SPEED_OF_LIGHT;
  info->is_dn = dn ? 1 : 0;
  info->observation_type =
      (q.method == FOMO_METHOD_THOMSON || q.nlambda <= 1) ? FOMO_OBS_IMAGING : FOMO_OBS_SPECTROSCOPIC;
}

namespace {

struct Layout {
  size_t off = 0;
  size_t take(size_t bytes, size_t align = 256) {
    off = (off + align - 1) & ~(align - 1);
    size_t r = off;
    off += bytes;
    return r;
  }
};

struct ViewKey {
  int snapshot, method, nx, ny, nz, L;
  double l, b, width;
  bool operator<(const ViewKey& o) const {
    return std::tie(snapshot, method, nx, ny, nz, L, l, b, width) <
           std::tie(o.snapshot, o.method, o.nx, o.ny, o.nz, o.L, o.l, o.b, o.width);
  }
};

}  // namespace

std::string workload_class(const PlanGroup& G, const SnapRec& snap) {
  // autotuner key: method, mode, lines, bins, LOS samples and snapshot size (log2 buckets)
  std::ostringstream k;
  int lg = 0;
  for (int64_t n = snap.n; n > 1; n >>= 1) ++lg;
  k << (G.method == FOMO_METHOD_THOMSON ? "thomson"
        : (G.method == FOMO_METHOD_PROJECTION ? (G.imaging ? "proj-imaging" : "proj-spectral")
                                              : (G.imaging ? "imaging" : "spectral"))) << ":nl" << G.nl << ":L"
    << G.maxL << ":nz" << G.maxnz << ":n2^" << lg;
  return k.str();
}

// Plan a batch.  Requests are grouped into launches by (snapshot, method,
// imaging); inside a launch, requests with the same view (angles, resolution,
// width) become lines of one view and share the neighbour search.  All
// descriptors of all launches get disjoint places in one staging blob and in
// the scratch arena of `scr`, so a plan can be captured in a CUDA graph.
int plan_batch(fomo_ctx* ctx, const fomo_request* reqs, int nreq, float* const* d_out, int32_t* const* d_nn,
               ScratchSet* scr, Plan* plan) {
  NvtxRange range("fomo: plan");
  plan->groups.clear();
  plan->view_of_req.assign(nreq, -1);
  plan->nviews_total = 0;
  for (int r = 0; r < nreq; ++r) {
    int rc = validate(ctx, reqs[r]);
    if (rc) return rc;
    if (!d_out[r]) return set_err(ctx, FOMO_EINVAL, "null output buffer");
  }
  {
    std::map<std::tuple<int, int, int>, int> gi;
    for (int r = 0; r < nreq; ++r) {
      const fomo_request& q = reqs[r];
      int imaging = (q.method == FOMO_METHOD_THOMSON || q.nlambda <= 1) ? 1 : 0;
      auto k = std::make_tuple(q.snapshot, q.method, imaging);
      auto it = gi.find(k);
      if (it == gi.end()) {
        gi[k] = (int)plan->groups.size();
        PlanGroup G;
        G.snapshot = q.snapshot;
        G.method = q.method;
        G.imaging = imaging;
        plan->groups.push_back(G);
        it = gi.find(k);
      }
      plan->groups[it->second].reqs.push_back(r);
    }
  }
  // launches with less work first (a server completes their requests sooner)
  {
    auto work = [&](const PlanGroup& G) {
      double w = 0.0;
      for (int r : G.reqs) w += (double)reqs[r].nx * reqs[r].ny * reqs[r].nz;
      return w;
    };
    std::stable_sort(plan->groups.begin(), plan->groups.end(),
                     [&](const PlanGroup& a, const PlanGroup& b) { return work(a) < work(b); });
  }
  Layout L;
  const size_t hdr = L.take(0);
  (void)hdr;
  // pass 1: views, sizes, payloads, layout
  for (PlanGroup& G : plan->groups) {
    SnapRec& snap = ctx->snaps[G.snapshot];
    const int line_cap = G.imaging ? 8 : 4;
    std::map<ViewKey, std::vector<int>> vm;
    for (int r : G.reqs) {
      const fomo_request& q = reqs[r];
      ViewKey k{q.snapshot, q.method, q.nx, q.ny, q.nz, q.method == FOMO_METHOD_THOMSON ? 1 : q.nlambda, q.l, q.b,
                q.method == FOMO_METHOD_THOMSON ? 0.0 : q.lambda_width};
      auto it = vm.find(k);
      if (it != vm.end() && (int)it->second.size() >= line_cap) {
        G.vreqs.push_back(it->second);  // full: start another view with the same key
        vm.erase(it);
      }
      vm[k].push_back(r);
    }
    for (auto& kv : vm) G.vreqs.push_back(kv.second);
    G.nv = (int)G.vreqs.size();
    G.nl = 1;
    G.maxL = 1;
    G.maxnz = 1;
    G.maxnx = 2;
    G.maxny = 2;
    for (auto& v : G.vreqs) {
      G.nl = std::max(G.nl, (int)v.size());
      const fomo_request& q = reqs[v[0]];
      G.maxL = std::max(G.maxL, q.method == FOMO_METHOD_THOMSON ? 1 : q.nlambda);
      G.maxnz = std::max(G.maxnz, q.nz);
      G.maxnx = std::max(G.maxnx, q.nx);
      G.maxny = std::max(G.maxny, q.ny);
    }
    if (G.method == FOMO_METHOD_THOMSON) {
      int rc = get_thomson_payload(ctx, snap, &G.totpol);
      if (rc) return rc;
    } else {
      G.ew.assign(nreq, nullptr);
      for (int r : G.reqs) {
        int rc = get_payload(ctx, G.snapshot, reqs[r].table, G.imaging, reqs[r].abundratio, &G.ew[r]);
        if (rc) return rc;
      }
    }
    // march configuration: explicit setting, else the autotuned choice, else 8x4
    G.tw = ctx->tile_w;
    G.th = ctx->tile_h;
    G.bps = ctx->blocks_per_sm;
    G.rscale = ctx->rscale;
    if (G.tw <= 0 || G.th <= 0) {
      G.tw = 8;
      G.th = 4;
      auto t = ctx->tuned.find(workload_class(G, snap));
      if (t != ctx->tuned.end()) {
        G.tw = t->second.tile_w;
        G.th = t->second.tile_h;
        if (ctx->blocks_per_sm == 0) G.bps = t->second.blocks_per_sm;
        if (ctx->rscale == 0.0f) G.rscale = t->second.rscale;
      }
    }
    G.o_views = L.take(sizeof(ViewDesc) * G.nv);
    G.o_lines = L.take(sizeof(LineDesc) * (size_t)G.nv * G.nl);
    G.o_off = L.take(sizeof(int64_t) * (G.nv + 1));
    G.o_nnp = L.take(sizeof(int32_t*) * G.nv);
    size_t lam_total = 0;
    for (auto& v : G.vreqs) lam_total += (size_t)v.size() * (size_t)G.maxL;
    G.o_lam = L.take(sizeof(float) * std::max<size_t>(lam_total, 1));
  }
  plan->host_bytes = L.off;  // the staged (uploaded) part
  for (PlanGroup& G : plan->groups) {
    SnapRec& snap = ctx->snaps[G.snapshot];
    G.o_ktab = L.take(sizeof(double3) * (size_t)G.nv * G.maxnz);
    G.o_xy = L.take(sizeof(double) * (size_t)G.nv * (G.maxnx + G.maxny));
    G.o_ctr = L.take(sizeof(unsigned long long) * kCtrCount);
    int64_t items = 0;
    for (auto& v : G.vreqs) {
      const fomo_request& q = reqs[v[0]];
      items += (int64_t)((q.nx + G.tw - 1) / G.tw) * G.tw * (int64_t)((q.ny + G.th - 1) / G.th) * G.th;
    }
    G.deferred_cap = deferred_capacity(items, G.maxnz);
    G.o_def = L.take(sizeof(DeferredRec) * (size_t)G.deferred_cap);
    G.hard_cap = hard_capacity(items, G.maxnz);
    G.o_hard = L.take(sizeof(uint2) * (size_t)G.hard_cap);
    // the searches and the emission run as separate passes through a
    // neighbour buffer (each pass at its own occupancy; the emission pass runs
    // last, so no sample is added with atomics); at most ctx->npos_cap
    // entries, the launch marching in item chunks beyond that
    G.npos_items = 0;
    G.o_npos = 0;
    G.o_far = 0;
    if (G.method != FOMO_METHOD_PROJECTION) {
      const int64_t cap_items = std::max<int64_t>(1, ctx->npos_cap / G.maxnz);
      G.npos_items = std::min<int64_t>(items, cap_items);
      G.o_npos = L.take(sizeof(int32_t) * (size_t)G.npos_items * G.maxnz);
      G.o_far = L.take(sizeof(int32_t) * (size_t)G.deferred_cap);
    }
    G.o_s2 = G.method == FOMO_METHOD_THOMSON ? L.take(sizeof(float) * (size_t)G.nv * snap.n) : 0;
  }
  plan->dev_bytes = L.off;
  int rc = scr->arena.reserve(ctx, plan->dev_bytes);
  if (rc) return rc;
  rc = scr->staging.reserve(ctx, plan->host_bytes);
  if (rc) return rc;
  if (scr->staging.copy_done) cudaEventSynchronize(scr->staging.copy_done);  // previous upload has run
  char* hb = scr->staging.base;
  char* db = scr->arena.base;
  std::memset(hb, 0, plan->host_bytes);
  // pass 2: fill the staged descriptors
  int vbase = 0;
  for (PlanGroup& G : plan->groups) {
    ViewDesc* hv = reinterpret_cast<ViewDesc*>(hb + G.o_views);
    LineDesc* hl = reinterpret_cast<LineDesc*>(hb + G.o_lines);
    int64_t* hoff = reinterpret_cast<int64_t*>(hb + G.o_off);
    int32_t** hnn = reinterpret_cast<int32_t**>(hb + G.o_nnp);
    float* hlam = reinterpret_cast<float*>(hb + G.o_lam);
    double* dxy = reinterpret_cast<double*>(db + G.o_xy);
    size_t lam_pos = 0;
    hoff[0] = 0;
    G.any_nn = false;
    for (int v = 0; v < G.nv; ++v) {
      const fomo_request& q0 = reqs[G.vreqs[v][0]];
      const TableHost* t0 = uses_table(q0.method) ? &ctx->tables[q0.table].h : nullptr;
      fill_view_host(q0, t0 ? t0->lambda0 : 0.0, G.tw, G.th, &hv[v]);
      hv[v].xt = dxy + (size_t)v * (G.maxnx + G.maxny);
      hv[v].yt = hv[v].xt + G.maxnx;
      const int64_t items =
          (int64_t)((q0.nx + G.tw - 1) / G.tw) * G.tw * (int64_t)((q0.ny + G.th - 1) / G.th) * G.th;
      hoff[v + 1] = hoff[v] + items;
      for (int li = 0; li < (int)G.vreqs[v].size(); ++li) {
        const int r = G.vreqs[v][li];
        const fomo_request& q = reqs[r];
        LineDesc& LD = hl[(size_t)v * G.nl + li];
        LD.out = d_out[r];
        if (uses_table(q.method)) {
          const TableHost& t = ctx->tables[q.table].h;
          LD.ew = G.ew[r];
          LD.lambda0 = t.lambda0;
          LD.lwa = q.lambda_width * t.lambda0 / FOMO_SPEED_OF_LIGHT;  // nn:116
          LD.shift_k = (float)(t.lambda0 / FOMO_SPEED_OF_LIGHT);
          LD.is_dn = t.is_dn ? 1 : 0;
          line_window(LD.lwa, q.nlambda, t.lambda0, ctx->snaps[G.snapshot].vmax,
                      payload_wmax(ctx, G.snapshot, q.table, G.imaging, q.abundratio), &LD.wstart, &LD.nw);
          const int Lq = q.nlambda;
          float* lam = hlam + lam_pos;
          for (int il = 0; il < Lq && Lq > 1; ++il)
            lam[il] = (float)(double(il) / (Lq - 1) * LD.lwa - LD.lwa / 2.);  // nn:200
          LD.lam = reinterpret_cast<const float*>(db + G.o_lam) + lam_pos;
          lam_pos += G.maxL;
        } else {
          LD.ew = nullptr;
          LD.is_dn = 0;
        }
        plan->view_of_req[r] = vbase + v;
        if (q.method == FOMO_METHOD_PROJECTION) {
          // the projection accumulates into the output with atomics: zeroed first
          G.zero_outs.push_back({d_out[r], sizeof(float) * cube_elems(q)});
          if (d_nn && d_nn[r])
            return set_err(ctx, FOMO_EINVAL, "a projection render has no per-sample neighbour indices");
        }
        if (d_nn && d_nn[r]) {
          hnn[v] = d_nn[r];
          G.any_nn = true;
        }
      }
    }
    G.total_items = hoff[G.nv];
    G.item_off.assign(hoff, hoff + G.nv + 1);
    G.vcost.assign(G.nv, 0.0);
    G.out_bytes = 0;
    for (int v = 0; v < G.nv; ++v) {
      const fomo_request& q0 = reqs[G.vreqs[v][0]];
      G.vcost[v] = (double)q0.nx * q0.ny * q0.nz;
      for (int r : G.vreqs[v]) {
        G.vcost[v] += (double)cube_elems(reqs[r]);
        G.out_bytes += cube_elems(reqs[r]) * sizeof(float);
      }
    }
    G.max_nw = 1;
    for (int v = 0; v < G.nv; ++v)
      for (int li = 0; li < (int)G.vreqs[v].size(); ++li) G.max_nw = std::max(G.max_nw, hl[(size_t)v * G.nl + li].nw);
    G.vbase = vbase;
    vbase += G.nv;
  }
  plan->nviews_total = vbase;
  plan->arena_base = db;
  return FOMO_OK;
}

// Enqueue a planned batch on stream s: one descriptor upload, then per launch
// view set-up and the persistent march.
// Cut points [0 = c0 < c1 < ... = nv] of the view ranges a launch marches in
// when its cubes download as they complete: about equal shares of the views'
// cost, one range per 256 MB of cubes, 8 at most.
static std::vector<int> view_ranges(const PlanGroup& G, bool split, double range_cost) {
  if (split && range_cost > 0.0) {
    // ranges of about range_cost each (views in plan order: smaller images first)
    std::vector<int> cuts{0};
    double acc = 0.0;
    for (int v = 0; v < G.nv; ++v) {
      if (v > cuts.back() && acc >= range_cost) {
        cuts.push_back(v);
        acc = 0.0;
      }
      acc += G.vcost[v];
    }
    cuts.push_back(G.nv);
    return cuts;
  }
  const size_t n = split ? std::min<size_t>({8, (size_t)G.nv, std::max<size_t>(1, G.out_bytes >> 28)}) : 1;
  double total = 0.0;
  for (double c : G.vcost) total += c;
  std::vector<int> cuts{0};
  double acc = 0.0;
  for (int v = 0; v < G.nv; ++v) {
    if (v > cuts.back() && cuts.size() < n && acc >= total * (double)cuts.size() / (double)n) cuts.push_back(v);
    acc += G.vcost[v];
  }
  cuts.push_back(G.nv);
  return cuts;
}

int issue_plan(fomo_ctx* ctx, const Plan& plan, ScratchSet* scr, cudaStream_t s, const RangeDone* done,
               double range_cost) {
  NvtxRange range("fomo: launch");
  char* db = scr->arena.base;
  // Under stream capture an ordinary event record is only a capture-internal
  // dependency: the staging event is then recorded after the graph launch,
  // and the timing events become external event-record nodes.
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cs);
  const bool capturing = cs == cudaStreamCaptureStatusActive;
  auto record_timing = [&](cudaEvent_t ev) {
    return capturing ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal) : cudaEventRecord(ev, s);
  };
  cudaError_t e = cudaMemcpyAsync(db, scr->staging.base, plan.host_bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && scr->staging.copy_done && !capturing) e = cudaEventRecord(scr->staging.copy_done, s);
  if (ctx->kernel_timing && !capturing) ctx->timer.n = 0;  // the breakdown covers this render
  for (const PlanGroup& G : plan.groups) {
    if (e != cudaSuccess) break;
    SnapRec& snap = ctx->snaps[G.snapshot];
    e = cudaMemsetAsync(db + G.o_ctr, 0, sizeof(unsigned long long) * kCtrCount, s);
    ViewDesc* dv = reinterpret_cast<ViewDesc*>(db + G.o_views);
    if (e == cudaSuccess) e = launch_view_init(dv, G.nv, s);
    SnapDev sd = snap_dev(snap);
    float* s2 = G.method == FOMO_METHOD_THOMSON ? reinterpret_cast<float*>(db + G.o_s2) : nullptr;
    if (e == cudaSuccess) e = launch_view_extents(sd, dv, G.nv, s2, s);
    double3* ktab = reinterpret_cast<double3*>(db + G.o_ktab);
    if (e == cudaSuccess) e = launch_view_finalize(dv, G.nv, ktab, G.maxnz, s);
    MarchArgs a;
    std::memset(&a, 0, sizeof(a));
    a.snap = sd;
    a.views = dv;
    a.ray_offset = reinterpret_cast<const int64_t*>(db + G.o_off);
    a.lines = reinterpret_cast<const LineDesc*>(db + G.o_lines);
    a.nviews = G.nv;
    a.nlines = G.nl;
    a.item_base = 0;
    a.total_items = G.total_items;
    a.counter = reinterpret_cast<unsigned long long*>(db + G.o_ctr);
    a.deferred = reinterpret_cast<DeferredRec*>(db + G.o_def);
    a.deferred_cap = G.deferred_cap;
    a.far_list = G.o_far ? reinterpret_cast<int32_t*>(db + G.o_far) : nullptr;
    a.hard = reinterpret_cast<uint2*>(db + G.o_hard);
    a.hard_cap = G.hard_cap;
    a.npos = G.o_npos ? reinterpret_cast<int32_t*>(db + G.o_npos) : nullptr;
    a.npos_cap = G.o_npos ? G.npos_items * (int64_t)G.maxnz : 0;
    a.nn_idx = G.any_nn ? reinterpret_cast<int32_t* const*>(db + G.o_nnp) : nullptr;
    a.s2 = s2;
    a.totpol = G.totpol;
    a.stats = ctx->march_stats;
    a.rscale = G.rscale;
    a.stop = scr->stop;
    if (e == cudaSuccess && scr->ev0 && ctx->time_march) e = record_timing(scr->ev0);
    MarchTimer* timer = (ctx->kernel_timing && !capturing) ? &ctx->timer : nullptr;
    int rc = FOMO_OK;
    if (G.method == FOMO_METHOD_PROJECTION) {
      for (const auto& z : G.zero_outs)
        if (e == cudaSuccess) e = cudaMemsetAsync(z.first, 0, z.second, s);
      if (e == cudaSuccess) e = launch_projection(sd, dv, a.lines, G.nv, G.nl, G.imaging, ctx->sm_count, s);
      if (e == cudaSuccess && done) rc = (*done)(G, 0, G.nv);
    } else if (e == cudaSuccess) {
      // the march over view ranges: each range's rays are a contiguous run of
      // work items, with the work counters cleared before it
      // a view range marches in item chunks when its neighbour buffer would
      // exceed the buffer's capacity (the buffer is indexed from item_base)
      const std::vector<int> cuts = view_ranges(G, done != nullptr, range_cost);
      bool first = true;
      for (size_t k = 0; k + 1 < cuts.size() && e == cudaSuccess && rc == FOMO_OK; ++k) {
        const int64_t i0 = G.item_off[cuts[k]], i1 = G.item_off[cuts[k + 1]];
        int64_t step = G.npos_items > 0 ? G.npos_items : (i1 - i0);
        // ranges of bounded work also split a large view's rays into launches
        // of about range_cost, so that other streams' kernels start in between
        if (range_cost > 0.0) step = std::min<int64_t>(step, std::max<int64_t>(1024, (int64_t)(range_cost / G.maxnz)));
        for (int64_t b = i0; b < i1 && e == cudaSuccess; b += step) {
          if (!first) e = cudaMemsetAsync(db + G.o_ctr, 0, sizeof(unsigned long long) * kCtrCount, s);
          first = false;
          a.item_base = b;
          a.total_items = std::min(i1, b + step);
          if (e == cudaSuccess)
            e = launch_march(a, ktab, G.maxnz, G.max_nw, ctx->sm_count, s, G.bps,
                             G.method == FOMO_METHOD_THOMSON || G.imaging, timer);
        }
        if (e == cudaSuccess && done) rc = (*done)(G, cuts[k], cuts[k + 1]);
      }
    }
    if (rc) return rc;
    if (e == cudaSuccess && scr->ev1 && ctx->time_march) e = record_timing(scr->ev1);
  }
  if (e != cudaSuccess) return cuda_err(ctx, e, "render launch");
  return FOMO_OK;
}

int enqueue_batch(fomo_ctx* ctx, const fomo_request* reqs, int nreq, float* const* d_out, int32_t* const* d_nn,
                  cudaStream_t s, std::vector<ViewDesc>* views_out, std::vector<int>* view_of_req,
                  const RangeDone* done) {
  Plan plan;
  int rc = plan_batch(ctx, reqs, nreq, d_out, d_nn, &ctx->scratch, &plan);
  if (rc) return rc;
  rc = order_streams(ctx, s);
  if (rc) return rc;
  rc = issue_plan(ctx, plan, &ctx->scratch, s, done);
  if (rc) return rc;
  if (view_of_req) *view_of_req = plan.view_of_req;
  if (views_out) {
    views_out->assign(plan.nviews_total, ViewDesc{});
    ctx->view_readback.clear();
    for (const PlanGroup& G : plan.groups)
      ctx->view_readback.push_back({reinterpret_cast<ViewDesc*>(ctx->scratch.arena.base + G.o_views),
                                    (size_t)G.vbase, G.nv});
  }
  return FOMO_OK;
}

// A line of the autotuner's cache file: "<class> tile_w tile_h blocks_per_sm
// rscale ms" (lines without rscale, from before it was tuned, keep the default).
bool parse_tune_line(const std::string& line, std::string* key, TuneChoice* c) {
  std::istringstream ls(line);
  std::vector<double> v;
  if (!(ls >> *key)) return false;
  double x;
  while (ls >> x) v.push_back(x);
  if (v.size() != 4 && v.size() != 5) return false;
  c->tile_w = (int)v[0];
  c->tile_h = (int)v[1];
  c->blocks_per_sm = (int)v[2];
  c->rscale = v.size() == 5 ? (float)v[3] : 0.0f;
  return c->tile_w > 0 && c->tile_h > 0 && c->blocks_per_sm >= 0 && c->rscale >= 0.0f;
}

void load_tune_cache(fomo_ctx* ctx, const char* path) {
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    std::string k;
    TuneChoice c;
    if (parse_tune_line(line, &k, &c)) ctx->tuned[k] = c;
  }
}

int finish_views(fomo_ctx* ctx, std::vector<ViewDesc>* views) {
  for (auto& rb : ctx->view_readback) {
    cudaError_t e = cudaMemcpy(views->data() + rb.base, rb.dev, sizeof(ViewDesc) * rb.count, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      ctx->view_readback.clear();
      return cuda_err(ctx, e, "view readback");
    }
  }
  ctx->view_readback.clear();
  return FOMO_OK;
}

}  // namespace fomo

// =========================================================================
// C ABI
// =========================================================================

extern "C" {

const char* fomo_version(void) { return kVersion; }

int fomo_ctx_create(int device, size_t hbm_budget_bytes, fomo_ctx** out) {
  if (!out) return FOMO_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    return FOMO_ENODEVICE;
  }
  if (device < 0 || device >= ndev) return FOMO_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return FOMO_ENODEVICE;
  fomo_ctx* ctx = new fomo_ctx();
  ctx->device = device;
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  ctx->sm_count = prop.multiProcessorCount;
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  ctx->budget = hbm_budget_bytes ? hbm_budget_bytes : (size_t)(0.9 * (double)fr);
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      ctx->scratch.init() != cudaSuccess || cudaMalloc(&ctx->stats_dev, 256) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->order_ev, cudaEventDisableTiming) != cudaSuccess) {
    delete ctx;
    return FOMO_EDEVICE;
  }
  if (const char* tc = std::getenv("FOMO_TUNE_CACHE")) load_tune_cache(ctx, tc);
  if (const char* nc = std::getenv("FOMO_NPOS_CAP")) {
    const long long v = std::atoll(nc);  // neighbour-buffer entries (4 B each) per launch
    if (v > 0) ctx->npos_cap = v;
  }
  if (const char* ms = std::getenv("FOMO_MARCH_STATS")) {
    if (ms[0] == '1' && cudaMalloc(&ctx->march_stats, sizeof(unsigned long long) * kStatCount) == cudaSuccess) {
      cudaMemset(ctx->march_stats, 0, sizeof(unsigned long long) * kStatCount);
      ctx->print_stats = true;
    }
  }
  if (const char* co = std::getenv("FOMO_CELL_OCCUPANCY")) {
    const double v = std::atof(co);  // target points per grid cell of the snapshots built afterwards
    if (v >= 0.25 && v <= 64.0) {
      ctx->cell_occupancy = v;
      ctx->occupancy_set = true;
    }
  }
  if (const char* fa = std::getenv("FOMO_INJECT_ALLOC_FAILURE")) ctx->fail_alloc_at = std::atol(fa);
  const char* tm = std::getenv("FOMO_TIME_MARCH");
  ctx->time_march = !(tm && tm[0] == '0');
  *out = ctx;
  return FOMO_OK;
}

int fomo_ctx_destroy(fomo_ctx* ctx) {
  if (!ctx) return FOMO_EINVAL;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& kv : ctx->graphs) {
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  }
  for (auto& kv : ctx->payloads) dev_free(ctx, kv.second);
  for (auto& kv : ctx->snaps) {
    dev_free(ctx, kv.second.block);
    dev_free(ctx, kv.second.totpol);
  }
  for (auto& kv : ctx->tables) dev_free(ctx, kv.second.d);
  dev_free(ctx, ctx->scratch.arena.base);
  dev_free(ctx, ctx->out_arena.base);
  release_free_blocks(ctx);
  if (ctx->stats_dev) cudaFree(ctx->stats_dev);
  if (ctx->timer.ev) {
    for (int i = 0; i < ctx->timer.cap; ++i) cudaEventDestroy(ctx->timer.ev[i]);
    delete[] ctx->timer.ev;
    delete[] ctx->timer.kind;
  }
  if (ctx->march_stats && !ctx->print_stats) cudaFree(ctx->march_stats);
  if (ctx->march_stats && ctx->print_stats) {
    unsigned long long h[kStatCount] = {0};
    cudaMemcpy(h, ctx->march_stats, sizeof(h), cudaMemcpyDeviceToHost);
    std::fprintf(stderr,
                 "fomo march stats: segments %llu candidates %llu rows %llu points_loaded %llu not_gathered %llu "
                 "fallbacks %llu (ambiguous %llu no_candidate %llu far %llu deferred %llu records %llu hard %llu) "
                 "samples %llu scanned %llu ties %llu\n",
                 h[kStatSegments], h[kStatCandidates], h[kStatRows], h[kStatPointsLoaded], h[kStatNotGathered],
                 h[kStatFallbacks], h[kStatFbAmb], h[kStatFbNoCand], h[kStatFbFar], h[kStatFbUnion],
                 h[kStatDeferredRecs], h[kStatHard], h[kStatSamples], h[kStatScanned], h[kStatTies]);
    cudaFree(ctx->march_stats);
  }
  ctx->scratch.release();
  for (cudaEvent_t ev : ctx->range_ev) cudaEventDestroy(ev);
  if (ctx->copy_stream) {
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
  }
  cudaEventDestroy(ctx->order_ev);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return FOMO_OK;
}

const char* fomo_last_error(const fomo_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int fomo_ctx_memory(const fomo_ctx* ctx, size_t* used, size_t* budget) {
  if (!ctx) return FOMO_EINVAL;
  if (used) *used = ctx->used;
  if (budget) *budget = ctx->budget;
  return FOMO_OK;
}

int fomo_ctx_synchronize(fomo_ctx* ctx) {
  if (!ctx) return FOMO_EINVAL;
  cudaSetDevice(ctx->device);
  FOMO_CUDA(cudaStreamSynchronize(ctx->stream), "synchronize");
  return check_device_words(ctx);
}

int fomo_host_register(fomo_ctx* ctx, void* ptr, size_t bytes) {
  if (!ctx || !ptr) return FOMO_EINVAL;
  FOMO_CUDA(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault), "cudaHostRegister");
  return FOMO_OK;
}

int fomo_host_unregister(fomo_ctx* ctx, void* ptr) {
  if (!ctx || !ptr) return FOMO_EINVAL;
  FOMO_CUDA(cudaHostUnregister(ptr), "cudaHostUnregister");
  return FOMO_OK;
}

int fomo_snapshot_create(fomo_ctx* ctx, int64_t n, const float* x, const float* y, const float* z, const float* n_e,
                         const float* T, const float* vx, const float* vy, const float* vz, int* id) {
  if (!ctx || !id) return FOMO_EINVAL;
  if (n <= 0 || n >= ((int64_t)1 << 31) - 1) return set_err(ctx, FOMO_EINVAL, "npoints must be in [1, 2^31-2]");
  if (!x || !y || !n_e || !T || !vx || !vy || !vz) return set_err(ctx, FOMO_EINVAL, "null input array");
  cudaSetDevice(ctx->device);
  const float* host[8] = {x, y, z, n_e, T, vx, vy, vz};
  SnapRec r;
  int rc = build_snapshot(ctx, n, host, &r);
  if (rc) return rc;
  rc = check_device_words(ctx);
  if (rc) {
    dev_free(ctx, r.block);
    return rc;
  }
  int nid = ctx->next_id++;
  ctx->snaps[nid] = r;
  *id = nid;
  return FOMO_OK;
}

int fomo_snapshot_create_device(fomo_ctx* ctx, int64_t n, const float* x, const float* y, const float* z,
                                const float* n_e, const float* T, const float* vx, const float* vy, const float* vz,
                                int* id) {
  if (!ctx || !id) return FOMO_EINVAL;
  const float* arrs[8] = {x, y, z, n_e, T, vx, vy, vz};
  for (const float* p : arrs) {
    if (!p) continue;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess || at.type != cudaMemoryTypeDevice) {
      cudaGetLastError();
      return set_err(ctx, FOMO_EINVAL, "fomo_snapshot_create_device needs device arrays");
    }
  }
  return fomo_snapshot_create(ctx, n, x, y, z, n_e, T, vx, vy, vz, id);
}

int fomo_abundance_ratio(fomo_ctx* ctx, const char* abund_file, const char* standard_file, const char* ion,
                         double* ratio) {
  if (!abund_file || !standard_file || !ion || !ratio) return FOMO_EINVAL;
  double a = 0, b = 0;
  std::string err;
  if (!abundance_of(abund_file, ion, &a, &err) || !abundance_of(standard_file, ion, &b, &err))
    return ctx ? set_err(ctx, FOMO_ETABLE, err) : FOMO_ETABLE;
  *ratio = a / b;
  return FOMO_OK;
}

int fomo_snapshot_destroy(fomo_ctx* ctx, int id) {
  if (!ctx) return FOMO_EINVAL;
  auto it = ctx->snaps.find(id);
  if (it == ctx->snaps.end()) return set_err(ctx, FOMO_ENOTFOUND, "unknown snapshot id");
  cudaStreamSynchronize(ctx->stream);
  for (auto p = ctx->payloads.begin(); p != ctx->payloads.end();) {
    if (std::get<0>(p->first) == id) {
      dev_free(ctx, p->second);
      p = ctx->payloads.erase(p);
    } else {
      ++p;
    }
  }
  dev_free(ctx, it->second.block);
  dev_free(ctx, it->second.totpol);
  ctx->snaps.erase(it);
  return FOMO_OK;
}

int fomo_snapshot_get_info(fomo_ctx* ctx, int id, fomo_snapshot_info* info) {
  if (!ctx || !info) return FOMO_EINVAL;
  auto it = ctx->snaps.find(id);
  if (it == ctx->snaps.end()) return set_err(ctx, FOMO_ENOTFOUND, "unknown snapshot id");
  const SnapRec& r = it->second;
  info->npoints = r.n;
  info->grid_dims[0] = r.g.dx;
  info->grid_dims[1] = r.g.dy;
  info->grid_dims[2] = r.g.dz;
  info->cell_edge = r.g.h;
  info->aabb[0] = r.g.minx;
  info->aabb[1] = r.g.miny;
  info->aabb[2] = r.g.minz;
  info->aabb[3] = r.g.maxx;
  info->aabb[4] = r.g.maxy;
  info->aabb[5] = r.g.maxz;
  info->device_bytes = r.bytes;
  return FOMO_OK;
}

int fomo_table_create(fomo_ctx* ctx, const char* ion, double lambda0, double atweight, const char* unit, int nt,
                      int nrho, const float* logT, const float* logn, const float* G, int* id) {
  if (!ctx || !id || !logT || !logn || !G) return FOMO_EINVAL;
  if (nt < 2 || nrho < 2) return set_err(ctx, FOMO_ETABLE, "table needs nt >= 2 and nrho >= 2");
  cudaSetDevice(ctx->device);
  TableHost t;
  t.ion = ion ? ion : "";
  t.unit = unit ? unit : "";
  t.lambda0 = lambda0;
  t.atweight = atweight;
  t.nt = nt;
  t.nrho = nrho;
  t.logT.assign(logT, logT + nt);
  t.logn.assign(logn, logn + nrho);
  t.G.assign(G, G + (size_t)nt * nrho);
  return upload_table(ctx, std::move(t), id);
}

int fomo_table_load(fomo_ctx* ctx, const char* path, int* id) {
  if (!ctx || !path || !id) return FOMO_EINVAL;
  std::ifstream f(path, std::ios::binary);
  if (!f) return set_err(ctx, FOMO_EIO, std::string("Error: no CHIANTI G(T) file exists: ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  TableHost t;
  std::string err;
  int rc = parse_table_text(ss.str(), &t, &err);
  if (rc) return set_err(ctx, rc, err);
  cudaSetDevice(ctx->device);
  return upload_table(ctx, std::move(t), id);
}

int fomo_table_destroy(fomo_ctx* ctx, int id) {
  if (!ctx) return FOMO_EINVAL;
  auto it = ctx->tables.find(id);
  if (it == ctx->tables.end()) return set_err(ctx, FOMO_ENOTFOUND, "unknown table id");
  cudaStreamSynchronize(ctx->stream);
  for (auto p = ctx->payloads.begin(); p != ctx->payloads.end();) {
    if (std::get<1>(p->first) == id) {
      dev_free(ctx, p->second);
      p = ctx->payloads.erase(p);
    } else {
      ++p;
    }
  }
  dev_free(ctx, it->second.d);
  ctx->tables.erase(it);
  return FOMO_OK;
}

int fomo_table_get_info(fomo_ctx* ctx, int id, double* lambda0, double* atweight, int* nt, int* nrho, int* is_dn,
                        char* ion, int ion_cap, char* unit, int unit_cap) {
  if (!ctx) return FOMO_EINVAL;
  auto it = ctx->tables.find(id);
  if (it == ctx->tables.end()) return set_err(ctx, FOMO_ENOTFOUND, "unknown table id");
  const TableHost& t = it->second.h;
  if (lambda0) *lambda0 = t.lambda0;
  if (atweight) *atweight = t.atweight;
  if (nt) *nt = t.nt;
  if (nrho) *nrho = t.nrho;
  if (is_dn) *is_dn = t.is_dn ? 1 : 0;
  if (ion && ion_cap > 0) std::snprintf(ion, (size_t)ion_cap, "%s", t.ion.c_str());
  if (unit && unit_cap > 0) std::snprintf(unit, (size_t)unit_cap, "%s", t.unit.c_str());
  return FOMO_OK;
}

int fomo_render_batch_device(fomo_ctx* ctx, const fomo_request* reqs, int nreq, float* const* d_outs, void* stream) {
  if (!ctx || !reqs || nreq <= 0 || !d_outs) return FOMO_EINVAL;
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  return enqueue_batch(ctx, reqs, nreq, d_outs, nullptr, s, nullptr, nullptr);
}

int fomo_render_device(fomo_ctx* ctx, const fomo_request* req, float* d_out_cube, int32_t* d_out_nn_idx,
                       fomo_view_info* info, void* stream) {
  if (!ctx || !req || !d_out_cube) return FOMO_EINVAL;
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  std::vector<ViewDesc> views;
  std::vector<int> vof;
  float* outs[1] = {d_out_cube};
  int32_t* nns[1] = {d_out_nn_idx};
  int rc = enqueue_batch(ctx, req, 1, outs, nns, s, info ? &views : nullptr, &vof);
  if (rc) return rc;
  if (info) {
    FOMO_CUDA(cudaStreamSynchronize(s), "render");
    rc = check_device_words(ctx);
    if (rc) return rc;
    rc = finish_views(ctx, &views);
    if (rc) return rc;
    const TableHost* t = uses_table(req->method) ? &ctx->tables[req->table].h : nullptr;
    view_info_from(views[vof[0]], *req, t, info);
  }
  return FOMO_OK;
}

int fomo_render_batch(fomo_ctx* ctx, const fomo_request* reqs, int nreq, float* const* outs, fomo_view_info* infos) {
  if (!ctx || !reqs || nreq <= 0 || !outs) return FOMO_EINVAL;
  NvtxRange range("fomo: render batch to host");
  cudaSetDevice(ctx->device);
  for (int r = 0; r < nreq; ++r) {
    int rc = validate(ctx, reqs[r]);
    if (rc) return rc;
    if (!outs[r]) return set_err(ctx, FOMO_EINVAL, "null output buffer");
  }
  // device outputs in the output arena
  std::vector<size_t> off(nreq);
  size_t total = 0;
  for (int r = 0; r < nreq; ++r) {
    off[r] = total;
    total += (cube_elems(reqs[r]) * sizeof(float) + 255) & ~size_t(255);
  }
  int rc = ctx->out_arena.reserve(ctx, total);
  if (rc) return rc;
  if (!ctx->copy_stream) FOMO_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking), "copy stream");
  std::vector<float*> d(nreq);
  for (int r = 0; r < nreq; ++r) d[r] = reinterpret_cast<float*>(ctx->out_arena.base + off[r]);
  // The cubes of each range of views download on the copy stream while the
  // next range marches.  A range's downloads are issued after the next
  // range's march is queued: into pageable memory they return only when done.
  std::vector<int> pending;  // requests of the range before
  size_t nev = 0;
  auto download = [&](const std::vector<int>& rs) -> int {
    for (int r : rs)
      FOMO_CUDA(cudaMemcpyAsync(outs[r], d[r], cube_elems(reqs[r]) * sizeof(float), cudaMemcpyDeviceToHost,
                                ctx->copy_stream),
                "cube download");
    return FOMO_OK;
  };
  RangeDone done = [&](const PlanGroup& G, int v0, int v1) -> int {
    if (nev == ctx->range_ev.size()) {
      cudaEvent_t ev = nullptr;
      FOMO_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "range event");
      ctx->range_ev.push_back(ev);
    }
    const cudaEvent_t ev = ctx->range_ev[nev++];
    FOMO_CUDA(cudaEventRecord(ev, ctx->stream), "range event");
    int rc2 = download(pending);
    pending.clear();
    FOMO_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ev, 0), "range wait");
    for (int v = v0; v < v1; ++v) pending.insert(pending.end(), G.vreqs[v].begin(), G.vreqs[v].end());
    return rc2;
  };
  std::vector<ViewDesc> views;
  std::vector<int> vof;
  rc = enqueue_batch(ctx, reqs, nreq, d.data(), nullptr, ctx->stream, infos ? &views : nullptr, &vof, &done);
  if (rc == FOMO_OK) rc = download(pending);
  // the caller's buffers must not be written after return, error or not
  const cudaError_t e1 = cudaStreamSynchronize(ctx->copy_stream);
  const cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
  if (rc) return rc;
  FOMO_CUDA(e1 != cudaSuccess ? e1 : e2, "render");
  rc = check_device_words(ctx);
  if (rc) return rc;
  if (ctx->time_march) cudaEventElapsedTime(&ctx->last_ms, ctx->scratch.ev0, ctx->scratch.ev1);
  if (infos) {
    rc = finish_views(ctx, &views);
    if (rc) return rc;
    for (int r = 0; r < nreq; ++r) {
      const TableHost* t = uses_table(reqs[r].method) ? &ctx->tables[reqs[r].table].h : nullptr;
      view_info_from(views[vof[r]], reqs[r], t, &infos[r]);
    }
  }
  return FOMO_OK;
}

int fomo_render(fomo_ctx* ctx, const fomo_request* req, float* out_cube, int32_t* out_nn_idx, fomo_view_info* info) {
  if (!ctx || !req || !out_cube) return FOMO_EINVAL;
  NvtxRange range("fomo: render to host");
  cudaSetDevice(ctx->device);
  int rc = validate(ctx, *req);
  if (rc) return rc;
  const size_t cube_bytes = (cube_elems(*req) * sizeof(float) + 255) & ~size_t(255);
  const size_t nn_bytes = out_nn_idx ? (size_t)req->nx * req->ny * req->nz * sizeof(int32_t) : 0;
  rc = ctx->out_arena.reserve(ctx, cube_bytes + nn_bytes);
  if (rc) return rc;
  float* d_cube = reinterpret_cast<float*>(ctx->out_arena.base);
  int32_t* d_nn = out_nn_idx ? reinterpret_cast<int32_t*>(ctx->out_arena.base + cube_bytes) : nullptr;
  std::vector<ViewDesc> views;
  std::vector<int> vof;
  float* outs[1] = {d_cube};
  int32_t* nns[1] = {d_nn};
  rc = enqueue_batch(ctx, req, 1, outs, nns, ctx->stream, info ? &views : nullptr, &vof);
  if (rc) return rc;
  FOMO_CUDA(cudaMemcpyAsync(out_cube, d_cube, cube_elems(*req) * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
            "cube download");
  if (d_nn)
    FOMO_CUDA(cudaMemcpyAsync(out_nn_idx, d_nn, nn_bytes, cudaMemcpyDeviceToHost, ctx->stream), "index download");
  FOMO_CUDA(cudaStreamSynchronize(ctx->stream), "render");
  rc = check_device_words(ctx);
  if (rc) return rc;
  if (ctx->time_march) cudaEventElapsedTime(&ctx->last_ms, ctx->scratch.ev0, ctx->scratch.ev1);
  if (info) {
    rc = finish_views(ctx, &views);
    if (rc) return rc;
    const TableHost* t = uses_table(req->method) ? &ctx->tables[req->table].h : nullptr;
    view_info_from(views[vof[0]], *req, t, info);
  }
  return FOMO_OK;
}

int fomo_emission(fomo_ctx* ctx, int snapshot, int table, int imaging, double abundratio, float* eps, float* fwhm) {
  if (!ctx || !eps || !fwhm) return FOMO_EINVAL;
  cudaSetDevice(ctx->device);
  auto sit = ctx->snaps.find(snapshot);
  if (sit == ctx->snaps.end()) return set_err(ctx, FOMO_ENOTFOUND, "unknown snapshot id");
  const float2* ew = nullptr;
  int rc = get_payload(ctx, snapshot, table, imaging ? 1 : 0, abundratio, &ew);
  if (rc) return rc;
  const int64_t n = sit->second.n;
  rc = ctx->out_arena.reserve(ctx, sizeof(float) * 2 * (size_t)n);
  if (rc) return rc;
  float* a = reinterpret_cast<float*>(ctx->out_arena.base);
  float* b = a + n;
  FOMO_CUDA(launch_unsort_payload(sit->second.pts, ew, n, a, b, ctx->stream), "emission unsort");
  FOMO_CUDA(cudaMemcpyAsync(eps, a, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream), "emission download");
  FOMO_CUDA(cudaMemcpyAsync(fwhm, b, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream), "emission download");
  FOMO_CUDA(cudaStreamSynchronize(ctx->stream), "emission");
  return check_device_words(ctx);
}

int fomo_thomson_emission(fomo_ctx* ctx, int snapshot, float* tot, float* pol) {
  if (!ctx || !tot || !pol) return FOMO_EINVAL;
  cudaSetDevice(ctx->device);
  auto sit = ctx->snaps.find(snapshot);
  if (sit == ctx->snaps.end()) return set_err(ctx, FOMO_ENOTFOUND, "unknown snapshot id");
  const float2* tp = nullptr;
  int rc = get_thomson_payload(ctx, sit->second, &tp);
  if (rc) return rc;
  const int64_t n = sit->second.n;
  rc = ctx->out_arena.reserve(ctx, sizeof(float) * 2 * (size_t)n);
  if (rc) return rc;
  float* a = reinterpret_cast<float*>(ctx->out_arena.base);
  float* b = a + n;
  FOMO_CUDA(launch_unsort_payload(sit->second.pts, tp, n, a, b, ctx->stream), "Thomson unsort");
  FOMO_CUDA(cudaMemcpyAsync(tot, a, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream), "Thomson download");
  FOMO_CUDA(cudaMemcpyAsync(pol, b, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream), "Thomson download");
  FOMO_CUDA(cudaStreamSynchronize(ctx->stream), "Thomson emission");
  return FOMO_OK;
}

int fomo_set_march_config(fomo_ctx* ctx, int tile_w, int tile_h, int blocks_per_sm) {
  if (!ctx || tile_w < 0 || tile_h < 0 || blocks_per_sm < 0) return FOMO_EINVAL;
  if ((tile_w == 0) != (tile_h == 0)) return set_err(ctx, FOMO_EINVAL, "set both tile dimensions or neither");
  ctx->tile_w = tile_w;
  ctx->tile_h = tile_h;
  ctx->blocks_per_sm = blocks_per_sm;
  return FOMO_OK;
}

int fomo_set_profiling(fomo_ctx* ctx, int kernel_timing, int counters) {
  if (!ctx) return FOMO_EINVAL;
  cudaSetDevice(ctx->device);
  static_assert(kKCount == FOMO_KERNEL_COUNT, "kernel kinds of include/fomo_gpu.h");
  static_assert(kStatCount == FOMO_COUNTER_COUNT, "counters of include/fomo_gpu.h");
  if (kernel_timing && !ctx->timer.ev) {
    const int cap = 4096;
    ctx->timer.ev = new cudaEvent_t[cap]();
    ctx->timer.kind = new int[cap]();
    for (int i = 0; i < cap; ++i) {
      if (cudaEventCreate(&ctx->timer.ev[i]) != cudaSuccess) {
        for (int k = 0; k < i; ++k) cudaEventDestroy(ctx->timer.ev[k]);
        delete[] ctx->timer.ev;
        delete[] ctx->timer.kind;
        ctx->timer.ev = nullptr;
        ctx->timer.kind = nullptr;
        return cuda_err(ctx, cudaGetLastError(), "profiling events");
      }
    }
    ctx->timer.cap = cap;
  }
  ctx->kernel_timing = kernel_timing != 0;
  ctx->timer.n = 0;
  if (counters && !ctx->march_stats) {
    FOMO_CUDA(cudaMalloc(&ctx->march_stats, sizeof(unsigned long long) * kStatCount), "profiling counters");
    FOMO_CUDA(cudaMemset(ctx->march_stats, 0, sizeof(unsigned long long) * kStatCount), "profiling counters");
  } else if (!counters && ctx->march_stats && !ctx->print_stats) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->march_stats);
    ctx->march_stats = nullptr;
  }
  return FOMO_OK;
}

int fomo_profile_read(fomo_ctx* ctx, float* kernel_ms, int nk, uint64_t* counters, int nc) {
  if (!ctx || nk < 0 || nc < 0) return FOMO_EINVAL;
  cudaSetDevice(ctx->device);
  if (kernel_ms) {
    for (int k = 0; k < nk; ++k) kernel_ms[k] = 0.0f;
    const MarchTimer& t = ctx->timer;
    if (t.n > 0) FOMO_CUDA(cudaEventSynchronize(t.ev[t.n - 1]), "profiling events");
    for (int i = 1; i < t.n; ++i) {
      if (t.kind[i] < 0 || t.kind[i] >= nk) continue;
      float ms = 0.0f;
      FOMO_CUDA(cudaEventElapsedTime(&ms, t.ev[i - 1], t.ev[i]), "profiling events");
      kernel_ms[t.kind[i]] += ms;
    }
  }
  if (counters) {
    for (int k = 0; k < nc; ++k) counters[k] = 0;
    if (ctx->march_stats) {
      unsigned long long h[kStatCount] = {0};
      FOMO_CUDA(cudaDeviceSynchronize(), "profiling counters");  // the render may be on a caller's stream
      FOMO_CUDA(cudaMemcpy(h, ctx->march_stats, sizeof(h), cudaMemcpyDeviceToHost), "profiling counters");
      FOMO_CUDA(cudaMemset(ctx->march_stats, 0, sizeof(h)), "profiling counters");
      for (int k = 0; k < nc && k < kStatCount; ++k) counters[k] = h[k];
    }
  }
  return FOMO_OK;
}

int fomo_last_march_ms(fomo_ctx* ctx, float* ms) {
  if (!ctx || !ms) return FOMO_EINVAL;
  // events around the last march issued from the context's scratch set
  // (direct launches and graph replays alike)
  if (!ctx->time_march) return set_err(ctx, FOMO_EINVAL, "march timing disabled (FOMO_TIME_MARCH=0)");
  FOMO_CUDA(cudaEventSynchronize(ctx->scratch.ev1), "march timing");
  float t = 0;
  FOMO_CUDA(cudaEventElapsedTime(&t, ctx->scratch.ev0, ctx->scratch.ev1), "march timing");
  ctx->last_ms = t;
  *ms = t;
  return FOMO_OK;
}

}  // extern "C"
