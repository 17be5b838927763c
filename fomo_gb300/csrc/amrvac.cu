// AMRVAC snapshots straight into a resident snapshot: the ingestion of the
// reference's AMRVAC example (fomo-c/example/example_mpi_amrvac/
// read_amrvac_files.cpp), which reads a data file and pushes every cell into a
// FoMoObject one point at a time.
//
// Host: the data file's header, its tree ("forest") and leaf blocks are
// parsed; the leaves are ordered as the reference orders them (level-1 blocks
// in Morton order, or x fastest for pre-2017 files with amrvac_version "old",
// each walked depth first through the tree, :20-44 and :183-226); the blocks'
// values are repacked into one aligned array (version 3/4 files put two
// ghost-cell counts per dimension before each block).
// Device: one thread per cell computes the cell's position and n, T, v in
// FP64 in the reference's operation order (fomo_from_amrvac, :228-299; explicit
// __dadd_rn/__dmul_rn/__ddiv_rn, so no FMA contraction changes a rounding) and
// rounds them to FP32 as the DataCube stores them.  The arrays then go through
// the regular snapshot build (spatial index, resident on the device).
//
// Reference quirks kept for parity: T uses the first two momentum and magnetic
// components only (std::inner_product over [1, 3) and [5, 7), :266-268); the
// cell's second coordinate index is k / nx0 % nx0 (:254).  Reference faults
// not kept: a version-3 file is read by the version-3 reader only (the
// reference's dispatch falls through to the pre-2017 reader afterwards,
// :700-713), and variable names are the 16-byte fields of the file (the
// reference reads them as unterminated C strings).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/fomo_gpu.h"
#include "fomo_consts.h"
#include "fomo_device.cuh"
#include "runtime_internal.h"

namespace fomo {
namespace {

struct AmrvacGrid {
  int ndim = 0, nw = 0, nleafs = 0;
  int nx[3] = {1, 1, 1};
  double xprobmin[3] = {0, 0, 0};
  double cellsize[3] = {0, 0, 0};
  double gamma = 0.0;
  std::vector<int4> leaves;    // level, 1-based index at that level
  std::vector<double> blocks;  // nleafs x nw x nglev1, each block variable-major as in the file
  int64_t nglev1() const { return (int64_t)nx[0] * nx[1] * (ndim == 3 ? nx[2] : 1); }
};

// mortonEncode_for (FoMo-amrvac.h:13-19): bit i of x, y, z to bits 3i, 3i+1, 3i+2.
uint64_t morton3(unsigned x, unsigned y, unsigned z) {
  uint64_t r = 0;
  for (int i = 0; i < 21; ++i)
    r |= ((uint64_t)((x >> i) & 1u) << (3 * i)) | ((uint64_t)((y >> i) & 1u) << (3 * i + 1)) |
         ((uint64_t)((z >> i) & 1u) << (3 * i + 2));
  return r;
}

// loopthroughleafs (:20-44), depth first; false when the tree is shorter
// than its walk.
bool walk_leaves(const std::vector<int>& forest, int64_t& pos, int level, int ndim, int i0, int i1, int i2,
                 std::vector<int4>& out) {
  ++pos;
  if (pos >= (int64_t)forest.size()) return false;
  if (forest[pos]) {
    out.push_back(make_int4(level, i0, i1, i2));
    return true;
  }
  for (int i = 0; i < (1 << ndim); ++i) {
    const int n0 = 2 * (i0 - 1) + 1 + i % 2;
    const int n1 = ndim == 2 ? 2 * (i1 - 1) + 1 + i / 2 : 2 * (i1 - 1) + 1 + (i / 2) % 2;
    const int n2 = ndim == 2 ? 1 : 2 * (i2 - 1) + 1 + i / 4;
    if (!walk_leaves(forest, pos, level + 1, ndim, n0, n1, n2, out)) return false;
  }
  return true;
}

template <typename T>
bool get(const std::string& buf, size_t off, T* v) {
  if (off + sizeof(T) > buf.size()) return false;
  std::memcpy(v, buf.data() + off, sizeof(T));
  return true;
}

// A 16-byte name field: trailing blanks and NULs removed.
std::string name16(const std::string& buf, size_t off) {
  std::string s = off + 16 <= buf.size() ? buf.substr(off, 16) : std::string();
  while (!s.empty() && (s.back() == ' ' || s.back() == '\0')) s.pop_back();
  const size_t z = s.find('\0');
  return z == std::string::npos ? s : s.substr(0, z);
}

// read_amrvac_par_file (:50-112): the first "nxlone<d>", "xprobmin<d>",
// "xprobmax<d>"; the value starts after the next tab, newline, '=' or blank.
bool par_value(const std::string& text, const std::string& key, double* v) {
  const size_t at = text.find(key);
  if (at == std::string::npos) return false;
  const size_t start = text.find_first_of("\t\n= ", at + 1);
  if (start == std::string::npos) return false;
  *v = std::strtod(text.c_str() + start + 1, nullptr);
  return true;
}

int parse_amrvac(const char* datfile, const char* amrvacpar, const char* amrvac_version, int gamma_pos,
                 AmrvacGrid* G, std::string* err) {
  std::ifstream f(datfile, std::ios::binary);
  if (!f) {
    *err = std::string(".dat file not found at ") + datfile;
    return FOMO_EIO;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string buf = ss.str();
  auto bad = [&](const char* what) {
    *err = std::string("AMRVAC data file ") + datfile + ": " + what;
    return FOMO_ETABLE;
  };
  int version = 0;
  if (!get(buf, 0, &version)) return bad("too short");
  int nxlone[3] = {1, 1, 1}, nparents = 0, neqpar = 0;
  double xprobmax[3] = {0, 0, 0};
  size_t treeoff = 0, blockoff = 0;
  int64_t nforest = 0;
  bool ghosts = false;
  if (version == 3 || version == 4) {
    // read_amrvac_new_dat_file (:430-528), read_amrvac_dat_file_v4 (:535-683)
    int hdr[10];
    for (int i = 0; i < 10; ++i)
      if (!get(buf, 4 * i, &hdr[i])) return bad("truncated header");
    treeoff = (size_t)hdr[1];
    blockoff = (size_t)hdr[2];
    G->nw = hdr[3];
    G->ndim = hdr[5];
    G->nleafs = hdr[7];
    nparents = hdr[8];
    if (G->ndim < 2 || G->ndim > 3) return bad("only 2-D and 3-D data are read");
    size_t off = 48;
    for (int i = 0; i < G->ndim; ++i, off += 8) get(buf, off, &G->xprobmin[i]);
    for (int i = 0; i < G->ndim; ++i, off += 8) get(buf, off, &xprobmax[i]);
    for (int i = 0; i < G->ndim; ++i, off += 4) get(buf, off, &nxlone[i]);
    for (int i = 0; i < G->ndim; ++i, off += 4) get(buf, off, &G->nx[i]);
    off += 16 * (size_t)G->nw + 16;  // variable names, physics module
    if (!get(buf, off, &neqpar) || neqpar < 0) return bad("truncated equation parameters");
    off += 4;
    for (int i = 0; i < neqpar; ++i) {
      double v = 0;
      if (!get(buf, off + 8 * (size_t)i, &v)) return bad("truncated equation parameters");
      // the last parameter named "gamma" (:503-511); version 4 compares the
      // name's first five characters only (:637-646)
      const std::string nm = name16(buf, off + 8 * (size_t)neqpar + 16 * (size_t)i);
      if (version == 4 ? nm.substr(0, 5) == "gamma" : nm == "gamma") G->gamma = v;
    }
    if (G->gamma == 0.0) return bad("no value for gamma found");
    nforest = (int64_t)nparents + G->nleafs;
    ghosts = true;  // two ghost-cell counts per dimension before each block (:159-177)
  } else {
    // read_amrvac_old_dat_file (:301-418): the header at the end of the file
    if (buf.size() < 36) return bad("too short");
    const size_t tail = buf.size() - 8 - 7 * 4;
    int t[7];
    for (int i = 0; i < 7; ++i) get(buf, tail + 4 * i, &t[i]);
    G->nleafs = t[0];
    G->ndim = t[2];
    G->nw = t[4];
    neqpar = t[5];
    if (G->ndim < 2 || G->ndim > 3) return bad("only 2-D and 3-D data are read");
    if (neqpar < 0 || gamma_pos < 0 || gamma_pos >= neqpar) return bad("gamma_eqparposition out of range");
    const size_t eqoff = tail - 8 * (size_t)neqpar;
    const size_t nxoff = eqoff - 4 * (size_t)G->ndim;
    for (int i = 0; i < G->ndim; ++i) get(buf, nxoff + 4 * i, &G->nx[i]);
    get(buf, eqoff + 8 * (size_t)gamma_pos, &G->gamma);
    blockoff = 0;
    treeoff = (size_t)G->nleafs * G->nw * G->nglev1() * 8;
    if (treeoff > nxoff) return bad("blocks larger than the file");
    nforest = (int64_t)(nxoff - treeoff) / 4;
    std::ifstream pf(amrvacpar ? amrvacpar : "");
    if (!pf) {
      *err = std::string("amrvac.par file not found at ") + (amrvacpar ? amrvacpar : "(null)");
      return FOMO_EIO;
    }
    std::stringstream ps;
    ps << pf.rdbuf();
    const std::string text = ps.str();
    const char* keys[3] = {"nxlone", "xprobmin", "xprobmax"};
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < G->ndim; ++i) {
        double v = 0;
        if (!par_value(text, std::string(keys[j]) + std::to_string(i + 1), &v)) {
          *err = std::string(amrvacpar) + " does not contain the key " + keys[j] + std::to_string(i + 1);
          return FOMO_ETABLE;
        }
        if (j == 0) nxlone[i] = (int)v;
        if (j == 1) G->xprobmin[i] = v;
        if (j == 2) xprobmax[i] = v;
      }
  }
  if (G->nleafs <= 0 || G->nw < 8) return bad("expected MHD data (rho, m1..m3, e, b1..b3) in at least one block");
  for (int i = 0; i < G->ndim; ++i)
    if (G->nx[i] <= 0 || nxlone[i] <= 0) return bad("bad block or domain size");
  // blocksandsize (:114-129)
  int nblocks[3] = {1, 1, 1};
  for (int i = 0; i < G->ndim; ++i) {
    if (nxlone[i] % G->nx[i] != 0) return bad("non-integer number of blocks");
    nblocks[i] = nxlone[i] / G->nx[i];
    G->cellsize[i] = (xprobmax[i] - G->xprobmin[i]) / nxlone[i];
  }
  std::vector<int> forest((size_t)std::max<int64_t>(nforest, 0));
  for (int64_t i = 0; i < nforest; ++i)
    if (!get(buf, treeoff + 4 * (size_t)i, &forest[(size_t)i])) return bad("truncated tree");
  // the leaves in the reference's order
  int64_t pos = -1;
  G->leaves.clear();
  const bool xfast = !(version == 3 || version == 4) && std::string(amrvac_version ? amrvac_version : "") == "old";
  if (!(version == 3 || version == 4) && !xfast && std::string(amrvac_version ? amrvac_version : "") != "gitlab") {
    *err = std::string("The stated AMRVAC implementation ") + (amrvac_version ? amrvac_version : "(null)") +
           " is not known (\"old\" or \"gitlab\").";
    return FOMO_EINVAL;
  }
  std::vector<int4> order;  // level-1 blocks, 0-based
  for (int k = 0; k < nblocks[2]; ++k)
    for (int j = 0; j < nblocks[1]; ++j)
      for (int i = 0; i < nblocks[0]; ++i) order.push_back(make_int4(i, j, k, 0));
  if (!xfast)
    std::stable_sort(order.begin(), order.end(), [](const int4& a, const int4& b) {
      return morton3(a.x, a.y, a.z) < morton3(b.x, b.y, b.z);
    });
  for (const int4& o : order)
    if (!walk_leaves(forest, pos, 1, G->ndim, o.x + 1, o.y + 1, o.z + 1, G->leaves)) return bad("tree shorter than its walk");
  if ((int)G->leaves.size() != G->nleafs) return bad("the tree's leaves do not match nleafs");
  // the blocks, repacked contiguous and 8-byte aligned
  const int64_t per = (int64_t)G->nw * G->nglev1();
  G->blocks.resize((size_t)(per * G->nleafs));
  size_t off = blockoff;
  for (int b = 0; b < G->nleafs; ++b) {
    if (ghosts) off += 8 * (size_t)G->ndim;
    if (off + 8 * (size_t)per > buf.size()) return bad("truncated blocks");
    std::memcpy(G->blocks.data() + (size_t)b * per, buf.data() + off, 8 * (size_t)per);
    off += 8 * (size_t)per;
  }
  return FOMO_OK;
}

struct AmrvacConst {
  int ndim, nw, nx0, nx1, nx2;
  int64_t nglev1, npts;
  double xprobmin[3], cellsize[3];
  double gamma, n_unit, Teunit, L_unit, V_unit;
};

// fomo_from_amrvac (:228-299): cell k of leaf b.
__global__ void amrvac_cells_kernel(const double* __restrict__ blocks, const int4* __restrict__ leaves, AmrvacConst c,
                                    float* __restrict__ x, float* __restrict__ y, float* __restrict__ z,
                                    float* __restrict__ ne, float* __restrict__ T, float* __restrict__ vx,
                                    float* __restrict__ vy, float* __restrict__ vz) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < c.npts; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = p / c.nglev1, k = p - b * c.nglev1;
    const int4 lf = leaves[b];
    const double p2 = ldexp(1.0, lf.x - 1);  // pow(2, level - 1), exact
    const int idx[3] = {lf.y, lf.z, lf.w};
    const int nx[3] = {c.nx0, c.nx1, c.nx2};
    const int64_t lc[3] = {1 + k % c.nx0, 1 + k / c.nx0 % c.nx0, 1 + k / c.nx0 / c.nx1};
    double cc[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < c.ndim; ++j) {
      // bottomleft = xprobmin + (idx - 1) * cellsize * nx / 2^(level-1); local cell size cellsize / 2^(level-1)
      const double bl = __dadd_rn(c.xprobmin[j],
                                  __ddiv_rn(__dmul_rn(__dmul_rn((double)(idx[j] - 1), c.cellsize[j]), (double)nx[j]), p2));
      const double lcs = __ddiv_rn(c.cellsize[j], p2);
      cc[j] = __dmul_rn(__dadd_rn(bl, __dmul_rn(__dsub_rn((double)lc[j], .5), lcs)), c.L_unit);
    }
    const double* v = blocks + FOMO_IDX(b, c.npts / c.nglev1, kSitePts) * (int64_t)c.nw * c.nglev1 + k;
    const double rho = v[0], m1 = v[c.nglev1], m2 = v[2 * c.nglev1], m3 = v[3 * c.nglev1];
    const double e = v[4 * c.nglev1], b1 = v[5 * c.nglev1], b2 = v[6 * c.nglev1];
    const double kin = __ddiv_rn(__ddiv_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(m1, m1)), __dmul_rn(m2, m2)), rho), 2.0);
    const double mag = __ddiv_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(b1, b1)), __dmul_rn(b2, b2)), 2.0);
    const double pr = __dmul_rn(__dsub_rn(c.gamma, 1.0), __dsub_rn(__dsub_rn(e, kin), mag));
    x[p] = __double2float_rn(cc[0]);
    y[p] = __double2float_rn(cc[1]);
    z[p] = __double2float_rn(cc[2]);
    ne[p] = __double2float_rn(__dmul_rn(rho, c.n_unit));
    T[p] = __double2float_rn(__dmul_rn(__ddiv_rn(pr, rho), c.Teunit));
    vx[p] = __double2float_rn(__dmul_rn(__ddiv_rn(m1, rho), c.V_unit));
    vy[p] = __double2float_rn(__dmul_rn(__ddiv_rn(m2, rho), c.V_unit));
    vz[p] = __double2float_rn(__dmul_rn(__ddiv_rn(m3, rho), c.V_unit));
  }
}

// Parse the file and compute the points on the device into d8 (8 arrays of
// npts floats: x, y, z, n, T, vx, vy, vz) allocated here; the caller frees it.
int amrvac_points(fomo_ctx* ctx, const char* datfile, const char* amrvacpar, const char* amrvac_version,
                  int gamma_pos, double n_unit, double Teunit, double L_unit, float** d8, int64_t* npts,
                  int* ndim) {
  AmrvacGrid G;
  std::string err;
  int rc = parse_amrvac(datfile, amrvacpar, amrvac_version, gamma_pos, &G, &err);
  if (rc) return set_err(ctx, rc, err);
  AmrvacConst c;
  std::memset(&c, 0, sizeof(c));
  c.ndim = G.ndim;
  c.nw = G.nw;
  c.nx0 = G.nx[0];
  c.nx1 = G.nx[1];
  c.nx2 = G.nx[2];
  c.nglev1 = G.nglev1();
  c.npts = c.nglev1 * G.nleafs;
  if (c.npts >= ((int64_t)1 << 31) - 1) return set_err(ctx, FOMO_EINVAL, "AMRVAC snapshot has 2^31 or more cells");
  for (int i = 0; i < 3; ++i) {
    c.xprobmin[i] = G.xprobmin[i];
    c.cellsize[i] = G.cellsize[i];
  }
  c.gamma = G.gamma;
  c.n_unit = n_unit;
  c.Teunit = Teunit;
  c.L_unit = L_unit;
  // V_unit = sqrt(R_spec Teunit), R_spec = k_B / (0.5 m_p) (:14-16, :233)
  c.V_unit = std::sqrt(FOMO_BOLTZMANN / (0.5e0 * FOMO_MASS_PROTON) * Teunit);
  void* dblk = nullptr;
  void* dlf = nullptr;
  void* dout = nullptr;
  rc = dev_alloc(ctx, &dblk, sizeof(double) * G.blocks.size());
  if (!rc) rc = dev_alloc(ctx, &dlf, sizeof(int4) * G.leaves.size());
  if (!rc) rc = dev_alloc(ctx, &dout, sizeof(float) * 8 * (size_t)c.npts);
  cudaError_t e = cudaSuccess;
  if (!rc) {
    cudaStream_t s = ctx->stream;
    e = cudaMemcpyAsync(dblk, G.blocks.data(), sizeof(double) * G.blocks.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dlf, G.leaves.data(), sizeof(int4) * G.leaves.size(), cudaMemcpyHostToDevice, s);
    float* o = static_cast<float*>(dout);
    const int64_t n = c.npts;
    if (e == cudaSuccess) {
      const int threads = 256;
      const int64_t blocks = std::min<int64_t>((n + threads - 1) / threads, (int64_t)ctx->sm_count * 16);
      amrvac_cells_kernel<<<(unsigned)std::max<int64_t>(blocks, 1), threads, 0, s>>>(
          static_cast<const double*>(dblk), static_cast<const int4*>(dlf), c, o, o + n, o + 2 * n, o + 3 * n,
          o + 4 * n, o + 5 * n, o + 6 * n, o + 7 * n);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the host copies of the blocks are released below
  }
  dev_free(ctx, dblk);
  dev_free(ctx, dlf);
  if (rc || e != cudaSuccess) {
    dev_free(ctx, dout);
    return rc ? rc : cuda_err(ctx, e, "AMRVAC cells");
  }
  *d8 = static_cast<float*>(dout);
  *npts = c.npts;
  *ndim = c.ndim;
  return FOMO_OK;
}

}  // namespace

FOMO_DEFINE_CHECK_READER(check_word_amrvac)

}  // namespace fomo

using namespace fomo;

extern "C" int fomo_snapshot_from_amrvac(fomo_ctx* ctx, const char* datfile, const char* amrvacpar,
                                         const char* amrvac_version, int gamma_eqparposition, double n_unit,
                                         double Teunit, double L_unit, int* id) {
  if (!ctx || !datfile || !id) return FOMO_EINVAL;
  cudaSetDevice(ctx->device);
  float* d = nullptr;
  int64_t n = 0;
  int ndim = 0;
  int rc = amrvac_points(ctx, datfile, amrvacpar, amrvac_version, gamma_eqparposition, n_unit, Teunit, L_unit, &d,
                         &n, &ndim);
  if (rc) return rc;
  const float* arr[8];
  for (int k = 0; k < 8; ++k) arr[k] = d + (size_t)k * n;
  if (ndim == 2) arr[2] = nullptr;  // 2-D data: z = 0 (fomo-nearestneighbour.cpp:82)
  SnapRec r;
  rc = build_snapshot(ctx, n, arr, &r);
  dev_free(ctx, d);
  if (rc) return rc;
  const int nid = ctx->next_id++;
  ctx->snaps[nid] = r;
  *id = nid;
  return FOMO_OK;
}

extern "C" int fomo_amrvac_points(fomo_ctx* ctx, const char* datfile, const char* amrvacpar,
                                  const char* amrvac_version, int gamma_eqparposition, double n_unit, double Teunit,
                                  double L_unit, int64_t cap, int64_t* npoints, int* ndim, float* x, float* y,
                                  float* z, float* n_e, float* T, float* vx, float* vy, float* vz) {
  if (!ctx || !datfile || !npoints || !ndim) return FOMO_EINVAL;
  cudaSetDevice(ctx->device);
  float* d = nullptr;
  int64_t n = 0;
  int rc = amrvac_points(ctx, datfile, amrvacpar, amrvac_version, gamma_eqparposition, n_unit, Teunit, L_unit, &d, &n,
                         ndim);
  if (rc) return rc;
  *npoints = n;
  if (!x) {
    dev_free(ctx, d);
    return FOMO_OK;  // the size query
  }
  if (n > cap) {
    dev_free(ctx, d);
    return set_err(ctx, FOMO_EINVAL, "output arrays hold fewer points than the snapshot has");
  }
  float* outs[8] = {x, y, z, n_e, T, vx, vy, vz};
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 8 && e == cudaSuccess; ++k)
    if (outs[k]) e = cudaMemcpy(outs[k], d + (size_t)k * n, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost);
  dev_free(ctx, d);
  if (e != cudaSuccess) return cuda_err(ctx, e, "AMRVAC points download");
  return check_device_words(ctx);
}
