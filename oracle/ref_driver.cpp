// Test-harness driver for the reference FoMo-C library built from its own,
// unmodified sources (see oracle/Makefile, target `ref`).  It drives the
// reference through its public API exactly as a user program does
// (fomo-c/example/example.cpp:28-114): FoMoObject::setdata, setchiantifile,
// setabundfile, setrendermethod, setresolution, render(l,b), readrendering().
// The extern "C" entry points below only marshal plain arrays so the Python
// tests can generate golden vectors from the reference itself.
//
// This file is test infrastructure: nothing in the product library links it.
#include <algorithm>
#include <cstring>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "FoMo.h"
#include "FoMo-internal.h"  // has no include guard and needs FoMo.h first
#include "FoMo-amrvac.h"    // the reference's AMRVAC reader (its example directory)

namespace {

// The reference prints progress to std::cout on every call; silence it.
struct QuietCout {
  std::ostringstream sink;
  std::streambuf* saved;
  QuietCout() : saved(std::cout.rdbuf(sink.rdbuf())) {}
  ~QuietCout() { std::cout.rdbuf(saved); }
};

std::string g_error;

FoMo::DataCube make_datacube(long n, const float* x, const float* y, const float* z, const float* ne,
                             const float* T, const float* vx, const float* vy, const float* vz) {
  FoMo::tgrid grid(3);
  grid[0].assign(x, x + n);
  grid[1].assign(y, y + n);
  grid[2].assign(z, z + n);
  FoMo::tvars vars(5);
  vars[0].assign(ne, ne + n);
  vars[1].assign(T, T + n);
  vars[2].assign(vx, vx + n);
  vars[3].assign(vy, vy + n);
  vars[4].assign(vz, vz + n);
  std::vector<std::string> units = {"Mm", "Mm", "Mm", "cm^{-3}", "K", "m s^{-1}", "m s^{-1}", "m s^{-1}"};
  FoMo::DataCube cube(3);
  cube.setdata(grid, vars, &units);
  return cube;
}

void copy_out(const FoMo::tphysvar& v, float* out) {
  if (out) std::memcpy(out, v.data(), v.size() * sizeof(float));
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_error.c_str(); }

// emissionfromdatacube (fomo-CHIANTI.cpp:228-322): per-point [eps, fwhm].
// imaging != 0 selects FoMo::Imaging, else FoMo::Spectroscopic.
int ref_emission(long n, const float* x, const float* y, const float* z, const float* ne, const float* T,
                 const float* vx, const float* vy, const float* vz, const char* table_path,
                 const char* abund_path, int imaging, float* eps, float* fwhm, double* lambda0_out) {
  try {
    QuietCout quiet;
    FoMo::DataCube cube = make_datacube(n, x, y, z, ne, T, vx, vy, vz);
    FoMo::GoftCube g = FoMo::emissionfromdatacube(cube, table_path, abund_path,
                                                  imaging ? FoMo::Imaging : FoMo::Spectroscopic);
    copy_out(g.readvar(0), eps);
    copy_out(g.readvar(1), fwhm);
    if (lambda0_out) *lambda0_out = g.readlambda0();
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return -1;
  }
}

// thomsonfromdatacube (fomo-thomson.cpp:60-92): per-point [n*tot, n*pol].
int ref_thomson_emission(long n, const float* x, const float* y, const float* z, const float* ne,
                         const float* T, const float* vx, const float* vy, const float* vz, float* tot,
                         float* pol) {
  try {
    QuietCout quiet;
    FoMo::DataCube cube = make_datacube(n, x, y, z, ne, T, vx, vy, vz);
    FoMo::GoftCube g = FoMo::thomsonfromdatacube(cube);
    copy_out(g.readvar(0), tot);
    copy_out(g.readvar(1), pol);
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return -1;
  }
}

// FoMoObject::render(l, b) (fomo-object.cpp:374-455) with the given method
// string ("NearestNeighbour" or "Thomson").  Outputs the rendered intensity
// (readvar(0)), optionally the per-element grid (readgrid()), and
// meta = [x_pixel, y_pixel, z_pixel, lambda_pixel, lambda_width(m/s), l, b,
//         observationtype, lambda0, is_dn_units].
int ref_render(const char* method, long n, const float* x, const float* y, const float* z, const float* ne,
               const float* T, const float* vx, const float* vy, const float* vz, const char* table_path,
               const char* abund_path, double l, double b, int nx, int ny, int nz, int nlambda,
               double lambda_width, float* intens, float* gx, float* gy, float* glambda, double* meta) {
  try {
    QuietCout quiet;
    FoMo::FoMoObject obj;
    FoMo::DataCube cube = make_datacube(n, x, y, z, ne, T, vx, vy, vz);
    FoMo::tgrid grid = cube.readgrid();
    FoMo::tvars vars;
    for (int i = 0; i < cube.readnvars(); ++i) vars.push_back(cube.readvar(i));
    std::vector<std::string> units = cube.readunit();
    obj.setdata(grid, vars, &units);
    if (table_path && table_path[0]) obj.setchiantifile(table_path);
    obj.setabundfile(abund_path && abund_path[0] ? abund_path : "/empty");
    obj.setrendermethod(method);
    obj.setwriteoutbinary(false);
    obj.setwriteouttext(false);
    obj.setoutfile("");
    obj.setresolution(nx, ny, nz, nlambda, lambda_width);
    obj.render(l, b);
    FoMo::RenderCube r = obj.readrendering();
    copy_out(r.readvar(0), intens);
    FoMo::tgrid rg = r.readgrid();
    if (gx && rg.size() > 0) copy_out(rg[0], gx);
    if (gy && rg.size() > 1) copy_out(rg[1], gy);
    if (glambda && rg.size() > 2) copy_out(rg[2], glambda);
    if (meta) {
      int rx, ry, rz, rl;
      double rw, ll, bb;
      r.readresolution(rx, ry, rz, rl, rw);
      r.readangles(ll, bb);
      meta[0] = rx;
      meta[1] = ry;
      meta[2] = rz;
      meta[3] = rl;
      meta[4] = rw;
      meta[5] = ll;
      meta[6] = bb;
      meta[7] = static_cast<double>(r.readobservationtype());
      meta[8] = r.readlambda0();
      std::vector<std::string> ru = r.readunit();
      meta[9] = (!ru.empty() && ru.back().find("DN") != std::string::npos) ? 1.0 : 0.0;
    }
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return -1;
  }
}

// GoftCube::writegoftcube (fomo-io.cpp:248-287) of a rendered cube, for
// pinning the on-disk text (.txt) and binary (.dat) formats.  options is the
// reference's write-option bitset as an integer (bit0 binary, bit1 text).
int ref_render_and_write(const char* method, long n, const float* x, const float* y, const float* z,
                         const float* ne, const float* T, const float* vx, const float* vy, const float* vz,
                         const char* table_path, double l, double b, int nx, int ny, int nz, int nlambda,
                         double lambda_width, int options, const char* out_path) {
  try {
    QuietCout quiet;
    FoMo::FoMoObject obj;
    FoMo::DataCube cube = make_datacube(n, x, y, z, ne, T, vx, vy, vz);
    FoMo::tgrid grid = cube.readgrid();
    FoMo::tvars vars;
    for (int i = 0; i < cube.readnvars(); ++i) vars.push_back(cube.readvar(i));
    std::vector<std::string> units = cube.readunit();
    obj.setdata(grid, vars, &units);
    if (table_path && table_path[0]) obj.setchiantifile(table_path);
    obj.setrendermethod(method);
    obj.setwriteoutbinary(false);
    obj.setwriteouttext(false);
    obj.setresolution(nx, ny, nz, nlambda, lambda_width);
    obj.render(l, b);
    FoMo::RenderCube r = obj.readrendering();
    r.setwriteoptions(std::bitset<FoMo::noptions>(static_cast<unsigned long>(options)));
    r.writegoftcube(out_path);
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return -1;
  }
}

// The reference's AMRVAC snapshot reader (fomo-c/example/example_mpi_amrvac/
// read_amrvac_files.cpp, compiled unmodified into this library): read a data
// file into a FoMoObject and copy its DataCube out (coordinates, then n, T,
// vx, vy, vz; z is left untouched for 2-D data).  -3 when cap is too small.
int ref_amrvac_read(const char* datfile, const char* parfile, const char* amrvac_version, int gamma_eqparposition,
                    double n_unit, double Teunit, double L_unit, long cap, int* ndim, long* npts, float* x,
                    float* y, float* z, float* ne, float* T, float* vx, float* vy, float* vz) {
  try {
    QuietCout quiet;
    FoMo::FoMoObject obj = read_amrvac_dat_file(datfile, parfile, amrvac_version, gamma_eqparposition, n_unit,
                                                Teunit, L_unit);
    FoMo::DataCube cube = obj.readdatacube();
    FoMo::tgrid grid = cube.readgrid();
    *ndim = (int)grid.size();
    *npts = grid.empty() ? 0 : (long)grid[0].size();
    if (*npts > cap) return -3;
    float* c[3] = {x, y, z};
    for (int d = 0; d < *ndim && d < 3; ++d) std::copy(grid[d].begin(), grid[d].end(), c[d]);
    float* v[5] = {ne, T, vx, vy, vz};
    for (int i = 0; i < 5; ++i) {
      FoMo::tphysvar var = cube.readvar(i);
      std::copy(var.begin(), var.end(), v[i]);
    }
    return 0;
  } catch (const std::exception& e) {
    g_error = e.what();
    return -1;
  }
}

}  // extern "C"
