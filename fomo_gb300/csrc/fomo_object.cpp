// The FoMo C++ object interface (include/FoMo.h) on top of the C ABI of
// fomo_gpu.h: the containers, their element-wise operations, and FoMoObject,
// whose render() runs the GPU renderers.  The writers and the reader of
// rendered cubes are in fomo_io.cpp.
//
// Behaviour follows the reference object by object:
//   containers        fomo-c/src/fomo-datacube.cpp:13-279, fomo-goftcube.cpp:14-113,
//                     fomo-rendercube.cpp:20-149 (defaults, unit bookkeeping)
//   operations        fomo-c/src/fomo-operations.cpp:8-114 (FP32 result per element)
//   FoMoObject        fomo-c/src/fomo-object.cpp:14-455 (setters, render flow)
//   emission cube     fomo-CHIANTI.cpp:296-321, fomo-thomson.cpp:60-92 (vars, units, names)
//   rendered cube     fomo-nearestneighbour.cpp:119-128,209-211,233-279 and
//                     fomo-thomson.cpp:224-232,343-363 (grid, units, scaling)
//   per-view files    fomo-nearestneighbour.cpp:285-306, fomo-thomson.cpp:371-392
// Differences (an exception instead of exit(), the GPU method names, the
// resident snapshot) are listed in FoMo.h.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <mutex>
#include <sstream>
#include <stdexcept>

#include "../../include/FoMo-amrvac.h"
#include "../../include/FoMo.h"
#include "../../include/fomo_gpu.h"
#include "fomo_consts.h"

namespace FoMo {

// ------------------------------------------------------------ operations

tphysvar pow(const double base, tphysvar const& in) {
  tphysvar out(in.size());
  for (size_t i = 0; i < in.size(); ++i) out[i] = (float)std::pow(base, (double)in[i]);
  return out;
}

static void same_size(tphysvar const& a, tphysvar const& b) {
  if (a.size() != b.size()) throw std::invalid_argument("FoMo: element-wise operation on vectors of different sizes");
}

tphysvar operator/(tphysvar const& a, tphysvar const& b) {
  same_size(a, b);
  tphysvar out(a.size());
  for (size_t i = 0; i < a.size(); ++i) out[i] = a[i] / b[i];
  return out;
}

tphysvar operator*(tphysvar const& a, tphysvar const& b) {
  same_size(a, b);
  tphysvar out(a.size());
  for (size_t i = 0; i < a.size(); ++i) out[i] = a[i] * b[i];
  return out;
}

tphysvar operator*=(tphysvar const& a, tphysvar const& b) { return a * b; }

tphysvar log10(tphysvar const& in) {
  tphysvar out(in.size());
  for (size_t i = 0; i < in.size(); ++i) {
    if (in[i] <= 0) {
      std::cerr << "Warning: some densities were <= 0 at position " << i << std::endl;
      out[i] = 0;
    } else {
      out[i] = std::log10(in[i]);  // the float overload
    }
  }
  return out;
}

tphysvar sqrt(tphysvar const& in) {
  tphysvar out(in.size());
  for (size_t i = 0; i < in.size(); ++i) out[i] = std::sqrt(in[i]);
  return out;
}

tphysvar operator*(double const& c, tphysvar const& in) {
  tphysvar out(in.size());
  for (size_t i = 0; i < in.size(); ++i) out[i] = (float)(c * (double)in[i]);
  return out;
}

// ------------------------------------------------------------ DataCube

DataCube::DataCube(const int indim) : dim(indim), nvars(0), ng(0) {
  grid.resize(dim);
  unit.resize(dim + nvars);
}

DataCube::~DataCube() {}

int DataCube::readdim() const { return (int)dim; }
int DataCube::readngrid() const { return (int)ng; }
int DataCube::readnvars() const { return (int)nvars; }
std::vector<std::string> DataCube::readunit() const { return unit; }
tgrid DataCube::readgrid() const { return grid; }

tphysvar DataCube::readvar(const unsigned int nvar) const {
  if (nvar >= nvars) throw std::out_of_range("FoMo: DataCube::readvar index beyond nvars");
  return vars.at(nvar);
}

void DataCube::setdim(const int indim) {
  dim = indim;
  grid.resize(indim);
  unit.resize(dim + nvars);
}

void DataCube::setnvars(const int innvars) {
  if (innvars < 0) throw std::invalid_argument("FoMo: negative number of variables");
  nvars = innvars;
  vars.resize(innvars);
  unit.resize(dim + nvars);
}

void DataCube::setngrid(const int inngrid) {
  if (inngrid < 0) throw std::invalid_argument("FoMo: negative number of grid points");
  ng = inngrid;
  for (unsigned int i = 0; i < dim; ++i) grid.at(i).resize(inngrid);
}

// The variables' units survive a new grid; the grid's units are replaced only
// when given (fomo-datacube.cpp:114-148).
void DataCube::setgrid(tgrid ingrid, std::vector<std::string>* inunit) {
  if (ingrid.empty()) throw std::invalid_argument("FoMo: grid of dimension 0");
  std::vector<std::string> varunits;
  if (unit.size() > dim) varunits.assign(unit.begin() + dim, unit.end());
  dim = (unsigned int)ingrid.size();
  const size_t n = ingrid[0].size();
  for (unsigned int i = 1; i < dim; ++i)
    if (ingrid[i].size() != n) throw std::invalid_argument("FoMo: grid coordinates of different lengths");
  grid = std::move(ingrid);
  ng = (unsigned int)n;
  if (inunit) {
    if (inunit->size() != dim) throw std::invalid_argument("FoMo: one unit per grid coordinate expected");
    unit = *inunit;
    unit.insert(unit.end(), varunits.begin(), varunits.end());
  }
}

void DataCube::setvar(const unsigned int nvar, const tphysvar var, std::string inunit) {
  if (nvar >= vars.size()) throw std::out_of_range("FoMo: DataCube::setvar index beyond nvars");
  vars.at(nvar) = var;
  unit.at(dim + nvar) = inunit;
}

void DataCube::setdata(tgrid& ingrid, tvars& indata, std::vector<std::string>* unitvec) {
  setgrid(ingrid);
  if (!indata.empty()) {
    setnvars((int)indata.size());
    for (unsigned int i = 0; i < nvars; ++i) {
      if (indata[i].size() != ng) throw std::invalid_argument("FoMo: variable length differs from the grid");
      setvar(i, indata[i]);
    }
  }
  if (unitvec) {
    if (unitvec->size() != dim + nvars) throw std::invalid_argument("FoMo: dim + nvars units expected");
    unit = *unitvec;
  }
}

void DataCube::push_back(std::vector<double> coordinate, std::vector<double> variables,
                         std::vector<std::string>* unitvec) {
  if (ng == 0) {
    tgrid g;
    for (double c : coordinate) g.push_back(tcoord(1, (float)c));
    tvars v;
    for (double x : variables) v.push_back(tphysvar(1, (float)x));
    setdata(g, v, unitvec);
    return;
  }
  if (coordinate.size() != dim || variables.size() != nvars)
    throw std::invalid_argument("FoMo: data point with a different number of coordinates or variables");
  for (unsigned int i = 0; i < dim; ++i) grid.at(i).push_back((float)coordinate[i]);
  for (unsigned int i = 0; i < nvars; ++i) vars.at(i).push_back((float)variables[i]);
  ++ng;
}

// ------------------------------------------------------------ GoftCube

static const char* const kDefaultTable = "../chiantitables/goft_table_fe_12_0194_abco.dat";

GoftCube::GoftCube(const int indim)
    : DataCube(), chiantifile(kDefaultTable), abundfile("/empty"), lambda0(193.509),
      writeoptions(std::string("0010")) {
  dim = indim;
  grid.resize(indim);
  ng = 0;
  nvars = 0;
}

GoftCube::GoftCube(DataCube incube)
    : DataCube(), chiantifile(kDefaultTable), abundfile("/empty"), lambda0(193.509),
      writeoptions(std::string("0010")) {
  dim = incube.readdim();
  ng = incube.readngrid();
  grid = incube.readgrid();
  nvars = 0;
}

void GoftCube::setchiantifile(const std::string inchianti) { chiantifile = inchianti; }
void GoftCube::setabundfile(const std::string inabund) { abundfile = inabund; }
std::string GoftCube::readchiantifile() { return chiantifile; }
std::string GoftCube::readabundfile() { return abundfile; }
double GoftCube::readlambda0() { return lambda0; }
void GoftCube::setlambda0(const double l0) { lambda0 = l0; }
std::bitset<noptions> GoftCube::getwriteoptions() { return writeoptions; }
void GoftCube::setwriteoptions(std::bitset<noptions> o) { writeoptions = o; }
void GoftCube::setwriteoutbinary(const bool v) { writeoptions[0] = v; }
void GoftCube::setwriteouttext(const bool v) { writeoptions[1] = v; }
void GoftCube::setwriteoutzip(const bool v) { writeoptions[2] = v; }
void GoftCube::setwriteoutdeletefiles(const bool v) { writeoptions[3] = v; }

// ------------------------------------------------------------ RenderCube

// Built from a GoftCube as fomo-rendercube.cpp:20-35 does: the names, rest
// wavelength, grid and write options are copied; dimension, point count and
// units keep the defaults of a fresh 3-D cube.
RenderCube::RenderCube(GoftCube goftcube)
    : GoftCube(3), l(0), b(0), x_pixel(101), y_pixel(102), z_pixel(300), lambda_pixel(30), lambda_width(200000),
      rendermethod("NearestNeighbour"), observationtype(Spectroscopic) {
  chiantifile = goftcube.readchiantifile();
  abundfile = goftcube.readabundfile();
  lambda0 = goftcube.readlambda0();
  grid = goftcube.readgrid();
  writeoptions = goftcube.getwriteoptions();
}

void RenderCube::setresolution(const int& nx, const int& ny, const int& nz, const int& nlambda,
                               const double& lambdawidth) {
  x_pixel = nx;
  y_pixel = ny;
  z_pixel = nz;
  lambda_pixel = nlambda;
  lambda_width = lambdawidth;
  // a width below 1 is taken as Angstrom (fomo-rendercube.cpp:74-84)
  if (lambdawidth < 1.) {
    std::cout << "******Warning! In newer versions of FoMo, the spectral window is given in m/s, rather than Angstrom."
              << std::endl;
    lambda_width = lambdawidth * FOMO_SPEED_OF_LIGHT / lambda0;
    std::cout << "******The input value of " << lambdawidth << " was converted to " << lambda_width << "m/s"
              << std::endl;
  } else if (lambdawidth < 1000.) {
    std::cout << "******Warning! Your spectral window width was set to a small value. Are you sure it is in m/s?"
              << std::endl;
  }
}

void RenderCube::readresolution(int& nx, int& ny, int& nz, int& nlambda, double& lambdawidth) {
  nx = x_pixel;
  ny = y_pixel;
  nz = z_pixel;
  nlambda = lambda_pixel;
  lambdawidth = lambda_width;
}

void RenderCube::setangles(const double inl, const double inb) {
  l = inl;
  b = inb;
}

void RenderCube::readangles(double& outl, double& outb) {
  outl = l;
  outb = b;
}

void RenderCube::setrendermethod(const std::string m) { rendermethod = m; }
std::string RenderCube::readrendermethod() { return rendermethod; }
void RenderCube::setobservationtype(FoMoObservationType t) { observationtype = t; }
FoMoObservationType RenderCube::readobservationtype() { return observationtype; }

// ------------------------------------------------------------ GPU side

namespace {

enum class Method { kNN, kThomson, kProjection };

// The render methods of this library; the reference's CPU names select the
// GPU renderers too.  Others raise, as the reference exits (fomo-object.cpp:430-434).
Method method_of(const std::string& m) {
  if (m == "NearestNeighbour" || m == "NearestNeighbourGPU") return Method::kNN;
  if (m == "Thomson" || m == "ThomsonGPU") return Method::kThomson;
  if (m == "Projection") return Method::kProjection;
  if (m == "CGAL" || m == "CGAL2D")
    throw std::runtime_error("FoMo: render method " + m + " is not available in this library");
  throw std::runtime_error("Error: unknown rendering method.");
}

// One context per process (device FOMO_DEVICE, default 0); it lives until exit.
fomo_ctx* shared_context() {
  static std::mutex mu;
  static fomo_ctx* ctx = nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!ctx) {
    int dev = 0;
    if (const char* s = std::getenv("FOMO_DEVICE")) dev = std::atoi(s);
    fomo_ctx* c = nullptr;
    const int rc = fomo_ctx_create(dev, 0, &c);
    if (rc != FOMO_OK)
      throw std::runtime_error("FoMo: no usable CUDA device for the GPU renderers (fomo_ctx_create returned " +
                               std::to_string(rc) + ")");
    ctx = c;
  }
  return ctx;
}

void check(fomo_ctx* ctx, int rc, const char* what) {
  if (rc != FOMO_OK) throw std::runtime_error(std::string("FoMo GPU ") + what + ": " + fomo_last_error(ctx));
}

// lambda0 from the first line of a G(T) table (fomo-CHIANTI.cpp:123-141)
double table_lambda0(const std::string& path) {
  std::ifstream in(path);
  if (!in) throw std::runtime_error("Error: no CHIANTI G(T) file exists: " + path);
  std::string ion;
  double l0 = 0;
  in >> ion >> l0;
  if (!in) throw std::runtime_error("FoMo: malformed CHIANTI G(T) file header: " + path);
  return l0;
}

// The file name of view (l, b): outfile + "l" + degrees + "b" + degrees + ".txt",
// three digits, zero-filled (fomo-nearestneighbour.cpp:294-301).
std::string view_file(const std::string& outfile, double l, double b) {
  std::stringstream ss;
  ss << outfile << "l" << std::setfill('0') << std::setw(3) << std::round(l / FOMO_PI * 180.) << "b"
     << std::setfill('0') << std::setw(3) << std::round(b / FOMO_PI * 180.) << ".txt";
  return ss.str();
}

}  // namespace

struct FoMoObject::Device {
  fomo_ctx* ctx = nullptr;
  int snap = -1;
  unsigned long long gen = ~0ull;
  int64_t npoints = 0;
  std::map<std::string, int> tables;  // loaded G(T) tables by path
  double abundratio = 1.0;            // of the last render
  ~Device() {
    if (!ctx) return;
    if (snap >= 0) fomo_snapshot_destroy(ctx, snap);
    for (auto& kv : tables) fomo_table_destroy(ctx, kv.second);
  }
};

// ------------------------------------------------------------ FoMoObject

FoMoObject::FoMoObject(const int indim) : datacube(indim), goftcube(datacube), rendering(goftcube) {}
FoMoObject::~FoMoObject() {}

void FoMoObject::setrendermethod(const std::string m) { rendering.setrendermethod(m); }
std::string FoMoObject::readrendermethod() { return rendering.readrendermethod(); }
DataCube FoMoObject::readdatacube() { return datacube; }
RenderCube FoMoObject::readrendering() { return rendering; }

void FoMoObject::setabundfile(const std::string inabund) {
  goftcube.setabundfile(inabund);
  rendering.setabundfile(inabund);
}
std::string FoMoObject::readabundfile() { return goftcube.readabundfile(); }

void FoMoObject::setchiantifile(const std::string inchianti) {
  const double l0 = table_lambda0(inchianti);
  goftcube.setlambda0(l0);
  goftcube.setchiantifile(inchianti);
  rendering.setlambda0(l0);
  rendering.setchiantifile(inchianti);
}
std::string FoMoObject::readchiantifile() { return goftcube.readchiantifile(); }

// The reference passes no units on here (fomo-object.cpp:137-142); neither do we.
void FoMoObject::push_back_datapoint(std::vector<double> coordinate, std::vector<double> variables,
                                     std::vector<std::string>* unitvec) {
  (void)unitvec;
  datacube.push_back(coordinate, variables);
  ++data_gen_;
}

void FoMoObject::setdata(tgrid& ingrid, tvars& indata, std::vector<std::string>* unitvec) {
  datacube.setdata(ingrid, indata, unitvec);
  ++data_gen_;
}

void FoMoObject::setrenderingdata(tgrid ingrid, tvars invars) { rendering.setdata(ingrid, invars); }
void FoMoObject::setobservationtype(FoMoObservationType t) { rendering.setobservationtype(t); }
FoMoObservationType FoMoObject::readobservationtype() { return rendering.readobservationtype(); }
void FoMoObject::setoutfile(const std::string s) { outfile = s; }

void FoMoObject::setresolution(const int& nx, const int& ny, const int& nz, const int& nlambda, const double& width) {
  rendering.setresolution(nx, ny, nz, nlambda, width);
}
void FoMoObject::readresolution(int& nx, int& ny, int& nz, int& nlambda, double& width) {
  rendering.readresolution(nx, ny, nz, nlambda, width);
}

void FoMoObject::setwriteoptions(std::bitset<noptions> o) {
  rendering.setwriteoptions(o);
  goftcube.setwriteoptions(o);
}
void FoMoObject::setwriteoutbinary(const bool v) {
  rendering.setwriteoutbinary(v);
  goftcube.setwriteoutbinary(v);
}
void FoMoObject::setwriteouttext(const bool v) {
  rendering.setwriteouttext(v);
  goftcube.setwriteouttext(v);
}
void FoMoObject::setwriteoutzip(const bool v) {
  rendering.setwriteoutzip(v);
  goftcube.setwriteoutzip(v);
}
void FoMoObject::setwriteoutdeletefiles(const bool v) {
  rendering.setwriteoutdeletefiles(v);
  goftcube.setwriteoutdeletefiles(v);
}

// The emission cube of the last render: the per-point emissivity and line
// width (or the Thomson terms), read back from the device on first use.
GoftCube FoMoObject::readgoftcube() {
  if (goft_pending_ && device_ && device_->snap >= 0) {
    fomo_ctx* ctx = device_->ctx;
    const size_t n = (size_t)device_->npoints;
    tphysvar a(n), w(n);
    const bool thomson = goftcube.readchiantifile() == "thomson scattering";
    tgrid g = datacube.grid;
    tvars v;
    if (thomson) {
      check(ctx, fomo_thomson_emission(ctx, device_->snap, a.data(), w.data()), "Thomson terms");
      v.push_back(a);
      v.push_back(w);
      goftcube.setdata(g, v);  // no units given (fomo-thomson.cpp:85)
    } else {
      auto it = device_->tables.find(goftcube.readchiantifile());
      if (it == device_->tables.end()) throw std::runtime_error("FoMo: table of the last render is not loaded");
      const bool imaging = rendering.readobservationtype() == Imaging;
      check(ctx, fomo_emission(ctx, device_->snap, it->second, imaging ? 1 : 0, device_->abundratio, a.data(),
                               w.data()),
            "emission");
      char unit[256] = {0};
      check(ctx, fomo_table_get_info(ctx, it->second, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0, unit,
                                     (int)sizeof(unit)),
            "table info");
      // units: the grid's, the table's, Angstrom, then the velocities' (fomo-CHIANTI.cpp:301-314)
      std::vector<std::string> du = datacube.unit;
      std::vector<std::string> units(du.begin(), du.begin() + datacube.dim);
      units.push_back(unit);
      units.push_back("\\AA{}");
      v.push_back(a);
      v.push_back(w);
      for (unsigned int i = 2; i < datacube.nvars; ++i) {
        v.push_back(datacube.vars[i]);
        units.push_back(du.at(datacube.dim + i));
      }
      goftcube.setdata(g, v, &units);
    }
    goft_pending_ = false;
  }
  return goftcube;
}

void FoMoObject::render(const double l, const double b) { render(std::vector<double>{l}, std::vector<double>{b}); }

void FoMoObject::render(const std::vector<double> lvec, const std::vector<double> bvec) {
  int nx, ny, nz, nl;
  double width;
  rendering.readresolution(nx, ny, nz, nl, width);
  rendering.setobservationtype(nl <= 1 ? Imaging : Spectroscopic);
  const std::string mname = rendering.readrendermethod();
  const Method method = method_of(mname);
  const std::bitset<noptions> wopt = goftcube.getwriteoptions();
  const bool thomson = method == Method::kThomson;
  const bool imaging = rendering.readobservationtype() == Imaging;

  if (!device_) device_ = std::make_shared<Device>();
  Device& D = *device_;
  if (!D.ctx) D.ctx = shared_context();
  fomo_ctx* ctx = D.ctx;

  // the snapshot stays resident while the data do not change
  if (D.snap < 0 || D.gen != data_gen_) {
    if (D.snap >= 0) {
      fomo_snapshot_destroy(ctx, D.snap);
      D.snap = -1;
    }
    const size_t n = datacube.ng;
    if (n == 0) throw std::runtime_error("FoMo: no data points to render");
    if (datacube.dim < 2 || datacube.dim > 3) throw std::runtime_error("FoMo: data must be 2-D or 3-D");
    const unsigned int need = thomson ? 1 : 5;
    if (datacube.nvars < need)
      throw std::runtime_error("FoMo: the data need the variables n, T, vx, vy, vz (in that order)");
    const tphysvar zero(n, 0.0f);
    auto var = [&](unsigned int i) -> const float* {
      return i < datacube.nvars ? datacube.vars[i].data() : zero.data();
    };
    int id = -1;
    check(ctx,
          fomo_snapshot_create(ctx, (int64_t)n, datacube.grid[0].data(), datacube.grid[1].data(),
                               datacube.dim == 3 ? datacube.grid[2].data() : nullptr, var(0), var(1), var(2), var(3),
                               var(4), &id),
          "snapshot upload");
    D.snap = id;
    D.gen = data_gen_;
    D.npoints = (int64_t)n;
  }

  // the emission cube's names (fomo-CHIANTI.cpp:316-318, fomo-thomson.cpp:86-89)
  int table = -1;
  double abundratio = 1.0;
  GoftCube goft(datacube);
  if (thomson) {
    goft.setchiantifile("thomson scattering");
    goft.setabundfile("thomson scattering");
    goft.setlambda0(0.);
  } else {
    const std::string tf = rendering.readchiantifile();
    auto it = D.tables.find(tf);
    if (it == D.tables.end()) {
      check(ctx, fomo_table_load(ctx, tf.c_str(), &table), "table");
      D.tables[tf] = table;
    } else {
      table = it->second;
    }
    // abundance renormalisation of spectroscopic renders (fomo-CHIANTI.cpp:
    // 264-273) against the standard abundances the tables were made with.  The
    // reference's built-in copy of those is an empty string at the point of use
    // (fomo-CHIANTI.cpp:21), so any file but "/empty" fails there; here the
    // standard file is FOMO_STANDARD_ABUND, and without it the same error.
    const std::string af = rendering.readabundfile();
    if (!imaging && af != "/empty") {
      const char* std_file = std::getenv("FOMO_STANDARD_ABUND");
      if (!std_file || !*std_file)
        throw std::runtime_error("Error: invalid CHIANTI abundance file (set FOMO_STANDARD_ABUND to the standard "
                                 "abundance file the G(T) tables were computed with)");
      char ion[64] = {0};
      check(ctx, fomo_table_get_info(ctx, table, nullptr, nullptr, nullptr, nullptr, nullptr, ion, (int)sizeof(ion),
                                     nullptr, 0),
            "table info");
      check(ctx, fomo_abundance_ratio(ctx, af.c_str(), std_file, ion, &abundratio), "abundance");
    }
    goft.setchiantifile(tf);
    goft.setabundfile(af);
    goft.setlambda0(rendering.readlambda0());
  }
  goft.setwriteoptions(wopt);
  D.abundratio = abundratio;
  goftcube = goft;
  goft_pending_ = true;

  // all views of lvec x bvec in batched launches of at most ~1 GiB of cubes
  struct View {
    double l, b;
  };
  std::vector<View> views;
  for (double lv : lvec)
    for (double bv : bvec) views.push_back({lv, bv});
  const int L = thomson ? 1 : (nl < 1 ? 1 : nl);
  const size_t cube_elems = (size_t)nx * (size_t)ny * (size_t)L;
  const size_t per_batch = std::max<size_t>(1, ((size_t)1 << 28) / std::max<size_t>(cube_elems, 1));
  // a RenderCube built from the emission cube copies its names and options;
  // its grid is replaced by the image grid, so start from the names only
  GoftCube meta;
  meta.setchiantifile(goftcube.readchiantifile());
  meta.setabundfile(goftcube.readabundfile());
  meta.setlambda0(goftcube.readlambda0());
  meta.setwriteoptions(wopt);
  RenderCube last(meta);
  for (size_t v0 = 0; v0 < views.size(); v0 += per_batch) {
    const size_t nv = std::min(per_batch, views.size() - v0);
    std::vector<fomo_request> reqs(nv);
    std::vector<std::vector<float>> cubes(nv, std::vector<float>(cube_elems));
    std::vector<float*> outs(nv);
    std::vector<fomo_view_info> infos(nv);
    for (size_t k = 0; k < nv; ++k) {
      fomo_request& q = reqs[k];
      q.snapshot = D.snap;
      q.table = thomson ? 0 : table;
      q.method = thomson ? FOMO_METHOD_THOMSON
                         : (method == Method::kProjection ? FOMO_METHOD_PROJECTION : FOMO_METHOD_NN);
      q.nx = nx;
      q.ny = ny;
      q.nz = nz;
      q.nlambda = L;
      q.l = views[v0 + k].l;
      q.b = views[v0 + k].b;
      q.lambda_width = width;
      q.abundratio = abundratio;
      outs[k] = cubes[k].data();
    }
    check(ctx, fomo_render_batch(ctx, reqs.data(), (int)nv, outs.data(), infos.data()), "render");
    for (size_t k = 0; k < nv; ++k) {
      const fomo_view_info& I = infos[k];
      RenderCube rc(meta);
      // image grid (nn:123-127, 151-153, 209-211); x and y are stored as FP32
      const size_t np = (size_t)nx * ny;
      tgrid g(L > 1 ? 3 : 2, tcoord(np * L));
      for (int i = 0; i < ny; ++i) {
        const double y = double(i) / (ny - 1) * (I.maxy - I.miny) + I.miny;
        for (int j = 0; j < nx; ++j) {
          const double x = double(j) / (nx - 1) * (I.maxx - I.minx) + I.minx;
          const size_t base = ((size_t)i * nx + j) * L;
          for (int il = 0; il < L; ++il) {
            g[0][base + il] = (float)x;
            g[1][base + il] = (float)y;
            if (L > 1) {
              const double lv = double(il) / (L - 1) * I.lambda_width_A - I.lambda_width_A / 2.;
              g[2][base + il] = (float)(lv + I.lambda0);
            }
          }
        }
      }
      tvars data;
      data.push_back(tphysvar(cubes[k].begin(), cubes[k].end()));
      if (thomson) {
        rc.setdata(g, data);  // no units (fomo-thomson.cpp:359)
        rc.setrendermethod("Thomson");
        rc.setresolution(nx, ny, nz, 1, 100000.);
        rc.setobservationtype(Imaging);
      } else {
        std::vector<std::string> units{"Mm", "Mm"};
        if (L > 1) units.push_back("\\AA{}");
        units.push_back("erg cm^{-2} s^{-1} \\AA{}^{-1}");
        if (I.is_dn) {
          // instrument units: arcsec grid, per-pixel intensity (nn:254-265)
          units[0] = "arcsec";
          units[1] = "arcsec";
          g[0] = operator*(1. / FOMO_MM_PER_ARCSEC, g[0]);
          g[1] = operator*(1. / FOMO_MM_PER_ARCSEC, g[1]);
          units.back() = "DN s^{-1} pixel^{-1}";
        }
        rc.setdata(g, data, &units);
        rc.setrendermethod("NearestNeighbour");
        rc.setresolution(nx, ny, nz, L, width);
        rc.setobservationtype(L == 1 ? Imaging : Spectroscopic);
      }
      rc.setangles(views[v0 + k].l, views[v0 + k].b);
      rc.writegoftcube(view_file(outfile, views[v0 + k].l, views[v0 + k].b));
      last = std::move(rc);
    }
  }
  // the last view's cube (a fresh one when lvec or bvec is empty)
  last.setrendermethod(mname);
  last.setobservationtype(rendering.readobservationtype());
  rendering = last;
}

}  // namespace FoMo

// ---------------------------------------------------------------- AMRVAC

void read_amrvac_par_file(const char* amrvacpar, const int ndim, std::vector<int>& nxlone,
                          std::vector<double>& xprobmin, std::vector<double>& xprobmax) {
  std::ifstream in(amrvacpar ? amrvacpar : "");
  if (!in) throw std::runtime_error(std::string("amrvac.par file not found at ") + (amrvacpar ? amrvacpar : "(null)"));
  std::stringstream ss;
  ss << in.rdbuf();
  const std::string text = ss.str();
  nxlone.assign(ndim, 0);
  xprobmin.assign(ndim, 0.0);
  xprobmax.assign(ndim, 0.0);
  const char* keys[3] = {"nxlone", "xprobmin", "xprobmax"};
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < ndim; ++i) {
      const std::string key = keys[j] + std::to_string(i + 1);
      const size_t at = text.find(key);
      const size_t start = at == std::string::npos ? at : text.find_first_of("\t\n= ", at + 1);
      if (start == std::string::npos)
        throw std::runtime_error(std::string(amrvacpar) + " does not contain the key " + key);
      const char* v = text.c_str() + start + 1;
      if (j == 0) nxlone[i] = std::atoi(v);
      if (j == 1) xprobmin[i] = std::strtod(v, nullptr);
      if (j == 2) xprobmax[i] = std::strtod(v, nullptr);
    }
}

FoMo::FoMoObject read_amrvac_dat_file(const char* datfile, const char* amrvacpar, std::string amrvac_version,
                                      const int gamma_eqparposition, const double n_unit, const double Teunit,
                                      const double L_unit) {
  fomo_ctx* ctx = FoMo::shared_context();
  int64_t n = 0;
  int ndim = 0;
  FoMo::check(ctx,
        fomo_amrvac_points(ctx, datfile, amrvacpar, amrvac_version.c_str(), gamma_eqparposition, n_unit, Teunit,
                           L_unit, 0, &n, &ndim, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                           nullptr),
        "AMRVAC reader");
  FoMo::tgrid grid(ndim, FoMo::tcoord((size_t)n));
  FoMo::tvars vars(5, FoMo::tphysvar((size_t)n));
  std::vector<float> zeros(ndim == 2 ? (size_t)n : 0);
  FoMo::check(ctx,
        fomo_amrvac_points(ctx, datfile, amrvacpar, amrvac_version.c_str(), gamma_eqparposition, n_unit, Teunit,
                           L_unit, n, &n, &ndim, grid[0].data(), grid[1].data(),
                           ndim == 3 ? grid[2].data() : zeros.data(), vars[0].data(), vars[1].data(), vars[2].data(),
                           vars[3].data(), vars[4].data()),
        "AMRVAC reader");
  FoMo::FoMoObject object;
  object.setdata(grid, vars);
  return object;
}
