// FoMo.h -- the C++ object interface of FoMo-C, rendered on a GB300.
//
// Source-compatible with the reference's public header (fomo-c/src/FoMo.h:
// namespace FoMo, the tcoord/tgrid/tphysvar/tvars vectors, the element-wise
// tphysvar operations, DataCube, GoftCube, RenderCube and FoMoObject with the
// same member signatures), so that a program written against FoMo-C -- e.g.
// fomo-c/example/example.cpp -- compiles unchanged against this header and
// links against libfomo_gpu.so.
//
// What differs from the reference:
//   * FoMoObject::render runs on the GPU through the C ABI of fomo_gpu.h.  The
//     method names "NearestNeighbour" and "NearestNeighbourGPU" select the
//     nearest-neighbour renderer, "Thomson" and "ThomsonGPU" the Thomson pB
//     renderer, "Projection" the projection renderer (each point added to the
//     pixel nearest its projection).  The emissivity (or Thomson terms) is computed on the device
//     from the DataCube and kept resident with the snapshot while the data do
//     not change; several (l, b) views render in one batched launch.
//   * Errors throw std::runtime_error (the reference prints and exits): an
//     unknown or unavailable method, a missing or malformed table, a failed
//     imaging-table check, no usable CUDA device.
//   * "CGAL" and "CGAL2D" are not part of this library.
//   * Gzipped output (setwriteoutzip) is a valid .gz stream written with
//     stored deflate blocks; its uncompressed content is byte-identical.
//
// The device is FOMO_DEVICE (environment; default 0), shared by every
// FoMoObject of the process.
#ifndef FOMO_H
#define FOMO_H

#include <bitset>
#include <memory>
#include <string>
#include <vector>

namespace FoMo {

// Storage types: every coordinate and physical variable is an FP32 vector of
// the number of grid points; a grid / a variable set is a vector of those.
typedef std::vector<float> tcoord;
typedef std::vector<tcoord> tgrid;
typedef std::vector<float> tphysvar;
typedef std::vector<tphysvar> tvars;

// Element-wise operations on tphysvar (each result element rounded to FP32,
// as fomo-c/src/fomo-operations.cpp does).
tphysvar pow(const double, tphysvar const&);
tphysvar operator/(tphysvar const&, tphysvar const&);
tphysvar operator*(tphysvar const&, tphysvar const&);
tphysvar operator*=(tphysvar const&, tphysvar const&);
tphysvar log10(tphysvar const&);
tphysvar operator*(double const&, tphysvar const&);
tphysvar sqrt(tphysvar const&);

// Model data: dim coordinates and nvars physical variables at ng points, with
// one unit string per coordinate and per variable.
class DataCube {
  friend class FoMoObject;  // uploads the data without copying them

 protected:
  unsigned int dim;
  unsigned int nvars;
  unsigned int ng;
  FoMo::tgrid grid;
  FoMo::tvars vars;
  std::vector<std::string> unit;
  void setgrid(tgrid ingrid, std::vector<std::string>* inunit = NULL);
  void setvar(const unsigned int, const tphysvar, std::string inunit = "");

 public:
  DataCube(const int = 3);
  ~DataCube();
  int readdim() const;
  int readngrid() const;
  int readnvars() const;
  std::vector<std::string> readunit() const;
  tgrid readgrid() const;
  tphysvar readvar(const unsigned int) const;
  void setdim(const int indim);
  void setnvars(const int innvars);
  void setngrid(const int inngrid);
  void setdata(tgrid& ingrid, tvars& indata, std::vector<std::string>* unitvec = NULL);
  void push_back(std::vector<double> coordinate, std::vector<double> variables,
                 std::vector<std::string>* unitvec = NULL);
};

// Number of write options of a GoftCube: binary, text, gzip, delete-after-gzip.
const int noptions = 4;

// A DataCube with the emission table, abundance file, rest wavelength and
// write options it was (or will be) processed with.
class GoftCube : public DataCube {
 protected:
  std::string chiantifile;
  std::string abundfile;
  double lambda0;
  std::bitset<noptions> writeoptions;

 public:
  GoftCube(const int = 3);
  GoftCube(DataCube datacube);
  void setchiantifile(const std::string inchianti);
  void setabundfile(const std::string inabund);
  std::string readchiantifile();
  std::string readabundfile();
  double readlambda0();
  void setlambda0(const double lambda0);
  void writegoftcube(const std::string);
  void readgoftcube(const std::string);
  std::bitset<noptions> getwriteoptions();
  void setwriteoptions(std::bitset<noptions> options);
  void setwriteoutbinary(const bool = true);
  void setwriteouttext(const bool = true);
  void setwriteoutzip(const bool = true);
  void setwriteoutdeletefiles(const bool = true);
};

// Spectroscopic when lambda_pixel > 1, Imaging otherwise (set by render()).
enum FoMoObservationType { ObservationTypeNotDefined, Spectroscopic, Imaging };

// A rendering: the image grid (x, y[, lambda]) and intensity, with the view
// angles, resolution, method and observation type that produced it.
class RenderCube : public GoftCube {
 protected:
  double l;
  double b;
  int x_pixel;
  int y_pixel;
  int z_pixel;
  int lambda_pixel;
  double lambda_width;
  std::string rendermethod;
  FoMoObservationType observationtype;

 public:
  RenderCube(GoftCube goftcube);
  void setresolution(const int& x_pixel, const int& y_pixel, const int& z_pixel, const int& lambda_pixel,
                     const double& lambda_width);
  void readresolution(int& x_pixel, int& y_pixel, int& z_pixel, int& lambda_pixel, double& lambda_width);
  void setangles(const double l, const double b);
  void readangles(double& l, double& b);
  void setrendermethod(const std::string inrendermethod);
  std::string readrendermethod();
  void setobservationtype(FoMoObservationType);
  FoMoObservationType readobservationtype();
};

// The main object: load data (push_back_datapoint / setdata), choose table,
// method and resolution, render(l, b), read the rendering.
class FoMoObject {
 protected:
  std::string outfile;
  FoMo::DataCube datacube;
  FoMo::GoftCube goftcube;
  FoMo::RenderCube rendering;

 public:
  FoMoObject(const int = 3);
  ~FoMoObject();
  void render(const double = 0, const double = 0);
  void render(const std::vector<double> lvec, const std::vector<double> bvec);
  void setrenderingdata(tgrid ingrid, tvars invars);
  FoMo::DataCube readdatacube();
  FoMo::RenderCube readrendering();
  FoMo::GoftCube readgoftcube();
  void setrendermethod(const std::string inrendermethod);
  std::string readrendermethod();
  void setchiantifile(const std::string inchianti);
  void setabundfile(const std::string inabund);
  std::string readchiantifile();
  std::string readabundfile();
  void setoutfile(const std::string outfile);
  void push_back_datapoint(std::vector<double> coordinate, std::vector<double> variables,
                           std::vector<std::string>* unitvec = NULL);
  void setdata(tgrid& ingrid, tvars& indata, std::vector<std::string>* unitvec = NULL);
  void setobservationtype(FoMoObservationType);
  FoMoObservationType readobservationtype();
  void setresolution(const int& x_pixel, const int& y_pixel, const int& z_pixel, const int& lambda_pixel,
                     const double& lambda_width);
  void readresolution(int& x_pixel, int& y_pixel, int& z_pixel, int& lambda_pixel, double& lambda_width);
  void setwriteoptions(std::bitset<noptions> options);
  void setwriteoutbinary(const bool = true);
  void setwriteouttext(const bool = true);
  void setwriteoutzip(const bool = true);
  void setwriteoutdeletefiles(const bool = true);

 private:
  struct Device;                   // the snapshot resident on the GPU (shared by copies)
  std::shared_ptr<Device> device_;
  unsigned long long data_gen_ = 0;  // bumped by every change of datacube
  bool goft_pending_ = false;        // goftcube metadata set, its vars not yet read back
};

}  // namespace FoMo

#endif  // FOMO_H
