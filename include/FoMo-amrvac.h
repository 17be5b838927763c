// FoMo-amrvac.h -- reading AMRVAC snapshots into a FoMoObject, as the
// reference's AMRVAC example declares it (fomo-c/example/example_mpi_amrvac/
// FoMo-amrvac.h:7-9), so that its user programs compile unchanged.
//
// read_amrvac_dat_file parses the data file on the host and computes every
// cell's position and n, T, v on the GPU (fomo_amrvac_points in fomo_gpu.h,
// the same FP64 arithmetic as the reference's fomo_from_amrvac), then loads the
// points into the object (setdata).  Errors throw std::runtime_error where the
// reference exits.
#ifndef FOMO_AMRVAC_H
#define FOMO_AMRVAC_H

#include <string>
#include <vector>

#include "FoMo.h"

// The nxlone<d>, xprobmin<d>, xprobmax<d> of an amrvac.par file
// (read_amrvac_files.cpp:50-112).
void read_amrvac_par_file(const char* amrvacpar, const int ndim, std::vector<int>& nxlone,
                          std::vector<double>& xprobmin, std::vector<double>& xprobmax);

// An AMRVAC data file as a FoMoObject (read_amrvac_files.cpp:685-715):
// versions 3 and 4 carry their domain; older files need amrvacpar, the
// amrvac_version "old" or "gitlab" and the position of gamma among the
// equation parameters.  n_unit in cm^-3, Teunit in K, L_unit in Mm per code
// length.
FoMo::FoMoObject read_amrvac_dat_file(const char* datfile, const char* amrvacpar, std::string amrvac_version,
                                      const int gamma_eqparposition, const double n_unit, const double Teunit,
                                      const double L_unit);

#endif
