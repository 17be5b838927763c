// A FoMo-C user program of the reference's AMRVAC example kind
// (fomo-c/example/example_mpi_amrvac/example_mpi_amrvac.cpp:36): read an AMRVAC
// data file into a FoMoObject with read_amrvac_dat_file, then write the
// object's data cube (x, y[, z], n, T, vx, vy, vz as FP32 columns) to OUT as raw
// bytes and print "ndim npoints".
//
//   amrvac_points DATFILE PARFILE VERSION GAMMAPOS N_UNIT TE_UNIT L_UNIT OUT
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <stdexcept>

#include "FoMo-amrvac.h"
#include "FoMo.h"

int main(int argc, char* argv[]) {
  if (argc < 9) {
    std::cerr << "usage: amrvac_points DATFILE PARFILE VERSION GAMMAPOS N_UNIT TE_UNIT L_UNIT OUT" << std::endl;
    return 1;
  }
  try {
    FoMo::FoMoObject object = read_amrvac_dat_file(argv[1], argv[2], argv[3], std::atoi(argv[4]),
                                                   std::atof(argv[5]), std::atof(argv[6]), std::atof(argv[7]));
    FoMo::DataCube cube = object.readdatacube();
    FoMo::tgrid grid = cube.readgrid();
    FILE* f = std::fopen(argv[8], "wb");
    if (!f) throw std::runtime_error("cannot write the output file");
    for (const FoMo::tcoord& c : grid) std::fwrite(c.data(), sizeof(float), c.size(), f);
    for (int i = 0; i < 5; ++i) {
      FoMo::tphysvar v = cube.readvar(i);
      std::fwrite(v.data(), sizeof(float), v.size(), f);
    }
    std::fclose(f);
    std::cout << grid.size() << " " << (grid.empty() ? 0 : grid[0].size()) << std::endl;
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << std::endl;
    return 2;
  }
}
