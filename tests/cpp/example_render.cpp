// A FoMo-C user program, compiled unchanged against include/FoMo.h.
//
// It follows the flow of the reference's example program
// (fomo-c/example/example.cpp:28-114): read points (x, y, z, n, T, vx, vy, vz
// per line) into a FoMoObject with push_back_datapoint, choose the table,
// abundance file, method, observation type and resolution, render(l, b), read
// the rendering back and write it.  Arguments:
//
//   example_render DATA TABLE METHOD L B NX NY NZ NLAMBDA WIDTH OUT [OPTIONS [ABUND]]
//
// OUT is the file the rendering is written to with writegoftcube (write
// options OPTIONS, default 3 = binary + text); the per-view file that render()
// itself writes (default options: text) goes to OUT's directory as
// "view-l<deg>b<deg>.txt".  ABUND is the abundance file (default "/empty":
// the tables' own abundances).  Errors are reported on stderr with exit code 2.
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "FoMo.h"

int main(int argc, char* argv[]) {
  if (argc < 12) {
    std::cerr << "usage: example_render DATA TABLE METHOD L B NX NY NZ NLAMBDA WIDTH OUT [OPTIONS]" << std::endl;
    return 1;
  }
  try {
    FoMo::FoMoObject Object;
    std::ifstream in(argv[1]);
    if (!in.is_open()) throw std::runtime_error(std::string("cannot open ") + argv[1]);
    std::vector<std::string> unitvec{"Mm", "Mm", "Mm", "cm^{-3}", "K", "m s^{-1}", "m s^{-1}", "m s^{-1}"};
    double v;
    while (true) {
      std::vector<double> coordinates, variables;
      for (int i = 0; i < 3 && (in >> v); ++i) coordinates.push_back(v);
      for (int i = 0; i < 5 && (in >> v); ++i) variables.push_back(v);
      if (coordinates.size() != 3 || variables.size() != 5) break;
      Object.push_back_datapoint(coordinates, variables, &unitvec);
    }
    const std::string method = argv[3];
    if (method.find("Thomson") == std::string::npos) Object.setchiantifile(argv[2]);
    Object.setabundfile(argc > 13 ? argv[13] : "/empty");
    Object.setrendermethod(method);
    Object.setobservationtype(FoMo::Spectroscopic);
    const int nx = std::atoi(argv[6]), ny = std::atoi(argv[7]), nz = std::atoi(argv[8]), nl = std::atoi(argv[9]);
    const double width = std::atof(argv[10]);
    Object.setresolution(nx, ny, nz, nl, width);
    const std::string out = argv[11];
    const size_t slash = out.rfind('/');
    Object.setoutfile((slash == std::string::npos ? std::string() : out.substr(0, slash + 1)) + "view-");
    Object.render(std::atof(argv[4]), std::atof(argv[5]));

    FoMo::RenderCube rendercube = Object.readrendering();
    int rx, ry, rz, rl;
    double rw;
    rendercube.readresolution(rx, ry, rz, rl, rw);
    std::cout << "resolution " << rx << " " << ry << " " << rz << " " << rl << " " << rw << std::endl;
    std::cout << "method " << rendercube.readrendermethod() << std::endl;
    std::cout << "observationtype " << (int)rendercube.readobservationtype() << std::endl;
    std::cout << "points " << rendercube.readngrid() << std::endl;
    const int options = argc > 12 ? std::atoi(argv[12]) : 3;
    rendercube.setwriteoptions(std::bitset<FoMo::noptions>((unsigned long)options));
    rendercube.writegoftcube(out);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << std::endl;
    return 2;
  }
}
