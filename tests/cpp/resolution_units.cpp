// RenderCube::setresolution's unit rule as a FoMo-C user meets it through
// FoMoObject (fomo-rendercube.cpp:67-85): a spectral window below 1 is taken
// as Angstrom and converted to m/s with c / lambda0 of the rendering, where
// lambda0 is set only by setchiantifile (fomo-object.cpp:110-116), so the
// order of the two calls matters.  Prints the stored widths, one per line:
//
//   1. setchiantifile(TABLE), then setresolution(..., 0.6)   -> 0.6 c / lambda0(TABLE)
//   2. setresolution(..., 0.6) first, then setchiantifile     -> 0.6 c / 193.509 (the default)
//   3. setresolution(..., 150000)                             -> 150000 (already m/s)
//
//   resolution_units TABLE
#include <cstdio>
#include <iostream>

#include "FoMo.h"

static double width_of(FoMo::FoMoObject& o) {
  int nx, ny, nz, nl;
  double w;
  o.readresolution(nx, ny, nz, nl, w);
  return w;
}

int main(int argc, char* argv[]) {
  if (argc < 2) {
    std::cerr << "usage: resolution_units TABLE" << std::endl;
    return 1;
  }
  FoMo::FoMoObject a;
  a.setchiantifile(argv[1]);
  a.setresolution(8, 6, 10, 16, 0.6);
  FoMo::FoMoObject b;
  b.setresolution(8, 6, 10, 16, 0.6);
  b.setchiantifile(argv[1]);
  FoMo::FoMoObject c;
  c.setchiantifile(argv[1]);
  c.setresolution(8, 6, 10, 16, 150000.);
  std::printf("%.17g\n%.17g\n%.17g\n", width_of(a), width_of(b), width_of(c));
  return 0;
}
