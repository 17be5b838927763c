// Reads a FoMo cube file with GoftCube::readgoftcube and writes it back with
// writegoftcube under the given write options (FoMo.h; no GPU involved).
//
//   roundtrip_cube IN OUT OPTIONS
#include <bitset>
#include <cstdlib>
#include <iostream>
#include <stdexcept>

#include "FoMo.h"

int main(int argc, char* argv[]) {
  if (argc < 4) {
    std::cerr << "usage: roundtrip_cube IN OUT OPTIONS" << std::endl;
    return 1;
  }
  try {
    FoMo::GoftCube cube;
    cube.readgoftcube(argv[1]);
    cube.setwriteoptions(std::bitset<FoMo::noptions>((unsigned long)std::atoi(argv[3])));
    cube.writegoftcube(argv[2]);
    std::cout << cube.readdim() << " " << cube.readngrid() << " " << cube.readnvars() << std::endl;
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << std::endl;
    return 2;
  }
}
