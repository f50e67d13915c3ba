// luxum -- command-line drop-in for the reference's main() (main.cc:53-72).
//
//   luxum [parameters.yaml] [--dir D] [--print-every N] [--quiet] [--no-material]
//
// Reads parameters.yaml from the working directory by default (reader.cc:70), runs the
// driver maxwell::solve would pick on one GPU, and writes that driver's HDF5 file
// (Ey_data_2d.h5, Ez_data.h5 or Ez_data2.h5) into the working directory.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "luxum.hpp"

int main(int argc, char** argv) {
  std::string path = "parameters.yaml", dir = ".";
  int print_every = 1;
  bool quiet = false, material = true;
  for (int i = 1; i < argc; i++) {
    if (!std::strcmp(argv[i], "--dir") && i + 1 < argc) dir = argv[++i];
    else if (!std::strcmp(argv[i], "--print-every") && i + 1 < argc) print_every = std::atoi(argv[++i]);
    else if (!std::strcmp(argv[i], "--quiet")) quiet = true;
    else if (!std::strcmp(argv[i], "--no-material")) material = false;
    else if (!std::strcmp(argv[i], "--help") || !std::strcmp(argv[i], "-h")) {
      std::printf("usage: luxum [parameters.yaml] [--dir D] [--print-every N] [--quiet] [--no-material]\n");
      return 0;
    } else path = argv[i];
  }
  try {
    luxum::reader inputData(path.c_str());
    luxum::maxwell solver(inputData);
    solver.dir = dir;
    solver.print_every = print_every;
    solver.quiet = quiet;
    solver.require_material = material;
    solver.solve();
  } catch (const luxum::error& e) {
    std::fprintf(stderr, "luxum: %s\n", e.what());
    return 1;
  }
  return 0;
}
