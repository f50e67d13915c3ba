// lx_hdf5.cpp -- placeholder until the on-disk HDF5 layout lands.
#include "lx_hdf5.h"

namespace lx {
Hdf5Writer::~Hdf5Writer() { close(); }
std::string Hdf5Writer::open(const char*, const int ext[3]) {
  for (int a = 0; a < 3; a++) ext_[a] = ext[a];
  return "HDF5 output not available yet";
}
std::string Hdf5Writer::write(int, const double*) { return "HDF5 output not available yet"; }
std::string Hdf5Writer::close() { return ""; }
}  // namespace lx
