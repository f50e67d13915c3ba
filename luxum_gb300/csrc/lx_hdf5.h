// lx_hdf5.h -- minimal HDF5 writer/reader for the snapshot layout of fileio.cc:60-212.
#pragma once
#include <cstdio>
#include <string>
#include <vector>

namespace lx {

// Appends one 3-D native-double dataset "t=<step>" per write to a single file (or named
// datasets of their own extents: checkpoints).
class Hdf5Writer {
 public:
  ~Hdf5Writer();
  std::string open(const char* path, const int ext[3]);
  std::string write(int t, const double* data);  // dataset "t=<t>" (fileio.cc:186-187)
  // ext: this dataset's extents (nullptr: the file's, from open)
  std::string write_named(const std::string& name, const double* data, const int* ext = nullptr);
  std::string close();

 private:
  struct Entry {
    std::string name;
    unsigned long long addr, bytes;
    int ext[3];
  };
  std::string failed(const char* what) const;  // "<what> failed on <path>: <errno text>"
  std::FILE* f_ = nullptr;
  std::string path_;
  int ext_[3] = {0, 0, 0};
  unsigned long long eof_ = 0;
  std::vector<Entry> entries_;
};

// Reads a little-endian float64/float32 dataset of rank <= 3 (contiguous layout) of an HDF5
// file with superblock 0/1; shape is right-aligned (rank 2 -> {1, n0, n1}).  Empty = ok.
std::string hdf5_read(const char* path, const char* dataset, std::vector<double>& data, int shape[3]);

}  // namespace lx
