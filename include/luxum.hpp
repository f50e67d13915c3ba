// luxum.hpp -- header-only C++ facade over the C ABI, shaped like the reference's classes so
// that a program written against Luxum's main.cc (main.cc:53-72) keeps its structure:
//
//     luxum::reader inputData;              // reader::reader, reader.cc:55-58
//     luxum::maxwell solver(inputData);     // maxwell::maxwell, maxwell.cc:60-148
//     solver.solve();                       // maxwell::solve, maxwell.cc:157-174
//
// The parallel and grid objects of the reference (parallel.cc:57-77, grid.cc:58-95) have no
// counterpart: one GPU holds the whole grid.  solve() runs the driver maxwell::solve picks
// (planar/3-D x PML/no PML) with that driver's output file and cadence, prints
// "t: <t>, max: <max|E|^2>" like the drivers do, and "Time taken: <s> sec" at the end.
// Failures throw luxum::error (the reference prints and calls exit(0)).
#pragma once
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "luxum.h"

namespace luxum {

struct error : std::runtime_error {
  lx_status status;
  error(lx_status st, const std::string& m) : std::runtime_error(m), status(st) {}
};

inline void check(lx_status st, const lx_sim* sim = nullptr) {
  if (st != LX_OK) throw error(st, lx_last_error(sim));
}

// Class reader: the parsed and checked parameters.yaml (reader.h:50-174).
class reader {
 public:
  lx_params p;
  explicit reader(const char* path = "parameters.yaml") { check(lx_params_from_yaml(path, &p)); }
  explicit reader(const lx_params& params) : p(params) {}
};

// Class maxwell: one simulation and the reference driver's time loop.
class maxwell {
 public:
  explicit maxwell(const reader& in) : p_(in.p) {
    if (p_.monitor_every == 0) p_.monitor_every = 1;  // the drivers take the max every step
    check(lx_sim_create(&p_, &sim_));
  }
  ~maxwell() { lx_sim_destroy(sim_); }
  maxwell(const maxwell&) = delete;
  maxwell& operator=(const maxwell&) = delete;

  lx_sim* handle() { return sim_; }

  // Print the "t: ..., max: ..." line of every print_every-th step (1 = every step, as the
  // reference prints).
  int print_every = 1;
  bool quiet = false;
  // Directory for the driver's output files and the 3-D PML driver's material files.
  std::string dir = ".";
  // solve3d_pml needs airplane_100_{x,y,z}.h5 (three_dim_pml.cc:109-118); when false and
  // the files are missing the run uses vacuum instead of failing.
  bool require_material = true;

  void solve() {
    const bool planar = p_.isPlanar != 0, pml = p_.usePML != 0;
    if (planar) {
      // Ey every 10 steps (two_dim_pml.cc:184) or every 20 from t = 100 (two_dim.cc:140)
      check(lx_sim_set_hdf5_output(sim_, pml ? 10 : 20, pml ? 0 : 100, LX_EY, (dir + "/Ey_data_2d.h5").c_str()),
            sim_);
    } else if (pml) {
      load_material();
      check(lx_sim_set_hdf5_output(sim_, 3, 0, LX_ETOTAL, (dir + "/Ez_data.h5").c_str()), sim_);  // :279
    } else {
      check(lx_sim_set_hdf5_output(sim_, 10, 0, LX_ETOTAL, (dir + "/Ez_data2.h5").c_str()), sim_);  // :192
    }
    const auto t0 = std::chrono::steady_clock::now();
    // Steps run in chunks; the max of each step comes back from the device series once per
    // chunk.  solve_planar prints, after its E update, the max of step t itself
    // (two_dim.cc:126-137).  The other three drivers print, at the top of step t, the max left
    // by step t-1 (two_dim_pml.cc:135-141, three_dim.cc:91-97, three_dim_pml.cc:167-173); at
    // t = 0 they print an uninitialised local_max, here 0 (the max of the zero initial fields).
    const bool same_step = planar && !pml;
    const int chunk = 100;
    check(lx_sim_set_max_series(sim_, chunk), sim_);
    std::vector<int> ts(chunk);
    std::vector<double> ms(chunk);
    double prev = 0.0;
    int done = 0;
    while (done < p_.num_timesteps) {
      const int n = std::min(chunk, p_.num_timesteps - done);
      check(lx_sim_step(sim_, n), sim_);
      int rows = 0;
      check(lx_sim_read_max_series(sim_, ts.data(), ms.data(), chunk, &rows), sim_);
      for (int r = 0; r < rows; r++) {
        const double shown = same_step ? ms[r] : prev;
        if (!quiet && print_every > 0 && ts[r] % print_every == 0) std::printf("t: %d, max: %g\n", ts[r], shown);
        prev = ms[r];
      }
      done += n;
    }
    check(lx_sim_sync(sim_), sim_);
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (!quiet) std::printf("Time taken: %g sec\n", sec);
  }

 private:
  // Cb = dt/(eps0*(1+F*1e6)) from the "data" dataset of one file per E component
  // (three_dim_pml.cc:109-128).
  void load_material() {
    const char* names[3] = {"airplane_100_x.h5", "airplane_100_y.h5", "airplane_100_z.h5"};
    for (int c = 0; c < 3; c++) {
      const std::string path = dir + "/" + names[c];
      int shp[3];
      if (lx_hdf5_read(path.c_str(), "data", nullptr, 0, shp) != LX_OK) {
        if (require_material) throw error(LX_ERR_IO, std::string(lx_last_error(nullptr)) + " (material of E component)");
        continue;
      }
      int want[3];
      check(lx_sim_field_shape(sim_, c, want), sim_);
      if (shp[0] != want[0] || shp[1] != want[1] || shp[2] != want[2])
        throw error(LX_ERR_INVALID, path + ": dataset shape does not match the component's staggered extent");
      std::vector<double> F((size_t)shp[0] * shp[1] * shp[2]);
      check(lx_hdf5_read(path.c_str(), "data", F.data(), F.size(), shp));
      check(lx_sim_set_material(sim_, c, F.data(), F.size(), 1e6), sim_);
    }
  }

  lx_params p_;
  lx_sim* sim_ = nullptr;
};

}  // namespace luxum
