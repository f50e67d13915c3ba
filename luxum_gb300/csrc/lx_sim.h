// lx_sim.h -- host-side state of one simulation handle (C++ only; not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "luxum.h"
#include "lx_internal.h"

namespace lx {

class Hdf5Writer;  // lx_hdf5.cpp

// One snapshot consumer: a user callback or an HDF5 file for one component.
struct Output {
  int every = 0;
  int first = 0;
  unsigned mask = 0;
  lx_snapshot_fn fn = nullptr;
  void* user = nullptr;
  Hdf5Writer* h5 = nullptr;  // owned
  int h5_comp = -1;
};

struct SnapSlot {
  double* dev = nullptr;   // compact staging (device)
  double* host = nullptr;  // pinned
  size_t cap = 0;          // doubles
  cudaEvent_t ev_d2h = nullptr;
  bool busy = false;
};

struct DftPlane {
  int axis = 0, index = 0, nfreq = 0, every = 1, na = 0, nb = 0;
  int comps[4] = {0, 0, 0, 0};
  std::vector<double> omega;
  double* d_omega = nullptr;
  double* d_acc = nullptr;
  double* d_flux = nullptr;  // flux result + per-chunk partial sums
  double* d_phase = nullptr;  // phase factors of the current sample (4 x kMaxDftFreq)
  size_t n_acc = 0;  // doubles
};

struct SnapJob {
  int slot, t;
  unsigned mask;
  size_t off[7];
};

// Makes a handle's device current for the length of an entry point and gives the caller's
// device back on return.  A handle's streams and memory belong to the device that was current
// when it was created; a caller on another device would otherwise launch on the wrong one.
class DeviceGuard {
 public:
  explicit DeviceGuard(int device) {
    int cur = -1;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != device && cudaSetDevice(device) == cudaSuccess) prev_ = cur;
  }
  ~DeviceGuard() {
    if (prev_ >= 0) cudaSetDevice(prev_);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;

 private:
  int prev_ = -1;
};

// Host-side constants of maxwell::maxwell (maxwell.cc:60-148).
struct Consts {
  double epsilon0, mew0, S, c, dt, dx, dy, dz, sigma, init;
  double a_max, k_max, m_pml, ma_pml, sigma_optimal, sigma_max, d_pml;
  double H_dir[3], E_dir[3], k[3];
  int p1, q1, r1, p2, q2, r2;
  int st[3], en[3];  // plane_wave_initialise start/end per axis
};

}  // namespace lx

struct lx_sim {
  lx_params p;
  lx_batch* batch = nullptr;  // the batch this handle is a member of
  int device = 0;             // CUDA device current when the handle was created
  lx::Consts k;
  std::string err;
  int planar = 0, pml = 0, uniform = 0, prec = 0, tfsf = 0;
  int Nx = 0, Ny = 0, Nz = 0, Nzp = 0;
  size_t ncell = 0;   // Nx*Ny*Nzp
  size_t tsize = 0;   // bytes per field element
  size_t csize = 0;   // bytes per compute element
  int ext[7][3] = {};  // staggered extents (component 6 = |E|^2, Ez-shaped)
  // device state
  void* E[3] = {};
  void* H[3] = {};
  void* Cbs[3] = {};
  void* prof[3][6] = {};  // per axis: bE cE rkE bH cH rkH (compute precision)
  void* psiH[3][2] = {};
  void* psiE[3][2] = {};
  // Single-sweep handles (float compute) keep a second copy of the state.  Stepped
  // alone they run in ping-pong mode (pp): after t steps the state lives in buffer t & 1
  // (buffer 0 = E, H, psiH, psiE above, buffer 1 here).  In a batch they are updated in place
  // in buffer 0 (pp = 0); set_pp moves the state when the mode changes.
  int sweep = 0;
  int pp = 0;
  void* E1[3] = {};
  void* H1[3] = {};
  void* psiH1[3][2] = {};
  void* psiE1[3][2] = {};
  size_t psiH_n[3][2] = {}, psiE_n[3][2] = {};
  lx::Slab slab[3] = {};
  void* tab = nullptr;
  int tab_total = 0;
  lx::PatchSet setsH[3][2] = {}, setsE[3][2] = {};
  unsigned long long* d_max = nullptr;
  unsigned* d_fault = nullptr;  // in d_max's allocation: set by a kernel whose bounded wait ran out
  // max|E|^2 series: one slot per monitored step (device), the step of each slot (host)
  unsigned long long* d_series = nullptr;
  int series_cap = 0;
  std::vector<int> series_t;
  void* etotal = nullptr;
  double* xfer = nullptr;  // compact staging for field/material transfers
  size_t xfer_cap = 0;
  double cbs_scale = 1.0;  // 1/dx in difference units, 1 otherwise, divided by hscale
  double hscale = 1.0;     // H is stored as H*hscale (FP16 storage: the impedance of free space)
  double cb0 = 0.0;        // dt/epsilon0
  // point source
  int src_kind = -1;
  long long src_idx = 0;
  // streams
  cudaStream_t own = nullptr, side = nullptr, stream = nullptr;
  int t = 0;
  double last_max = 0.0;
  // probes
  int nprobes = 0, probe_cap = 0, probe_rows = 0;
  int* d_probe_ijk = nullptr;
  double* d_probe = nullptr;
  // DFT plane monitors
  std::vector<lx::DftPlane> dfts;
  // snapshots
  std::vector<lx::Output> outputs;
  lx::SnapSlot slots[2];
  std::deque<lx::SnapJob> jobs;
  std::mutex mu;
  std::condition_variable cv;
  std::thread writer;
  bool writer_on = false, stop = false;
  std::string writer_err;
  int pending = 0;
  // counters
  uint64_t n_kernels = 0, n_h2d = 0, n_d2h = 0;
};

namespace lx {
// Device array of component `comp` (LX_EX..LX_ETOTAL) in the buffer that holds the current
// state: buffer t & 1 for a handle stepped alone in ping-pong mode, else buffer 0.  With
// `other`, the buffer that does not.  Null when the handle keeps no such array.  Every reader
// of a handle's fields takes its source from here.
void* comp_ptr(lx_sim* s, int comp, bool other = false);
}  // namespace lx
