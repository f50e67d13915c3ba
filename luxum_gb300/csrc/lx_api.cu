// lx_api.cu -- implementation of the C ABI in include/luxum.h.
//
// Host code here is compiled with -ffp-contract=off: the constants and CPML profiles are
// computed with the reference's expressions (maxwell.cc:60-148, 997-1280) and must round
// the same way on x86-64 and aarch64 hosts.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "luxum.h"
#include "lx_hdf5.h"
#include "lx_internal.h"
#include "lx_kernels.h"
#include "lx_sim.h"

using lx::PatchSet;
using lx::Slab;

static thread_local std::string g_err;

namespace lx {
lx_status set_thread_error(const char* msg, lx_status st) {
  g_err = msg;
  return st;
}
}  // namespace lx

// Device memory of handles and batches comes from the device's stream-ordered pool: creating
// and destroying handles (the serving loop does so continuously) then neither pays for a
// fresh cudaMalloc nor synchronises the device as cudaFree does.  Freed blocks stay in the
// pool for reuse (release threshold raised once per process); cudaMemPoolTrimTo on the
// device's default pool returns them.
static void keep_pool_memory() {
  static bool done = false;
  if (done) return;
  int dev = 0;
  cudaMemPool_t pool;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done = true;
}

extern "C" LX_API lx_status lx_trim_device_memory(void) {
  int dev = 0;
  cudaMemPool_t pool;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaDeviceGetDefaultMemPool(&pool, dev);
  if (e == cudaSuccess) e = cudaMemPoolTrimTo(pool, 0);
  if (e != cudaSuccess) return lx::set_thread_error((std::string("lx_trim_device_memory: ") + cudaGetErrorString(e)).c_str(), LX_ERR_CUDA);
  return LX_OK;
}

static void dfree(void* p, cudaStream_t st) {
  if (p) cudaFreeAsync(p, st);
}

// Reserved bytes of the device's default pool at construction; on destruction the pool is
// trimmed back to them.  Tuning creates and frees thousands of twin allocations: left in the
// pool, they slowed every later handle creation of the serving loop threefold (5 -> 14 s of
// worker time over a 1000-request stream).
class PoolMark {
 public:
  PoolMark() {
    int dev = 0;
    uint64_t v = 0;
    ok_ = cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool_, dev) == cudaSuccess &&
          cudaMemPoolGetAttribute(pool_, cudaMemPoolAttrReservedMemCurrent, &v) == cudaSuccess;
    keep_ = (size_t)v;
  }
  ~PoolMark() {
    if (ok_) cudaMemPoolTrimTo(pool_, keep_);
  }
  PoolMark(const PoolMark&) = delete;
  PoolMark& operator=(const PoolMark&) = delete;

 private:
  cudaMemPool_t pool_ = nullptr;
  size_t keep_ = 0;
  bool ok_ = false;
};

static lx_status fail(lx_sim* s, lx_status st, const std::string& msg) {
  if (s) s->err = msg;
  g_err = msg;
  return st;
}

#define CK(...)                                                                                       \
  do {                                                                                                \
    cudaError_t e_ = (__VA_ARGS__);                                                                        \
    if (e_ != cudaSuccess)                                                                            \
      return fail(s, e_ == cudaErrorMemoryAllocation ? LX_ERR_OOM : LX_ERR_CUDA,                      \
                  std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(e_));                              \
  } while (0)

extern "C" LX_API const char* lx_version(void) { return "luxum-gb300 0.1 (sm_103a)"; }

extern "C" LX_API const char* lx_last_error(const lx_sim* s) { return s ? s->err.c_str() : g_err.c_str(); }

extern "C" LX_API void lx_params_init(lx_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->dx = p->dy = p->dz = 1e-3;
  p->S = 0.5;
  p->npX = p->npY = p->n_threads = 1;
  p->precision = LX_PREC_FP64;
  p->pw_sigma = pow(10, -4) / 0.5;  // maxwell.cc:71
  p->cpml_mode = LX_CPML_REFERENCE;
  p->source_kind = LX_SRC_CW_HARD;
  p->src_tw = 1.0;
  p->sigma = 0.65;
  p->sigma_m = 3;
  p->kappa = 1;
  p->a_m = 1;
}

// ------------------------------------------------------------------ validation

// reader::checkData (reader.cc:141-162) plus every index range or division the reference
// would read out of bounds, divide by zero on, or turn into NaN profiles.
static lx_status validate(const lx_params* p, std::string& why) {
  char b[256];
  if (p->npX < 1 || p->npY < 1) { why = "Number of Procs must be >= 1"; return LX_ERR_INVALID; }
  if ((p->Nx - 2) % p->npX != 0) {
    why = "ERROR: Condition-- (Number of points - 2) mod Number of processors --is not satisfied in X-direction";
    return LX_ERR_INVALID;
  }
  if ((p->Ny - 2) % p->npY != 0) {
    why = "ERROR: Condition-- (Number of points - 2) mod Number of processors --is not satisfied in Y-direction";
    return LX_ERR_INVALID;
  }
  if (p->isPlanar && p->Ny != 1) { why = "ERROR: Please put number of grid points in Y-direction as 1 for planar solutions."; return LX_ERR_INVALID; }
  if (p->isPlanar && p->npY != 1) { why = "ERROR: Please put number of processors in Y-direction as 1 for planar solutions."; return LX_ERR_INVALID; }
  if (p->Nx < 3 || p->Nz < 3 || (!p->isPlanar && p->Ny < 3)) { why = "grid must have at least 3 points per used axis"; return LX_ERR_INVALID; }
  if ((double)p->Nx * (p->isPlanar ? 1 : p->Ny) * p->Nz > 4.0e9) { why = "grid larger than 4e9 cells"; return LX_ERR_INVALID; }
  if (!(p->dx > 0) || !(p->dz > 0) || (!p->isPlanar && !(p->dy > 0)) || !(p->S > 0)) { why = "resolutions and Courant factor must be > 0"; return LX_ERR_INVALID; }
  if (p->num_timesteps < 0) { why = "Number of timesteps must be >= 0"; return LX_ERR_INVALID; }
  if (p->usePW) {
    if (p->x1_pw < 1 || p->x2_pw > p->Nx - 2 || p->x1_pw > p->x2_pw ||
        p->z1_pw < 1 || p->z2_pw > p->Nz - 2 || p->z1_pw > p->z2_pw ||
        (!p->isPlanar && (p->y1_pw < 1 || p->y2_pw > p->Ny - 2 || p->y1_pw > p->y2_pw))) {
      std::snprintf(b, sizeof b,
                    "total-field box must satisfy 1 <= x1 <= x2 <= Nx-2 (and y, z alike): the reference indexes "
                    "plane x1-1 and edits curl cells it never recomputes otherwise (got x %d..%d y %d..%d z %d..%d)",
                    p->x1_pw, p->x2_pw, p->y1_pw, p->y2_pw, p->z1_pw, p->z2_pw);
      why = b;
      return LX_ERR_INVALID;
    }
    double hx = p->ky_pw * p->Ez_pw - p->kz_pw * p->Ey_pw;
    double hy = p->kz_pw * p->Ex_pw - p->kx_pw * p->Ez_pw;
    double hz = p->kx_pw * p->Ey_pw - p->ky_pw * p->Ex_pw;
    if (hx == 0 && hy == 0 && hz == 0) { why = "k x E is zero: H direction undefined (maxwell.cc:94-102 divides by |k x E|)"; return LX_ERR_INVALID; }
    if (!(p->pw_sigma > 0)) { why = "plane-wave pulse width must be > 0"; return LX_ERR_INVALID; }
  }
  if (p->usePML) {
    double d0 = p->d_pml / p->dx, d2 = p->d_pml / p->dz, d1 = p->isPlanar ? 2.0 : p->d_pml / p->dy;
    if (!(d0 > 1) || !(d1 > 1) || !(d2 > 1)) { why = "Thickness of PML must exceed one cell (the profiles divide by d-1)"; return LX_ERR_INVALID; }
    if (p->sigma_m != std::floor(p->sigma_m)) {
      why = "m value of sigma must be an integer: the reference raises a negative base to it outside the layer (NaN profiles)";
      return LX_ERR_INVALID;
    }
  }
  if (p->usePS) {
    if (p->source_kind != LX_SRC_CW_HARD && p->source_kind != LX_SRC_PULSE_SOFT) { why = "unknown source kind"; return LX_ERR_INVALID; }
    if (p->isPlanar && p->source_kind == LX_SRC_CW_HARD) {
      why = "planar point source: the reference writes E->Vz, which planar grids do not have (vfield.cc:69-71)";
      return LX_ERR_UNSUPPORTED;
    }
    int zext = p->isPlanar ? p->Nz : p->Nz - 1;
    if (p->Nz_source < 0 || p->Nz_source >= zext) { why = "Source Z Pos outside the Ez extent (the reference does not range-check z)"; return LX_ERR_INVALID; }
    if (p->source_kind == LX_SRC_PULSE_SOFT && !(p->src_tw > 0)) { why = "pulse width must be > 0"; return LX_ERR_INVALID; }
  }
  if (p->precision < LX_PREC_FP64 || p->precision > LX_PREC_FP16S) { why = "unknown precision"; return LX_ERR_INVALID; }
  if (p->monitor_every < 0) { why = "monitor_every must be >= 0"; return LX_ERR_INVALID; }
  return LX_OK;
}

// ------------------------------------------------------------------ profiles (host)

// Position array of sigma_fn/k_fn/a_fn (maxwell.cc:1026-1035): index (+0.5 for H), offset 0.
static double prof_pos(int i, bool is_E) { return is_E ? (double)(i + 0) : ((double)i + 0.5) + 0; }

struct AxisProf {
  std::vector<double> kE, bE, cE, kH, bH, cH;
};

// sigma/k/a/b/c of maxwell.cc:997-1280 for one axis (N global points, spacing delta).
static void axis_profiles(const lx::Consts& K, int cpml_mode, int N, double delta, AxisProf& out) {
  const double d = K.d_pml / delta;
  for (int is_E = 1; is_E >= 0; --is_E) {
    int n = is_E ? N : N - 1;
    std::vector<double> sg(n), kk(n), aa(n), bb(n), cc(n);
    for (int i = 0; i < n; i++) {
      double temp = prof_pos(i, is_E);
      double w = 0.0;  // sigma_fn :1038-1040
      w = (double)(temp <= (d - 1)) * pow((((d - 1) - temp) / (d - 1)), K.m_pml) * K.sigma_max + (double)(temp > (d - 1)) * w;
      w = (double)(temp >= (N - d)) * pow((temp - N + d) / (d - 1), K.m_pml) * K.sigma_max + (double)(temp < (N - d)) * w;
      sg[i] = w;
      w = 1;  // k_fn :1100-1102
      w = (double)(temp <= (d - 1)) * (pow((((d - 1) - temp) / (d - 1)), K.m_pml) * (K.k_max - 1) + 1) + (double)(temp > (d - 1)) * w;
      w = (double)(temp >= (N - d)) * (pow((temp - N + d) / (d - 1), K.m_pml) * (K.k_max - 1) + 1) + (double)(temp < (N - d)) * w;
      kk[i] = w;
      w = 0.0;  // a_fn :1163-1165
      w = (double)(temp <= (d - 1)) * pow((temp / (d - 1)), K.ma_pml) * K.a_max + (double)(temp > (d - 1)) * w;
      w = (double)(temp >= (N - d)) * pow((N - 1 - temp) / (d - 1), K.ma_pml) * K.a_max + (double)(temp < (N - d)) * w;
      aa[i] = w;
      // b_fn :1215 (reference sign on a) or the textbook sign
      if (cpml_mode == LX_CPML_STANDARD)
        bb[i] = exp(-((sg[i] / kk[i] / K.epsilon0) + (aa[i] / K.epsilon0)) * K.dt);
      else
        bb[i] = exp(-((sg[i] / kk[i] / K.epsilon0) - (aa[i] / K.epsilon0)) * K.dt);
      // c_fn :1271-1278
      cc[i] = (sg[i] == 0) ? 0.0 : sg[i] / (sg[i] * kk[i] + pow(kk[i], 2) * aa[i]) * (bb[i] - 1);
    }
    if (is_E) { out.kE = kk; out.bE = bb; out.cE = cc; }
    else { out.kH = kk; out.bH = bb; out.cH = cc; }
  }
}

// Largest run of cells where neither the E nor the H profile is active -> packed slab.
static Slab make_slab(const AxisProf& a, int N) {
  std::vector<char> act(N, 0);
  for (int u = 0; u < N; u++) act[u] = (a.cE[u] != 0.0 || a.kE[u] != 1.0);
  for (int u = 0; u < N - 1; u++) act[u] |= (a.cH[u] != 0.0 || a.kH[u] != 1.0);
  int best_a = 0, best_b = 0, u = 0;
  while (u < N) {
    if (act[u]) { u++; continue; }
    int v = u;
    while (v < N && !act[v]) v++;
    if (v - u > best_b - best_a) { best_a = u; best_b = v; }
    u = v;
  }
  Slab s;
  if (best_b - best_a == 0) { s.lo = N; s.hi0 = N; s.n = N; }  // active everywhere
  else { s.lo = best_a; s.hi0 = best_b; s.n = best_a + (N - best_b); }
  return s;
}

// ------------------------------------------------------------------ TF/SF plane sets

static PatchSet mkset(const lx_sim* s, int axis, int pl0, int pl1, double pos0, double pos1, double sg0, double sg1,
                      double dir, double neg, double dn, int hcurl, const int lo[3], const int hi[3],
                      const double off[3]) {
  PatchSet ps;
  std::memset(&ps, 0, sizeof ps);
  ps.axis = axis;
  ps.plane[0] = pl0;
  ps.plane[1] = pl1;
  ps.pos_n[0] = pos0;
  ps.pos_n[1] = pos1;
  ps.sign[0] = sg0;
  ps.sign[1] = sg1;
  ps.dir = dir;
  ps.neg = neg;
  ps.dn = dn;
  ps.hcurl = hcurl;
  ps.scale = hcurl ? s->hscale : 1.0;
  // the constant part of every entry of this set, in the order the reference applies it
  // (maxwell.cc:289 and siblings: * E_dir / d, or / d / c / mu0 for the H-curl lines)
  double f = neg * dir / dn;
  if (hcurl) f = f / s->k.c / s->k.mew0;
  if (s->uniform) f = f * dn;  // difference units
  if (ps.scale != 1.0) f = f * ps.scale;
  ps.factor = f;
  bool empty = false;
  for (int b = 0; b < 3; b++) {
    ps.lo[b] = lo[b];
    ps.hi[b] = hi[b];
    ps.off[b] = off[b];
    if (b != axis && hi[b] < lo[b]) empty = true;
  }
  // the wave varies along in-plane axis b when its k component is non-zero (planar: no y term)
  int run = 1;
  for (int b = 2; b >= 0; b--) {
    bool varies = (b != axis) && (s->planar ? (b != 1 && s->k.k[b] != 0.0) : (s->k.k[b] != 0.0));
    ps.n[b] = varies ? (hi[b] - lo[b] + 1) : 1;
    ps.stride[b] = varies ? run : 0;
    run *= ps.n[b];
  }
  ps.plane_len = run;
  ps.active = (!empty && dir != 0.0) ? 1 : 0;
  return ps;
}

static void build_sets(lx_sim* s) {
  const lx::Consts& K = s->k;
  const int p1 = K.p1, p2 = K.p2, q1 = K.q1, q2 = K.q2, r1 = K.r1, r2 = K.r2;
  const int sx = K.st[0], ex = K.en[0], sy = K.st[1], ey = K.en[1], sz = K.st[2], ez = K.en[2];
  const double Ex = K.E_dir[0], Ey = K.E_dir[1], Ez = K.E_dir[2];
  const double Hx = K.H_dir[0], Hy = K.H_dir[1], Hz = K.H_dir[2];
  const double dx = K.dx, dy = K.dy, dz = K.dz;
  std::memset(s->setsH, 0, sizeof s->setsH);
  std::memset(s->setsE, 0, sizeof s->setsE);
  if (s->planar) {
    // maxwell.cc:516-591 (planar, adv curls)
    { int lo[3] = {sx, 0, 0}, hi[3] = {ex, 0, 0}; double off[3] = {0, 0, 0};
      s->setsH[0][1] = mkset(s, 2, r1 - 1, r2, r1, r2, +1, -1, Ey, 1, dz, 0, lo, hi, off); }   // :539-553
    { int lo[3] = {0, 0, sz}, hi[3] = {0, 0, ez}; double off[3] = {0, 0, 0};
      s->setsH[2][0] = mkset(s, 0, p1 - 1, p2, p1, p2, +1, -1, Ey, 1, dx, 0, lo, hi, off); }   // :519-534
    { int lo[3] = {0, 0, sz}, hi[3] = {0, 0, ez}; double off[3] = {0, 0, 0};
      s->setsE[1][1] = mkset(s, 0, p1, p2, p1 - 0.5, p2 + 0.5, -1, +1, Hz, -1, dx, 1, lo, hi, off); }  // :559-572
    { int lo[3] = {sx, 0, 0}, hi[3] = {ex, 0, 0}; double off[3] = {0, 0, 0};
      s->setsE[1][0] = mkset(s, 2, r1, r2, r1 - 0.5, r2 + 0.5, -1, +1, Hx, -1, dz, 1, lo, hi, off); }  // :577-590
  } else {
    // maxwell.cc:597-701 (E-curl sets for the H update, t - 0.5)
    { int lo[3] = {sx, 0, sz}, hi[3] = {ex, 0, ez - 1}; double off[3] = {0, 0, 0.5};
      s->setsH[0][0] = mkset(s, 1, q1 - 1, q2, q1, q2, -1, +1, Ez, 1, dy, 0, lo, hi, off); }  // :642-664
    { int lo[3] = {sx, sy, 0}, hi[3] = {ex, ey - 1, 0}; double off[3] = {0, 0.5, 0};
      s->setsH[0][1] = mkset(s, 2, r1 - 1, r2, r1, r2, -1, +1, Ey, 1, dz, 0, lo, hi, off); }  // :678-700
    { int lo[3] = {sx, sy, 0}, hi[3] = {ex - 1, ey, 0}; double off[3] = {0.5, 0, 0};
      s->setsH[1][0] = mkset(s, 2, r1 - 1, r2, r1, r2, -1, +1, Ex, 1, dz, 0, lo, hi, off); }  // :671-692
    { int lo[3] = {0, sy, sz}, hi[3] = {0, ey, ez - 1}; double off[3] = {0, 0, 0.5};
      s->setsH[1][1] = mkset(s, 0, p1 - 1, p2, p1, p2, -1, +1, Ez, 1, dx, 0, lo, hi, off); }  // :607-628
    { int lo[3] = {0, sy, sz}, hi[3] = {0, ey - 1, ez}; double off[3] = {0, 0.5, 0};
      s->setsH[2][0] = mkset(s, 0, p1 - 1, p2, p1, p2, -1, +1, Ey, 1, dx, 0, lo, hi, off); }  // :600-621
    { int lo[3] = {sx, 0, sz}, hi[3] = {ex - 1, 0, ez}; double off[3] = {0.5, 0, 0};
      s->setsH[2][1] = mkset(s, 1, q1 - 1, q2, q1, q2, -1, +1, Ex, 1, dy, 0, lo, hi, off); }  // :635-656
    // maxwell.cc:707-809 (H-curl sets for the E update, t)
    { int lo[3] = {sx, 0, sz}, hi[3] = {ex - 1, 0, ez}; double off[3] = {0.5, 0, 0};
      s->setsE[0][0] = mkset(s, 1, q1, q2, q1 - 0.5, q2 + 0.5, -1, +1, Hz, 1, dy, 1, lo, hi, off); }  // :743-764
    { int lo[3] = {sx, sy, 0}, hi[3] = {ex - 1, ey, 0}; double off[3] = {0.5, 0, 0};
      s->setsE[0][1] = mkset(s, 2, r1, r2, r1 - 0.5, r2 + 0.5, -1, +1, Hy, 1, dz, 1, lo, hi, off); }  // :779-800
    { int lo[3] = {sx, sy, 0}, hi[3] = {ex, ey - 1, 0}; double off[3] = {0, 0.5, 0};
      s->setsE[1][0] = mkset(s, 2, r1, r2, r1 - 0.5, r2 + 0.5, -1, +1, Hx, 1, dz, 1, lo, hi, off); }  // :786-807
    { int lo[3] = {0, sy, sz}, hi[3] = {0, ey - 1, ez}; double off[3] = {0, 0.5, 0};
      s->setsE[1][1] = mkset(s, 0, p1, p2, p1 - 0.5, p2 + 0.5, -1, +1, Hz, 1, dx, 1, lo, hi, off); }  // :708-729
    { int lo[3] = {0, sy, sz}, hi[3] = {0, ey, ez - 1}; double off[3] = {0, 0, 0.5};
      s->setsE[2][0] = mkset(s, 0, p1, p2, p1 - 0.5, p2 + 0.5, -1, +1, Hy, 1, dx, 1, lo, hi, off); }  // :715-736
    { int lo[3] = {sx, 0, sz}, hi[3] = {ex, 0, ez - 1}; double off[3] = {0, 0, 0.5};
      s->setsE[2][1] = mkset(s, 1, q1, q2, q1 - 0.5, q2 + 0.5, -1, +1, Hx, 1, dy, 1, lo, hi, off); }  // :750-771
  }
  int off = 0;
  for (int h = 0; h < 2; h++)
    for (int c = 0; c < 3; c++)
      for (int part = 0; part < 2; part++) {
        PatchSet& ps = h == 0 ? s->setsH[c][part] : s->setsE[c][part];
        if (!ps.active) continue;
        ps.tab = off;
        off += 2 * ps.plane_len;
      }
  s->tab_total = off;
}

// plane_wave_initialise maxwell.cc:825-913 for one axis
static void pw_clip(int a1, int a2, int cs, int ce, int* st, int* en) {
  if (a1 > ce) { *st = -1; *en = -1; }
  else if (a1 >= cs) { *st = a1; *en = (a2 > ce) ? ce : a2; }
  else if (a2 > ce) { *st = cs; *en = ce; }
  else if (a2 >= cs) { *st = cs; *en = a2; }
  else { *st = -1; *en = -1; }
}

// ------------------------------------------------------------------ create / destroy

static size_t elsize(int prec) { return prec == LX_PREC_FP64 ? 8 : (prec == LX_PREC_FP32 ? 4 : 2); }

template <class C>
static lx_status upload_vec(lx_sim* s, void** dst, const std::vector<double>& v) {
  std::vector<C> tmp(v.size());
  for (size_t q = 0; q < v.size(); q++) tmp[q] = (C)v[q];
  CK(cudaMallocAsync(dst, tmp.size() * sizeof(C) + 16, s->own));
  CK(cudaMemcpyAsync(*dst, tmp.data(), tmp.size() * sizeof(C), cudaMemcpyHostToDevice, s->own));
  s->n_h2d += tmp.size() * sizeof(C);
  return LX_OK;
}

static void compute_extents(lx_sim* s) {
  const int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz;
  std::memset(s->ext, 0, sizeof s->ext);
  if (s->planar) {
    int ey[3] = {Nx, 1, Nz}, hx[3] = {Nx, 1, Nz - 1}, hz[3] = {Nx - 1, 1, Nz};  // vfield.cc:64-70
    std::memcpy(s->ext[LX_EY], ey, sizeof ey);
    std::memcpy(s->ext[LX_HX], hx, sizeof hx);
    std::memcpy(s->ext[LX_HZ], hz, sizeof hz);
  } else {
    int e[6][3] = {{Nx - 1, Ny, Nz}, {Nx, Ny - 1, Nz}, {Nx, Ny, Nz - 1},      // vfield.cc:81-83
                   {Nx, Ny - 1, Nz - 1}, {Nx - 1, Ny, Nz - 1}, {Nx - 1, Ny - 1, Nz}};  // vfield.cc:76-78
    std::memcpy(s->ext, e, sizeof e);
    s->ext[LX_ETOTAL][0] = Nx;
    s->ext[LX_ETOTAL][1] = Ny;
    s->ext[LX_ETOTAL][2] = Nz - 1;
  }
}

static size_t ext_n(const lx_sim* s, int c) { return (size_t)s->ext[c][0] * s->ext[c][1] * s->ext[c][2]; }

static void stop_writer(lx_sim* s);

// Completes a batch chunk in flight that this handle is a member of, before the handle's
// own state is read, written or stepped.  A blow-up is reported by the batch's own wait and
// shows in this handle's max|E|^2; only CUDA errors are returned here.
extern "C" LX_API lx_status lx_batch_wait(lx_batch* b);
extern "C" LX_API lx_status lx_batch_remove(lx_batch* b, lx_sim* s);
static void batch_member_changed(lx_batch* b);
static lx_status settle(lx_sim* s) {
  if (!s->batch) return LX_OK;
  const lx_status st = lx_batch_wait(s->batch);
  return st == LX_ERR_BLOWUP ? LX_OK : st;
}

extern "C" LX_API void lx_sim_destroy(lx_sim* s) {
  if (!s) return;
  lx::DeviceGuard dg_(s->device);
  if (s->batch) lx_batch_remove(s->batch, s);
  stop_writer(s);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->side) cudaStreamSynchronize(s->side);
  cudaStream_t fs = s->own;
  for (int c = 0; c < 3; c++) {
    dfree(s->E[c], fs); dfree(s->H[c], fs); dfree(s->Cbs[c], fs);
    dfree(s->E1[c], fs); dfree(s->H1[c], fs);
    for (int q = 0; q < 6; q++) dfree(s->prof[c][q], fs);
    for (int q = 0; q < 2; q++) { dfree(s->psiH[c][q], fs); dfree(s->psiE[c][q], fs); }
    for (int q = 0; q < 2; q++) { dfree(s->psiH1[c][q], fs); dfree(s->psiE1[c][q], fs); }
  }
  dfree(s->tab, fs); dfree(s->d_max, fs); dfree(s->d_series, fs); dfree(s->etotal, fs); dfree(s->xfer, fs);
  dfree(s->d_probe_ijk, fs); dfree(s->d_probe, fs);
  for (auto& sl : s->slots) {
    dfree(sl.dev, fs);
    if (sl.host) cudaFreeHost(sl.host);
    if (sl.ev_d2h) cudaEventDestroy(sl.ev_d2h);
  }
  for (auto& o : s->outputs) delete o.h5;
  for (auto& d : s->dfts) {
    dfree(d.d_omega, fs);
    dfree(d.d_acc, fs);
    dfree(d.d_flux, fs);
    dfree(d.d_phase, fs);
  }
  if (s->own) {
    cudaStreamSynchronize(s->own);
    cudaStreamDestroy(s->own);
  }
  if (s->side) cudaStreamDestroy(s->side);
  delete s;
}

static lx_status alloc_zero(lx_sim* s, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) return LX_OK;
  CK(cudaMallocAsync(p, bytes, s->own));
  CK(cudaMemsetAsync(*p, 0, bytes, s->own));
  return LX_OK;
}

template <class C>
static lx_status create_typed(lx_sim* s) {
  const lx::Consts& K = s->k;
  const size_t fb = s->ncell * s->tsize;
  lx_status st;
  // fields (field.cc:77-85 zero-initialises every component)
  for (int c = 0; c < 3; c++) {
    if (s->planar && c != 1) continue;
    if ((st = alloc_zero(s, &s->E[c], fb))) return st;
    if (s->sweep && (st = alloc_zero(s, &s->E1[c], fb))) return st;
    if ((st = alloc_zero(s, &s->Cbs[c], s->ncell * sizeof(C)))) return st;
  }
  for (int c = 0; c < 3; c++) {
    if (s->planar && c == 1) continue;
    if ((st = alloc_zero(s, &s->H[c], fb))) return st;
    if (s->sweep && (st = alloc_zero(s, &s->H1[c], fb))) return st;
  }
  // Cb = dt/epsilon0 (two_dim.cc:81, two_dim_pml.cc:116, three_dim.cc:54)
  s->cb0 = K.dt / K.epsilon0;
  for (int c = 0; c < 3; c++) {
    if (!s->Cbs[c]) continue;
    int lo[3] = {0, 0, 0}, hi[3] = {s->ext[c][0], s->ext[c][1], s->ext[c][2]};
    CK(lx::launch_eps_box<C>((C*)s->Cbs[c], s->ext[c], s->Ny, s->Nzp, lo, hi, s->cb0 * s->cbs_scale, s->stream));
    s->n_kernels++;
  }
  // CPML profiles and slabs
  if (s->pml) {
    for (int a = 0; a < 3; a++) {
      if (s->planar && a == 1) continue;
      const int N = a == 0 ? s->p.Nx : (a == 1 ? s->p.Ny : s->p.Nz);
      const double delta = a == 0 ? s->p.dx : (a == 1 ? s->p.dy : s->p.dz);
      AxisProf ap;
      axis_profiles(K, s->p.cpml_mode, N, delta, ap);
      s->slab[a] = make_slab(ap, N);
      std::vector<double> rkE(ap.kE.size()), rkH(ap.kH.size());
      for (size_t q = 0; q < rkE.size(); q++) rkE[q] = 1.0 / ap.kE[q];
      for (size_t q = 0; q < rkH.size(); q++) rkH[q] = 1.0 / ap.kH[q];
      if ((st = upload_vec<C>(s, &s->prof[a][0], ap.bE))) return st;
      if ((st = upload_vec<C>(s, &s->prof[a][1], ap.cE))) return st;
      if ((st = upload_vec<C>(s, &s->prof[a][2], rkE))) return st;
      if ((st = upload_vec<C>(s, &s->prof[a][3], ap.bH))) return st;
      if ((st = upload_vec<C>(s, &s->prof[a][4], ap.cH))) return st;
      if ((st = upload_vec<C>(s, &s->prof[a][5], rkH))) return st;
    }
    // psi arrays: [component][part] -> axis of that part's derivative
    const int axH[3][2] = {{1, 2}, {2, 0}, {0, 1}};  // Hx: d/dy, d/dz; Hy: d/dz, d/dx; Hz: d/dx, d/dy
    const int axE[3][2] = {{1, 2}, {2, 0}, {0, 1}};  // Ex: d/dy, d/dz; Ey: d/dz, d/dx; Ez: d/dx, d/dy
    auto psi_size = [&](int axis) -> size_t {
      const Slab& sl = s->slab[axis];
      if (sl.n == 0) return 0;
      if (axis == 0) return (size_t)sl.n * s->Ny * s->Nzp;
      if (axis == 1) return (size_t)s->Nx * sl.n * s->Nzp;
      return (size_t)s->Nx * s->Ny * sl.n;
    };
    for (int c = 0; c < 3; c++)
      for (int part = 0; part < 2; part++) {
        bool useH = !s->planar || (c == 0 && part == 1) || (c == 2 && part == 0);
        bool useE = !s->planar || (c == 1);
        if (s->planar && (axH[c][part] == 1)) useH = false;
        if (s->planar && (axE[c][part] == 1)) useE = false;
        if (useH) {
          s->psiH_n[c][part] = psi_size(axH[c][part]);
          if ((st = alloc_zero(s, &s->psiH[c][part], s->psiH_n[c][part] * sizeof(C)))) return st;
          if (s->sweep && (st = alloc_zero(s, &s->psiH1[c][part], s->psiH_n[c][part] * sizeof(C)))) return st;
        }
        if (useE) {
          s->psiE_n[c][part] = psi_size(axE[c][part]);
          if ((st = alloc_zero(s, &s->psiE[c][part], s->psiE_n[c][part] * sizeof(C)))) return st;
          if (s->sweep && (st = alloc_zero(s, &s->psiE1[c][part], s->psiE_n[c][part] * sizeof(C)))) return st;
        }
      }
  }
  if (s->tfsf) {
    build_sets(s);
    CK(cudaMallocAsync(&s->tab, (size_t)(s->tab_total > 0 ? s->tab_total : 1) * sizeof(C), s->own));
  }
  CK(cudaMallocAsync(&s->d_max, 64, s->own));
  CK(cudaMemsetAsync(s->d_max, 0, 64, s->own));
  s->d_fault = reinterpret_cast<unsigned*>(s->d_max + 1);
  return LX_OK;
}

// Host-side set-up shared by lx_sim_create and lx_params_device_bytes: grid, constants
// (maxwell.cc:60-148), plane-wave clipping, point source.
static void setup_host(lx_sim* s, const lx_params* p) {
  s->p = *p;
  s->planar = p->isPlanar != 0;
  s->pml = p->usePML != 0;
  s->tfsf = p->usePW != 0;
  s->prec = p->precision;
  s->tsize = elsize(p->precision);
  s->csize = p->precision == LX_PREC_FP64 ? 8 : 4;
  // grid::grid grid.cc:83-93, single rank
  s->Nx = (p->Nx - 2) / 1 + 2;
  s->Ny = s->planar ? 1 : (p->Ny - 2) / 1 + 2;
  s->Nz = p->Nz;
  const int per = (int)(128 / s->tsize);
  s->Nzp = (s->Nz + per - 1) / per * per;
  s->ncell = (size_t)s->Nx * s->Ny * s->Nzp;
  compute_extents(s);
  // Planar handles with float compute step in one sweep over two state buffers; FP64 is bound
  // by the FP64 pipe, where the sweep's recomputed halos would only add work.  3-D float
  // handles take the single-sweep kernel (lx_sweep3d.cu) when LUXUM_SWEEP3=1: it runs ahead
  // of the two-sweep kernels on grids without CPML and TF/SF and behind them with both.
  // LUXUM_TWO_SWEEP=1 keeps new handles on the in-place two-sweep kernels (A/B checks).
  {
    const char* two = std::getenv("LUXUM_TWO_SWEEP");
    const char* s3 = std::getenv("LUXUM_SWEEP3");
    s->sweep = p->precision != LX_PREC_FP64 && !(two && two[0] == '1') &&
               (s->planar || (s3 && s3[0] == '1'));
  }

  // maxwell::maxwell maxwell.cc:60-148
  lx::Consts& K = s->k;
  std::memset(&K, 0, sizeof K);
  K.epsilon0 = 8.85 * pow(10, -12);
  K.mew0 = M_PI * 4 * pow(10, -7);
  K.S = p->S;
  K.c = 1 / pow(K.epsilon0 * K.mew0, 0.5);
  K.dt = K.S * p->dx / K.c;
  K.dx = p->dx;
  K.dy = p->dy;
  K.dz = p->dz;
  K.sigma = p->pw_sigma;
  K.init = p->off_pw;
  if (s->pml) {
    K.a_max = p->a_max;
    K.k_max = p->kappa;
    K.m_pml = p->sigma_m;
    K.ma_pml = p->a_m;
    K.sigma_optimal = 0.8 * (K.m_pml + 1) / K.dx / pow(K.mew0 / K.epsilon0, 0.5);
    K.sigma_max = K.sigma_optimal * p->sigma;
    K.d_pml = p->d_pml;
  }
  if (s->tfsf) {
    K.E_dir[0] = p->Ex_pw; K.E_dir[1] = p->Ey_pw; K.E_dir[2] = p->Ez_pw;
    K.k[0] = p->kx_pw; K.k[1] = p->ky_pw; K.k[2] = p->kz_pw;
    K.H_dir[0] = K.k[1] * K.E_dir[2] - K.k[2] * K.E_dir[1];
    K.H_dir[1] = K.k[2] * K.E_dir[0] - K.k[0] * K.E_dir[2];
    K.H_dir[2] = K.k[0] * K.E_dir[1] - K.k[1] * K.E_dir[0];
    double H_abs = pow(pow(K.H_dir[0], 2) + pow(K.H_dir[1], 2) + pow(K.H_dir[2], 2), 0.5);
    for (int a = 0; a < 3; a++) K.H_dir[a] = K.H_dir[a] / H_abs;
    K.p1 = p->x1_pw; K.q1 = p->y1_pw; K.r1 = p->z1_pw;
    K.p2 = p->x2_pw; K.q2 = p->y2_pw; K.r2 = p->z2_pw;
    pw_clip(K.p1, K.p2, 0, s->Nx - 1, &K.st[0], &K.en[0]);
    if (s->planar) pw_clip(K.q1, K.q2, 0, 0, &K.st[1], &K.en[1]);
    else pw_clip(K.q1, K.q2, 0, s->Ny - 1, &K.st[1], &K.en[1]);
    pw_clip(K.r1, K.r2, 0, s->Nz - 1, &K.st[2], &K.en[2]);
  }
  s->uniform = s->planar ? (p->dx == p->dz) : (p->dx == p->dy && p->dx == p->dz);
  // FP16 storage keeps H as H * sqrt(mu0/eps0), the same order as E: stored H then stays
  // in binary16's normal range.  Cb absorbs 1/hscale, Db and the H-curl TF/SF lines hscale.
  s->hscale = p->precision == LX_PREC_FP16S ? pow(K.mew0 / K.epsilon0, 0.5) : 1.0;
  s->cbs_scale = (s->uniform ? 1.0 / p->dx : 1.0) / s->hscale;

  // point source: check_global_limits (maxwell.cc:944-959) skips it silently off the grid
  if (p->usePS) {
    int x = p->Nx_source, y = s->planar ? 0 : p->Ny_source, z = p->Nz_source;
    bool inside = x >= 0 && y >= 0 && x <= s->Nx - 1 && y <= (s->planar ? 0 : s->Ny - 1);
    if (inside) {
      s->src_kind = p->source_kind == LX_SRC_CW_HARD ? 0 : 1;
      s->src_idx = ((long long)x * s->Ny + y) * s->Nzp + z;
    }
  }

}

extern "C" LX_API lx_status lx_sim_create(const lx_params* p, lx_sim** out) {
  if (!p || !out) return fail(nullptr, LX_ERR_INVALID, "null argument");
  *out = nullptr;
  std::string why;
  lx_status st = validate(p, why);
  if (st) return fail(nullptr, st, why);
  lx_sim* s = new (std::nothrow) lx_sim();
  if (!s) return fail(nullptr, LX_ERR_OOM, "host allocation failed");
  keep_pool_memory();
  setup_host(s, p);
  cudaGetDevice(&s->device);

  // The handle's own stream takes the device's highest priority: what a new handle queues
  // while a batch chunk runs (its allocations' memsets, boxes, DFT set-up, in the serving loop)
  // is then scheduled ahead of the chunk's pending blocks rather than behind them.
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  cudaError_t e = cudaStreamCreateWithPriority(&s->own, cudaStreamNonBlocking, prio_hi);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    std::string m = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
    lx_sim_destroy(s);
    return fail(nullptr, LX_ERR_CUDA, m);
  }
  s->stream = s->own;
  st = (s->csize == 8) ? create_typed<double>(s) : create_typed<float>(s);
  s->pp = s->sweep;
  if (st == LX_OK) {
    e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) st = fail(s, LX_ERR_CUDA, std::string("create: ") + cudaGetErrorString(e));
  }
  if (st) {
    std::string m = s->err;
    lx_sim_destroy(s);
    return fail(nullptr, st, m);
  }
  *out = s;
  return LX_OK;
}

extern "C" LX_API lx_status lx_params_field_shape(const lx_params* p, int comp, int shape[3]) {
  if (!p || !shape || comp < 0 || comp > LX_ETOTAL) return fail(nullptr, LX_ERR_INVALID, "bad argument");
  std::string why;
  lx_status st = validate(p, why);
  if (st) return fail(nullptr, st, why);
  lx_sim tmp;
  setup_host(&tmp, p);
  for (int a = 0; a < 3; a++) shape[a] = tmp.ext[comp][a];
  return LX_OK;
}

extern "C" LX_API lx_status lx_params_device_bytes(const lx_params* p, size_t* bytes) {
  if (!p || !bytes) return fail(nullptr, LX_ERR_INVALID, "null argument");
  std::string why;
  lx_status st = validate(p, why);
  if (st) return fail(nullptr, st, why);
  lx_sim tmp;
  setup_host(&tmp, p);
  size_t b = 0;
  const int nE = tmp.planar ? 1 : 3, nH = tmp.planar ? 2 : 3, nbuf = tmp.sweep ? 2 : 1;
  b += (size_t)nbuf * (nE + nH) * tmp.ncell * tmp.tsize + (size_t)nE * tmp.ncell * tmp.csize;
  if (tmp.pml) {
    for (int a = 0; a < 3; a++) {
      if (tmp.planar && a == 1) continue;
      const int N = a == 0 ? p->Nx : (a == 1 ? p->Ny : p->Nz);
      const double delta = a == 0 ? p->dx : (a == 1 ? p->dy : p->dz);
      AxisProf ap;
      axis_profiles(tmp.k, p->cpml_mode, N, delta, ap);
      tmp.slab[a] = make_slab(ap, N);
      b += (size_t)(6 * N) * tmp.csize + 96;
      const Slab& sl = tmp.slab[a];
      const size_t plane = a == 0 ? (size_t)tmp.Ny * tmp.Nzp : (a == 1 ? (size_t)tmp.Nx * tmp.Nzp : (size_t)tmp.Nx * tmp.Ny);
      // psi arrays whose derivative runs along this axis: 4 in 3-D (2 H + 2 E), 2 in planar
      b += (size_t)nbuf * (tmp.planar ? 2 : 4) * sl.n * plane * tmp.csize;
    }
  }
  if (tmp.tfsf) {
    build_sets(&tmp);
    b += (size_t)tmp.tab_total * tmp.csize;
  }
  *bytes = b + 64;
  return LX_OK;
}

extern "C" LX_API lx_status lx_params_step_bytes(const lx_params* p, double* bytes) {
  if (!p || !bytes) return fail(nullptr, LX_ERR_INVALID, "null argument");
  std::string why;
  lx_status st = validate(p, why);
  if (st) return fail(nullptr, st, why);
  lx_sim tmp;
  setup_host(&tmp, p);
  const double cells = (double)p->Nx * (tmp.planar ? 1 : p->Ny) * p->Nz;
  const int nF = tmp.planar ? 3 : 6, nE = tmp.planar ? 1 : 3;
  double b = cells * (2.0 * nF * tmp.tsize + (double)nE * tmp.csize);
  if (tmp.pml) {
    const double ext[3] = {(double)p->Nx, tmp.planar ? 1.0 : (double)p->Ny, (double)p->Nz};
    for (int a = 0; a < 3; a++) {
      if (tmp.planar && a == 1) continue;
      const int N = a == 0 ? p->Nx : (a == 1 ? p->Ny : p->Nz);
      const double delta = a == 0 ? p->dx : (a == 1 ? p->dy : p->dz);
      AxisProf ap;
      axis_profiles(tmp.k, p->cpml_mode, N, delta, ap);
      const Slab sl = make_slab(ap, N);
      // psi arrays whose derivative runs along axis a: 2 H + 2 E in 3-D, 1 + 1 in planar
      b += 2.0 * (tmp.planar ? 2 : 4) * sl.n * (cells / ext[a]) * tmp.csize;
    }
  }
  *bytes = b;
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_reset(lx_sim* s) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  lx::DeviceGuard dg_(s->device);
  lx_status st = lx_sim_sync(s);
  if (st) return st;
  const size_t fb = s->ncell * s->tsize;
  for (int c = 0; c < 3; c++) {
    for (void* f : {s->E[c], s->H[c], s->E1[c], s->H1[c]})
      if (f) CK(cudaMemsetAsync(f, 0, fb, s->stream));
    for (int q = 0; q < 2; q++) {
      for (void* f : {s->psiH[c][q], s->psiH1[c][q]})
        if (f) CK(cudaMemsetAsync(f, 0, s->psiH_n[c][q] * s->csize, s->stream));
      for (void* f : {s->psiE[c][q], s->psiE1[c][q]})
        if (f) CK(cudaMemsetAsync(f, 0, s->psiE_n[c][q] * s->csize, s->stream));
    }
  }
  if (s->etotal) CK(cudaMemsetAsync(s->etotal, 0, s->ncell * s->csize, s->stream));
  for (auto& d : s->dfts) CK(cudaMemsetAsync(d.d_acc, 0, d.n_acc * sizeof(double), s->stream));
  s->t = 0;
  s->probe_rows = 0;
  s->series_t.clear();
  s->last_max = 0.0;
  return LX_OK;
}

// ------------------------------------------------------------------ transfers

static lx_status ensure_xfer(lx_sim* s) {
  if (s->xfer) return LX_OK;
  size_t m = 0;
  for (int c = 0; c < 7; c++) m = std::max(m, ext_n(s, c));
  CK(cudaMallocAsync(&s->xfer, m * sizeof(double) + 64, s->own));
  CK(cudaStreamSynchronize(s->own));
  s->xfer_cap = m;
  return LX_OK;
}

// The buffer holding the current state (buffer t & 1 in ping-pong mode, else 0), and the other.
static bool odd_state(const lx_sim* s) { return s->pp && (s->t & 1); }

void* lx::comp_ptr(lx_sim* s, int comp, bool other) {
  const bool b1 = odd_state(s) != other;
  if (comp >= LX_EX && comp <= LX_EZ) return b1 ? s->E1[comp] : s->E[comp];
  if (comp >= LX_HX && comp <= LX_HZ) return b1 ? s->H1[comp - 3] : s->H[comp - 3];
  if (comp == LX_ETOTAL) return other ? nullptr : s->etotal;
  return nullptr;
}

using lx::comp_ptr;

static void* psi_ptr(lx_sim* s, bool h, int a, int q, bool other = false) {
  const bool b1 = odd_state(s) != other;
  if (h) return b1 ? s->psiH1[a][q] : s->psiH[a][q];
  return b1 ? s->psiE1[a][q] : s->psiE[a][q];
}

// Switches a single-sweep handle between ping-pong mode (stepped alone: the state after t
// steps in buffer t & 1) and in-place mode (batched: the state in buffer 0).  At odd t the
// state moves between the buffers, one device copy of the fields and psi.
static lx_status set_pp(lx_sim* s, bool on) {
  if (!s->sweep || (s->pp != 0) == on) return LX_OK;
  if (s->t & 1) {
    const size_t fb = s->ncell * s->tsize;
    auto move = [&](void* b0, void* b1, size_t bytes) -> lx_status {
      if (!b0 || !bytes) return LX_OK;
      CK(cudaMemcpyAsync(on ? b1 : b0, on ? b0 : b1, bytes, cudaMemcpyDeviceToDevice, s->stream));
      return LX_OK;
    };
    lx_status st;
    for (int c = 0; c < 3; c++) {
      if ((st = move(s->E[c], s->E1[c], fb))) return st;
      if ((st = move(s->H[c], s->H1[c], fb))) return st;
      for (int q = 0; q < 2; q++) {
        if ((st = move(s->psiH[c][q], s->psiH1[c][q], s->psiH_n[c][q] * s->csize))) return st;
        if ((st = move(s->psiE[c][q], s->psiE1[c][q], s->psiE_n[c][q] * s->csize))) return st;
      }
    }
  }
  s->pp = on;
  return LX_OK;
}

static lx_status gather(lx_sim* s, int comp, double* dst) {
  void* src = comp_ptr(s, comp);
  const double mul = (comp >= LX_HX && comp <= LX_HZ) ? 1.0 / s->hscale : 1.0;
  if (comp == LX_ETOTAL) {
    // |E|^2 is kept in compute precision
    if (s->csize == 8) CK(lx::launch_gather<double>((const double*)src, dst, s->ext[comp], s->Ny, s->Nzp, mul, s->stream));
    else CK(lx::launch_gather<float>((const float*)src, dst, s->ext[comp], s->Ny, s->Nzp, mul, s->stream));
  } else if (s->prec == LX_PREC_FP64) {
    CK(lx::launch_gather<double>((const double*)src, dst, s->ext[comp], s->Ny, s->Nzp, mul, s->stream));
  } else if (s->prec == LX_PREC_FP32) {
    CK(lx::launch_gather<float>((const float*)src, dst, s->ext[comp], s->Ny, s->Nzp, mul, s->stream));
  } else {
    CK(lx::launch_gather<__half>((const __half*)src, dst, s->ext[comp], s->Ny, s->Nzp, mul, s->stream));
  }
  s->n_kernels++;
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_field_shape(const lx_sim* s, int comp, int shape[3]) {
  if (!s || !shape || comp < 0 || comp > LX_ETOTAL) return fail((lx_sim*)s, LX_ERR_INVALID, "bad component");
  for (int a = 0; a < 3; a++) shape[a] = s->ext[comp][a];
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_read_field(lx_sim* s, int comp, double* host, size_t n) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  if (comp < 0 || comp > LX_ETOTAL) return fail(s, LX_ERR_INVALID, "bad component");
  const size_t m = ext_n(s, comp);
  if (n != m) return fail(s, LX_ERR_INVALID, "buffer size does not match the component's staggered extent");
  if (m == 0) return LX_OK;
  if (comp == LX_ETOTAL && !s->etotal) return fail(s, LX_ERR_STATE, "|E|^2 is only kept when a snapshot asks for it");
  lx_status st = ensure_xfer(s);
  if (st) return st;
  if ((st = gather(s, comp, s->xfer))) return st;
  CK(cudaMemcpyAsync(host, s->xfer, m * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->n_d2h += m * sizeof(double);
  return LX_OK;
}

static lx_status scatter(lx_sim* s, int comp, void* dst, bool compute_prec, int mode, double a, double scale) {
  const int* ext = s->ext[comp];
  if (compute_prec || s->prec == LX_PREC_FP64 || s->prec == LX_PREC_FP32) {
    bool dbl = compute_prec ? s->csize == 8 : s->prec == LX_PREC_FP64;
    if (dbl) CK(lx::launch_scatter<double>(s->xfer, (double*)dst, ext, s->Ny, s->Nzp, mode, a, s->k.dt, s->k.epsilon0, scale, s->stream));
    else CK(lx::launch_scatter<float>(s->xfer, (float*)dst, ext, s->Ny, s->Nzp, mode, a, s->k.dt, s->k.epsilon0, scale, s->stream));
  } else {
    CK(lx::launch_scatter<__half>(s->xfer, (__half*)dst, ext, s->Ny, s->Nzp, mode, a, s->k.dt, s->k.epsilon0, scale, s->stream));
  }
  s->n_kernels++;
  return LX_OK;
}

static lx_status upload(lx_sim* s, const double* host, size_t m) {
  lx_status st = ensure_xfer(s);
  if (st) return st;
  CK(cudaMemcpyAsync(s->xfer, host, m * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  s->n_h2d += m * sizeof(double);
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_write_field(lx_sim* s, int comp, const double* host, size_t n) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  if (comp < 0 || comp > LX_HZ) return fail(s, LX_ERR_INVALID, "bad component");
  const size_t m = ext_n(s, comp);
  if (n != m) return fail(s, LX_ERR_INVALID, "buffer size does not match the component's staggered extent");
  if (m == 0) return LX_OK;
  lx_status st = upload(s, host, m);
  if (st) return st;
  const bool hcomp = comp >= LX_HX && comp <= LX_HZ;
  if ((st = scatter(s, comp, comp_ptr(s, comp), false, hcomp && s->hscale != 1.0 ? 1 : 0, s->hscale, 0.0))) return st;
  // single-sweep handles: the other buffer too, so that the values stay the state whichever
  // buffer the step count selects (a checkpoint load sets the step count afterwards)
  if (s->sweep && (st = scatter(s, comp, comp_ptr(s, comp, true), false, hcomp && s->hscale != 1.0 ? 1 : 0, s->hscale, 0.0)))
    return st;
  CK(cudaStreamSynchronize(s->stream));
  return LX_OK;
}

// ------------------------------------------------------------------ checkpoints

namespace {
const char* kCompName[6] = {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz"};

// lx_params with the members a resumed run may change (step count, threads, decomposition,
// monitor cadence) cleared, for the compatibility check.
std::vector<double> params_key(const lx_params& p0) {
  lx_params p = p0;
  p.num_timesteps = 0;
  p.n_threads = 0;
  p.npX = p.npY = 0;
  p.monitor_every = 0;
  std::vector<double> v((sizeof(lx_params) + 7) / 8, 0.0);
  std::memcpy(v.data(), &p, sizeof p);
  return v;
}

// raw device array of compute-precision values <-> doubles on the host
lx_status raw_to_host(lx_sim* s, const void* dev, size_t n, std::vector<double>& out) {
  out.resize(n);
  if (!n) return LX_OK;
  if (s->csize == 8) {
    CK(cudaMemcpyAsync(out.data(), dev, n * 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
  } else {
    std::vector<float> f(n);
    CK(cudaMemcpyAsync(f.data(), dev, n * 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    for (size_t q = 0; q < n; q++) out[q] = f[q];
  }
  s->n_d2h += n * s->csize;
  return LX_OK;
}

lx_status raw_to_device(lx_sim* s, void* dev, const std::vector<double>& in) {
  const size_t n = in.size();
  if (!n) return LX_OK;
  if (s->csize == 8) {
    CK(cudaMemcpyAsync(dev, in.data(), n * 8, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
  } else {
    std::vector<float> f(n);
    for (size_t q = 0; q < n; q++) f[q] = (float)in[q];
    CK(cudaMemcpyAsync(dev, f.data(), n * 4, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
  }
  s->n_h2d += n * s->csize;
  return LX_OK;
}
}  // namespace

extern "C" LX_API lx_status lx_sim_save(lx_sim* s, const char* path) {
  if (!s || !path) return fail(s, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(s->device);
  lx_status st = lx_sim_sync(s);
  if (st) return st;
  if ((st = ensure_xfer(s))) return st;
  lx::Hdf5Writer w;
  std::string m = w.open(path, s->ext[LX_EY]);
  if (!m.empty()) return fail(s, LX_ERR_IO, m);
  std::vector<double> host;
  auto put = [&](const std::string& name, const std::vector<double>& v, const int* ext) -> lx_status {
    const std::string e = w.write_named(name, v.data(), ext);
    return e.empty() ? LX_OK : fail(s, LX_ERR_IO, e);
  };
  // fields in the snapshot layout (physical values, staggered extents, C order)
  for (int c = 0; c < 6; c++) {
    const size_t n = ext_n(s, c);
    if (!n) continue;
    host.resize(n);
    if ((st = lx_sim_read_field(s, c, host.data(), n))) return st;
    if ((st = put(kCompName[c], host, s->ext[c]))) return st;
  }
  // per-cell coefficients as stored (Cb in the engine's units)
  for (int c = 0; c < 3; c++) {
    const size_t n = ext_n(s, c);
    if (!n) continue;
    if (s->csize == 8) CK(lx::launch_gather<double>((const double*)s->Cbs[c], s->xfer, s->ext[c], s->Ny, s->Nzp, 1.0, s->stream));
    else CK(lx::launch_gather<float>((const float*)s->Cbs[c], s->xfer, s->ext[c], s->Ny, s->Nzp, 1.0, s->stream));
    host.resize(n);
    CK(cudaMemcpyAsync(host.data(), s->xfer, n * 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if ((st = put(std::string("Cb_") + kCompName[c], host, s->ext[c]))) return st;
  }
  // CPML psi on the slabs and DFT accumulators, raw
  for (int a = 0; a < 3; a++)
    for (int q = 0; q < 2; q++) {
      for (int h = 0; h < 2; h++) {
        const size_t n = h ? s->psiH_n[a][q] : s->psiE_n[a][q];
        if (!n) continue;
        if ((st = raw_to_host(s, psi_ptr(s, h, a, q), n, host))) return st;
        const int ext[3] = {1, 1, (int)n};
        if ((st = put(std::string(h ? "psiH_" : "psiE_") + char('0' + a) + char('0' + q), host, ext))) return st;
      }
    }
  for (size_t d = 0; d < s->dfts.size(); d++) {
    const lx::DftPlane& D = s->dfts[d];
    host.resize(D.n_acc);
    CK(cudaMemcpyAsync(host.data(), D.d_acc, D.n_acc * 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    const int ext[3] = {1, 1, (int)D.n_acc};
    if ((st = put("dft_" + std::to_string(d), host, ext))) return st;
  }
  const std::vector<double> state = {(double)s->t, s->last_max, (double)s->prec, (double)s->dfts.size()};
  const int sext[3] = {1, 1, (int)state.size()};
  if ((st = put("engine_state", state, sext))) return st;
  const std::vector<double> key = params_key(s->p);
  const int kext[3] = {1, 1, (int)key.size()};
  if ((st = put("engine_params", key, kext))) return st;
  m = w.close();
  if (!m.empty()) return fail(s, LX_ERR_IO, m);
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_load(lx_sim* s, const char* path) {
  if (!s || !path) return fail(s, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(s->device);
  lx_status st = lx_sim_sync(s);
  if (st) return st;
  std::vector<double> v;
  int shp[3];
  auto get = [&](const std::string& name, size_t n) -> lx_status {
    const std::string e = lx::hdf5_read(path, name.c_str(), v, shp);
    if (!e.empty()) return fail(s, LX_ERR_IO, name + ": " + e);
    if (v.size() != n) return fail(s, LX_ERR_INVALID, name + ": size does not match this handle");
    return LX_OK;
  };
  const std::vector<double> key = params_key(s->p);
  if ((st = get("engine_params", key.size()))) return st;
  if (std::memcmp(v.data(), key.data(), key.size() * 8) != 0)
    return fail(s, LX_ERR_INVALID, "checkpoint was written by a handle with other parameters");
  if ((st = get("engine_state", 4))) return st;
  const std::vector<double> state = v;
  if ((int)state[2] != s->prec) return fail(s, LX_ERR_INVALID, "checkpoint precision differs");
  if ((size_t)state[3] != s->dfts.size()) return fail(s, LX_ERR_INVALID, "checkpoint has another number of DFT planes");
  for (size_t d = 0; d < s->dfts.size(); d++)
    if ((st = get("dft_" + std::to_string(d), s->dfts[d].n_acc))) return st;
  for (int c = 0; c < 6; c++) {
    const size_t n = ext_n(s, c);
    if (!n) continue;
    if ((st = get(kCompName[c], n))) return st;
    if ((st = lx_sim_write_field(s, c, v.data(), n))) return st;
  }
  for (int c = 0; c < 3; c++) {
    const size_t n = ext_n(s, c);
    if (!n) continue;
    if ((st = get(std::string("Cb_") + kCompName[c], n))) return st;
    if ((st = upload(s, v.data(), n))) return st;
    if ((st = scatter(s, c, s->Cbs[c], true, 0, 1.0, 0.0))) return st;
  }
  for (int a = 0; a < 3; a++)
    for (int q = 0; q < 2; q++)
      for (int h = 0; h < 2; h++) {
        const size_t n = h ? s->psiH_n[a][q] : s->psiE_n[a][q];
        if (!n) continue;
        if ((st = get(std::string(h ? "psiH_" : "psiE_") + char('0' + a) + char('0' + q), n))) return st;
        if ((st = raw_to_device(s, psi_ptr(s, h, a, q), v))) return st;
        if (s->sweep && (st = raw_to_device(s, psi_ptr(s, h, a, q, true), v))) return st;
      }
  for (size_t d = 0; d < s->dfts.size(); d++) {
    if ((st = get("dft_" + std::to_string(d), s->dfts[d].n_acc))) return st;
    CK(cudaMemcpyAsync(s->dfts[d].d_acc, v.data(), v.size() * 8, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
  }
  s->t = (int)state[0];
  s->last_max = state[1];
  s->probe_rows = 0;
  return LX_OK;
}

static lx_status check_cb_comp(lx_sim* s, int comp, size_t n) {
  if (comp < LX_EX || comp > LX_EZ || !s->Cbs[comp]) return fail(s, LX_ERR_INVALID, "Cb exists for Ex, Ey, Ez (planar: Ey only)");
  if (n != ext_n(s, comp)) return fail(s, LX_ERR_INVALID, "buffer size does not match the component's staggered extent");
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_set_cb(lx_sim* s, int comp, const double* cb, size_t n) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  lx_status st = check_cb_comp(s, comp, n);
  if (st) return st;
  if ((st = upload(s, cb, n))) return st;
  if ((st = scatter(s, comp, s->Cbs[comp], true, 1, s->cbs_scale, 0.0))) return st;
  CK(cudaStreamSynchronize(s->stream));
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_set_material(lx_sim* s, int comp, const double* F, size_t n, double scale) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  lx_status st = check_cb_comp(s, comp, n);
  if (st) return st;
  if ((st = upload(s, F, n))) return st;
  if ((st = scatter(s, comp, s->Cbs[comp], true, 2, s->cbs_scale, scale))) return st;
  CK(cudaStreamSynchronize(s->stream));
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_set_eps_box(lx_sim* s, const int lo[3], const int hi[3], double eps_r) {
  if (!s || !lo || !hi) return fail(s, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  if (!(eps_r > 0)) return fail(s, LX_ERR_INVALID, "eps_r must be > 0");
  const double val = s->k.dt / (s->k.epsilon0 * eps_r) * s->cbs_scale;
  for (int c = 0; c < 3; c++) {
    if (!s->Cbs[c]) continue;
    if (s->csize == 8) CK(lx::launch_eps_box<double>((double*)s->Cbs[c], s->ext[c], s->Ny, s->Nzp, lo, hi, val, s->stream));
    else CK(lx::launch_eps_box<float>((float*)s->Cbs[c], s->ext[c], s->Ny, s->Nzp, lo, hi, val, s->stream));
    s->n_kernels++;
  }
  CK(cudaStreamSynchronize(s->stream));
  return LX_OK;
}

// ------------------------------------------------------------------ probes

extern "C" LX_API lx_status lx_sim_set_probes(lx_sim* s, const int* ijk, int nprobes, int cap) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  lx::DeviceGuard dg_(s->device);
  if (s->batch)
    return fail(s, LX_ERR_STATE, "remove the handle from its batch first: batched members keep no snapshot outputs or probes");
  if (nprobes < 0 || nprobes > lx::kMaxProbes || cap < 0) return fail(s, LX_ERR_INVALID, "0..64 probes, capacity >= 0");
  CK(cudaStreamSynchronize(s->stream));
  dfree(s->d_probe_ijk, s->own);
  dfree(s->d_probe, s->own);
  s->d_probe_ijk = nullptr;
  s->d_probe = nullptr;
  s->nprobes = 0;
  s->probe_cap = 0;
  s->probe_rows = 0;
  if (nprobes == 0 || cap == 0) return LX_OK;
  CK(cudaMallocAsync(&s->d_probe_ijk, sizeof(int) * 3 * nprobes, s->own));
  CK(cudaMemcpyAsync(s->d_probe_ijk, ijk, sizeof(int) * 3 * nprobes, cudaMemcpyHostToDevice, s->own));
  CK(cudaMallocAsync(&s->d_probe, sizeof(double) * 6 * (size_t)nprobes * cap, s->own));
  CK(cudaMemsetAsync(s->d_probe, 0, sizeof(double) * 6 * (size_t)nprobes * cap, s->own));
  CK(cudaStreamSynchronize(s->own));
  s->nprobes = nprobes;
  s->probe_cap = cap;
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_read_probes(lx_sim* s, double* host, size_t n, int* rows) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  const size_t m = (size_t)s->probe_rows * s->nprobes * 6;
  if (rows) *rows = s->probe_rows;
  if (n < m) return fail(s, LX_ERR_INVALID, "probe buffer too small");
  if (m == 0) return LX_OK;
  CK(cudaMemcpyAsync(host, s->d_probe, m * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->n_d2h += m * sizeof(double);
  return LX_OK;
}

// ------------------------------------------------------------------ DFT plane monitors

extern "C" LX_API lx_status lx_sim_add_dft_plane(lx_sim* s, int axis, int index, int nfreq, const double* omega,
                                                 int every, int* id) {
  if (!s || !omega || !id) return fail(s, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  if (axis < 0 || axis > 2 || (s->planar && axis == 1)) return fail(s, LX_ERR_INVALID, "axis must be 0, 1 or 2 (planar: 0 or 2)");
  const int N[3] = {s->Nx, s->Ny, s->Nz};
  if (index < 0 || index >= N[axis]) return fail(s, LX_ERR_INVALID, "plane index outside the grid");
  if (nfreq < 1 || nfreq > lx::kMaxDftFreq || every < 1) return fail(s, LX_ERR_INVALID, "1..256 frequencies, every >= 1");
  static const int kComps[3][4] = {{LX_EY, LX_EZ, LX_HY, LX_HZ}, {LX_EZ, LX_EX, LX_HZ, LX_HX}, {LX_EX, LX_EY, LX_HX, LX_HY}};
  lx::DftPlane d;
  d.axis = axis;
  d.index = index;
  d.nfreq = nfreq;
  d.every = every;
  d.na = axis == 0 ? s->Ny : s->Nx;
  d.nb = axis == 2 ? s->Ny : s->Nz;
  for (int q = 0; q < 4; q++) d.comps[q] = kComps[axis][q];
  d.omega.assign(omega, omega + nfreq);
  d.n_acc = (size_t)nfreq * 4 * d.na * d.nb * 2;
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaMallocAsync(&d.d_omega, nfreq * sizeof(double), s->own));
  CK(cudaMemcpyAsync(d.d_omega, omega, nfreq * sizeof(double), cudaMemcpyHostToDevice, s->own));
  CK(cudaMallocAsync(&d.d_acc, d.n_acc * sizeof(double), s->own));
  CK(cudaMemsetAsync(d.d_acc, 0, d.n_acc * sizeof(double), s->own));
  CK(cudaMallocAsync(&d.d_phase, 4 * lx::kMaxDftFreq * sizeof(double), s->own));
  CK(cudaStreamSynchronize(s->own));
  s->n_h2d += nfreq * sizeof(double);
  s->dfts.push_back(d);
  *id = (int)s->dfts.size() - 1;
  if (s->batch) batch_member_changed(s->batch);  // the batch samples the new plane from its next step
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_read_dft(lx_sim* s, int id, double* host, size_t n) {
  if (!s || !host) return fail(s, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  if (id < 0 || id >= (int)s->dfts.size()) return fail(s, LX_ERR_INVALID, "no such DFT plane");
  const lx::DftPlane& d = s->dfts[id];
  if (n != d.n_acc) return fail(s, LX_ERR_INVALID, "buffer size must be nfreq*4*na*nb*2");
  CK(cudaMemcpyAsync(host, d.d_acc, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->n_d2h += n * sizeof(double);
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_dft_flux(lx_sim* s, int id, double* flux, int nfreq) {
  if (!s || !flux) return fail(s, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  if (id < 0 || id >= (int)s->dfts.size()) return fail(s, LX_ERR_INVALID, "no such DFT plane");
  lx::DftPlane& d = s->dfts[id];
  if (nfreq != d.nfreq) return fail(s, LX_ERR_INVALID, "nfreq does not match the plane");
  const double sp[3] = {s->p.dx, s->p.dy, s->p.dz};
  double dA;
  if (s->planar) dA = d.axis == 0 ? sp[2] : sp[0];
  else dA = d.axis == 0 ? sp[1] * sp[2] : (d.axis == 1 ? sp[2] * sp[0] : sp[0] * sp[1]);
  const long long nc = (long long)d.na * d.nb;
  if (!d.d_flux) {
    const long long nchunk = (nc + 1023) / 1024;
    CK(cudaMallocAsync(&d.d_flux, sizeof(double) * (d.nfreq + d.nfreq * nchunk), s->own));
    CK(cudaStreamSynchronize(s->own));
  }
  // deterministic on-device reduction: per-chunk partial sums, then chunks in order
  CK(lx::launch_dft_flux(d.d_acc, d.nfreq, nc, d.d_flux + d.nfreq, dA, d.d_flux, s->stream));
  CK(cudaMemcpyAsync(flux, d.d_flux, sizeof(double) * d.nfreq, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->n_kernels += 2;
  s->n_d2h += sizeof(double) * d.nfreq;
  return LX_OK;
}

// ------------------------------------------------------------------ snapshots

static void writer_main(lx_sim* s) {
  cudaSetDevice(s->device);
  for (;;) {
    lx::SnapJob job;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv.wait(lk, [&] { return s->stop || !s->jobs.empty(); });
      if (s->jobs.empty() && s->stop) return;
      job = s->jobs.front();
      s->jobs.pop_front();
    }
    lx::SnapSlot& sl = s->slots[job.slot];
    cudaError_t e = cudaEventSynchronize(sl.ev_d2h);
    std::string err;
    if (e != cudaSuccess) err = std::string("snapshot copy: ") + cudaGetErrorString(e);
    if (err.empty()) {
      for (auto& o : s->outputs) {
        if (o.every <= 0 || job.t < o.first || job.t % o.every != 0) continue;
        for (int c = 0; c < 7; c++) {
          if (!(o.mask & (1u << c)) || !(job.mask & (1u << c))) continue;
          const double* data = sl.host + job.off[c];
          if (o.fn) o.fn(o.user, job.t, c, data, s->ext[c]);
          if (o.h5) {
            std::string m = o.h5->write(job.t, data);
            if (!m.empty() && err.empty()) err = m;
          }
        }
      }
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      sl.busy = false;
      s->pending--;
      if (!err.empty() && s->writer_err.empty()) s->writer_err = err;
    }
    s->cv.notify_all();
  }
}

static void stop_writer(lx_sim* s) {
  if (!s->writer_on) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  s->writer.join();
  s->writer_on = false;
  s->stop = false;
}

static lx_status add_output(lx_sim* s, const lx::Output& o) {
  lx_status st = lx_sim_sync(s);
  if (st) return st;
  s->outputs.push_back(o);
  // size the staging slots for the union of all outputs' components
  unsigned all = 0;
  for (auto& q : s->outputs) all |= q.mask;
  size_t need = 0;
  for (int c = 0; c < 7; c++)
    if (all & (1u << c)) need += ext_n(s, c);
  for (auto& sl : s->slots) {
    if (sl.cap >= need) continue;
    dfree(sl.dev, s->own);
    if (sl.host) cudaFreeHost(sl.host);
    sl.dev = nullptr;
    sl.host = nullptr;
    CK(cudaMallocAsync(&sl.dev, need * sizeof(double), s->own));
    CK(cudaHostAlloc(&sl.host, need * sizeof(double), cudaHostAllocDefault));
    if (!sl.ev_d2h) CK(cudaEventCreateWithFlags(&sl.ev_d2h, cudaEventDisableTiming));
    sl.cap = need;
  }
  if ((all & (1u << LX_ETOTAL)) && !s->etotal) {
    if (s->planar) return fail(s, LX_ERR_INVALID, "|E|^2 snapshots exist for 3-D grids only");
    CK(cudaMallocAsync(&s->etotal, s->ncell * s->csize, s->own));
    CK(cudaMemsetAsync(s->etotal, 0, s->ncell * s->csize, s->own));
  }
  CK(cudaStreamSynchronize(s->own));
  if (!s->writer_on) {
    s->writer = std::thread(writer_main, s);
    s->writer_on = true;
  }
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_set_snapshots(lx_sim* s, int every, unsigned mask, lx_snapshot_fn fn, void* user) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  lx::DeviceGuard dg_(s->device);
  if (s->batch)
    return fail(s, LX_ERR_STATE, "remove the handle from its batch first: batched members keep no snapshot outputs or probes");
  if (every < 0 || (every > 0 && !fn)) return fail(s, LX_ERR_INVALID, "every >= 0 and a callback are required");
  for (int c = 0; c < 7; c++)
    if ((mask & (1u << c)) && ext_n(s, c) == 0) return fail(s, LX_ERR_INVALID, "component absent on this grid");
  lx_status st = lx_sim_sync(s);
  if (st) return st;
  for (auto it = s->outputs.begin(); it != s->outputs.end();) {
    if (it->fn) it = s->outputs.erase(it);
    else ++it;
  }
  if (every == 0) return LX_OK;
  lx::Output o;
  o.every = every;
  o.mask = mask & 0x7f;
  o.fn = fn;
  o.user = user;
  return add_output(s, o);
}

extern "C" LX_API lx_status lx_sim_set_hdf5_output(lx_sim* s, int every, int first, int comp, const char* path) {
  if (!s || !path) return fail(s, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(s->device);
  if (s->batch)
    return fail(s, LX_ERR_STATE, "remove the handle from its batch first: batched members keep no snapshot outputs or probes");
  if (every <= 0 || first < 0 || comp < 0 || comp > LX_ETOTAL || ext_n(s, comp) == 0)
    return fail(s, LX_ERR_INVALID, "bad cadence or component");
  lx::Output o;
  o.every = every;
  o.first = first;
  o.mask = 1u << comp;
  o.h5 = new lx::Hdf5Writer();
  std::string m = o.h5->open(path, s->ext[comp]);
  if (!m.empty()) {
    delete o.h5;
    return fail(s, LX_ERR_IO, m);
  }
  o.h5_comp = comp;
  return add_output(s, o);
}

// Gathers the due components into a free staging slot and queues the copy to pinned memory.
static lx_status snapshot(lx_sim* s, int t, unsigned mask) {
  int slot = -1;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv.wait(lk, [&] { return !s->slots[0].busy || !s->slots[1].busy; });
    slot = !s->slots[0].busy ? 0 : 1;
    s->slots[slot].busy = true;
    s->pending++;
  }
  lx::SnapSlot& sl = s->slots[slot];
  lx::SnapJob job;
  job.slot = slot;
  job.t = t;
  job.mask = mask;
  size_t off = 0;
  for (int c = 0; c < 7; c++) {
    job.off[c] = off;
    if (!(mask & (1u << c))) continue;
    lx_status st = gather(s, c, sl.dev + off);
    if (st) return st;
    off += ext_n(s, c);
  }
  // the side stream copies once the gathers on the compute stream are done
  cudaEvent_t ev;
  CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  CK(cudaEventRecord(ev, s->stream));
  CK(cudaStreamWaitEvent(s->side, ev, 0));
  CK(cudaEventDestroy(ev));
  CK(cudaMemcpyAsync(sl.host, sl.dev, off * sizeof(double), cudaMemcpyDeviceToHost, s->side));
  CK(cudaEventRecord(sl.ev_d2h, s->side));
  // The compute stream does not wait for this copy: the slot is reused only after the
  // writer has synchronised on ev_d2h and cleared `busy`, which the wait above checks.
  s->n_d2h += off * sizeof(double);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->jobs.push_back(job);
  }
  s->cv.notify_all();
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_sync(lx_sim* s) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaStreamSynchronize(s->side));
  std::unique_lock<std::mutex> lk(s->mu);
  s->cv.wait(lk, [&] { return s->pending == 0; });
  if (!s->writer_err.empty()) {
    std::string m = s->writer_err;
    s->writer_err.clear();
    lk.unlock();
    return fail(s, LX_ERR_IO, m);
  }
  return LX_OK;
}

// ------------------------------------------------------------------ stepping

template <class T, class C>
static lx::StepParams<T, C> step_params(lx_sim* s) {
  lx::StepParams<T, C> p;
  std::memset(&p, 0, sizeof p);
  p.Nx = s->Nx; p.Ny = s->Ny; p.Nz = s->Nz; p.Nzp = s->Nzp;
  p.sj = s->Nzp;
  p.si = (long long)s->Ny * s->Nzp;
  for (int c = 0; c < 3; c++) {
    p.E[c] = (T*)s->E[c];
    p.H[c] = (T*)s->H[c];
    p.E1[c] = (T*)s->E1[c];
    p.H1[c] = (T*)s->H1[c];
    p.Cbs[c] = (const C*)s->Cbs[c];
  }
  const double Db = s->k.dt / s->k.mew0;  // Db arrays = dt/mew0 (two_dim_pml.cc:117, three_dim_pml.cc:130-132)
  p.Dbs = (C)((s->uniform ? Db * (1.0 / s->p.dx) : Db) * s->hscale);
  p.rd[0] = (C)(1.0 / s->p.dx);
  p.rd[1] = (C)(s->planar ? 0.0 : 1.0 / s->p.dy);
  p.rd[2] = (C)(1.0 / s->p.dz);
  p.pml = s->pml;
  for (int a = 0; a < 3; a++) {
    p.slab[a] = s->slab[a];
    if (!s->pml) { p.slab[a].lo = 0; p.slab[a].hi0 = 1 << 30; p.slab[a].n = 0; }
    p.bE[a] = (const C*)s->prof[a][0];
    p.cE[a] = (const C*)s->prof[a][1];
    p.rkE[a] = (const C*)s->prof[a][2];
    p.bH[a] = (const C*)s->prof[a][3];
    p.cH[a] = (const C*)s->prof[a][4];
    p.rkH[a] = (const C*)s->prof[a][5];
  }
  if (s->planar) { p.slab[1].lo = 0; p.slab[1].hi0 = 1 << 30; p.slab[1].n = 0; }
  for (int c = 0; c < 3; c++)
    for (int q = 0; q < 2; q++) {
      p.psiH[c][q] = (C*)s->psiH[c][q];
      p.psiE[c][q] = (C*)s->psiE[c][q];
      p.psiH1[c][q] = (C*)s->psiH1[c][q];
      p.psiE1[c][q] = (C*)s->psiE1[c][q];
      p.setsH[c][q] = s->setsH[c][q];
      p.setsE[c][q] = s->setsE[c][q];
    }
  p.tfsf = s->tfsf && s->tab_total > 0;
  p.tab = (const C*)s->tab;
  // plane lists of the block skip test: per axis, the planes any active set of that half step
  // sits on (two per axis: the low and high face)
  for (int a = 0; a < 3; a++)
    for (int q = 0; q < 2; q++) p.planesH[a][q] = p.planesE[a][q] = -2;
  for (int c = 0; c < 3; c++)
    for (int q = 0; q < 2; q++) {
      const lx::PatchSet& h = s->setsH[c][q];
      const lx::PatchSet& e = s->setsE[c][q];
      if (h.active) { p.planesH[h.axis][0] = h.plane[0]; p.planesH[h.axis][1] = h.plane[1]; }
      if (e.active) { p.planesE[e.axis][0] = e.plane[0]; p.planesE[e.axis][1] = e.plane[1]; }
    }
  return p;
}

// The parameter block of a single-sweep step that reads buffer 1 and writes buffer 0.
template <class T, class C>
static void swap_buffers(lx::StepParams<T, C>& p) {
  for (int c = 0; c < 3; c++) {
    std::swap(p.E[c], p.E1[c]);
    std::swap(p.H[c], p.H1[c]);
    for (int q = 0; q < 2; q++) {
      std::swap(p.psiH[c][q], p.psiH1[c][q]);
      std::swap(p.psiE[c][q], p.psiE1[c][q]);
    }
  }
}

// Optional per-launch timing of run_steps (lx_sim_time_kernels).
struct KernelTimer {
  cudaEvent_t ev[2];
  double sum[4] = {0, 0, 0, 0};
  int cnt[4] = {0, 0, 0, 0};
};

static lx::PrologueParams make_prologue(lx_sim* s) {
  lx::PrologueParams pp;
  std::memset(&pp, 0, sizeof pp);
  pp.nsets = 12;
  for (int c = 0; c < 3; c++)
    for (int q = 0; q < 2; q++) {
      pp.sets[c * 2 + q] = s->setsH[c][q];
      pp.sets[6 + c * 2 + q] = s->setsE[c][q];
    }
  pp.tab = s->tab;
  pp.tab_total = (s->tfsf && s->tab_total > 0) ? s->tab_total : 0;
  pp.planar = s->planar;
  pp.dx = s->k.dx; pp.dy = s->k.dy; pp.dz = s->k.dz;
  pp.kx = s->k.k[0]; pp.ky = s->k.k[1]; pp.kz = s->k.k[2];
  pp.init = s->k.init; pp.c = s->k.c; pp.dt = s->k.dt; pp.mu0 = s->k.mew0; pp.pw_sigma = s->k.sigma;
  pp.inv_sigma = 1.0 / s->k.sigma;
  pp.scale_units = s->uniform ? 0.0 : 1.0;
  pp.src_kind = s->src_kind;
  pp.src_idx = s->src_idx;
  pp.src_field = s->planar ? s->E[1] : s->E[2];
  pp.src_field1 = s->pp ? (s->planar ? s->E1[1] : s->E1[2]) : nullptr;  // ping-pong mode: used at odd t
  pp.src_amp_i = (int)s->p.amp_source;  // maxwell.cc:142-143 store them in int members
  pp.src_omega_i = (int)s->p.omega_source;
  pp.src_amp = s->p.amp_source;
  pp.src_omega = s->p.omega_source;
  pp.src_t0 = s->p.src_t0;
  pp.src_tw = s->p.src_tw;
  pp.prec = s->prec;
  return pp;
}

template <class T, class C>
static lx_status run_steps(lx_sim* s, int nsteps, KernelTimer* kt = nullptr) {
  if (!s->batch) {  // stepped alone: single-sweep handles take the ping-pong kernel
    const lx_status st = set_pp(s, true);
    if (st) return st;
  }
  lx::StepParams<T, C> sp = step_params<T, C>(s);
  sp.fault = s->d_fault;
  lx::PrologueParams pp = make_prologue(s);
  T* pf[6];  // the components after the current step (buffer (t+1) & 1 in ping-pong mode)
  auto post_step = [&](int t) {
    const bool b1 = s->pp && ((t + 1) & 1);
    for (int c = 0; c < 3; c++) {
      pf[c] = (T*)(b1 ? s->E1[c] : s->E[c]);
      pf[3 + c] = (T*)(b1 ? s->H1[c] : s->H[c]);
    }
  };
  lx::ProbeParams prb;
  std::memset(&prb, 0, sizeof prb);
  prb.nprobes = s->nprobes;
  prb.Ny = s->Ny;
  prb.Nzp = s->Nzp;
  for (int c = 0; c < 6; c++)
    for (int a = 0; a < 3; a++) prb.ext[c][a] = s->ext[c][a];
  prb.ijk = s->d_probe_ijk;
  prb.hmul = 1.0 / s->hscale;

  unsigned long long* last_slot = s->d_max;
  for (int q = 0; q < nsteps; q++) {
    const int t = s->t;
    bool mon = (q == nsteps - 1) || (s->p.monitor_every > 0 && (t + 1) % s->p.monitor_every == 0);
    unsigned snap = 0;
    for (auto& o : s->outputs)
      if (o.every > 0 && t >= o.first && t % o.every == 0) snap |= o.mask;
    auto tic = [&]() -> lx_status {
      if (kt) CK(cudaEventRecord(kt->ev[0], s->stream));
      return LX_OK;
    };
    auto toc = [&](int which) -> lx_status {
      if (!kt) return LX_OK;
      CK(cudaEventRecord(kt->ev[1], s->stream));
      CK(cudaEventSynchronize(kt->ev[1]));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, kt->ev[0], kt->ev[1]));
      kt->sum[which] += ms;
      kt->cnt[which]++;
      return LX_OK;
    };
    lx_status st;
    unsigned long long* slot = s->d_max;
    if (mon && s->d_series && (int)s->series_t.size() < s->series_cap) {
      slot = s->d_series + s->series_t.size();
      s->series_t.push_back(t);
    }
    if (mon) last_slot = slot;
    if (pp.tab_total > 0 || s->src_kind >= 0 || mon) {
      pp.t = t;
      pp.max_slot = mon ? slot : nullptr;
      if ((st = tic())) return st;
      if (s->csize == 8) CK(lx::launch_prologue<double>(pp, s->stream));
      else CK(lx::launch_prologue<float>(pp, s->stream));
      if ((st = toc(0))) return st;
      s->n_kernels++;
    }
    sp.max_slot = mon ? slot : nullptr;
    sp.etotal = (snap & (1u << LX_ETOTAL)) ? (C*)s->etotal : nullptr;
    bool swept = false;
    if constexpr (sizeof(C) == 4) {
      if (s->pp) {  // one launch: H and E of the step, state t & 1 -> (t+1) & 1
        lx::StepParams<T, C> sw = sp;
        if (t & 1) swap_buffers(sw);
        if ((st = tic())) return st;
        if (s->planar) CK(lx::launch_step_sweep2<T, C>(sw, s->uniform, s->stream));
        else CK(lx::launch_step_sweep3<T, C>(sw, s->uniform, s->stream));
        if ((st = toc(1))) return st;
        s->n_kernels += 1;
        swept = true;
      }
    }
    if (!swept) {
      if ((st = tic())) return st;
      CK(lx::launch_step<T, C>(sp, s->planar, s->uniform, true, s->stream));
      if ((st = toc(1))) return st;
      if ((st = tic())) return st;
      CK(lx::launch_step<T, C>(sp, s->planar, s->uniform, false, s->stream));
      if ((st = toc(2))) return st;
      s->n_kernels += 2;
    }
    post_step(t);
    for (auto& d : s->dfts) {
      if (t % d.every != 0) continue;
      lx::DftParams dp;
      std::memset(&dp, 0, sizeof dp);
      dp.axis = d.axis; dp.index = d.index; dp.na = d.na; dp.nb = d.nb; dp.Ny = s->Ny; dp.Nzp = s->Nzp;
      dp.nfreq = d.nfreq; dp.t = t; dp.dt = s->k.dt; dp.weight = (double)d.every;
      dp.omega = d.d_omega; dp.acc = d.d_acc; dp.phase = d.d_phase; dp.hmul = 1.0 / s->hscale;
      T* f4[4];
      for (int q = 0; q < 4; q++) {
        f4[q] = pf[d.comps[q]];
        for (int a = 0; a < 3; a++) dp.ext[q][a] = s->ext[d.comps[q]][a];
      }
      CK(lx::launch_dft<T>(dp, f4, s->stream));
      s->n_kernels += 2;  // phase factors, accumulation
    }
    if (s->nprobes > 0 && s->probe_rows < s->probe_cap) {
      prb.row = s->probe_rows++;
      if ((st = tic())) return st;
      CK(lx::launch_probes<T>(prb, pf, s->d_probe, s->stream));
      if ((st = toc(3))) return st;
      s->n_kernels++;
    }
    s->t++;
    if (snap) {
      lx_status st = snapshot(s, t, snap);
      if (st) return st;
    }
  }
  if (nsteps > 0) {
    unsigned long long bits = 0;
    unsigned fault = 0;
    CK(cudaMemcpyAsync(&bits, last_slot, sizeof bits, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(&fault, s->d_fault, sizeof fault, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    s->n_d2h += sizeof bits + sizeof fault;
    if (fault) {
      CK(cudaMemsetAsync(s->d_fault, 0, sizeof fault, s->stream));
      return fail(s, LX_ERR_CUDA, "a sweep kernel's bounded wait for a staged plane ran out; the step's fields are not valid");
    }
    double v;
    std::memcpy(&v, &bits, sizeof v);
    s->last_max = v;
    if (!std::isfinite(v)) {
      char b[128];
      std::snprintf(b, sizeof b, "max|E|^2 is not finite after step %d", s->t);
      return fail(s, LX_ERR_BLOWUP, b);
    }
  }
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_step(lx_sim* s, int nsteps) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  if (nsteps < 0) return fail(s, LX_ERR_INVALID, "nsteps must be >= 0");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->writer_err.empty()) {
      std::string m = s->writer_err;
      s->writer_err.clear();
      return fail(s, LX_ERR_IO, m);
    }
  }
  if (s->prec == LX_PREC_FP64) return run_steps<double, double>(s, nsteps);
  if (s->prec == LX_PREC_FP32) return run_steps<float, float>(s, nsteps);
  return run_steps<__half, float>(s, nsteps);
}

extern "C" LX_API lx_status lx_sim_time_kernels(lx_sim* s, int nsteps, double out_ms[4]) {
  if (!s || !out_ms) return fail(s, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  if (nsteps < 1) return fail(s, LX_ERR_INVALID, "nsteps must be >= 1");
  KernelTimer kt;
  CK(cudaEventCreate(&kt.ev[0]));
  CK(cudaEventCreate(&kt.ev[1]));
  lx_status st;
  if (s->prec == LX_PREC_FP64) st = run_steps<double, double>(s, nsteps, &kt);
  else if (s->prec == LX_PREC_FP32) st = run_steps<float, float>(s, nsteps, &kt);
  else st = run_steps<__half, float>(s, nsteps, &kt);
  cudaEventDestroy(kt.ev[0]);
  cudaEventDestroy(kt.ev[1]);
  for (int q = 0; q < 4; q++) out_ms[q] = kt.cnt[q] ? kt.sum[q] / kt.cnt[q] : 0.0;
  return st;
}

extern "C" LX_API int lx_sim_timestep(const lx_sim* s) { return s ? s->t : -1; }

extern "C" LX_API lx_status lx_sim_set_max_series(lx_sim* s, int capacity) {
  if (!s || capacity < 0) return fail(s, LX_ERR_INVALID, "capacity must be >= 0");
  lx::DeviceGuard dg_(s->device);
  if (s->batch) return fail(s, LX_ERR_STATE, "batched members keep no max series");
  lx_status st = lx_sim_sync(s);
  if (st) return st;
  dfree(s->d_series, s->own);
  s->d_series = nullptr;
  s->series_cap = 0;
  s->series_t.clear();
  if (capacity > 0) {
    CK(cudaMallocAsync(&s->d_series, sizeof(unsigned long long) * capacity, s->own));
    CK(cudaStreamSynchronize(s->own));
    s->series_cap = capacity;
  }
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_read_max_series(lx_sim* s, int* steps, double* values, int capacity, int* rows) {
  if (!s || !rows) return fail(s, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(s->device);
  lx_status st = lx_sim_sync(s);
  if (st) return st;
  const int n = (int)s->series_t.size();
  *rows = n;
  if (n == 0) return LX_OK;
  if (!steps || !values || capacity < n) return fail(s, LX_ERR_INVALID, "buffers hold fewer entries than the series");
  std::vector<unsigned long long> bits(n);
  CK(cudaMemcpyAsync(bits.data(), s->d_series, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->n_d2h += sizeof(unsigned long long) * n;
  for (int q = 0; q < n; q++) {
    steps[q] = s->series_t[q];
    std::memcpy(&values[q], &bits[q], sizeof(double));
  }
  s->series_t.clear();
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_max_e2(lx_sim* s, double* out) {
  if (!s || !out) return fail(s, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(s->device);
  { const lx_status st_ = settle(s); if (st_) return st_; }
  *out = s->last_max;
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_set_stream(lx_sim* s, void* stream) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  lx::DeviceGuard dg_(s->device);
  lx_status st = lx_sim_sync(s);
  if (st) return st;
  s->stream = stream ? (cudaStream_t)stream : s->own;
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_info(const lx_sim* s, lx_info* info) {
  if (!s || !info) return fail((lx_sim*)s, LX_ERR_INVALID, "null argument");
  std::memset(info, 0, sizeof *info);
  info->cells = (size_t)s->Nx * s->Ny * s->Nz;
  size_t b = 0;
  for (int c = 0; c < 3; c++) {
    for (void* f : {s->E[c], s->H[c], s->E1[c], s->H1[c]})
      if (f) b += s->ncell * s->tsize;
    if (s->Cbs[c]) b += s->ncell * s->csize;
    for (int q = 0; q < 2; q++) {
      info->psi_h_entries += s->psiH_n[c][q];
      info->psi_e_entries += s->psiE_n[c][q];
    }
  }
  b += (s->sweep ? 2 : 1) * (info->psi_h_entries + info->psi_e_entries) * s->csize;
  if (s->etotal) b += s->ncell * s->csize;
  b += s->xfer_cap * sizeof(double) + (size_t)s->tab_total * s->csize;
  for (auto& sl : s->slots) b += sl.cap * sizeof(double);
  for (auto& d : s->dfts) b += d.n_acc * sizeof(double);
  b += (size_t)s->probe_cap * s->nprobes * 6 * sizeof(double);
  info->device_bytes = b;
  for (int a = 0; a < 3; a++) info->slab[a] = s->pml ? s->slab[a].n : 0;
  info->uniform = s->uniform;
  info->field_bytes = (int)s->tsize;
  return LX_OK;
}

extern "C" LX_API lx_status lx_sim_counters(const lx_sim* s, uint64_t* kernels, uint64_t* h2d, uint64_t* d2h) {
  if (!s) return fail(nullptr, LX_ERR_INVALID, "null handle");
  if (kernels) *kernels = s->n_kernels;
  if (h2d) *h2d = s->n_h2d;
  if (d2h) *d2h = s->n_d2h;
  return LX_OK;
}

extern "C" LX_API lx_status lx_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return fail(nullptr, LX_ERR_INVALID, "null argument");
  cudaError_t e = cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocDefault);
  if (e != cudaSuccess) return fail(nullptr, LX_ERR_OOM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
  return LX_OK;
}

extern "C" LX_API void lx_host_free(void* ptr) {
  if (ptr) cudaFreeHost(ptr);
}

// ------------------------------------------------------------------ batches

struct lx_batch {
  std::vector<lx_sim*> sims;
  int device = 0;  // CUDA device current at lx_batch_create; every member lives on it
  int prec = -1;
  int chunk = 100;
  bool dirty = true;
  cudaStream_t stream = nullptr;
  // 3-D members of at least kSoloCells cells take one kernel pair each, with their parameter
  // block passed by value (the constant bank, as for a handle stepped alone), spread over the
  // batch stream and kLanes - 1 more so that the members' kernels overlap.  Planar members with
  // float compute of at least kSoloCells2 cells take the single-sweep kernel the same way, in
  // their two buffers (ping-pong mode); smaller members share the batched launches in place.
  static constexpr long long kSoloCells = 1LL << 18;
  // (2^21 cells: a member's sweep takes ~15 us; at 2^18 the launches of the 256-lens batch's
  // larger half cost more than the single sweep saves, 103 -> 96 Gcell/s)
  static constexpr long long kSoloCells2 = 1LL << 21;
  static constexpr int kLanes = 4;
  cudaStream_t lanes[kLanes - 1] = {};
  cudaEvent_t lane_ev[kLanes] = {};  // [0] fork, [1..] joins
  struct Group {  // members sharing (planar, uniform, solo): one update launch per half step
    bool planar = false, uniform = false;
    bool solo = false;              // members launched one by one (kSoloCells / kSoloCells2 and larger)
    std::vector<char> host_params;  // solo groups: the members' parameter blocks
    int march = lx::kMarch3;   // cells each thread walks along x
    std::vector<int> members;  // batch-global indices
    void* d_params = nullptr;
    int* d_first = nullptr;
    int4* d_tiles = nullptr;
    int nblocks = 0;
  };
  int march2d = lx::kMarch2, march3d = lx::kMarch3;  // per dimension (lx_batch_set_march / autotune)
  std::vector<lx_tune_entry> table;  // march per member class (lx_batch_set_tune_table / autotune)
  struct DftClass {  // DFT planes that sample at the same batch steps
    int every = 1, phase = 0;
    lx::DftParams* d_planes = nullptr;
    int* d_bfirst = nullptr;
    int2* d_map = nullptr;
    int nplanes = 0, nblocks = 0;
  };
  std::vector<Group> groups;
  std::vector<DftClass> dft;
  lx::PrologueParams* d_pps = nullptr;
  int max_entries = 0;
  int* d_ts = nullptr;
  unsigned long long* d_slots = nullptr;
  long long step = 0;  // batch steps taken (DFT sampling classes are phases of it)
  cudaGraphExec_t exec = nullptr;
  int exec_steps = 0;
  long long chunks_since_rebuild = 0;  // a chunk is captured only when the one before had the same members
  long long exec_base_mod = -1;
  bool graphable = true;
  std::vector<int> host_ts;
  int pending = 0;  // steps enqueued since the last wait
  std::string err;
};

static void batch_member_changed(lx_batch* b) { b->dirty = true; }

// A member launched one by one, with no tile shape: 3-D members of kSoloCells cells or more,
// planar single-sweep members of kSoloCells2 cells or more.
static bool batch_alone(const lx_sim* s) {
  return s->planar ? s->sweep && (long long)s->Nx * s->Nz >= lx_batch::kSoloCells2
                   : (long long)s->Nx * s->Ny * s->Nz >= lx_batch::kSoloCells;
}

// The tile-shape class of a handle: dimension, floor(log4(cells)), precision, x slab depth.
static lx_tune_entry tune_class_of(const lx_sim* s) {
  lx_tune_entry e{};
  const double cells = (double)s->Nx * s->Ny * s->Nz;
  int sc = 0;
  while (sc < 15 && cells >= std::ldexp(1.0, 2 * (sc + 1))) sc++;
  e.planar = s->planar ? 1 : 0;
  e.size_class = sc;
  e.precision = s->p.precision;
  const int d = s->pml ? s->slab[0].lo : 0;
  e.slab_class = d <= 0 ? 0 : d <= 8 ? 1 : d <= 16 ? 2 : 3;
  return e;
}

static bool same_class(const lx_tune_entry& a, const lx_tune_entry& b) {
  return a.planar == b.planar && a.size_class == b.size_class && a.precision == b.precision &&
         a.slab_class == b.slab_class;
}

static void table_put(lx_batch* b, const lx_tune_entry& e) {
  for (auto& x : b->table)
    if (same_class(x, e)) {
      x.march = e.march;
      return;
    }
  b->table.push_back(e);
}

// The march of a batched member: its class's table entry, else the per-dimension march.
static int batch_march(const lx_batch* b, const lx_sim* s) {
  const lx_tune_entry k = tune_class_of(s);
  for (const auto& x : b->table)
    if (same_class(x, k)) return x.march;
  return s->planar ? b->march2d : b->march3d;
}

static void batch_free_device(lx_batch* b) {
  for (auto& g : b->groups) {
    dfree(g.d_params, b->stream);
    dfree(g.d_first, b->stream);
    dfree(g.d_tiles, b->stream);
  }
  b->groups.clear();
  for (auto& d : b->dft) {
    dfree(d.d_planes, b->stream);
    dfree(d.d_bfirst, b->stream);
    dfree(d.d_map, b->stream);
  }
  b->dft.clear();
  dfree(b->d_pps, b->stream);
  dfree(b->d_ts, b->stream);
  dfree(b->d_slots, b->stream);
  b->d_pps = nullptr;
  b->d_ts = nullptr;
  b->d_slots = nullptr;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->exec_steps = 0;
}

static lx_status bfail(lx_batch* b, lx_status st, const std::string& m) {
  if (b) b->err = m;
  return fail(nullptr, st, m);
}

#define BCK(...)                                                                                      \
  do {                                                                                                \
    cudaError_t e_ = (__VA_ARGS__);                                                                   \
    if (e_ != cudaSuccess) return bfail(b, e_ == cudaErrorMemoryAllocation ? LX_ERR_OOM : LX_ERR_CUDA, \
                                        std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(e_));   \
  } while (0)

extern "C" LX_API lx_status lx_batch_create(lx_batch** out) {
  if (!out) return fail(nullptr, LX_ERR_INVALID, "null argument");
  lx_batch* b = new (std::nothrow) lx_batch();
  if (!b) return fail(nullptr, LX_ERR_OOM, "host allocation failed");
  keep_pool_memory();
  cudaGetDevice(&b->device);
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  for (int l = 0; e == cudaSuccess && l < lx_batch::kLanes - 1; l++)
    e = cudaStreamCreateWithFlags(&b->lanes[l], cudaStreamNonBlocking);
  for (int l = 0; e == cudaSuccess && l < lx_batch::kLanes; l++)
    e = cudaEventCreateWithFlags(&b->lane_ev[l], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    for (int l = 0; l < lx_batch::kLanes - 1; l++)
      if (b->lanes[l]) cudaStreamDestroy(b->lanes[l]);
    for (int l = 0; l < lx_batch::kLanes; l++)
      if (b->lane_ev[l]) cudaEventDestroy(b->lane_ev[l]);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return fail(nullptr, LX_ERR_CUDA, std::string("batch create: ") + cudaGetErrorString(e));
  }
  *out = b;
  return LX_OK;
}

extern "C" LX_API void lx_batch_destroy(lx_batch* b) {
  if (!b) return;
  lx::DeviceGuard dg_(b->device);
  cudaStreamSynchronize(b->stream);
  for (auto* s : b->sims) s->batch = nullptr;
  batch_free_device(b);
  cudaStreamSynchronize(b->stream);
  cudaStreamDestroy(b->stream);
  for (int l = 0; l < lx_batch::kLanes - 1; l++) cudaStreamDestroy(b->lanes[l]);
  for (int l = 0; l < lx_batch::kLanes; l++) cudaEventDestroy(b->lane_ev[l]);
  delete b;
}

extern "C" LX_API int lx_batch_size(const lx_batch* b) { return b ? (int)b->sims.size() : 0; }

extern "C" LX_API lx_status lx_batch_set_chunk(lx_batch* b, int steps) {
  if (!b || steps < 0) return fail(nullptr, LX_ERR_INVALID, "chunk must be >= 0");
  lx::DeviceGuard dg_(b->device);
  b->chunk = steps;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->exec_steps = 0;
  return LX_OK;
}

extern "C" LX_API lx_status lx_batch_wait(lx_batch* b);

extern "C" LX_API lx_status lx_batch_add(lx_batch* b, lx_sim* s) {
  if (!b || !s) return fail(nullptr, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(b->device);
  lx_status st = lx_batch_wait(b);
  if (st) return st;
  if (s->batch) return bfail(b, LX_ERR_INVALID, s->batch == b ? "handle already in this batch" : "handle is in another batch");
  if (s->device != b->device) return bfail(b, LX_ERR_INVALID, "the handle lives on another device than the batch");
  if (b->prec >= 0 && s->prec != b->prec) return bfail(b, LX_ERR_INVALID, "all members of a batch share one precision");
  if (!s->outputs.empty() || s->nprobes > 0 || s->d_series)
    return bfail(b, LX_ERR_UNSUPPORTED, "batched members cannot have snapshot outputs, probes or a max series");
  if ((st = lx_sim_sync(s))) return st;
  b->prec = s->prec;
  b->sims.push_back(s);
  s->batch = b;
  b->dirty = true;
  return LX_OK;
}

extern "C" LX_API lx_status lx_batch_remove(lx_batch* b, lx_sim* s) {
  if (!b || !s) return fail(nullptr, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(b->device);
  lx_status st = lx_batch_wait(b);
  if (st) return st;
  for (size_t q = 0; q < b->sims.size(); q++)
    if (b->sims[q] == s) {
      b->sims.erase(b->sims.begin() + q);
      s->batch = nullptr;
      b->dirty = true;
      if (b->sims.empty()) b->prec = -1;
      return LX_OK;
    }
  return bfail(b, LX_ERR_INVALID, "handle is not in this batch");
}

template <class T, class C>
static lx_status batch_rebuild(lx_batch* b) {
  batch_free_device(b);
  const int n = (int)b->sims.size();
  std::vector<lx::PrologueParams> pps(n);
  b->max_entries = 0;
  b->host_ts.resize(n);
  b->graphable = true;
  BCK(cudaMallocAsync(&b->d_slots, sizeof(unsigned long long) * (n > 0 ? n : 1), b->stream));
  std::vector<std::vector<lx::DftParams>> dft_planes;
  // Large planar single-sweep members step in their two buffers, the others in place in buffer 0;
  // a member whose mode changes at an odd step moves its state (one device copy).
  for (int q = 0; q < n; q++) {
    lx_sim* s = b->sims[q];
    const bool two = s->planar && batch_alone(s);
    lx_status st;
    if ((st = set_pp(s, two))) return st;
    BCK(cudaStreamSynchronize(s->stream));
  }
  for (int q = 0; q < n; q++) {
    lx_sim* s = b->sims[q];
    pps[q] = make_prologue(s);
    pps[q].max_slot = b->d_slots + q;
    b->max_entries = std::max(b->max_entries, pps[q].tab_total);
    b->host_ts[q] = s->t;
    T* pf[6] = {(T*)s->E[0], (T*)s->E[1], (T*)s->E[2], (T*)s->H[0], (T*)s->H[1], (T*)s->H[2]};
    for (auto& d : s->dfts) {
      lx::DftParams dp;
      std::memset(&dp, 0, sizeof dp);
      dp.axis = d.axis; dp.index = d.index; dp.na = d.na; dp.nb = d.nb; dp.Ny = s->Ny; dp.Nzp = s->Nzp;
      dp.nfreq = d.nfreq; dp.dt = s->k.dt; dp.weight = (double)d.every; dp.every_ = d.every;
      dp.omega = d.d_omega; dp.acc = d.d_acc; dp.phase = d.d_phase; dp.sim = q; dp.hmul = 1.0 / s->hscale;
      T* pf1[6] = {(T*)s->E1[0], (T*)s->E1[1], (T*)s->E1[2], (T*)s->H1[0], (T*)s->H1[1], (T*)s->H1[2]};
      for (int c = 0; c < 4; c++) {
        dp.f[c] = pf[d.comps[c]];
        dp.f1[c] = s->pp ? pf1[d.comps[c]] : nullptr;
        for (int a = 0; a < 3; a++) dp.ext[c][a] = s->ext[d.comps[c]][a];
      }
      // sampled at batch steps b' with (t + b' - step) % every == 0
      const int phase = (int)(((b->step - s->t) % d.every + d.every) % d.every);
      int ci = -1;
      for (size_t k = 0; k < b->dft.size(); k++)
        if (b->dft[k].every == d.every && b->dft[k].phase == phase) ci = (int)k;
      if (ci < 0) {
        b->dft.emplace_back();
        b->dft.back().every = d.every;
        b->dft.back().phase = phase;
        dft_planes.emplace_back();
        ci = (int)b->dft.size() - 1;
      }
      dft_planes[ci].push_back(dp);
      if (b->chunk > 0 && b->chunk % d.every != 0) b->graphable = false;
    }
    const bool solo = s->pp || (!s->planar && batch_alone(s));
    if (s->pp && b->chunk % 2) b->graphable = false;  // a captured chunk must keep each member's parity
    // batched members share a launch only with members of the same march (their classes' picks)
    const int march = solo ? (s->planar ? b->march2d : b->march3d) : batch_march(b, s);
    int gi = -1;
    for (size_t g = 0; g < b->groups.size(); g++)
      if (b->groups[g].planar == (bool)s->planar && b->groups[g].uniform == (bool)s->uniform &&
          b->groups[g].solo == solo && (solo || b->groups[g].march == march))
        gi = (int)g;
    if (gi < 0) {
      b->groups.emplace_back();
      b->groups.back().planar = s->planar;
      b->groups.back().uniform = s->uniform;
      b->groups.back().solo = solo;
      b->groups.back().march = march;
      gi = (int)b->groups.size() - 1;
    }
    b->groups[gi].members.push_back(q);
  }
  BCK(cudaMallocAsync(&b->d_pps, sizeof(lx::PrologueParams) * (n > 0 ? n : 1), b->stream));
  BCK(cudaMemcpyAsync(b->d_pps, pps.data(), sizeof(lx::PrologueParams) * n, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMallocAsync(&b->d_ts, sizeof(int) * (n > 0 ? n : 1), b->stream));
  BCK(cudaMemcpyAsync(b->d_ts, b->host_ts.data(), sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
  for (size_t k = 0; k < b->dft.size(); k++) {
    auto& cl = b->dft[k];
    const auto& planes = dft_planes[k];
    std::vector<int> bfirst(planes.size() + 1, 0);
    for (size_t q = 0; q < planes.size(); q++) bfirst[q + 1] = bfirst[q] + (int)((4LL * planes[q].na * planes[q].nb + 255) / 256);
    cl.nplanes = (int)planes.size();
    cl.nblocks = bfirst.back();
    BCK(cudaMallocAsync(&cl.d_planes, sizeof(lx::DftParams) * planes.size(), b->stream));
    BCK(cudaMemcpyAsync(cl.d_planes, planes.data(), sizeof(lx::DftParams) * planes.size(), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMallocAsync(&cl.d_bfirst, sizeof(int) * bfirst.size(), b->stream));
    BCK(cudaMemcpyAsync(cl.d_bfirst, bfirst.data(), sizeof(int) * bfirst.size(), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMallocAsync(&cl.d_map, sizeof(int2) * (cl.nblocks > 0 ? cl.nblocks : 1), b->stream));
    BCK(lx::launch_block_map(cl.d_bfirst, cl.nplanes, cl.nblocks, cl.d_map, b->stream));
  }
  for (auto& g : b->groups) {
    std::vector<lx::StepParams<T, C>> ps;
    std::vector<int> first(1, 0);
    for (int q : g.members) {
      lx_sim* s = b->sims[q];
      lx::StepParams<T, C> sp = step_params<T, C>(s);
      sp.max_slot = b->d_slots + q;
      sp.etotal = nullptr;
      ps.push_back(sp);
      const long long nb = (long long)first.back() + lx::batch_blocks(s->Nx, s->Ny, s->Nz, s->planar, g.march);
      if (nb > 0x7fffffffLL) return bfail(b, LX_ERR_INVALID, "batch too large for one launch");
      first.push_back((int)nb);
    }
    if (g.solo) {  // launched by value from the host copy: no device blocks or tile map
      g.host_params.assign((const char*)ps.data(), (const char*)(ps.data() + ps.size()));
      g.nblocks = 0;
      continue;
    }
    g.nblocks = first.back();
    BCK(cudaMallocAsync(&g.d_params, sizeof(lx::StepParams<T, C>) * ps.size(), b->stream));
    BCK(cudaMemcpyAsync(g.d_params, ps.data(), sizeof(lx::StepParams<T, C>) * ps.size(), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMallocAsync(&g.d_first, sizeof(int) * first.size(), b->stream));
    BCK(cudaMemcpyAsync(g.d_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice, b->stream));
    BCK(cudaMallocAsync(&g.d_tiles, sizeof(int4) * (g.nblocks > 0 ? g.nblocks : 1), b->stream));
    BCK(lx::launch_batch_tiles<T, C>((const lx::StepParams<T, C>*)g.d_params, g.d_first, (int)g.members.size(), g.nblocks,
                                     g.planar, g.march, g.d_tiles, b->stream));
  }
  b->dirty = false;
  return LX_OK;
}

template <class T, class C>
static lx_status batch_enqueue(lx_batch* b, long long step0, int nsteps) {
  const int n = (int)b->sims.size();
  // the members' device step counters advance once, after the chunk; step q runs at ts + q
  for (int q = 0; q < nsteps; q++) {
    BCK(lx::launch_prologue_batch<C>(b->d_pps, b->d_ts, q, n, b->max_entries, b->stream));
    for (auto& g : b->groups) {
      if (g.solo) {  // each member's H and E on one of the lanes; members are independent
        const auto* hp = (const lx::StepParams<T, C>*)g.host_params.data();
        const int L = std::min<int>(lx_batch::kLanes, (int)g.members.size());
        BCK(cudaEventRecord(b->lane_ev[0], b->stream));
        for (int l = 0; l < L - 1; l++) BCK(cudaStreamWaitEvent(b->lanes[l], b->lane_ev[0], 0));
        for (size_t m = 0; m < g.members.size(); m++) {
          cudaStream_t st = (m % L) ? b->lanes[m % L - 1] : b->stream;
          if constexpr (sizeof(C) == 4) {
            if (g.planar) {  // single sweep, state t & 1 -> (t+1) & 1
              lx::StepParams<T, C> sw = hp[m];
              if ((b->host_ts[g.members[m]] + q) & 1) swap_buffers(sw);
              BCK(lx::launch_step_sweep2<T, C>(sw, g.uniform, st));
              continue;
            }
          }
          BCK(lx::launch_step<T, C>(hp[m], g.planar, g.uniform, true, st));
          BCK(lx::launch_step<T, C>(hp[m], g.planar, g.uniform, false, st));
        }
        for (int l = 0; l < L - 1; l++) {
          BCK(cudaEventRecord(b->lane_ev[1 + l], b->lanes[l]));
          BCK(cudaStreamWaitEvent(b->stream, b->lane_ev[1 + l], 0));
        }
        continue;
      }
      BCK(lx::launch_batch_step<T, C>((const lx::StepParams<T, C>*)g.d_params, g.d_tiles, g.nblocks, g.planar,
                                      g.uniform, g.march, true, b->stream));
    }
    for (auto& g : b->groups)
      if (!g.solo)
        BCK(lx::launch_batch_step<T, C>((const lx::StepParams<T, C>*)g.d_params, g.d_tiles, g.nblocks, g.planar,
                                        g.uniform, g.march, false, b->stream));
    const long long bs = step0 + q;
    for (auto& cl : b->dft)
      if (bs % cl.every == cl.phase)
        BCK(lx::launch_dft_batch<T>(cl.d_planes, cl.d_map, cl.nplanes, cl.nblocks, b->d_ts, q, b->stream));
  }
  if (nsteps > 0) BCK(lx::launch_tick(b->d_ts, n, nsteps, b->stream));
  return LX_OK;
}

template <class T, class C>
static lx_status batch_run_async(lx_batch* b, int nsteps) {
  lx_status st;
  bool moved = false;
  for (size_t q = 0; q < b->sims.size() && !b->dirty; q++) moved |= (b->sims[q]->t != b->host_ts[q]);
  if (b->dirty || moved) {
    for (auto* s : b->sims) BCK(cudaStreamSynchronize(s->stream));  // members' own pending work first
    if ((st = batch_rebuild<T, C>(b))) return st;
    b->chunks_since_rebuild = 0;
  }
  int done = 0;
  if (b->chunk > 0 && b->graphable) {
    while (nsteps - done >= b->chunk) {
      // The first chunk after a change of members is launched directly: capturing and
      // instantiating a graph is host time before any of its work starts, while direct
      // launches run as they are issued.  A serving loop whose members change every chunk
      // never captures (1000-request stream: 55.4 -> 61.0 Gcell/s); a steady batch replays
      // a graph from its second chunk on.
      if (b->chunks_since_rebuild++ == 0) {
        if ((st = batch_enqueue<T, C>(b, b->step, b->chunk))) return st;
        b->step += b->chunk;
        done += b->chunk;
        continue;
      }
      const long long base_mod = b->step % b->chunk;
      if (!b->exec || b->exec_steps != b->chunk || b->exec_base_mod != base_mod) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
        cudaGraph_t g;
        BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        st = batch_enqueue<T, C>(b, b->step, b->chunk);
        cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
        if (st) return st;
        BCK(ce);
        ce = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        BCK(ce);
        b->exec_steps = b->chunk;
        b->exec_base_mod = base_mod;
      }
      BCK(cudaGraphLaunch(b->exec, b->stream));
      b->step += b->chunk;
      done += b->chunk;
    }
  }
  if (nsteps - done > 0) {
    if ((st = batch_enqueue<T, C>(b, b->step, nsteps - done))) return st;
    b->step += nsteps - done;
    b->chunks_since_rebuild++;
  }
  for (size_t q = 0; q < b->sims.size(); q++) {
    b->sims[q]->t += nsteps;
    b->host_ts[q] = b->sims[q]->t;
    b->sims[q]->n_kernels += (uint64_t)nsteps * 4;
  }
  b->pending += nsteps;
  return LX_OK;
}

extern "C" LX_API lx_status lx_batch_step_async(lx_batch* b, int nsteps) {
  if (!b || nsteps < 0) return fail(nullptr, LX_ERR_INVALID, "bad argument");
  lx::DeviceGuard dg_(b->device);
  if (b->sims.empty() || nsteps == 0) return LX_OK;
  if (b->prec == LX_PREC_FP64) return batch_run_async<double, double>(b, nsteps);
  if (b->prec == LX_PREC_FP32) return batch_run_async<float, float>(b, nsteps);
  return batch_run_async<__half, float>(b, nsteps);
}

extern "C" LX_API lx_status lx_batch_wait(lx_batch* b) {
  if (!b) return fail(nullptr, LX_ERR_INVALID, "null argument");
  lx::DeviceGuard dg_(b->device);
  if (b->pending == 0) return LX_OK;
  const int n = (int)b->sims.size();
  std::vector<unsigned long long> slots(n);
  if (n) BCK(cudaMemcpyAsync(slots.data(), b->d_slots, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  b->pending = 0;
  std::string bad;
  for (int q = 0; q < n; q++) {
    double v;
    std::memcpy(&v, &slots[q], sizeof v);
    b->sims[q]->last_max = v;
    if (!std::isfinite(v) && bad.empty()) bad = "member " + std::to_string(q) + ": max|E|^2 is not finite";
  }
  if (!bad.empty()) return bfail(b, LX_ERR_BLOWUP, bad);
  return LX_OK;
}

extern "C" LX_API lx_status lx_batch_step(lx_batch* b, int nsteps) {
  lx_status st = lx_batch_step_async(b, nsteps);
  if (st) return st;
  return lx_batch_wait(b);
}

static bool march_ok(int m) { return m == 1 || m == 2 || m == 4 || m == 8; }

extern "C" LX_API lx_status lx_batch_set_march(lx_batch* b, int planar_rows, int planes_3d) {
  if (!b || !march_ok(planar_rows) || !march_ok(planes_3d)) return fail(nullptr, LX_ERR_INVALID, "march must be 1, 2, 4 or 8");
  lx::DeviceGuard dg_(b->device);
  lx_status st = lx_batch_wait(b);
  if (st) return st;
  b->march2d = planar_rows;
  b->march3d = planes_3d;
  b->dirty = true;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->exec_steps = 0;
  return LX_OK;
}

extern "C" LX_API lx_status lx_batch_get_march(const lx_batch* b, int* planar_rows, int* planes_3d) {
  if (!b || !planar_rows || !planes_3d) return fail(nullptr, LX_ERR_INVALID, "null argument");
  *planar_rows = b->march2d;
  *planes_3d = b->march3d;
  return LX_OK;
}

// A scratch batch of zero-field twins (same parameters and Cb) of sampled handles, for timing
// tile shapes; the sampled handles themselves are never stepped.
struct TuneTwins {
  lx_batch* tb = nullptr;
  std::vector<lx_sim*> sims;
  TuneTwins() = default;
  TuneTwins(const TuneTwins&) = delete;
  TuneTwins& operator=(const TuneTwins&) = delete;
  ~TuneTwins() {
    if (tb) lx_batch_destroy(tb);
    for (auto* t : sims) lx_sim_destroy(t);
  }
};

// Twins of `sample`, each `copies` times, as members of one scratch batch (no graphs).
static lx_status make_twins(const std::vector<const lx_sim*>& sample, int copies, TuneTwins* tw) {
  lx_status st = lx_batch_create(&tw->tb);
  if (!st) st = lx_batch_set_chunk(tw->tb, 0);
  for (size_t q = 0; q < sample.size() * copies && !st; q++) {
    const lx_sim* src = sample[q % sample.size()];
    lx_sim* t = nullptr;
    st = lx_sim_create(&src->p, &t);
    if (st) break;
    tw->sims.push_back(t);
    for (int c = 0; c < 3 && !st; c++)
      if (src->Cbs[c] && ext_n(src, c))
        if (cudaMemcpyAsync(t->Cbs[c], src->Cbs[c], t->ncell * t->csize, cudaMemcpyDeviceToDevice, t->stream) != cudaSuccess)
          st = fail(nullptr, LX_ERR_CUDA, "copying Cb to a tuning twin failed");
    if (!st) st = lx_sim_sync(t);
    if (!st) st = lx_batch_add(tw->tb, t);
  }
  return st;
}

// Milliseconds for `steps` batched steps of the scratch batch with its current tile shapes:
// a rebuild and two warm-up steps, then the better of two timed runs (CUDA events on the
// batch stream).
static lx_status time_steps(lx_batch* tb, int steps, float* ms) {
  *ms = 0.f;
  lx_status st = lx_batch_step(tb, 2);
  if (st == LX_ERR_BLOWUP) st = LX_OK;  // zero fields cannot blow up; tolerate a source-driven twin
  if (st) return st;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    st = fail(nullptr, LX_ERR_CUDA, "cudaEventCreate failed");
  for (int rep = 0; rep < 2 && !st; rep++) {
    cudaEventRecord(e0, tb->stream);
    st = lx_batch_step_async(tb, steps);
    cudaEventRecord(e1, tb->stream);
    if (!st) st = lx_batch_wait(tb);
    if (st == LX_ERR_BLOWUP) st = LX_OK;
    float t = 0.f;
    if (!st && cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) st = fail(nullptr, LX_ERR_CUDA, "event timing failed");
    if (!st && (rep == 0 || t < *ms)) *ms = t;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return st;
}

// Drops the captured graph and regroups the members at the next step (a march changed).
static void batch_reshape(lx_batch* b) {
  b->dirty = true;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->exec_steps = 0;
}

extern "C" LX_API lx_status lx_sim_tune_class(const lx_sim* s, lx_tune_entry* key) {
  if (!s || !key) return fail(nullptr, LX_ERR_INVALID, "null argument");
  *key = tune_class_of(s);
  key->march = 0;
  return LX_OK;
}

extern "C" LX_API lx_status lx_batch_set_tune_table(lx_batch* b, const lx_tune_entry* e, int n) {
  if (!b || n < 0 || (n > 0 && !e)) return fail(nullptr, LX_ERR_INVALID, "bad table");
  for (int q = 0; q < n; q++)
    if (!march_ok(e[q].march) || e[q].planar < 0 || e[q].planar > 1 || e[q].size_class < 0 || e[q].size_class > 15 ||
        e[q].precision < LX_PREC_FP64 || e[q].precision > LX_PREC_FP16S || e[q].slab_class < 0 || e[q].slab_class > 3)
      return fail(nullptr, LX_ERR_INVALID, "bad table entry (march 1, 2, 4 or 8; classes as lx_sim_tune_class)");
  lx::DeviceGuard dg_(b->device);
  lx_status st = lx_batch_wait(b);
  if (st) return st;
  b->table.clear();
  for (int q = 0; q < n; q++) table_put(b, e[q]);
  batch_reshape(b);
  return LX_OK;
}

extern "C" LX_API lx_status lx_batch_get_tune_table(const lx_batch* b, lx_tune_entry* e, int cap, int* n) {
  if (!b || !n || cap < 0 || (cap > 0 && !e)) return fail(nullptr, LX_ERR_INVALID, "null argument");
  for (int q = 0; q < cap && q < (int)b->table.size(); q++) e[q] = b->table[q];
  *n = (int)b->table.size();
  return LX_OK;
}

extern "C" LX_API lx_status lx_batch_autotune(lx_batch* b, int steps, int* planar_rows, int* planes_3d) {
  if (!b || steps < 1) return fail(nullptr, LX_ERR_INVALID, "steps must be >= 1");
  lx::DeviceGuard dg_(b->device);
  lx_status st = lx_batch_wait(b);
  if (st) return st;
  // The classes of the batched members, and a sample of them within the cell budget that holds
  // at least one member of every class.
  const double budget = 1.5e8;
  std::vector<lx_tune_entry> classes;
  std::vector<double> total;
  std::vector<const lx_sim*> sample;
  double sampled = 0.0;
  for (auto* s : b->sims) {
    if (batch_alone(s)) continue;
    const lx_tune_entry k = tune_class_of(s);
    size_t c = 0;
    while (c < classes.size() && !same_class(classes[c], k)) c++;
    const double cells = (double)s->Nx * s->Ny * s->Nz;
    const bool first = c == classes.size();  // a class's first member is always sampled
    if (first) {
      classes.push_back(k);
      total.push_back(0.0);
    }
    total[c] += cells;
    if (first || sampled + cells <= budget) {
      sample.push_back(s);
      sampled += cells;
    }
  }
  if (classes.empty()) {
    if (planar_rows) *planar_rows = b->march2d;
    if (planes_3d) *planes_3d = b->march3d;
    return LX_OK;
  }
  // Time the whole sample together, so that a class's pick pays for the launch it splits off:
  // first one march for every class, then each class in turn (largest first) moved to each
  // other march, a move kept when it saves 2 %.
  PoolMark mark;  // destroyed after the twins: the pool gives their memory back
  TuneTwins tw;
  if ((st = make_twins(sample, 1, &tw))) return st;
  auto timed = [&](std::vector<lx_tune_entry>& tab, float* ms) -> lx_status {
    lx_status r = lx_batch_set_tune_table(tw.tb, tab.data(), (int)tab.size());
    return r ? r : time_steps(tw.tb, steps, ms);
  };
  const int cand[4] = {1, 2, 4, 8};
  std::vector<lx_tune_entry> cur = classes;
  float cur_ms = 0.f;
  for (int m : cand) {
    std::vector<lx_tune_entry> tab = classes;
    for (auto& e : tab) e.march = m;
    float ms = 0.f;
    if ((st = timed(tab, &ms))) return st;
    if (cur_ms == 0.f || ms < cur_ms) {
      cur_ms = ms;
      cur = tab;
    }
  }
  std::vector<size_t> order(classes.size());
  for (size_t c = 0; c < order.size(); c++) order[c] = c;
  std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return total[x] > total[y]; });
  if (classes.size() > 1)
    for (size_t c : order)
      for (int m : cand) {
        if (m == cur[c].march) continue;
        std::vector<lx_tune_entry> tab = cur;
        tab[c].march = m;
        float ms = 0.f;
        if ((st = timed(tab, &ms))) return st;
        if (ms < 0.98f * cur_ms) {
          cur_ms = ms;
          cur = tab;
        }
      }
  for (const auto& e : cur) table_put(b, e);
  int m2 = 0, m3 = 0;
  double big2 = -1.0, big3 = -1.0;
  for (size_t c = 0; c < cur.size(); c++) {
    double& big = cur[c].planar ? big2 : big3;
    if (total[c] > big) {
      big = total[c];
      (cur[c].planar ? m2 : m3) = cur[c].march;
    }
  }
  if ((st = lx_batch_set_march(b, m2 ? m2 : b->march2d, m3 ? m3 : b->march3d))) return st;
  if (planar_rows) *planar_rows = b->march2d;
  if (planes_3d) *planes_3d = b->march3d;
  return LX_OK;
}

extern "C" LX_API lx_status lx_batch_tune_member(lx_batch* b, const lx_sim* s, int steps, int* march) {
  if (!b || !s || steps < 1) return fail(nullptr, LX_ERR_INVALID, "null argument or steps < 1");
  if (march) *march = 0;
  if (s->device != b->device) return fail(nullptr, LX_ERR_INVALID, "handle lives on another device than the batch");
  if (b->prec >= 0 && s->prec != b->prec) return fail(nullptr, LX_ERR_INVALID, "handle precision differs from the batch's");
  lx::DeviceGuard dg_(b->device);
  lx_status st = lx_batch_wait(b);
  if (st) return st;
  if (batch_alone(s)) return LX_OK;
  // Twins of the handle alone, replicated to 2^24 cells or 64 twins: a batch of hundreds of
  // members fills the GPU many times over, and a sample that fills it once or less favours
  // short marches (16 twins of a 300^2 lens picked 2 where the full batch runs best at 8).
  // A pick other than the dimension's march must save 5 %, since members of one launch group
  // split by march.
  const double cells = (double)s->Nx * s->Ny * s->Nz;
  const int copies = (int)std::max(1.0, std::min(64.0, std::floor(16777216.0 / std::max(cells, 1.0))));
  PoolMark mark;  // destroyed after the twins: the pool gives their memory back
  TuneTwins tw;
  if ((st = make_twins({s}, copies, &tw))) return st;
  const int def = s->planar ? b->march2d : b->march3d;
  const int cand[4] = {1, 2, 4, 8};
  float t[4] = {}, t_def = 0.f;
  int bq = 0;
  for (int q = 0; q < 4; q++) {
    if ((st = lx_batch_set_march(tw.tb, cand[q], cand[q]))) return st;
    if ((st = time_steps(tw.tb, steps, &t[q]))) return st;
    if (cand[q] == def) t_def = t[q];
    if (t[q] < t[bq]) bq = q;
  }
  int best = cand[bq];
  if (best != def && t[bq] > 0.95f * t_def) best = def;
  lx_tune_entry e = tune_class_of(s);
  e.march = best;
  table_put(b, e);
  batch_reshape(b);
  if (march) *march = best;
  return LX_OK;
}
