// lx_kernels.cu -- sm_103a kernels of the Yee time step.
//
// One step = prologue (TF/SF incident tables for this step, point source, monitor reset)
//          -> H kernel (curl E + TF/SF + CPML psi_H + H update, fused)
//          -> E kernel (curl H + TF/SF + CPML psi_E + E update + max|E|^2, fused)
// This is the order of every reference driver (e.g. three_dim_pml.cc:158-276): point source,
// E-curl, TF/SF on the curl, H update with psi, H-curl, TF/SF, E update with psi, |E|^2 max.
//
// The reference materialises each curl in a full-grid array and patches it in a separate
// pass (vfield.cc:196-275, maxwell.cc:512-812).  Here the curl of a cell lives in registers:
// each thread forms the neighbour differences of its cell, adds the TF/SF increment if the
// cell lies on a total-field-box plane (one table load), runs the psi recursion only when
// the cell lies in a CPML slab, and writes the updated component.  Cells outside the slabs
// and off the planes do 4 FP64 operations per component (3 differences + 1 FMA), which is
// the bound on GB300, whose FP64 pipe (~0.6 T lane-ops/s) limits before HBM does.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include "lx_device.cuh"
#include "lx_internal.h"
#include "lx_kernels.h"

namespace lx {

// ------------------------------------------------------------------ prologue

// The entry before its plane's sign (curl - v or curl + v), in the table's type C.
template <class C>
__device__ C incident_value(const PrologueParams& p, const PatchSet& ps, int plane, int e, int t) {
  // table entry e of `plane` -> in-plane indices -> wave positions
  double pos[3];
  int rem = e;
#pragma unroll
  for (int b = 2; b >= 0; --b) {
    if (b == ps.axis) {
      pos[b] = ps.pos_n[plane];
      continue;
    }
    const int nb = ps.n[b];
    const int ib = rem % nb;
    rem /= nb;
    pos[b] = (double)(ps.lo[b] + ib) + ps.off[b];
  }
  // ((x*dx*kx + y*dy*ky + z*dz*kz) + init*dx) - t*c*dt   (maxwell.cc:289 and siblings;
  // the planar lines have no y term, maxwell.cc:206)
  double X;
  if (p.planar)
    X = __dadd_rn(__dmul_rn(__dmul_rn(pos[0], p.dx), p.kx), __dmul_rn(__dmul_rn(pos[2], p.dz), p.kz));
  else
    X = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(pos[0], p.dx), p.kx), __dmul_rn(__dmul_rn(pos[1], p.dy), p.ky)),
                  __dmul_rn(__dmul_rn(pos[2], p.dz), p.kz));
  const double tt = ps.hcurl ? (double)t : (double)t - 0.5;
  X = __dsub_rn(__dadd_rn(X, __dmul_rn(p.init, p.dx)), __dmul_rn(__dmul_rn(tt, p.c), p.dt));
  // exp(-X^2/sigma) times the set's constant factor: one exp and two multiplies per entry
  // (the reference divides by sigma, d, c and mu0 in turn; the products differ from its
  // quotients in the last bit only).  Float tables take the exponential in FP32: the position
  // arithmetic above, where x - c*t cancels, stays FP64, and the entry is stored as a float
  // either way.  The FP64 exp made the batched prologue of 256 lens simulations 23.6 us of an
  // 858 us step.
  const double a = -__dmul_rn(__dmul_rn(X, X), p.inv_sigma);
  if constexpr (sizeof(C) == 4) return (float)((double)expf((float)a) * ps.factor);
  else return __dmul_rn(exp(a), ps.factor);
}

template <class C>
__device__ __forceinline__ void prologue_body(const PrologueParams& p, const int t, C* tab_out, const int gid,
                                              const int gstride) {
  if (gid == 0) {
    if (p.max_slot) *p.max_slot = 0ull;
    void* const src_field = ((t & 1) && p.src_field1) ? p.src_field1 : p.src_field;  // the state step t reads
    if (p.src_kind == 0) {
      // amp_source*sin(omega_source*t*dt), int members (maxwell.h:203,206; three_dim_pml.cc:163)
      const int wt = (int)((unsigned)p.src_omega_i * (unsigned)t);
      const double v = (double)p.src_amp_i * sin((double)wt * p.dt);
      if (p.prec == 0) ((double*)src_field)[p.src_idx] = v;
      else if (p.prec == 1) ((float*)src_field)[p.src_idx] = (float)v;
      else ((__half*)src_field)[p.src_idx] = __double2half(v);
    } else if (p.src_kind == 1) {
      const double u = (t - p.src_t0) / p.src_tw;
      const double v = p.src_amp * exp(-(u * u)) * sin(p.src_omega * t * p.dt);
      if (p.prec == 0) ((double*)src_field)[p.src_idx] += v;
      else if (p.prec == 1) ((float*)src_field)[p.src_idx] += (float)v;
      else {
        __half* f = (__half*)src_field;
        f[p.src_idx] = __float2half_rn(__half2float(f[p.src_idx]) + (float)v);
      }
    }
  }
  // Work items: one per entry, except that a set whose planes are normal to an axis k has no
  // component along shares its values between the two planes (the normal position is
  // multiplied by 0 in X), so one item writes both.  The sets' work ranges are staged in
  // shared memory once per block, so an item finds its set without a walk through the
  // parameter block in global memory.
  __shared__ int w_end[12];
  __shared__ unsigned char w_shared[12];
  if (threadIdx.x < 12) {  // one thread per set: the loads run in parallel
    const int s = threadIdx.x;
    const double kn[3] = {p.kx, p.ky, p.kz};
    const bool on = p.tab_total > 0 && s < p.nsets && p.sets[s].active;
    const bool sh = on && kn[p.sets[s].axis] == 0.0;
    w_end[s] = on ? (sh ? 1 : 2) * p.sets[s].plane_len : 0;
    w_shared[s] = sh;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int s = 1; s < 12; ++s) w_end[s] += w_end[s - 1];
  __syncthreads();
  const int work = w_end[11];
  for (int e = gid; e < work; e += gstride) {
    int s = 0;
    while (e >= w_end[s]) ++s;
    const PatchSet& ps = p.sets[s];
    const int rem = e - (s ? w_end[s - 1] : 0);
    const int plane = rem >= ps.plane_len ? 1 : 0;
    const int q = rem - plane * ps.plane_len;
    const C v = incident_value<C>(p, ps, plane, q, t);
    tab_out[ps.tab + plane * ps.plane_len + q] = ps.sign[plane] < 0 ? -v : v;
    if (w_shared[s]) tab_out[ps.tab + ps.plane_len + q] = ps.sign[1] < 0 ? -v : v;
  }
}

template <class C>
__global__ void prologue_kernel(const PrologueParams p, C* tab_out) {
  prologue_body<C>(p, p.t, tab_out, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// Batched prologue: blockIdx.y selects the simulation.  Its step counter lives on the device
// and advances once per chunk, so that a captured chunk can be replayed: step k of a chunk
// runs at ts[sim] + k.
template <class C>
__global__ void prologue_batch_kernel(const PrologueParams* __restrict__ pps, const int* __restrict__ ts, int k) {
  const PrologueParams& p = pps[blockIdx.y];
  prologue_body<C>(p, ts[blockIdx.y] + k, (C*)p.tab, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

__global__ void tick_kernel(int* ts, int n, int steps) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) ts[s] += steps;
}

// ------------------------------------------------------------------ 3-D kernels

// H half-step over cell (i,j,k) for Hx, Hy, Hz (three_dim_pml.cc:176-213, three_dim.cc:101-132).
// A cell's loads (h_load) are all issued before its update and stores (h_apply).  (Threads
// that own two cells and issue both cells' loads first were tried: the doubled registers
// halve the resident blocks and the kernels ran 12-15 % slower.)
template <class C>
struct HCell {
  long long c;
  bool ux, uy, uz;
  C ex, ey, ez, ez_j, ey_k, ex_k, ez_i, ey_i, ex_j, hx, hy, hz;
};

template <class T, class C, bool FAST = false>
__device__ __forceinline__ void h_load(const StepParams<T, C>& p, const int i, const int j, const int k, HCell<C>& v) {
  const long long c = (long long)i * p.si + (long long)j * p.sj + k;
  const bool ux = FAST || (j < p.Ny - 1 && k < p.Nz - 1), uy = FAST || (i < p.Nx - 1 && k < p.Nz - 1),
             uz = FAST || (i < p.Nx - 1 && j < p.Ny - 1);
  v.c = c;
  v.ux = ux;
  v.uy = uy;
  v.uz = uz;
  // Every load is issued before any store: the field arrays may alias as far as the compiler
  // knows, so interleaving would serialise one memory round trip per component.
  v.ex = ld<T, C>(p.E[0] + c);
  v.ey = ld<T, C>(p.E[1] + c);
  v.ez = ld<T, C>(p.E[2] + c);
  v.ez_j = ux ? ld<T, C>(p.E[2] + c + p.sj) : C(0);
  v.ey_k = ux ? ld<T, C>(p.E[1] + c + 1) : C(0);
  v.ex_k = uy ? ld<T, C>(p.E[0] + c + 1) : C(0);
  v.ez_i = uy ? ld<T, C>(p.E[2] + c + p.si) : C(0);
  v.ey_i = uz ? ld<T, C>(p.E[1] + c + p.si) : C(0);
  v.ex_j = uz ? ld<T, C>(p.E[0] + c + p.sj) : C(0);
  v.hx = ux ? ld<T, C>(p.H[0] + c) : C(0);
  v.hy = uy ? ld<T, C>(p.H[1] + c) : C(0);
  v.hz = uz ? ld<T, C>(p.H[2] + c) : C(0);
}

template <class T, class C, bool UNI, bool FAST = false>
__device__ __forceinline__ void h_apply(const StepParams<T, C>& p, const int i, const int j, const int k, bool tf,
                                        const HCell<C>& v) {
  const long long c = v.c;
  const bool ux = FAST || v.ux, uy = FAST || v.uy, uz = FAST || v.uz;
  if (FAST) tf = false;
  const C ex = v.ex, ey = v.ey, ez = v.ez, ez_j = v.ez_j, ey_k = v.ey_k, ex_k = v.ex_k, ez_i = v.ez_i, ey_i = v.ey_i,
          ex_j = v.ex_j, hx = v.hx, hy = v.hy, hz = v.hz;
  int sx = -1, sy = -1, sz = -1;
  if (!FAST && p.pml) {
    sx = slab_index(p.slab[0], i);
    sy = slab_index(p.slab[1], j);
    sz = slab_index(p.slab[2], k);
  }
  C nhx = hx, nhy = hy, nhz = hz;
  // Hx: i < Nx, j < Ny-1, k < Nz-1; part 1 = dEz/dy (y profile), part 2 = dEy/dz (z profile)
  if (ux) {
    C d1 = ez_j - ez, d2 = ey_k - ey;
    if (!UNI) { d1 = mulC(d1, p.rd[1]); d2 = mulC(d2, p.rd[2]); }
    if (tf) {
      tfsf_apply<C>(p.setsH[0][0], p.tab, i, j, k, d1);
      tfsf_apply<C>(p.setsH[0][1], p.tab, i, j, k, d2);
    }
    if (sy >= 0) d1 = pml_term<C>(d1, p.psiH[0][0] + psi_index(1, p.slab[1], sy, i, j, k, p.Ny, p.Nzp), p.bH[1][j], p.cH[1][j], p.rkH[1][j]);
    if (sz >= 0) d2 = pml_term<C>(d2, p.psiH[0][1] + psi_index(2, p.slab[2], sz, i, j, k, p.Ny, p.Nzp), p.bH[2][k], p.cH[2][k], p.rkH[2][k]);
    nhx = fmaC(-p.Dbs, d1 - d2, hx);
  }
  // Hy: i < Nx-1, j < Ny, k < Nz-1; part 1 = dEx/dz (z), part 2 = dEz/dx (x)
  if (uy) {
    C d1 = ex_k - ex, d2 = ez_i - ez;
    if (!UNI) { d1 = mulC(d1, p.rd[2]); d2 = mulC(d2, p.rd[0]); }
    if (tf) {
      tfsf_apply<C>(p.setsH[1][0], p.tab, i, j, k, d1);
      tfsf_apply<C>(p.setsH[1][1], p.tab, i, j, k, d2);
    }
    if (sz >= 0) d1 = pml_term<C>(d1, p.psiH[1][0] + psi_index(2, p.slab[2], sz, i, j, k, p.Ny, p.Nzp), p.bH[2][k], p.cH[2][k], p.rkH[2][k]);
    if (sx >= 0) d2 = pml_term<C>(d2, p.psiH[1][1] + psi_index(0, p.slab[0], sx, i, j, k, p.Ny, p.Nzp), p.bH[0][i], p.cH[0][i], p.rkH[0][i]);
    nhy = fmaC(-p.Dbs, d1 - d2, hy);
  }
  // Hz: i < Nx-1, j < Ny-1, k < Nz; part 1 = dEy/dx (x), part 2 = dEx/dy (y)
  if (uz) {
    C d1 = ey_i - ey, d2 = ex_j - ex;
    if (!UNI) { d1 = mulC(d1, p.rd[0]); d2 = mulC(d2, p.rd[1]); }
    if (tf) {
      tfsf_apply<C>(p.setsH[2][0], p.tab, i, j, k, d1);
      tfsf_apply<C>(p.setsH[2][1], p.tab, i, j, k, d2);
    }
    if (sx >= 0) d1 = pml_term<C>(d1, p.psiH[2][0] + psi_index(0, p.slab[0], sx, i, j, k, p.Ny, p.Nzp), p.bH[0][i], p.cH[0][i], p.rkH[0][i]);
    if (sy >= 0) d2 = pml_term<C>(d2, p.psiH[2][1] + psi_index(1, p.slab[1], sy, i, j, k, p.Ny, p.Nzp), p.bH[1][j], p.cH[1][j], p.rkH[1][j]);
    nhz = fmaC(-p.Dbs, d1 - d2, hz);
  }
  if (ux) st<T, C>(p.H[0] + c, nhx);
  if (uy) st<T, C>(p.H[1] + c, nhy);
  if (uz) st<T, C>(p.H[2] + c, nhz);
}

template <class T, class C, bool UNI, bool FAST = false>
__device__ __forceinline__ void h_cell_3d(const StepParams<T, C>& p, const int i, const int j, const int k,
                                          const bool tf) {
  HCell<C> v;
  h_load<T, C, FAST>(p, i, j, k, v);
  h_apply<T, C, UNI, FAST>(p, i, j, k, tf, v);
}

// Resident blocks per SM asked of the compiler for the H kernel (a register cap): 8 for
// float compute (32 registers, 12-16 bytes spilled; FP16 storage 14 % faster than at 40
// registers), 5 for FP64 (its natural 48 registers; an explicit 1 lets the compiler take 54).
template <class C>
struct HMinBlocks {
  static constexpr int v = sizeof(C) == 4 ? 8 : 5;
};

// The z cells of a 3-D block.  Plain tiles are ZW consecutive cells (32, or 16 for float
// storage: a block is ZW z cells x 256/ZW y rows).  With zends (FP64 grids whose z CPML slabs
// are at most 16 cells wide; ZW = 32), tile 0 is the row's two ends, k in [0, 16) and
// [Nz-16, Nz), and tile m > 0 is [16 + 32(m-1), +32) up to Nz-16.  A 32-cell row's first and
// last tiles are half slab, and their warps run the z psi code with half the lanes idle; the
// end tile runs it once with all lanes busy, and sixteen doubles keep the other tiles on
// 128-byte lines.  Sixteen floats are half a line, so float storage takes 16-cell tiles
// instead: its slab tiles are whole slab, and half as many.  Each thread has one cell
// (valid = inside its tile's range).
struct ZTile {
  int k;
  bool valid;
  int lo0, n0, lo1, n1;  // the tile's cells: [lo0, lo0+n0) and [lo1, lo1+n1)
};

template <int ZW>
__device__ __forceinline__ ZTile z_tile(int Nz, bool ends) {
  ZTile z;
  const int lane = threadIdx.x;
  if (ZW != 32 || !ends) {
    z.lo0 = blockIdx.x * ZW;
    z.n0 = ZW;
    z.lo1 = z.n1 = 0;
    z.k = z.lo0 + lane;
    z.valid = z.k < Nz;
  } else if (blockIdx.x == 0) {
    z.lo0 = 0;
    z.n0 = 16;
    z.lo1 = Nz - 16;
    z.n1 = 16;
    z.k = lane < 16 ? lane : Nz - 32 + lane;
    z.valid = true;
  } else {
    z.lo0 = 16 + (blockIdx.x - 1) * 32;
    z.n0 = min(32, Nz - 16 - z.lo0);
    z.lo1 = z.n1 = 0;
    z.k = z.lo0 + lane;
    z.valid = lane < z.n0;
  }
  return z;
}

// Whether a 3-D block's tile (rows [j0, j0+nj)) meets a TF/SF plane.
__device__ __forceinline__ bool ztile_meets_planes(const int (&pl)[3][2], int i, int j0, int nj, const ZTile& z) {
  return tile_meets_planes(pl, i, 1, j0, nj, z.lo0, z.n0) || (z.n1 > 0 && tile_meets_planes(pl, i, 1, j0, nj, z.lo1, z.n1));
}

// One cell per thread; a block is ZW (z) x 256/ZW (y) cells of one x plane.  Blocks whose tile
// is interior take the cell code with every condition decided at compile time.
template <class T, class C, bool UNI, int ZW>
__global__ void __launch_bounds__(256, HMinBlocks<C>::v) h_kernel_3d(const StepParams<T, C> p) {
  constexpr int RY = 256 / ZW;
  const ZTile z = z_tile<ZW>(p.Nz, p.zends);
  const int k = z.k;
  const int j = blockIdx.y * RY + threadIdx.y;
  const int i = blockIdx.z;
  if (!z.valid || j >= p.Ny) return;
  const bool tf = p.tfsf && ztile_meets_planes(p.planesH, i, blockIdx.y * RY, RY, z);
  if (!tf && z.n1 == 0 && tile_is_interior(p.slab, p.pml, p.Nx, p.Ny, p.Nz, i, 1, blockIdx.y * RY, RY, z.lo0, z.n0))
    h_cell_3d<T, C, UNI, true>(p, i, j, k, false);
  else
    h_cell_3d<T, C, UNI>(p, i, j, k, tf);
}

// E half-step over cell (i,j,k) for Ex, Ey, Ez (three_dim_pml.cc:218-276, three_dim.cc:134-189).
// Only cells where the reference's H-curl is computed (vfield.cc:241-269: the transverse
// index in [1, N-2]) change; on the PEC walls the reference adds Cb*0 and psi stays 0.
// Returns the bit pattern of this cell's |E|^2 when monitoring (0 otherwise).
template <class C>
struct ECell {
  long long c;
  bool ux, uy, uz, mon;
  C hx, hy, hz, hz_j, hy_k, hx_k, hz_i, hy_i, hx_j, ex, ey, ez, cbx, cby, cbz;
};

template <class T, class C, bool MON, bool FAST = false>
__device__ __forceinline__ void e_load(const StepParams<T, C>& p, const int i, const int j, const int k, ECell<C>& v) {
  const long long c = (long long)i * p.si + (long long)j * p.sj + k;
  const bool ii = (i >= 1 && i < p.Nx - 1), jj = (j >= 1 && j < p.Ny - 1), kk = (k >= 1 && k < p.Nz - 1);
  const bool ux = FAST || (i < p.Nx - 1 && jj && kk), uy = FAST || (ii && j < p.Ny - 1 && kk),
             uz = FAST || (ii && jj && k < p.Nz - 1);
  const bool mon = MON && (FAST || (i < p.Nx - 1 && j < p.Ny - 1 && k < p.Nz - 1));
  v.c = c;
  v.ux = ux;
  v.uy = uy;
  v.uz = uz;
  v.mon = mon;
  // all loads first (see h_load)
  v.hx = ld<T, C>(p.H[0] + c);
  v.hy = ld<T, C>(p.H[1] + c);
  v.hz = ld<T, C>(p.H[2] + c);
  v.hz_j = ux ? ld<T, C>(p.H[2] + c - p.sj) : C(0);
  v.hy_k = ux ? ld<T, C>(p.H[1] + c - 1) : C(0);
  v.hx_k = uy ? ld<T, C>(p.H[0] + c - 1) : C(0);
  v.hz_i = uy ? ld<T, C>(p.H[2] + c - p.si) : C(0);
  v.hy_i = uz ? ld<T, C>(p.H[1] + c - p.si) : C(0);
  v.hx_j = uz ? ld<T, C>(p.H[0] + c - p.sj) : C(0);
  v.ex = (ux || mon) ? ld<T, C>(p.E[0] + c) : C(0);
  v.ey = (uy || mon) ? ld<T, C>(p.E[1] + c) : C(0);
  v.ez = (uz || mon) ? ld<T, C>(p.E[2] + c) : C(0);
  v.cbx = ux ? p.Cbs[0][c] : C(0);
  v.cby = uy ? p.Cbs[1][c] : C(0);
  v.cbz = uz ? p.Cbs[2][c] : C(0);
}

template <class T, class C, bool UNI, bool MON, bool FAST = false>
__device__ __forceinline__ typename MaxBits<C>::type e_apply(const StepParams<T, C>& p, const int i, const int j,
                                                             const int k, bool tf, const ECell<C>& v) {
  const long long c = v.c;
  const bool ux = FAST || v.ux, uy = FAST || v.uy, uz = FAST || v.uz, mon = MON && (FAST || v.mon);
  if (FAST) tf = false;
  const C hx = v.hx, hy = v.hy, hz = v.hz, hz_j = v.hz_j, hy_k = v.hy_k, hx_k = v.hx_k, hz_i = v.hz_i, hy_i = v.hy_i,
          hx_j = v.hx_j, ex = v.ex, ey = v.ey, ez = v.ez, cbx = v.cbx, cby = v.cby, cbz = v.cbz;
  int sx = -1, sy = -1, sz = -1;
  if (!FAST && p.pml) {
    sx = slab_index(p.slab[0], i);
    sy = slab_index(p.slab[1], j);
    sz = slab_index(p.slab[2], k);
  }
  C exn = ex, eyn = ey, ezn = ez;
  // Ex: i < Nx-1, j in [1,Ny-2], k in [1,Nz-2]; part 1 = dHz/dy (y), part 2 = dHy/dz (z)
  if (ux) {
    C d1 = hz - hz_j, d2 = hy - hy_k;
    if (!UNI) { d1 = mulC(d1, p.rd[1]); d2 = mulC(d2, p.rd[2]); }
    if (tf) {
      tfsf_apply<C>(p.setsE[0][0], p.tab, i, j, k, d1);
      tfsf_apply<C>(p.setsE[0][1], p.tab, i, j, k, d2);
    }
    if (sy >= 0) d1 = pml_term<C>(d1, p.psiE[0][0] + psi_index(1, p.slab[1], sy, i, j, k, p.Ny, p.Nzp), p.bE[1][j], p.cE[1][j], p.rkE[1][j]);
    if (sz >= 0) d2 = pml_term<C>(d2, p.psiE[0][1] + psi_index(2, p.slab[2], sz, i, j, k, p.Ny, p.Nzp), p.bE[2][k], p.cE[2][k], p.rkE[2][k]);
    exn = fmaC(cbx, d1 - d2, ex);
  }
  // Ey: i in [1,Nx-2], j < Ny-1, k in [1,Nz-2]; part 1 = dHx/dz (z), part 2 = dHz/dx (x)
  if (uy) {
    C d1 = hx - hx_k, d2 = hz - hz_i;
    if (!UNI) { d1 = mulC(d1, p.rd[2]); d2 = mulC(d2, p.rd[0]); }
    if (tf) {
      tfsf_apply<C>(p.setsE[1][0], p.tab, i, j, k, d1);
      tfsf_apply<C>(p.setsE[1][1], p.tab, i, j, k, d2);
    }
    if (sz >= 0) d1 = pml_term<C>(d1, p.psiE[1][0] + psi_index(2, p.slab[2], sz, i, j, k, p.Ny, p.Nzp), p.bE[2][k], p.cE[2][k], p.rkE[2][k]);
    if (sx >= 0) d2 = pml_term<C>(d2, p.psiE[1][1] + psi_index(0, p.slab[0], sx, i, j, k, p.Ny, p.Nzp), p.bE[0][i], p.cE[0][i], p.rkE[0][i]);
    eyn = fmaC(cby, d1 - d2, ey);
  }
  // Ez: i in [1,Nx-2], j in [1,Ny-2], k < Nz-1; part 1 = dHy/dx (x), part 2 = dHx/dy (y)
  if (uz) {
    C d1 = hy - hy_i, d2 = hx - hx_j;
    if (!UNI) { d1 = mulC(d1, p.rd[0]); d2 = mulC(d2, p.rd[1]); }
    if (tf) {
      tfsf_apply<C>(p.setsE[2][0], p.tab, i, j, k, d1);
      tfsf_apply<C>(p.setsE[2][1], p.tab, i, j, k, d2);
    }
    if (sx >= 0) d1 = pml_term<C>(d1, p.psiE[2][0] + psi_index(0, p.slab[0], sx, i, j, k, p.Ny, p.Nzp), p.bE[0][i], p.cE[0][i], p.rkE[0][i]);
    if (sy >= 0) d2 = pml_term<C>(d2, p.psiE[2][1] + psi_index(1, p.slab[1], sy, i, j, k, p.Ny, p.Nzp), p.bE[1][j], p.cE[1][j], p.rkE[1][j]);
    ezn = fmaC(cbz, d1 - d2, ez);
  }
  if (ux) st<T, C>(p.E[0] + c, exn);
  if (uy) st<T, C>(p.E[1] + c, eyn);
  if (uz) st<T, C>(p.E[2] + c, ezn);
  typename MaxBits<C>::type mbits = 0;
  if (mon) {
    // Etotal = Ez*Ez + Ey*Ey + Ex*Ex (three_dim_pml.cc:270), same association order
    const C e2 = fmaC(exn, exn, fmaC(eyn, eyn, ezn * ezn));
    if (p.etotal) p.etotal[c] = e2;
    mbits = MaxBits<C>::of(e2);
  }
  return mbits;
}

template <class T, class C, bool UNI, bool MON, bool FAST = false>
__device__ __forceinline__ typename MaxBits<C>::type e_cell_3d(const StepParams<T, C>& p, const int i, const int j,
                                                               const int k, const bool tf) {
  ECell<C> v;
  e_load<T, C, MON, FAST>(p, i, j, k, v);
  return e_apply<T, C, UNI, MON, FAST>(p, i, j, k, tf, v);
}

// Resident blocks per SM asked of the compiler for the 3-D E kernel: FP16 storage takes 8 (32
// registers, about 30 bytes spilled) together with the interior fast path, 0.3196 -> 0.3116 ms
// per 256^3 step (each alone was slower: the fast path 0.332, the cap 0.356); FP32 storage runs
// best at the compiler's own 40 (the cap cost it 4 %), and FP64 is bound by its pipe.
template <class T>
struct EMinBlocks {
  static constexpr int v = sizeof(T) == 2 ? 8 : 0;
};

template <class T, class C, bool UNI, bool MON, int ZW>
__global__ void __launch_bounds__(256, EMinBlocks<T>::v) e_kernel_3d(const StepParams<T, C> p) {
  constexpr int RY = 256 / ZW;
  const ZTile z = z_tile<ZW>(p.Nz, p.zends);
  const int k = z.k;
  const int j = blockIdx.y * RY + threadIdx.y;
  const int i = blockIdx.z;
  const bool tf = p.tfsf && ztile_meets_planes(p.planesE, i, blockIdx.y * RY, RY, z);
  typename MaxBits<C>::type mbits = 0;
  // The interior fast path pays for float compute (FP16 storage with the register cap above);
  // FP64 is bound by its pipe either way.
  constexpr bool kFast = sizeof(T) < 8;
  if (z.valid && j < p.Ny) {
    if (kFast && !tf && z.n1 == 0 && tile_is_interior(p.slab, p.pml, p.Nx, p.Ny, p.Nz, i, 1, blockIdx.y * RY, RY, z.lo0, z.n0))
      mbits = e_cell_3d<T, C, UNI, MON, kFast>(p, i, j, k, false);
    else
      mbits = e_cell_3d<T, C, UNI, MON>(p, i, j, k, tf);
  }
  if (MON && p.max_slot) block_max_atomic(mbits, p.max_slot);
}

// ------------------------------------------------------------------ planar kernels

// Planar H half-step (x-z plane, Ny = 1): Hx and Hz (two_dim_pml.cc:144-162, two_dim.cc:95-111).
// Loads (h2_load) are all issued before the update and stores (h2_apply).
template <class C>
struct HCell2 {
  long long c;
  bool ux, uz;
  C ey, ey_k, ey_i, hx, hz;
};

template <class T, class C, bool FAST = false>
__device__ __forceinline__ void h2_load(const StepParams<T, C>& p, const int i, const int k, HCell2<C>& v) {
  const long long c = (long long)i * p.si + k;
  const bool ux = FAST || k < p.Nz - 1, uz = FAST || i < p.Nx - 1;
  v.c = c;
  v.ux = ux;
  v.uz = uz;
  v.ey = ld<T, C>(p.E[1] + c);
  v.ey_k = ux ? ld<T, C>(p.E[1] + c + 1) : C(0);
  v.ey_i = uz ? ld<T, C>(p.E[1] + c + p.si) : C(0);
  v.hx = ux ? ld<T, C>(p.H[0] + c) : C(0);
  v.hz = uz ? ld<T, C>(p.H[2] + c) : C(0);
}

template <class T, class C, bool UNI, bool FAST = false>
__device__ __forceinline__ void h2_apply(const StepParams<T, C>& p, const int i, const int k, bool tf,
                                         const HCell2<C>& v) {
  const long long c = v.c;
  const bool ux = FAST || v.ux, uz = FAST || v.uz;
  if (FAST) tf = false;
  const C ey = v.ey, ey_k = v.ey_k, ey_i = v.ey_i, hx = v.hx, hz = v.hz;
  C nhx = hx, nhz = hz;
  // Hx: k < Nz-1; Hx -= Db*(-curl2/kappa - psi2), curl2 = dEy/dz (z profile)
  if (ux) {
    C d2 = ey_k - ey;
    if (!UNI) d2 = mulC(d2, p.rd[2]);
    if (tf) tfsf_apply<C>(p.setsH[0][1], p.tab, i, 0, k, d2);
    if (!FAST && p.pml) {
      const int sz = slab_index(p.slab[2], k);
      if (sz >= 0) d2 = pml_term<C>(d2, p.psiH[0][1] + (long long)i * p.slab[2].n + sz, p.bH[2][k], p.cH[2][k], p.rkH[2][k]);
    }
    nhx = fmaC(p.Dbs, d2, hx);
  }
  // Hz: i < Nx-1; Hz -= Db*(curl1/kappa + psi1), curl1 = dEy/dx (x profile)
  if (uz) {
    C d1 = ey_i - ey;
    if (!UNI) d1 = mulC(d1, p.rd[0]);
    if (tf) tfsf_apply<C>(p.setsH[2][0], p.tab, i, 0, k, d1);
    if (!FAST && p.pml) {
      const int sx = slab_index(p.slab[0], i);
      if (sx >= 0) d1 = pml_term<C>(d1, p.psiH[2][0] + (long long)sx * p.Nzp + k, p.bH[0][i], p.cH[0][i], p.rkH[0][i]);
    }
    nhz = fmaC(-p.Dbs, d1, hz);
  }
  if (ux) st<T, C>(p.H[0] + c, nhx);
  if (uz) st<T, C>(p.H[2] + c, nhz);
}

template <class T, class C, bool UNI, bool FAST = false>
__device__ __forceinline__ void h_cell_2d(const StepParams<T, C>& p, const int i, const int k, const bool tf) {
  HCell2<C> v;
  h2_load<T, C, FAST>(p, i, k, v);
  h2_apply<T, C, UNI, FAST>(p, i, k, tf, v);
}

// One cell per thread; a block is 32 (z) x 8 (x) cells.
template <class T, class C, bool UNI>
__global__ void __launch_bounds__(256) h_kernel_2d(const StepParams<T, C> p) {
  const int k = blockIdx.x * 32 + threadIdx.x;
  const int ib = blockIdx.y * 8, i = ib + threadIdx.y;
  if (k >= p.Nz || i >= p.Nx) return;
  const bool tf = p.tfsf && tile_meets_planes(p.planesH, ib, 8, 0, 1, blockIdx.x * 32, 32);
  if (!tf && tile_is_interior_2d(p.slab, p.pml, p.Nx, p.Nz, ib, 8, blockIdx.x * 32, 32))
    h_cell_2d<T, C, UNI, true>(p, i, k, false);
  else
    h_cell_2d<T, C, UNI>(p, i, k, tf);
}

// Planar E half-step: Ey (two_dim_pml.cc:164-181, two_dim.cc:113-128).  The reference loop
// covers i < Nx-1, k < Nz-1, but its H-curl is only computed for i, k in [1, N-2]
// (vfield.cc:376-381), so the other cells add Cb*0 and are skipped here.
template <class C>
struct ECell2 {
  long long c;
  bool u;
  C ey, hx, hx_k, hz, hz_i, cb;
};

template <class T, class C, bool MON, bool FAST = false>
__device__ __forceinline__ void e2_load(const StepParams<T, C>& p, const int i, const int k, ECell2<C>& v) {
  const long long c = (long long)i * p.si + k;
  const bool u = FAST || (i >= 1 && i < p.Nx - 1 && k >= 1 && k < p.Nz - 1);
  v.c = c;
  v.u = u;
  v.ey = (u || MON) ? ld<T, C>(p.E[1] + c) : C(0);
  v.hx = u ? ld<T, C>(p.H[0] + c) : C(0);
  v.hx_k = u ? ld<T, C>(p.H[0] + c - 1) : C(0);
  v.hz = u ? ld<T, C>(p.H[2] + c) : C(0);
  v.hz_i = u ? ld<T, C>(p.H[2] + c - p.si) : C(0);
  v.cb = u ? p.Cbs[1][c] : C(0);
}

template <class T, class C, bool UNI, bool MON, bool FAST = false>
__device__ __forceinline__ typename MaxBits<C>::type e2_apply(const StepParams<T, C>& p, const int i, const int k,
                                                              bool tf, const ECell2<C>& v) {
  const long long c = v.c;
  const C ey = v.ey;
  C eyn = ey;
  if (FAST) tf = false;
  if (FAST || v.u) {
    C d1 = v.hx - v.hx_k;  // dHx/dz (z profile)
    C d2 = v.hz - v.hz_i;  // dHz/dx (x profile)
    if (!UNI) { d1 = mulC(d1, p.rd[2]); d2 = mulC(d2, p.rd[0]); }
    if (tf) {
      tfsf_apply<C>(p.setsE[1][0], p.tab, i, 0, k, d1);
      tfsf_apply<C>(p.setsE[1][1], p.tab, i, 0, k, d2);
    }
    if (!FAST && p.pml) {
      const int sz = slab_index(p.slab[2], k), sx = slab_index(p.slab[0], i);
      if (sz >= 0) d1 = pml_term<C>(d1, p.psiE[1][0] + (long long)i * p.slab[2].n + sz, p.bE[2][k], p.cE[2][k], p.rkE[2][k]);
      if (sx >= 0) d2 = pml_term<C>(d2, p.psiE[1][1] + (long long)sx * p.Nzp + k, p.bE[0][i], p.cE[0][i], p.rkE[0][i]);
    }
    eyn = fmaC(v.cb, d1 - d2, ey);
    st<T, C>(p.E[1] + c, eyn);
  }
  // local_max = max(Ey*Ey) over the whole Ey array (two_dim_pml.cc:181)
  return MON ? MaxBits<C>::of(eyn * eyn) : typename MaxBits<C>::type(0);
}

template <class T, class C, bool UNI, bool MON, bool FAST = false>
__device__ __forceinline__ typename MaxBits<C>::type e_cell_2d(const StepParams<T, C>& p, const int i, const int k,
                                                               const bool tf) {
  ECell2<C> v;
  e2_load<T, C, MON, FAST>(p, i, k, v);
  return e2_apply<T, C, UNI, MON, FAST>(p, i, k, tf, v);
}

template <class T, class C, bool UNI, bool MON>
__global__ void __launch_bounds__(256) e_kernel_2d(const StepParams<T, C> p) {
  const int k = blockIdx.x * 32 + threadIdx.x;
  const int ib = blockIdx.y * 8, i = ib + threadIdx.y;
  const bool tf = p.tfsf && tile_meets_planes(p.planesE, ib, 8, 0, 1, blockIdx.x * 32, 32);
  const bool fast = !tf && tile_is_interior_2d(p.slab, p.pml, p.Nx, p.Nz, ib, 8, blockIdx.x * 32, 32);
  typename MaxBits<C>::type mbits = 0;
  if (k < p.Nz && i < p.Nx) {
    if (fast) mbits = e_cell_2d<T, C, UNI, MON, true>(p, i, k, false);
    else mbits = e_cell_2d<T, C, UNI, MON>(p, i, k, tf);
  }
  if (MON && p.max_slot) block_max_atomic(mbits, p.max_slot);
}

// ------------------------------------------------------------------ single-sweep planar step

// Planar step in one sweep, for float compute.  The two-sweep kernels above move 40 bytes per
// FP32 cell and step (H sweep: Ey read, Hx and Hz read and written; E sweep: Hx, Hz and Cb read,
// Ey read and written); one sweep moves the compulsory 28 (Ey, Hx, Hz and Cb read once, Ey, Hx
// and Hz written once).  A warp owns 32 z columns and R consecutive x rows and walks the rows in
// order.  At row i it forms H(i): Hx from Ey(i,k+1) (a shuffle) and Hz from Ey(i+1,k), the next
// row's value, which it keeps for the next iteration.  Then it forms E(i) from H(i), the Hx of
// column k-1 (a shuffle) and the Hz of row i-1, kept from the previous iteration.  Two values
// belong to other warps and are recomputed from the old state with the same code as their
// owners': Hz(i0-1) before the first row, and lane 0's Hx(i,k0-1).  State n is read from one
// buffer and state n+1 written to the other, so no warp sees a neighbour's new values, and every
// cell of the run is written (the cells a half step does not update keep their old value).  H
// enters E as stored (FP16 storage rounds it first), so the step matches the two-sweep kernels
// bit for bit.

// New Hx of planar cell (i,k), k < Nz-1: the arithmetic of h2_apply (two_dim_pml.cc:149-152).
// A null psi_out recomputes a neighbour's value and leaves its psi to the owner.
template <class T, class C, bool UNI, bool FAST>
__device__ __forceinline__ C hx2_value(const StepParams<T, C>& p, const C* psi_in, C* psi_out, int i, int k, C ey,
                                       C ey_k, C hx, bool tf) {
  C d2 = ey_k - ey;
  if (!UNI) d2 = mulC(d2, p.rd[2]);
  if (!FAST && tf) tfsf_apply<C>(p.setsH[0][1], p.tab, i, 0, k, d2);
  if (!FAST && p.pml) {
    const int sz = slab_index(p.slab[2], k);
    if (sz >= 0) {
      const long long q = (long long)i * p.slab[2].n + sz;
      const C ps = fmaC(p.bH[2][k], psi_in[q], p.cH[2][k] * d2);
      if (psi_out) psi_out[q] = ps;
      d2 = fmaC(d2, p.rkH[2][k], ps);
    }
  }
  return fmaC(p.Dbs, d2, hx);
}

// New Hz of planar cell (i,k), i < Nx-1 (two_dim_pml.cc:155-158).
template <class T, class C, bool UNI, bool FAST>
__device__ __forceinline__ C hz2_value(const StepParams<T, C>& p, const C* psi_in, C* psi_out, int i, int k, C ey,
                                       C ey_i, C hz, bool tf) {
  C d1 = ey_i - ey;
  if (!UNI) d1 = mulC(d1, p.rd[0]);
  if (!FAST && tf) tfsf_apply<C>(p.setsH[2][0], p.tab, i, 0, k, d1);
  if (!FAST && p.pml) {
    const int sx = slab_index(p.slab[0], i);
    if (sx >= 0) {
      const long long q = (long long)sx * p.Nzp + k;
      const C ps = fmaC(p.bH[0][i], psi_in[q], p.cH[0][i] * d1);
      if (psi_out) psi_out[q] = ps;
      d1 = fmaC(d1, p.rkH[0][i], ps);
    }
  }
  return fmaC(-p.Dbs, d1, hz);
}

// New Ey of planar cell (i,k), i and k in [1, N-2] (two_dim_pml.cc:164-176): e2_apply's arithmetic.
template <class T, class C, bool UNI, bool FAST>
__device__ __forceinline__ C ey2_value(const StepParams<T, C>& p, const C* pz_in, C* pz_out, const C* px_in, C* px_out,
                                       int i, int k, C ey, C hx, C hx_k, C hz, C hz_i, C cb, bool tf) {
  C d1 = hx - hx_k;  // dHx/dz (z profile)
  C d2 = hz - hz_i;  // dHz/dx (x profile)
  if (!UNI) { d1 = mulC(d1, p.rd[2]); d2 = mulC(d2, p.rd[0]); }
  if (!FAST && tf) {
    tfsf_apply<C>(p.setsE[1][0], p.tab, i, 0, k, d1);
    tfsf_apply<C>(p.setsE[1][1], p.tab, i, 0, k, d2);
  }
  if (!FAST && p.pml) {
    const int sz = slab_index(p.slab[2], k), sx = slab_index(p.slab[0], i);
    if (sz >= 0) {
      const long long q = (long long)i * p.slab[2].n + sz;
      const C ps = fmaC(p.bE[2][k], pz_in[q], p.cE[2][k] * d1);
      pz_out[q] = ps;
      d1 = fmaC(d1, p.rkE[2][k], ps);
    }
    if (sx >= 0) {
      const long long q = (long long)sx * p.Nzp + k;
      const C ps = fmaC(p.bE[0][i], px_in[q], p.cE[0][i] * d2);
      px_out[q] = ps;
      d2 = fmaC(d2, p.rkE[0][i], ps);
    }
  }
  return fmaC(cb, d1 - d2, ey);
}

// One warp's rows [i0, i1) of the 32 columns from k0; returns the bit pattern of its largest
// Ey^2 (the max over the whole Ey array, two_dim_pml.cc:181).
// The parameter block names the buffer read in E, H, psiH, psiE and the one written in E1,
// H1, psiH1, psiE1 (the host swaps them on odd steps).
template <class T, class C, bool UNI, bool FAST>
__device__ __forceinline__ typename MaxBits<C>::type step2_rows(const StepParams<T, C>& p, const int i0, const int i1,
                                                                const int k0, const bool tfH, const bool tfE) {
  const int lane = threadIdx.x;
  const int k = k0 + lane;
  const int Nx = p.Nx, Nz = p.Nz;
  const T* eyi = p.E[1];
  T* eyo = p.E1[1];
  const T* hxi = p.H[0];
  T* hxo = p.H1[0];
  const T* hzi = p.H[2];
  T* hzo = p.H1[2];
  const C* qhx = p.psiH[0][1];  // Hx, z part
  C* qhxo = p.psiH1[0][1];
  const C* qhz = p.psiH[2][0];  // Hz, x part
  C* qhzo = p.psiH1[2][0];
  const C* qez = p.psiE[1][0];  // Ey, z part
  C* qezo = p.psiE1[1][0];
  const C* qex = p.psiE[1][1];  // Ey, x part
  C* qexo = p.psiE1[1][1];
  const bool kin = FAST || k < Nz;
  const bool ux = FAST || k < Nz - 1;
  const bool ke = FAST || (k >= 1 && k < Nz - 1);
  const long long si = p.si;
  long long c = (long long)i0 * si + k;
  C ey = kin ? ld<T, C>(eyi + c) : C(0);
  C hz_p = C(0);  // new Hz of the row above
  if (i0 >= 1) {
    const C eym = kin ? ld<T, C>(eyi + c - si) : C(0);
    const C hzm = kin ? ld<T, C>(hzi + c - si) : C(0);
    hz_p = stored<T, C>(hz2_value<T, C, UNI, FAST>(p, qhz, nullptr, i0 - 1, k, eym, ey, hzm, tfH));
  }
  typename MaxBits<C>::type m = 0;
#pragma unroll 1
  for (int i = i0; i < i1; ++i, c += si) {
    const bool nx = FAST || i + 1 < Nx;
    const bool ue = ke && (FAST || (i >= 1 && i < Nx - 1));
    const C eyn = (kin && nx) ? ld<T, C>(eyi + c + si) : C(0);
    const C hx = kin ? ld<T, C>(hxi + c) : C(0);
    const C hz = kin ? ld<T, C>(hzi + c) : C(0);
    const C cb = (kin && ue) ? p.Cbs[1][c] : C(0);
    C ey_k = __shfl_down_sync(0xffffffffu, ey, 1);
    if (lane == 31) ey_k = (FAST || k + 1 < Nz) ? ld<T, C>(eyi + c + 1) : C(0);
    C hxh = C(0), eyh = C(0);  // lane 0: Hx and Ey of column k0-1
    if (lane == 0 && k0 >= 1) {
      hxh = ld<T, C>(hxi + c - 1);
      eyh = ld<T, C>(eyi + c - 1);
    }
    const C hxn = (kin && ux) ? stored<T, C>(hx2_value<T, C, UNI, FAST>(p, qhx, qhxo, i, k, ey, ey_k, hx, tfH)) : hx;
    const C hzn = (kin && nx) ? stored<T, C>(hz2_value<T, C, UNI, FAST>(p, qhz, qhzo, i, k, ey, eyn, hz, tfH)) : hz;
    C hx_k = __shfl_up_sync(0xffffffffu, hxn, 1);
    if (lane == 0)
      hx_k = k0 >= 1 ? stored<T, C>(hx2_value<T, C, UNI, FAST>(p, qhx, nullptr, i, k0 - 1, eyh, ey, hxh, tfH)) : C(0);
    const C eyw = (kin && ue) ? ey2_value<T, C, UNI, FAST>(p, qez, qezo, qex, qexo, i, k, ey, hxn, hx_k, hzn, hz_p, cb, tfE)
                              : ey;
    if (kin) {
      st<T, C>(hxo + c, hxn);
      st<T, C>(hzo + c, hzn);
      st<T, C>(eyo + c, eyw);
      const typename MaxBits<C>::type b = MaxBits<C>::of(eyw * eyw);
      m = b > m ? b : m;
    }
    hz_p = hzn;
    ey = eyn;
  }
  return m;
}

// A warp's run with its TF/SF and interior tests: H is formed on rows [i0-1, i1) and columns
// [k0-1, k0+32), E on rows [i0, i1) and columns [k0, k0+32).
template <class T, class C, bool UNI>
__device__ __forceinline__ typename MaxBits<C>::type step2_warp(const StepParams<T, C>& p, const int i0, const int i1,
                                                                const int k0) {
  const bool tfH = p.tfsf && tile_meets_planes(p.planesH, i0 - 1, i1 - i0 + 1, 0, 1, k0 - 1, 34);
  const bool tfE = p.tfsf && tile_meets_planes(p.planesE, i0, i1 - i0, 0, 1, k0, 32);
  if (!tfH && !tfE && tile_is_interior_2d(p.slab, p.pml, p.Nx, p.Nz, i0 - 1, i1 - i0 + 2, k0 - 1, 34))
    return step2_rows<T, C, UNI, true>(p, i0, i1, k0, false, false);
  return step2_rows<T, C, UNI, false>(p, i0, i1, k0, tfH, tfE);
}

// Register cap of the single-sweep kernel: 6 blocks of 256 per SM (40 registers, no spills).
constexpr int kSweepMinBlocks = 6;

// One simulation: a block is 32 z columns x 8 warps of R rows.
template <class T, class C, bool UNI, int R>
__global__ void __launch_bounds__(256, kSweepMinBlocks) step_kernel_2d(const StepParams<T, C> p) {
  const int k0 = blockIdx.x * 32;
  const int i0 = (blockIdx.y * 8 + threadIdx.y) * R;
  typename MaxBits<C>::type m = 0;
  if (i0 < p.Nx) m = step2_warp<T, C, UNI>(p, i0, min(i0 + R, p.Nx), k0);
  if (p.max_slot) block_max_atomic(m, p.max_slot);
}

// ------------------------------------------------------------------ batched update kernels

__device__ __forceinline__ int find_member(const int* __restrict__ first, int n, int t) {
  int lo = 0, hi = n;  // first[lo] <= t < first[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (first[mid] <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Block map of a batched launch: member m owns blocks [first[m], first[m+1]).  Built on the
// device once per change of membership, so that a block of the update kernels finds its
// member and tile with one 16-byte load: {member, a, b, c} with a = first x plane (3-D) or
// first x row (planar), b = first y row (3-D), c = first z cell.
template <class T, class C>
__global__ void batch_tiles_kernel(const StepParams<T, C>* __restrict__ ps, const int* __restrict__ first, int n,
                                   int nblocks, int planar, int march, int4* __restrict__ tiles) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nblocks; t += gridDim.x * blockDim.x) {
    const int m = find_member(first, n, t);
    const int lt = t - first[m];
    const StepParams<T, C>& p = ps[m];
    const int nkb = (p.Nz + 31) / 32;
    if (planar) {
      tiles[t] = make_int4(m, (lt / nkb) * 8 * march, 0, (lt % nkb) * 32);
    } else {
      const int njb = (p.Ny + 7) / 8;
      tiles[t] = make_int4(m, (lt / (nkb * njb)) * march, ((lt / nkb) % njb) * 8, (lt % nkb) * 32);
    }
  }
}

// DFT planes of a batch: block -> {plane, block within the plane}.
__global__ void block_map_kernel(const int* __restrict__ first, int n, int nblocks, int2* __restrict__ map) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nblocks; t += gridDim.x * blockDim.x) {
    const int m = find_member(first, n, t);
    map[t] = make_int2(m, t - first[m]);
  }
}

// Resident blocks per SM asked of the compiler for the batched 3-D kernels: 5 for float
// compute (48 registers instead of 72, a few spilled; 21.5 -> 30.1 Gcell/s on 16 CPML
// cubes), 3 (no effective cap) for FP64.
template <class C>
struct B3MinBlocks {
  static constexpr int v = sizeof(C) == 4 ? 5 : 3;
};

// 3-D members: a block is 32 z x 8 y cells over M consecutive x planes.
template <class T, class C, bool UNI, int M>
__global__ void __launch_bounds__(256, B3MinBlocks<C>::v) h_batch_3d(const StepParams<T, C>* __restrict__ ps, const int4* __restrict__ tiles) {
  const int4 tl = tiles[blockIdx.x];
  const StepParams<T, C>& p = ps[tl.x];
  const int k = tl.w + threadIdx.x, j = tl.z + threadIdx.y, i0 = tl.y;
  if (k >= p.Nz || j >= p.Ny) return;
  const bool tf = p.tfsf && tile_meets_planes(p.planesH, i0, M, tl.z, 8, tl.w, 32);
  const int i1 = min(i0 + M, p.Nx);
  if (!tf && tile_is_interior(p.slab, p.pml, p.Nx, p.Ny, p.Nz, i0, M, tl.z, 8, tl.w, 32)) {
#pragma unroll 1
    for (int i = i0; i < i1; ++i) h_cell_3d<T, C, UNI, true>(p, i, j, k, false);
  } else {
#pragma unroll 1
    for (int i = i0; i < i1; ++i) h_cell_3d<T, C, UNI>(p, i, j, k, tf);
  }
}

template <class T, class C, bool UNI, int M>
__global__ void __launch_bounds__(256, B3MinBlocks<C>::v) e_batch_3d(const StepParams<T, C>* __restrict__ ps, const int4* __restrict__ tiles) {
  const int4 tl = tiles[blockIdx.x];
  const StepParams<T, C>& p = ps[tl.x];
  const int k = tl.w + threadIdx.x, j = tl.z + threadIdx.y, i0 = tl.y;
  const bool tf = p.tfsf && tile_meets_planes(p.planesE, i0, M, tl.z, 8, tl.w, 32);
  typename MaxBits<C>::type mbits = 0;
  if (k < p.Nz && j < p.Ny) {
    const int i1 = min(i0 + M, p.Nx);
    if (!tf && tile_is_interior(p.slab, p.pml, p.Nx, p.Ny, p.Nz, i0, M, tl.z, 8, tl.w, 32)) {
#pragma unroll 1
      for (int i = i0; i < i1; ++i) {
        const typename MaxBits<C>::type b = e_cell_3d<T, C, UNI, true, true>(p, i, j, k, false);
        mbits = b > mbits ? b : mbits;
      }
    } else {
#pragma unroll 1
      for (int i = i0; i < i1; ++i) {
        const typename MaxBits<C>::type b = e_cell_3d<T, C, UNI, true>(p, i, j, k, tf);
        mbits = b > mbits ? b : mbits;
      }
    }
  }
  if (p.max_slot) block_max_atomic(mbits, p.max_slot);
}

// planar members: a block is 32 z cells x 8*M x rows.  Rows are walked one after the
// other: issuing all rows' loads first doubles the registers, halves the resident blocks and
// ran 25 % slower.  Interior tiles issue the next row's loads before the current row's update
// and stores: two rows in flight per thread at the same 32 registers (each row's cells are
// written only by their own thread, and the rows are 8 apart); the 256-lens batch ran 103 ->
// 111 Gcell/s.  The same in the general tiles took 46-48 registers and ran 90.
template <class T, class C, bool UNI, int M>
__global__ void __launch_bounds__(256) h_batch_2d(const StepParams<T, C>* __restrict__ ps, const int4* __restrict__ tiles) {
  const int4 tl = tiles[blockIdx.x];
  const StepParams<T, C>& p = ps[tl.x];
  const int k = tl.w + threadIdx.x;
  if (k >= p.Nz) return;
  const bool tf = p.tfsf && tile_meets_planes(p.planesH, tl.y, 8 * M, 0, 1, tl.w, 32);
  const bool fast = !tf && tile_is_interior_2d(p.slab, p.pml, p.Nx, p.Nz, tl.y, 8 * M, tl.w, 32);
  if (fast) {
    const int i0 = tl.y + threadIdx.y;
    HCell2<C> v[2];
    h2_load<T, C, true>(p, i0, k, v[0]);
#pragma unroll
    for (int r = 0; r < M; ++r) {
      if (r + 1 < M) h2_load<T, C, true>(p, i0 + 8 * (r + 1), k, v[(r + 1) & 1]);
      h2_apply<T, C, UNI, true>(p, i0 + 8 * r, k, false, v[r & 1]);
    }
    return;
  }
#pragma unroll 1
  for (int r = 0; r < M; ++r) {
    const int i = tl.y + threadIdx.y + 8 * r;
    if (i < p.Nx) h_cell_2d<T, C, UNI>(p, i, k, tf);
  }
}

// With float compute capped at 8 blocks per SM, 32 registers: left to itself the compiler took
// 40 for this kernel once the interior path prefetched, which leaves 6 blocks.  FP64 (doubles
// take register pairs) is left uncapped: at 32 registers it spilled 48 bytes.
template <class C>
struct E2BatchMinBlocks {
  static constexpr int v = sizeof(C) == 4 ? 8 : 1;
};
template <class T, class C, bool UNI, int M>
__global__ void __launch_bounds__(256, E2BatchMinBlocks<C>::v) e_batch_2d(const StepParams<T, C>* __restrict__ ps, const int4* __restrict__ tiles) {
  const int4 tl = tiles[blockIdx.x];
  const StepParams<T, C>& p = ps[tl.x];
  const int k = tl.w + threadIdx.x;
  const bool tf = p.tfsf && tile_meets_planes(p.planesE, tl.y, 8 * M, 0, 1, tl.w, 32);
  const bool fast = !tf && tile_is_interior_2d(p.slab, p.pml, p.Nx, p.Nz, tl.y, 8 * M, tl.w, 32);
  typename MaxBits<C>::type mbits = 0;
  if (fast && k < p.Nz) {  // interior tile: the next row's loads first (see h_batch_2d)
    const int i0 = tl.y + threadIdx.y;
    ECell2<C> v[2];
    e2_load<T, C, true, true>(p, i0, k, v[0]);
#pragma unroll
    for (int r = 0; r < M; ++r) {
      if (r + 1 < M) e2_load<T, C, true, true>(p, i0 + 8 * (r + 1), k, v[(r + 1) & 1]);
      const typename MaxBits<C>::type b = e2_apply<T, C, UNI, true, true>(p, i0 + 8 * r, k, false, v[r & 1]);
      mbits = b > mbits ? b : mbits;
    }
  } else if (k < p.Nz) {
#pragma unroll 1
    for (int r = 0; r < M; ++r) {
      const int i = tl.y + threadIdx.y + 8 * r;
      typename MaxBits<C>::type b = 0;
      if (i < p.Nx) b = e_cell_2d<T, C, UNI, true>(p, i, k, tf);
      mbits = b > mbits ? b : mbits;
    }
  }
  if (p.max_slot) block_max_atomic(mbits, p.max_slot);
}

// ------------------------------------------------------------------ data movement

// The three kernels below walk an (n0, n1, n2) block of a padded (Nx, Ny, Nzp) array one
// warp per (i, j) row: the row index fits 32 bits (the launchers hold n0*n1 to 2^30), one division
// per row gives (i, j), and the lanes stride the row's k.  An element-wise 64-bit q -> (i, j, k)
// split costs two 64-bit divisions per element, which the GPU emulates on the FP64 pipe.
constexpr int kRowWarps = 8;  // warps (rows in flight) per 256-thread block

__device__ __forceinline__ double as_double(double v) { return v; }
__device__ __forceinline__ double as_double(float v) { return (double)v; }
__device__ __forceinline__ double as_double(__half v) { return (double)__half2float(v); }

// padded storage -> dense double array of extent (n0,n1,n2)
template <class T>
__global__ void __launch_bounds__(256) gather_kernel(const T* __restrict__ src, double* __restrict__ dst, int n0,
                                                     int n1, int n2, int Ny, int Nzp, double mul) {
  const int lane = threadIdx.x & 31;
  const int rows = n0 * n1;
  const bool scale = mul != 1.0;
  for (int r = blockIdx.x * kRowWarps + (threadIdx.x >> 5); r < rows; r += gridDim.x * kRowWarps) {
    const int i = r / n1, j = r - i * n1;
    const T* s = src + ((long long)i * Ny + j) * Nzp;
    double* d = dst + (long long)r * n2;
    // two loops, so that a plain copy issues no FP64 compare or multiply per element (the FP64
    // pipe is the narrowest on this GPU)
    if (scale)
      for (int k = lane; k < n2; k += 32) d[k] = as_double(s[k]) * mul;
    else
      for (int k = lane; k < n2; k += 32) d[k] = as_double(s[k]);
  }
}

// dense double array -> padded storage (optionally Cb-style transform)
// mode 0: dst = v; mode 1: dst = v * a (Cb -> Cb/dx); mode 2: Cb = dt/(eps0*(1+F*scale)) * a
template <class T>
__global__ void __launch_bounds__(256) scatter_kernel(const double* __restrict__ src, T* __restrict__ dst, int n0,
                                                      int n1, int n2, int Ny, int Nzp, int mode, double a, double dt,
                                                      double eps0, double scale) {
  const int lane = threadIdx.x & 31;
  const int rows = n0 * n1;
  for (int r = blockIdx.x * kRowWarps + (threadIdx.x >> 5); r < rows; r += gridDim.x * kRowWarps) {
    const int i = r / n1, j = r - i * n1;
    const double* s = src + (long long)r * n2;
    T* d = dst + ((long long)i * Ny + j) * Nzp;
    for (int k = lane; k < n2; k += 32) {
      double v = s[k];
      if (mode == 2) {
        // epsilon0*(1+F*1000000) then dt/that (three_dim_pml.cc:122-128), no contraction
        const double e = __dmul_rn(eps0, __dadd_rn(1.0, __dmul_rn(v, scale)));
        v = __ddiv_rn(dt, e);
      }
      if (mode >= 1) v = __dmul_rn(v, a);
      if constexpr (sizeof(T) == 2) d[k] = __double2half(v);
      else d[k] = (T)v;
    }
  }
}

// Cb = dt/(eps0*eps_r) * a over the box [lo, hi) clipped to the extent
template <class C>
__global__ void __launch_bounds__(256) eps_box_kernel(C* dst, int n0, int n1, int n2, int Ny, int Nzp, int lo0,
                                                      int lo1, int lo2, int hi0, int hi1, int hi2, double val) {
  const int a0 = max(lo0, 0), a1 = max(lo1, 0), a2 = max(lo2, 0);
  const int b0 = min(hi0, n0), b1 = min(hi1, n1), b2 = min(hi2, n2);
  if (a0 >= b0 || a1 >= b1 || a2 >= b2) return;
  const int w1 = b1 - a1;
  const int rows = (b0 - a0) * w1;
  const int lane = threadIdx.x & 31;
  for (int r = blockIdx.x * kRowWarps + (threadIdx.x >> 5); r < rows; r += gridDim.x * kRowWarps) {
    const int di = r / w1;
    C* d = dst + ((long long)(a0 + di) * Ny + a1 + (r - di * w1)) * Nzp;
    for (int k = a2 + lane; k < b2; k += 32) d[k] = (C)val;
  }
}

template <class T>
__global__ void probe_kernel(const ProbeParams pp, const T* f0, const T* f1, const T* f2, const T* f3, const T* f4,
                             const T* f5, double* out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= pp.nprobes * 6) return;
  const int probe = q / 6, comp = q % 6;
  const T* f[6] = {f0, f1, f2, f3, f4, f5};
  const int i = pp.ijk[3 * probe], j = pp.ijk[3 * probe + 1], k = pp.ijk[3 * probe + 2];
  double v = 0.0;
  if (f[comp] && i >= 0 && j >= 0 && k >= 0 && i < pp.ext[comp][0] && j < pp.ext[comp][1] && k < pp.ext[comp][2]) {
    const T* src = f[comp] + ((long long)i * pp.Ny + j) * pp.Nzp + k;
    if constexpr (sizeof(T) == 2) v = (double)__half2float(*src);
    else v = (double)*src;
    if (comp >= 3 && pp.hmul != 1.0) v *= pp.hmul;
  }
  out[(long long)pp.row * pp.nprobes * 6 + q] = v;
}

// Phase factors of one sample of a DFT plane: cos/sin of omega*(t+1)*dt for the E
// components (sampled after the E update) and of omega*(t+0.5)*dt for the H components,
// formed once per plane and sample (the accumulating blocks then only read them).
__device__ __forceinline__ void dft_phase_body(const DftParams& d, const int t) {
  for (int f = threadIdx.x; f < d.nfreq; f += blockDim.x) {
    const double pe = __dmul_rn(d.omega[f], __dmul_rn((double)(t + 1), d.dt));
    const double ph = __dmul_rn(d.omega[f], __dmul_rn((double)t + 0.5, d.dt));
    double se, ce, sh, ch;
    sincos(pe, &se, &ce);
    sincos(ph, &sh, &ch);
    d.phase[f] = ce;
    d.phase[kMaxDftFreq + f] = se;
    d.phase[2 * kMaxDftFreq + f] = ch;
    d.phase[3 * kMaxDftFreq + f] = sh;
  }
}

__global__ void dft_phase_kernel(const DftParams d) { dft_phase_body(d, d.t); }

// Batched: one block per plane of a sampling class.
__global__ void dft_phase_batch_kernel(const DftParams* __restrict__ ds, const int* __restrict__ ts, int k) {
  const DftParams& d = ds[blockIdx.x];
  dft_phase_body(d, ts[d.sim] + k);
}

// Running DFT of the four tangential components on one plane.  Each thread owns one
// (component, cell) and updates its nfreq complex accumulators (coalesced along the cell),
// four frequencies at a time with their loads issued before their stores.
template <class T>
__device__ __forceinline__ void dft_body(const DftParams& d, const T* f0, const T* f1, const T* f2, const T* f3,
                                         const int lb) {
  __shared__ double cs[2][kMaxDftFreq], sn[2][kMaxDftFreq];
  for (int f = threadIdx.x; f < d.nfreq; f += blockDim.x) {
    cs[0][f] = d.phase[f];
    sn[0][f] = d.phase[kMaxDftFreq + f];
    cs[1][f] = d.phase[2 * kMaxDftFreq + f];
    sn[1][f] = d.phase[3 * kMaxDftFreq + f];
  }
  __syncthreads();
  const long long ncell = (long long)d.na * d.nb;
  const long long q = lb * (long long)blockDim.x + threadIdx.x;
  if (q >= 4 * ncell) return;
  const int comp = (int)(q / ncell);
  const long long cell = q % ncell;
  const int a = (int)(cell / d.nb), b = (int)(cell % d.nb);
  int u[3];
  u[d.axis] = d.index;
  u[d.axis == 0 ? 1 : 0] = a;
  u[d.axis == 2 ? 1 : 2] = b;
  const T* f = comp == 0 ? f0 : comp == 1 ? f1 : comp == 2 ? f2 : f3;
  double v = 0.0;
  if (f && u[0] < d.ext[comp][0] && u[1] < d.ext[comp][1] && u[2] < d.ext[comp][2]) {
    const T* src = f + ((long long)u[0] * d.Ny + u[1]) * d.Nzp + u[2];
    if constexpr (sizeof(T) == 2) v = (double)__half2float(*src);
    else v = (double)*src;
  }
  if (comp >= 2 && d.hmul != 1.0) v = __dmul_rn(v, d.hmul);
  v = __dmul_rn(v, d.weight);
  const int w = comp < 2 ? 0 : 1;
  double2* acc = reinterpret_cast<double2*>(d.acc) + (long long)comp * ncell + cell;
  const long long stride = 4 * ncell;  // from one frequency to the next
  int fq = 0;
  for (; fq + 4 <= d.nfreq; fq += 4) {
    double2 x[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) x[r] = acc[(fq + r) * stride];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      x[r].x = fma(v, cs[w][fq + r], x[r].x);
      x[r].y = fma(-v, sn[w][fq + r], x[r].y);
      acc[(fq + r) * stride] = x[r];
    }
  }
  for (; fq < d.nfreq; ++fq) {
    double2 x = acc[fq * stride];
    x.x = fma(v, cs[w][fq], x.x);
    x.y = fma(-v, sn[w][fq], x.y);
    acc[fq * stride] = x;
  }
}

template <class T>
__global__ void dft_kernel(const DftParams d, const T* f0, const T* f1, const T* f2, const T* f3) {
  dft_body<T>(d, f0, f1, f2, f3, blockIdx.x);
}

// Batched DFT planes: a flat launch over the planes sampled at this step; map gives each
// block its plane and its block within the plane.
template <class T>
__global__ void dft_batch_kernel(const DftParams* __restrict__ ds, const int2* __restrict__ map, const int* __restrict__ ts,
                                 int k) {
  const int2 bm = map[blockIdx.x];
  const DftParams& d = ds[bm.x];
  const int t = ts[d.sim] + k;
  if (t % d.every_ != 0) return;
  const void* const* f = (d.f1[0] || d.f1[1]) && ((t + 1) & 1) ? d.f1 : d.f;  // the state after step t
  dft_body<T>(d, (const T*)f[0], (const T*)f[1], (const T*)f[2], (const T*)f[3], bm.y);
}

// Net flux of a DFT plane per frequency: partial sums over fixed chunks of 1024 cells, then
// the chunks summed in order, so the result does not depend on scheduling.
__global__ void dft_flux_partial(const double* __restrict__ acc, int nfreq, long long ncell, double* __restrict__ part,
                                 int nchunk) {
  const int f = blockIdx.y, ch = blockIdx.x;
  const double2* a = reinterpret_cast<const double2*>(acc);
  double v = 0.0;
  const long long c0 = (long long)ch * 1024;
  for (long long c = c0 + threadIdx.x; c < c0 + 1024 && c < ncell; c += blockDim.x) {
    const double2 e1 = a[((long long)f * 4 + 0) * ncell + c], e2 = a[((long long)f * 4 + 1) * ncell + c];
    const double2 h1 = a[((long long)f * 4 + 2) * ncell + c], h2 = a[((long long)f * 4 + 3) * ncell + c];
    v += (e1.x * h2.x + e1.y * h2.y) - (e2.x * h1.x + e2.y * h1.y);
  }
  __shared__ double red[256];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(long long)f * nchunk + ch] = red[0];
}

__global__ void dft_flux_final(const double* __restrict__ part, int nfreq, int nchunk, double dA, double* __restrict__ out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nfreq) return;
  double v = 0.0;
  for (int c = 0; c < nchunk; ++c) v += part[(long long)f * nchunk + c];
  out[f] = v * dA;
}

// ------------------------------------------------------------------ launchers

// Blocks for a row-walking kernel: one warp per row, at most 16 blocks of 8 warps per SM.
static inline unsigned row_grid(long long rows) {
  const long long b = (rows + kRowWarps - 1) / kRowWarps;
  return (unsigned)(b < 152 * 16 ? b : 152 * 16);
}

static inline unsigned grid1d(long long n, int bs) {
  long long g = (n + bs - 1) / bs;
  if (g > 152LL * 64) g = 152LL * 64;
  return (unsigned)(g < 1 ? 1 : g);
}

template <class C>
cudaError_t launch_prologue(const PrologueParams& p, cudaStream_t s) {
  const int bs = 256;
  prologue_kernel<C><<<grid1d(p.tab_total > 0 ? p.tab_total : 1, bs), bs, 0, s>>>(p, (C*)p.tab);
  return cudaGetLastError();
}

// 16-cell z tiles for the 3-D E kernel with float storage (default); LUXUM_ZTILE=32 keeps the
// 32-cell tiles, read once per process.
static bool z16_tiles() {
  static const bool on = [] {
    const char* v = std::getenv("LUXUM_ZTILE");
    return !(v && std::strcmp(v, "32") == 0);
  }();
  return on;
}

template <class T, class C>
cudaError_t launch_step(const StepParams<T, C>& p, bool planar, bool uniform, bool h_half, cudaStream_t s) {
  // single simulations: one cell per thread (their parameters sit in the constant bank, and
  // walking several cells raises register use past what pays off)
  dim3 block(32, 8);
  const bool mon = p.max_slot || p.etotal;
  if (planar) {
    dim3 grid((p.Nz + 31) / 32, (p.Nx + 7) / 8, 1);
    if (h_half) {
      if (uniform) h_kernel_2d<T, C, true><<<grid, block, 0, s>>>(p);
      else h_kernel_2d<T, C, false><<<grid, block, 0, s>>>(p);
    } else if (mon) {
      if (uniform) e_kernel_2d<T, C, true, true><<<grid, block, 0, s>>>(p);
      else e_kernel_2d<T, C, false, true><<<grid, block, 0, s>>>(p);
    } else {
      if (uniform) e_kernel_2d<T, C, true, false><<<grid, block, 0, s>>>(p);
      else e_kernel_2d<T, C, false, false><<<grid, block, 0, s>>>(p);
    }
  } else {
    // FP64 with z CPML slabs of at most 16 cells: the rows' two ends share one tile (ZTile).
    // The E kernel with float storage takes 16-cell z tiles (LUXUM_ZTILE=32 keeps 32): on the
    // 256^3 drop-in grid E 0.2035 -> 0.189 ms (FP32), 0.200 -> 0.187 (FP16 storage), from its
    // CPML and TF/SF tiles; the H kernel ran 0.015 ms slower with them, CPML or not.
    StepParams<T, C> q = p;
    q.zends = sizeof(T) == 8 && p.pml && p.slab[2].n > 0 && p.slab[2].lo <= 16 && p.Nz - p.slab[2].hi0 <= 16 &&
              p.Nz >= 48;
    if (sizeof(T) < 8 && !h_half && z16_tiles()) {
      const dim3 block16(16, 16), grid16((p.Nz + 15) / 16, (p.Ny + 15) / 16, p.Nx);
      if (mon) {
        if (uniform) e_kernel_3d<T, C, true, true, 16><<<grid16, block16, 0, s>>>(q);
        else e_kernel_3d<T, C, false, true, 16><<<grid16, block16, 0, s>>>(q);
      } else {
        if (uniform) e_kernel_3d<T, C, true, false, 16><<<grid16, block16, 0, s>>>(q);
        else e_kernel_3d<T, C, false, false, 16><<<grid16, block16, 0, s>>>(q);
      }
      return cudaGetLastError();
    }
    dim3 grid(q.zends ? 1 + (p.Nz - 32 + 31) / 32 : (p.Nz + 31) / 32, (p.Ny + 7) / 8, p.Nx);
    if (h_half) {
      if (uniform) h_kernel_3d<T, C, true, 32><<<grid, block, 0, s>>>(q);
      else h_kernel_3d<T, C, false, 32><<<grid, block, 0, s>>>(q);
    } else if (mon) {
      if (uniform) e_kernel_3d<T, C, true, true, 32><<<grid, block, 0, s>>>(q);
      else e_kernel_3d<T, C, false, true, 32><<<grid, block, 0, s>>>(q);
    } else {
      if (uniform) e_kernel_3d<T, C, true, false, 32><<<grid, block, 0, s>>>(q);
      else e_kernel_3d<T, C, false, false, 32><<<grid, block, 0, s>>>(q);
    }
  }
  return cudaGetLastError();
}

template <class T, class C>
cudaError_t launch_step_sweep2(const StepParams<T, C>& p, bool uniform, cudaStream_t s) {
  // rows per warp: 16 where that still gives every SM 32 warps, fewer on small grids
  const long long cols = (p.Nz + 31) / 32;
  int R = 16;
  while (R > 2 && cols * ((p.Nx + R - 1) / R) < 152LL * 32) R /= 2;
  const dim3 block(32, 8), grid((unsigned)cols, (unsigned)((p.Nx + 8 * R - 1) / (8 * R)));
  switch (R * 2 + (uniform ? 1 : 0)) {
    case 32: step_kernel_2d<T, C, false, 16><<<grid, block, 0, s>>>(p); break;
    case 33: step_kernel_2d<T, C, true, 16><<<grid, block, 0, s>>>(p); break;
    case 16: step_kernel_2d<T, C, false, 8><<<grid, block, 0, s>>>(p); break;
    case 17: step_kernel_2d<T, C, true, 8><<<grid, block, 0, s>>>(p); break;
    case 8: step_kernel_2d<T, C, false, 4><<<grid, block, 0, s>>>(p); break;
    case 9: step_kernel_2d<T, C, true, 4><<<grid, block, 0, s>>>(p); break;
    case 4: step_kernel_2d<T, C, false, 2><<<grid, block, 0, s>>>(p); break;
    default: step_kernel_2d<T, C, true, 2><<<grid, block, 0, s>>>(p); break;
  }
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_gather(const T* src, double* dst, const int ext[3], int Ny, int Nzp, double mul, cudaStream_t s) {
  const long long rows = (long long)ext[0] * ext[1];
  if (rows == 0 || ext[2] == 0) return cudaSuccess;
  if (rows > (1LL << 30)) return cudaErrorInvalidValue;  // r + stride stays in int
  gather_kernel<T><<<row_grid(rows), 256, 0, s>>>(src, dst, ext[0], ext[1], ext[2], Ny, Nzp, mul);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_scatter(const double* src, T* dst, const int ext[3], int Ny, int Nzp, int mode, double a, double dt,
                           double eps0, double scale, cudaStream_t s) {
  const long long rows = (long long)ext[0] * ext[1];
  if (rows == 0 || ext[2] == 0) return cudaSuccess;
  if (rows > (1LL << 30)) return cudaErrorInvalidValue;  // r + stride stays in int
  scatter_kernel<T><<<row_grid(rows), 256, 0, s>>>(src, dst, ext[0], ext[1], ext[2], Ny, Nzp, mode, a, dt, eps0, scale);
  return cudaGetLastError();
}

template <class C>
cudaError_t launch_eps_box(C* dst, const int ext[3], int Ny, int Nzp, const int lo[3], const int hi[3], double val,
                           cudaStream_t s) {
  if ((long long)ext[0] * ext[1] > (1LL << 30)) return cudaErrorInvalidValue;
  eps_box_kernel<C><<<152 * 4, 256, 0, s>>>(dst, ext[0], ext[1], ext[2], Ny, Nzp, lo[0], lo[1], lo[2], hi[0], hi[1],
                                            hi[2], val);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_probes(const ProbeParams& pp, T* const f[6], double* out, cudaStream_t s) {
  const int n = pp.nprobes * 6;
  probe_kernel<T><<<(n + 127) / 128, 128, 0, s>>>(pp, f[0], f[1], f[2], f[3], f[4], f[5], out);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_dft(const DftParams& d, T* const f[4], cudaStream_t s) {
  const long long n = 4LL * d.na * d.nb;
  dft_phase_kernel<<<1, 128, 0, s>>>(d);
  dft_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, f[0], f[1], f[2], f[3]);
  return cudaGetLastError();
}

template <class T, class C>
cudaError_t launch_batch_tiles(const StepParams<T, C>* ps, const int* first, int n, int nblocks, bool planar, int march,
                               int4* tiles, cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  batch_tiles_kernel<T, C><<<grid1d(nblocks, 256), 256, 0, s>>>(ps, first, n, nblocks, planar ? 1 : 0, march, tiles);
  return cudaGetLastError();
}

template <class T, class C, int M>
static void batch_step_m(const StepParams<T, C>* ps, const int4* tiles, int nblocks, bool planar, bool uniform,
                         bool h_half, cudaStream_t s) {
  dim3 block(32, 8);
  if (planar) {
    if (h_half) {
      if (uniform) h_batch_2d<T, C, true, M><<<nblocks, block, 0, s>>>(ps, tiles);
      else h_batch_2d<T, C, false, M><<<nblocks, block, 0, s>>>(ps, tiles);
    } else {
      if (uniform) e_batch_2d<T, C, true, M><<<nblocks, block, 0, s>>>(ps, tiles);
      else e_batch_2d<T, C, false, M><<<nblocks, block, 0, s>>>(ps, tiles);
    }
  } else {
    if (h_half) {
      if (uniform) h_batch_3d<T, C, true, M><<<nblocks, block, 0, s>>>(ps, tiles);
      else h_batch_3d<T, C, false, M><<<nblocks, block, 0, s>>>(ps, tiles);
    } else {
      if (uniform) e_batch_3d<T, C, true, M><<<nblocks, block, 0, s>>>(ps, tiles);
      else e_batch_3d<T, C, false, M><<<nblocks, block, 0, s>>>(ps, tiles);
    }
  }
}

template <class T, class C>
cudaError_t launch_batch_step(const StepParams<T, C>* ps, const int4* tiles, int nblocks, bool planar, bool uniform,
                              int march, bool h_half, cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  switch (march) {
    case 1: batch_step_m<T, C, 1>(ps, tiles, nblocks, planar, uniform, h_half, s); break;
    case 2: batch_step_m<T, C, 2>(ps, tiles, nblocks, planar, uniform, h_half, s); break;
    case 4: batch_step_m<T, C, 4>(ps, tiles, nblocks, planar, uniform, h_half, s); break;
    case 8: batch_step_m<T, C, 8>(ps, tiles, nblocks, planar, uniform, h_half, s); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

int batch_blocks(int Nx, int Ny, int Nz, bool planar, int march) {
  if (planar) return ((Nz + 31) / 32) * ((Nx + 8 * march - 1) / (8 * march));
  return ((Nz + 31) / 32) * ((Ny + 7) / 8) * ((Nx + march - 1) / march);
}

cudaError_t launch_block_map(const int* first, int n, int nblocks, int2* map, cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  block_map_kernel<<<grid1d(nblocks, 256), 256, 0, s>>>(first, n, nblocks, map);
  return cudaGetLastError();
}

template <class C>
cudaError_t launch_prologue_batch(const PrologueParams* pps, const int* ts, int k, int nsims, int max_entries,
                                  cudaStream_t s) {
  if (nsims <= 0) return cudaSuccess;
  long long gx = (max_entries + 255) / 256;
  if (gx < 1) gx = 1;
  if (gx > 1024) gx = 1024;
  prologue_batch_kernel<C><<<dim3((unsigned)gx, (unsigned)nsims), 256, 0, s>>>(pps, ts, k);
  return cudaGetLastError();
}

cudaError_t launch_tick(int* ts, int n, int steps, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  tick_kernel<<<(n + 255) / 256, 256, 0, s>>>(ts, n, steps);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_dft_batch(const DftParams* ds, const int2* map, int nplanes, int nblocks, const int* ts, int k,
                             cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  dft_phase_batch_kernel<<<nplanes, 128, 0, s>>>(ds, ts, k);
  dft_batch_kernel<T><<<nblocks, 256, 0, s>>>(ds, map, ts, k);
  return cudaGetLastError();
}

cudaError_t launch_dft_flux(const double* acc, int nfreq, long long ncell, double* part, double dA, double* out,
                            cudaStream_t s) {
  const int nchunk = (int)((ncell + 1023) / 1024);
  dft_flux_partial<<<dim3(nchunk, nfreq), 256, 0, s>>>(acc, nfreq, ncell, part, nchunk);
  dft_flux_final<<<(nfreq + 63) / 64, 64, 0, s>>>(part, nfreq, nchunk, dA, out);
  return cudaGetLastError();
}

#define LX_INST(T, C)                                                                                                  \
  template cudaError_t launch_step<T, C>(const StepParams<T, C>&, bool, bool, bool, cudaStream_t);                   \
  template cudaError_t launch_gather<T>(const T*, double*, const int[3], int, int, double, cudaStream_t);                     \
  template cudaError_t launch_scatter<T>(const double*, T*, const int[3], int, int, int, double, double, double,      \
                                         double, cudaStream_t);                                                        \
  template cudaError_t launch_probes<T>(const ProbeParams&, T* const[6], double*, cudaStream_t);                   \
  template cudaError_t launch_dft<T>(const DftParams&, T* const[4], cudaStream_t);                                 \
  template cudaError_t launch_batch_tiles<T, C>(const StepParams<T, C>*, const int*, int, int, bool, int, int4*,    \
                                                cudaStream_t);                                                     \
  template cudaError_t launch_batch_step<T, C>(const StepParams<T, C>*, const int4*, int, bool, bool, int, bool,     \
                                               cudaStream_t);                                                          \
  template cudaError_t launch_dft_batch<T>(const DftParams*, const int2*, int, int, const int*, int, cudaStream_t);
LX_INST(double, double)
LX_INST(float, float)
LX_INST(__half, float)
template cudaError_t launch_step_sweep2<float, float>(const StepParams<float, float>&, bool, cudaStream_t);
template cudaError_t launch_step_sweep2<__half, float>(const StepParams<__half, float>&, bool, cudaStream_t);
template cudaError_t launch_prologue<double>(const PrologueParams&, cudaStream_t);
template cudaError_t launch_prologue<float>(const PrologueParams&, cudaStream_t);
template cudaError_t launch_prologue_batch<double>(const PrologueParams*, const int*, int, int, int, cudaStream_t);
template cudaError_t launch_prologue_batch<float>(const PrologueParams*, const int*, int, int, int, cudaStream_t);
template cudaError_t launch_eps_box<double>(double*, const int[3], int, int, const int[3], const int[3], double,
                                            cudaStream_t);
template cudaError_t launch_eps_box<float>(float*, const int[3], int, int, const int[3], const int[3], double,
                                           cudaStream_t);

}  // namespace lx
