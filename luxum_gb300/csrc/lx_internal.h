// lx_internal.h -- device-side data layout and kernel parameter blocks of the engine.
//
// Layout in HBM.  Every field component of one simulation lives in its own array of the
// common padded shape (Nx, Ny, Nzp), C order (z fastest), Nzp = Nz rounded up to 128 bytes
// of storage type.  A component only owns the cells of its staggered extent
// (field.cc:67-77: extent - 1 on every staggered axis); the remaining cells stay zero and
// are never written.  One shape for all six components lets a single index
// c = (i*Ny + j)*Nzp + k address every component at cell (i,j,k), so neighbour offsets are
// the constants 1, Nzp and Ny*Nzp.
//
// CPML psi is stored only on the slabs where a 1-D profile is active (c != 0 or kappa != 1):
// along axis a, indices [0, lo) and [hi0, N) are kept, packed to lo + (N - hi0) entries.
// Outside them the reference's psi stays exactly 0 (b = 1, c = 0), so dropping it is exact.
//
// Difference units.  With uniform spacing (dx = dy = dz, every reference fixture) curls are
// carried as plain neighbour differences (curl * dx); the 1/dx folds into the coefficients
// (Db/dx, Cb/dx), the TF/SF increments and psi, which removes two FP64 multiplies per
// component.  With non-uniform spacing the kernels multiply by 1/d per axis instead.
#pragma once
#include <cstddef>
#include <cstdint>

namespace lx {

constexpr int kMaxProbes = 64;
constexpr int kMaxDftFreq = 256;
// Default cells each thread of a batched update kernel walks through along x: planar rows 8
// apart, and 3-D planes (the autotuner's picks on the lens and 3-D cube workloads);
// lx_batch_autotune picks per batch among 1, 2, 4 and 8.
constexpr int kMarch2 = 8;
constexpr int kMarch3 = 8;

// Packed CPML slab along one axis.
struct Slab {
  int lo;   // indices [0, lo) are stored as 0..lo-1
  int hi0;  // indices [hi0, N) are stored as lo..lo+N-hi0-1
  int n;    // lo + N - hi0 (0: no psi on this axis)
};

__host__ __device__ inline int slab_index(const Slab& s, int u) {
  return u < s.lo ? u : (u >= s.hi0 ? u - s.hi0 + s.lo : -1);
}

// One TF/SF correction set: the two planes (low and high face of the total-field box)
// that feed one curl part of one component, with the in-plane index ranges of the
// reference loops (maxwell.cc:512-812) and the layout of its incident-value table.
struct PatchSet {
  int active;
  int axis;        // normal axis of the planes (0 = x, 1 = y, 2 = z)
  int plane[2];    // cell index along `axis` of the low and high plane
  int lo[3], hi[3];  // inclusive in-plane ranges (entry `axis` unused)
  int n[3];        // table extent per axis (1 on `axis` and on axes the wave does not vary along)
  int stride[3];   // table stride per axis (0 on collapsed axes)
  int tab;         // offset of the low plane's table in the table buffer
  int plane_len;   // entries per plane table (high plane at tab + plane_len)
  // incident-value expression of the table entries
  double pos_n[2];   // wave position along `axis` of each plane (e.g. p1, p2, p1-0.5, p2+0.5)
  double off[3];     // in-plane position offsets (0 or 0.5)
  double sign[2];    // -1 / +1 (curl = curl - v or curl + v)
  double dir;        // E_?_dir or H_?_dir
  double neg;        // 1, or -1 for the planar H-curl lines that multiply by (-1) first
  double dn;         // spacing along `axis` (the reference divides by it)
  int hcurl;         // 1: also divide by c and mu0 (H-curl lines)
  double scale;      // stored-H scale for H-curl lines (1 unless H is stored scaled)
  // neg * dir / dn (/ c / mu0 for H-curl lines) (* dn in difference units) * scale, formed
  // once on the host: a table entry is exp(-X^2 / sigma) * factor, signed per plane
  double factor;
};

// Parameters of the step prologue: TF/SF tables, point source, monitor reset.
struct PrologueParams {
  int nsets;          // 0..12
  PatchSet sets[12];  // [0,6): E-curl sets for the H update; [6,12): H-curl sets for the E update
  void* tab;          // table buffer (compute precision; entries evaluated in FP64)
  int tab_total;      // total entries over all active sets
  int planar;
  double dx, dy, dz, kx, ky, kz, init, c, dt, mu0, pw_sigma;
  double inv_sigma;    // 1 / pw_sigma
  double scale_units;  // 1 (curl units) or 0 = scale each entry by its plane spacing (difference units)
  int t;
  // point source
  int src_kind;       // -1 none, 0 hard CW, 1 additive pulse
  long long src_idx;  // linear index in the padded layout
  void* src_field;    // Ez (3D) or Ey (planar pulse)
  void* src_field1;   // its buffer 1 on single-sweep handles (used at odd t), else null
  int src_amp_i, src_omega_i;
  double src_amp, src_omega, src_t0, src_tw;
  int prec;           // storage precision of src_field
  unsigned long long* max_slot;  // reset to 0 when non-null
};

// Device pointers and constants of one 3-D or planar simulation, passed by value.
template <class T, class C>
struct StepParams {
  int Nx, Ny, Nz, Nzp;
  long long sj, si;  // strides of j and i
  T* E[3];
  T* H[3];
  const C* Cbs[3];  // Cb (curl units) or Cb/dx (difference units)
  C Dbs;            // Db or Db/dx
  C rd[3];          // 1/dx, 1/dy, 1/dz (non-uniform only)
  // CPML
  int pml;
  Slab slab[3];
  const C* bE[3];
  const C* cE[3];
  const C* rkE[3];
  const C* bH[3];
  const C* cH[3];
  const C* rkH[3];
  C* psiH[3][2];  // [component][part]
  C* psiE[3][2];
  // TF/SF
  int tfsf;
  int planesH[3][2];     // per axis, the planes any H-update set uses (-2 when none): block skip test
  int planesE[3][2];
  PatchSet setsH[3][2];  // [component][part]
  PatchSet setsE[3][2];
  const C* tab;
  // monitor / |E|^2 snapshot (E kernel)
  unsigned long long* max_slot;  // atomicMax of the bit pattern of max|E|^2 (non-negative)
  C* etotal;                     // when non-null, |E|^2 into the Ez-shaped array (3D)
  // Second copy of the state, held by planar float-compute handles (null for the others; the
  // in-place kernels ignore it).  For the single-sweep kernel, E, H, psiH, psiE name the copy
  // it reads and E1, H1, psiH1, psiE1 the one it writes.
  T* E1[3];
  T* H1[3];
  C* psiH1[3][2];
  C* psiE1[3][2];
  // Set by the single-simulation 3-D launch: 1 when a block's z tile 0 is the row's two
  // 16-cell ends (see ZTile in lx_kernels.cu), 0 for plain 32-cell tiles.
  int zends;
  // Set to nonzero by a kernel whose bounded wait for staged data ran out (null: not reported).
  unsigned* fault;
};

// Whether a block's tile [i0,i0+ni) x [j0,j0+nj) x [k0,k0+nk) meets any TF/SF plane of the
// given plane lists; blocks that do not skip every per-cell plane test.
__host__ __device__ inline bool tile_meets_planes(const int (&pl)[3][2], int i0, int ni, int j0, int nj, int k0, int nk) {
  bool t = false;
  for (int q = 0; q < 2; ++q) {
    t |= (unsigned)(pl[0][q] - i0) < (unsigned)ni;
    t |= (unsigned)(pl[1][q] - j0) < (unsigned)nj;
    t |= (unsigned)(pl[2][q] - k0) < (unsigned)nk;
  }
  return t;
}

// Whether a tile [i0,i0+ni) x [j0,j0+nj) x [k0,k0+nk) lies where every component of both
// half steps updates (every index in [1, N-2]) and no CPML slab reaches.  Such tiles (most
// of a grid) take the cell code with every per-cell condition decided at compile time.
__host__ __device__ inline bool axis_free(const Slab& s, int a, int n) { return s.n == 0 || (a >= s.lo && a + n <= s.hi0); }
__host__ __device__ inline bool tile_is_interior(const Slab (&sl)[3], bool pml, int Nx, int Ny, int Nz, int i0, int ni,
                                                 int j0, int nj, int k0, int nk) {
  if (i0 < 1 || i0 + ni > Nx - 1 || j0 < 1 || j0 + nj > Ny - 1 || k0 < 1 || k0 + nk > Nz - 1) return false;
  return !pml || (axis_free(sl[0], i0, ni) && axis_free(sl[1], j0, nj) && axis_free(sl[2], k0, nk));
}

// The same for a planar tile [i0,i0+ni) x [k0,k0+nk) (no y axis).
__host__ __device__ inline bool tile_is_interior_2d(const Slab (&sl)[3], bool pml, int Nx, int Nz, int i0, int ni,
                                                    int k0, int nk) {
  if (i0 < 1 || i0 + ni > Nx - 1 || k0 < 1 || k0 + nk > Nz - 1) return false;
  return !pml || (axis_free(sl[0], i0, ni) && axis_free(sl[2], k0, nk));
}

// Probe sampling of one step row.
struct ProbeParams {
  int nprobes, row, Ny, Nzp;
  double hmul;      // 1/hscale: stored H -> H
  int ext[6][3];    // staggered extents of the six components (0 for absent ones)
  const int* ijk;   // device array [nprobes][3]
};

// One DFT plane monitor (see lx_sim_add_dft_plane).
struct DftParams {
  int axis, index, na, nb, Ny, Nzp, nfreq, t;
  int sim;                // batched launches: index of the simulation's step counter
  const void* f[4];       // batched launches: the four sampled components
  const void* f1[4];      // ... in buffer 1, for members stepped in two buffers (null otherwise):
                          // the state after step t lives in buffer (t + 1) & 1
  int ext[4][3];          // extents of the four sampled components
  double dt, weight;
  double hmul;            // 1/hscale for the two H components
  int every_;             // batched launches: sampling cadence
  const double* omega;    // device [nfreq]
  double* phase;          // device [4][kMaxDftFreq]: cos, sin (E), cos, sin (H) of this sample
  double* acc;            // device [nfreq][4][na*nb][2]
};

}  // namespace lx
