// lx_sweep3d.cu -- single-sweep 3-D step for float compute (FP32 and FP16 storage).
//
// The two-sweep kernels (h_kernel_3d, e_kernel_3d) read E and H twice per step: the H sweep
// reads E and H and writes H, the E sweep reads H, E and Cb and writes E, 84 B per FP32 cell
// against the compulsory 60 (E, H and Cb read once, E and H written once) plus psi.  This
// kernel forms H and E of a step in one pass and moves the compulsory bytes.
//
// A block owns a tile of 8 y rows x 32 z columns and marches along x.  The tensor memory
// accelerator stages each plane into shared memory ahead of use (a ring of 4 planes filled
// by cp.async.bulk.tensor, completion on mbarriers): old E of the next plane on rows
// j0-1 .. j0+8, old H on rows j0-1 .. j0+7, both over columns k0-4 .. k0+35 (k0-8 .. k0+39 for
// FP16), and Cb.  Out-of-grid rows and columns arrive as zeros, so no copy needs a range
// check.  Every neighbour an update takes is then a shared-memory read: E at y+1 and z+1 for
// H, H at y-1 and z-1 (exchanged between the warps) for E.  The H of row j0-1 and column
// k0-1 belong to neighbouring tiles; a ninth warp recomputes them from the staged old state
// with the owners' arithmetic.  See step_kernel_3d for the order of a plane.
//
// State n is read from one buffer (E, H, psiH, psiE of the parameter block) and state n+1
// written to the other (E1, H1, psiH1, psiE1), so no block sees a neighbour's new values, and
// every cell of a tile is written (the cells a half step does not update with their old
// value).  H enters E as stored (FP16 storage rounds it first), so the step equals the
// two-sweep kernels bit for bit.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <utility>
#include <vector>

#include "lx_device.cuh"
#include "lx_internal.h"
#include "lx_kernels.h"

namespace lx {

// Tensor maps of the buffers a sweep launch reads: E and H of state n (boxes of the staged tile
// width over kTY + 2 and kTY + 1 rows), and Cb (32 x kTY).
struct Sweep3Maps {
  CUtensorMap e[3], h[3], cb[3];
};

namespace {

constexpr int kTY = 8;                    // rows (y) per block, one warp each
constexpr int kStages = 4;                // planes in flight per block
constexpr int kThreads = 32 * (kTY + 1);  // the row warps and one halo / producer warp
constexpr long long kSpin = 1LL << 20;    // bound of the tries of a wait on a staged plane (normally a few)

// ---- the arithmetic of h_apply for the H of a cell of another block (three_dim_pml.cc:176-213)

// psi = b*psi + c*d, with the old psi read and the new one left to its owner; returns
// d/kappa + psi (pml_term's arithmetic).
template <class C>
__device__ __forceinline__ C pml_in(C d, const C* in, long long q, C b, C cc, C rk) {
  const C ps = fmaC(b, in[q], cc * d);
  return fmaC(d, rk, ps);
}

template <class T, class C, bool UNI>
__device__ __forceinline__ C hy_old_state(const StepParams<T, C>& p, int i, int j, int k) {
  const long long c = (long long)i * p.si + (long long)j * p.sj + k;
  const C hy = ld<T, C>(p.H[1] + c);
  if (!(i < p.Nx - 1 && k < p.Nz - 1)) return hy;
  C d1 = ld<T, C>(p.E[0] + c + 1) - ld<T, C>(p.E[0] + c);      // dEx/dz (z profile)
  C d2 = ld<T, C>(p.E[2] + c + p.si) - ld<T, C>(p.E[2] + c);  // dEz/dx (x profile)
  if (!UNI) { d1 = mulC(d1, p.rd[2]); d2 = mulC(d2, p.rd[0]); }
  if (p.tfsf) {
    tfsf_apply<C>(p.setsH[1][0], p.tab, i, j, k, d1);
    tfsf_apply<C>(p.setsH[1][1], p.tab, i, j, k, d2);
  }
  const int sz = slab_index(p.slab[2], k), sx = slab_index(p.slab[0], i);
  if (sz >= 0) d1 = pml_in<C>(d1, p.psiH[1][0], psi_index(2, p.slab[2], sz, i, j, k, p.Ny, p.Nzp), p.bH[2][k], p.cH[2][k], p.rkH[2][k]);
  if (sx >= 0) d2 = pml_in<C>(d2, p.psiH[1][1], psi_index(0, p.slab[0], sx, i, j, k, p.Ny, p.Nzp), p.bH[0][i], p.cH[0][i], p.rkH[0][i]);
  return stored<T, C>(fmaC(-p.Dbs, d1 - d2, hy));
}

template <class T, class C, bool UNI>
__device__ __forceinline__ C hz_old_state(const StepParams<T, C>& p, int i, int j, int k) {
  const long long c = (long long)i * p.si + (long long)j * p.sj + k;
  const C hz = ld<T, C>(p.H[2] + c);
  if (!(i < p.Nx - 1 && j < p.Ny - 1)) return hz;
  C d1 = ld<T, C>(p.E[1] + c + p.si) - ld<T, C>(p.E[1] + c);  // dEy/dx (x profile)
  C d2 = ld<T, C>(p.E[0] + c + p.sj) - ld<T, C>(p.E[0] + c);  // dEx/dy (y profile)
  if (!UNI) { d1 = mulC(d1, p.rd[0]); d2 = mulC(d2, p.rd[1]); }
  if (p.tfsf) {
    tfsf_apply<C>(p.setsH[2][0], p.tab, i, j, k, d1);
    tfsf_apply<C>(p.setsH[2][1], p.tab, i, j, k, d2);
  }
  const int sx = slab_index(p.slab[0], i), sy = slab_index(p.slab[1], j);
  if (sx >= 0) d1 = pml_in<C>(d1, p.psiH[2][0], psi_index(0, p.slab[0], sx, i, j, k, p.Ny, p.Nzp), p.bH[0][i], p.cH[0][i], p.rkH[0][i]);
  if (sy >= 0) d2 = pml_in<C>(d2, p.psiH[2][1], psi_index(1, p.slab[1], sy, i, j, k, p.Ny, p.Nzp), p.bH[1][j], p.cH[1][j], p.rkH[1][j]);
  return stored<T, C>(fmaC(-p.Dbs, d1 - d2, hz));
}

// ---- staging

// Columns a staged field tile covers: k0 - XO .. k0 - XO + W - 1.  A TMA copy must start on a
// 16-byte boundary (XO * size is 16) and move whole 16-byte units (W * size).
template <class T>
struct TileCols;
template <>
struct TileCols<float> {
  static constexpr int XO = 4, W = 40;
};
template <>
struct TileCols<__half> {
  static constexpr int XO = 8, W = 48;
};

constexpr int round128(int n) { return (n + 127) / 128 * 128; }

// Byte layout of one stage (plane q): old E(q+1) on rows j0-1 .. j0+kTY, old H(q) on rows
// j0-1 .. j0+kTY-1 (both over the W columns), Cb(q) on rows j0 .. j0+kTY-1 over k0 .. k0+31.
// Every tile starts on a 128-byte boundary.
template <class T>
struct StageLayout {
  static constexpr int W = TileCols<T>::W;
  static constexpr int E_BYTES = (kTY + 2) * W * (int)sizeof(T);
  static constexpr int H_BYTES = (kTY + 1) * W * (int)sizeof(T);
  static constexpr int CB_BYTES = kTY * 32 * 4;
  static constexpr int E_OFF = 0, E_STRIDE = round128(E_BYTES);
  static constexpr int H_OFF = 3 * E_STRIDE, H_STRIDE = round128(H_BYTES);
  static constexpr int CB_OFF = H_OFF + 3 * H_STRIDE, CB_STRIDE = round128(CB_BYTES);
  static constexpr int BYTES = CB_OFF + 3 * CB_STRIDE;
  static constexpr int TX = 3 * (E_BYTES + H_BYTES + CB_BYTES);  // bytes the copies of a stage deliver
};

// The rest of the block's shared memory: new H exchanged between warps within a plane (by
// plane parity), the stage barriers.
template <class C>
struct Exchange {
  C hr[2][2][kTY + 1][32];  // [parity][Hz, Hx][row j0-1+r][lane]
  C hc[2][2][kTY];          // [parity][Hy, Hx][row j0+r] at column k0-1
  unsigned long long full[kStages];
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
// Waits, with a bound, for the phase of the given parity to complete; false when the bound ran out.
// Each try may suspend the warp for up to kSuspendNs instead of returning at once, so a waiting
// warp does not take issue slots from the warps that are computing.
constexpr unsigned kSuspendNs = 1000;
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned parity) {
  const unsigned a = smem_u32(b);
  for (long long it = 0; it < kSpin; ++it) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity), "r"(kSuspendNs)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load3(void* dst, const CUtensorMap* map, int x, int y, int z, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Issues the nine copies of plane q into stage `st` (one thread).
template <class T>
__device__ __forceinline__ void stage_plane(const Sweep3Maps& m, unsigned char* st, unsigned long long* bar, int q,
                                            int j0, int k0) {
  using L = StageLayout<T>;
  mbar_expect_tx(bar, L::TX);
  const int x = k0 - TileCols<T>::XO;
  for (int c = 0; c < 3; ++c) {
    tma_load3(st + L::E_OFF + c * L::E_STRIDE, &m.e[c], x, j0 - 1, q + 1, bar);
    tma_load3(st + L::H_OFF + c * L::H_STRIDE, &m.h[c], x, j0 - 1, q, bar);
    tma_load3(st + L::CB_OFF + c * L::CB_STRIDE, &m.cb[c], k0, j0, q, bar);
  }
}

template <class T, class C>
__device__ __forceinline__ C tile_at(const unsigned char* st, int off, int stride, int comp, int row, int col) {
  return ld<T, C>(reinterpret_cast<const T*>(st + off + comp * stride) + row * TileCols<T>::W + col);
}

// ---- TF/SF sets (bit 2c+q: H component c part q; 6+2c+q: E) that reach the block's cells,
// rows j0-1 .. j0+kTY-1 and columns k0-1 .. k0+31: y and z once per block, x per plane (a few
// comparisons: a per-plane pass over the twelve sets cost as much as the rest of the plane)

__device__ __forceinline__ bool set_reaches_yz(const PatchSet& ps, int jlo, int jhi, int klo, int khi) {
  if (!ps.active) return false;
  const bool y = ps.axis == 1 ? ((ps.plane[0] >= jlo && ps.plane[0] <= jhi) || (ps.plane[1] >= jlo && ps.plane[1] <= jhi))
                              : (ps.lo[1] <= jhi && ps.hi[1] >= jlo);
  const bool z = ps.axis == 2 ? ((ps.plane[0] >= klo && ps.plane[0] <= khi) || (ps.plane[1] >= klo && ps.plane[1] <= khi))
                              : (ps.lo[2] <= khi && ps.hi[2] >= klo);
  return y && z;
}
// Per block: the sets whose y and z extents reach the block's cells, split into those normal to
// x (they apply on their two x planes) and the others (they apply over an x range).
struct BlockSets {
  unsigned xn, other;    // set masks
  int xp[4];             // x planes of the x-normal sets (H sets: [0], [1]; E sets: [2], [3])
  int xlo, xhi;          // union of the other sets' x ranges
};
template <class T, class C>
__device__ __forceinline__ BlockSets block_sets(const StepParams<T, C>& p, int j0, int k0) {
  BlockSets bs;
  bs.xn = bs.other = 0;
  bs.xlo = 1 << 30;
  bs.xhi = -1;
  bs.xp[0] = p.planesH[0][0];
  bs.xp[1] = p.planesH[0][1];
  bs.xp[2] = p.planesE[0][0];
  bs.xp[3] = p.planesE[0][1];
  if (p.tfsf) {
#pragma unroll
    for (int b = 0; b < 12; ++b) {
      const PatchSet& ps = b < 6 ? p.setsH[b >> 1][b & 1] : p.setsE[(b - 6) >> 1][(b - 6) & 1];
      if (!set_reaches_yz(ps, j0 - 1, j0 + kTY - 1, k0 - 1, k0 + 31)) continue;
      if (ps.axis == 0) {
        bs.xn |= 1u << b;
      } else {
        bs.other |= 1u << b;
        bs.xlo = min(bs.xlo, ps.lo[0]);
        bs.xhi = max(bs.xhi, ps.hi[0]);
      }
    }
  }
  return bs;
}
// The sets that may apply at plane i (a superset: tfsf_apply checks each cell exactly).
__device__ __forceinline__ unsigned sets_at(const BlockSets& bs, int i) {
  unsigned m = (i >= bs.xlo && i <= bs.xhi) ? bs.other : 0u;
  if (bs.xn & 0x03Fu && (i == bs.xp[0] || i == bs.xp[1])) m |= bs.xn & 0x03Fu;
  if (bs.xn & 0xFC0u && (i == bs.xp[2] || i == bs.xp[3])) m |= bs.xn & 0xFC0u;
  return m;
}

// A difference of neighbours, scaled by 1/d of its axis with non-uniform spacing.
template <class C, bool UNI>
__device__ __forceinline__ C diff(C a, C b, C rd) {
  const C d = a - b;
  return UNI ? d : mulC(d, rd);
}

// One CPML psi term of a cell (pml_term's arithmetic): psi = b*psi + c*d, d -> d*(1/kappa) + psi.
template <class C>
struct Psi {
  bool on;
  const C* in;
  C* out;  // null for a recomputed neighbour: its owner stores the new psi
  long long q;
  const C *b, *cc, *rk;
  int u;  // profile index
};
template <class C>
__device__ __forceinline__ Psi<C> psi_term(bool on, const C* in, C* out, int axis, const Slab& sl, int s, int i, int j,
                                           int k, int Ny, int Nzp, const C* b, const C* cc, const C* rk, int u) {
  Psi<C> t;
  t.on = on && s >= 0;
  t.in = in;
  t.out = out;
  t.q = t.on ? psi_index(axis, sl, s, i, j, k, Ny, Nzp) : 0;
  t.b = b;
  t.cc = cc;
  t.rk = rk;
  t.u = u;
  return t;
}
// Applies N psi terms to their differences: every load of the N terms is issued first, then
// the arithmetic and the stores (a store between loads would keep the next term's loads
// waiting behind it, one memory round trip per term).
template <class C, int N>
__device__ __forceinline__ void psi_apply(const Psi<C> (&t)[N], C* const (&d)[N]) {
  C ps[N], b[N], cc[N], rk[N];
#pragma unroll
  for (int n = 0; n < N; ++n) {
    ps[n] = b[n] = cc[n] = rk[n] = C(0);
    if (t[n].on) {
      ps[n] = t[n].in[t[n].q];
      b[n] = t[n].b[t[n].u];
      cc[n] = t[n].cc[t[n].u];
      rk[n] = t[n].rk[t[n].u];
    }
  }
#pragma unroll
  for (int n = 0; n < N; ++n)
    if (t[n].on) {
      const C v = fmaC(b[n], ps[n], cc[n] * *d[n]);
      if (t[n].out) t[n].out[t[n].q] = v;
      *d[n] = fmaC(*d[n], rk[n], v);
    }
}

}  // namespace

// One block: the tile of kTY rows (j0 ..) x 32 columns (k0 ..), marching over planes i0 .. i1-1.
// Warps 0 .. kTY-1 update rows j0 + w; warp kTY recomputes the H of row j0-1 and of column k0-1
// that the row warps' E takes, and its lane 0 keeps the stage ring filled.  Per plane i:
//   all warps wait for stage i (old E(i+1), H(i), Cb(i)) and use stage i-1 (old E(i));
//   H phase: row warps form new H(i) of their row and post Hz, Hx; the halo warp posts row
//            j0-1 and column k0-1;
//   __syncthreads;  the producer refills stage i-1 (no longer read) with plane i-1+kStages;
//   E phase: row warps form new E(i), store E(i) and H(i) into the output buffer.
// The H exchange alternates between two copies by plane parity, so the next plane's H phase
// never overwrites what a slower warp still reads.  The arithmetic of every component follows
// h_apply and e_apply: two differences, the TF/SF increments, the CPML psi terms, one FMA; the
// TF/SF and CPML blocks run only on planes whose cells need them (block-uniform), and the
// update conditions of the grid edges only where a tile reaches one.
template <class T, class C, bool UNI, bool MON>
__global__ void __launch_bounds__(kThreads, 3)
    step_kernel_3d(const StepParams<T, C> p, const __grid_constant__ Sweep3Maps maps, int R) {
  using L = StageLayout<T>;
  constexpr int XO = TileCols<T>::XO;
  extern __shared__ __align__(128) unsigned char smem[];
  Exchange<C>& ex_ = *reinterpret_cast<Exchange<C>*>(smem + kStages * L::BYTES);
  const int lane = threadIdx.x, w = threadIdx.y;
  const int k0 = blockIdx.x * 32, j0 = blockIdx.y * kTY, i0 = blockIdx.z * R;
  const int i1 = min(i0 + R, p.Nx);
  const bool producer = w == kTY && lane == 0;
  if (producer) {
    for (int s = 0; s < kStages; ++s) mbar_init(&ex_.full[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  // stages 0 .. kStages-1: planes i0-1 (whose E(i0) the first plane takes) .. i0+kStages-2
  if (producer)
    for (int s = 0; s < kStages; ++s)
      if (i0 - 1 + s < i1) stage_plane<T>(maps, smem + s * L::BYTES, &ex_.full[s], i0 - 1 + s, j0, k0);

  const BlockSets bsets = block_sets(p, j0, k0);
  const bool edge_yz = !(j0 - 1 >= 1 && j0 + kTY <= p.Ny - 1 && k0 - 1 >= 1 && k0 + 32 <= p.Nz - 1);
  const bool psi_yz = p.pml && !(axis_free(p.slab[1], j0 - 1, kTY + 1) && axis_free(p.slab[2], k0 - 1, 33));
  const int k = k0 + lane;
  const int j = j0 + w;  // row warps
  const int sy = slab_index(p.slab[1], j), sz = slab_index(p.slab[2], k);
  const bool act = j < p.Ny && k < p.Nz;  // row warps: the cell exists
  long long c = (long long)i0 * p.si + (long long)j * p.sj + k;
  C hzm = C(0), hym = C(0);  // row warps: new Hz, Hy at i-1 of the cell
  if (w < kTY && act && i0 >= 1) {
    hzm = hz_old_state<T, C, UNI>(p, i0 - 1, j, k);
    hym = hy_old_state<T, C, UNI>(p, i0 - 1, j, k);
  }
  typename MaxBits<C>::type mbits = 0;
  bool fault = false;
#pragma unroll 1
  for (int i = i0; i < i1; ++i, c += p.si) {
    const int r = i - i0 + 1;  // stage ring position of plane i (plane i0-1 is position 0)
    const int cur = r % kStages, prv = (r - 1) % kStages, par = i & 1;
    // once a wait has run out, no further wait: the block runs its remaining planes without
    // storing and reports the fault
    if (!fault && i == i0) fault = !mbar_wait(&ex_.full[prv], 0);
    if (!fault) fault = !mbar_wait(&ex_.full[cur], (r / kStages) & 1);
    const unsigned char* sc = smem + cur * L::BYTES;  // E(i+1), H(i), Cb(i)
    const unsigned char* sp = smem + prv * L::BYTES;  // E(i)
    const unsigned tf = (bsets.xn | bsets.other) ? sets_at(bsets, i) : 0u;
    const int sx = slab_index(p.slab[0], i);
    const bool psi = psi_yz || (p.pml && sx >= 0);
    const bool edge = edge_yz || i < 1 || i + 1 > p.Nx - 1;
    C ex = C(0), ey = C(0), ez = C(0), nhx = C(0), nhy = C(0), nhz = C(0);
    if (w < kTY) {
      // ---- H phase, row warp: new H(i) of cell (i, j, k)
      const int row = w + 1, cx = lane + XO;
      ex = tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 0, row, cx);
      ey = tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 1, row, cx);
      ez = tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 2, row, cx);
      const C exj = tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 0, row + 1, cx);
      const C ezj = tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 2, row + 1, cx);
      const C exk = tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 0, row, cx + 1);
      const C eyk = tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 1, row, cx + 1);
      const C ey1 = tile_at<T, C>(sc, L::E_OFF, L::E_STRIDE, 1, row, cx);
      const C ez1 = tile_at<T, C>(sc, L::E_OFF, L::E_STRIDE, 2, row, cx);
      const C hx = tile_at<T, C>(sc, L::H_OFF, L::H_STRIDE, 0, row, cx);
      const C hy = tile_at<T, C>(sc, L::H_OFF, L::H_STRIDE, 1, row, cx);
      const C hz = tile_at<T, C>(sc, L::H_OFF, L::H_STRIDE, 2, row, cx);
      const bool uxh = !edge || (act && j < p.Ny - 1 && k < p.Nz - 1);
      const bool uyh = !edge || (act && i < p.Nx - 1 && k < p.Nz - 1);
      const bool uzh = !edge || (act && i < p.Nx - 1 && j < p.Ny - 1);
      C x1 = diff<C, UNI>(ezj, ez, p.rd[1]), x2 = diff<C, UNI>(eyk, ey, p.rd[2]);  // dEz/dy, dEy/dz
      C y1 = diff<C, UNI>(exk, ex, p.rd[2]), y2 = diff<C, UNI>(ez1, ez, p.rd[0]);  // dEx/dz, dEz/dx
      C z1 = diff<C, UNI>(ey1, ey, p.rd[0]), z2 = diff<C, UNI>(exj, ex, p.rd[1]);  // dEy/dx, dEx/dy
      if (tf) {
        if (tf & (1u << 0)) tfsf_apply<C>(p.setsH[0][0], p.tab, i, j, k, x1);
        if (tf & (1u << 1)) tfsf_apply<C>(p.setsH[0][1], p.tab, i, j, k, x2);
        if (tf & (1u << 2)) tfsf_apply<C>(p.setsH[1][0], p.tab, i, j, k, y1);
        if (tf & (1u << 3)) tfsf_apply<C>(p.setsH[1][1], p.tab, i, j, k, y2);
        if (tf & (1u << 4)) tfsf_apply<C>(p.setsH[2][0], p.tab, i, j, k, z1);
        if (tf & (1u << 5)) tfsf_apply<C>(p.setsH[2][1], p.tab, i, j, k, z2);
      }
      if (psi) {
        const Psi<C> t[6] = {
            psi_term<C>(uxh, p.psiH[0][0], p.psiH1[0][0], 1, p.slab[1], sy, i, j, k, p.Ny, p.Nzp, p.bH[1], p.cH[1], p.rkH[1], j),
            psi_term<C>(uxh, p.psiH[0][1], p.psiH1[0][1], 2, p.slab[2], sz, i, j, k, p.Ny, p.Nzp, p.bH[2], p.cH[2], p.rkH[2], k),
            psi_term<C>(uyh, p.psiH[1][0], p.psiH1[1][0], 2, p.slab[2], sz, i, j, k, p.Ny, p.Nzp, p.bH[2], p.cH[2], p.rkH[2], k),
            psi_term<C>(uyh, p.psiH[1][1], p.psiH1[1][1], 0, p.slab[0], sx, i, j, k, p.Ny, p.Nzp, p.bH[0], p.cH[0], p.rkH[0], i),
            psi_term<C>(uzh, p.psiH[2][0], p.psiH1[2][0], 0, p.slab[0], sx, i, j, k, p.Ny, p.Nzp, p.bH[0], p.cH[0], p.rkH[0], i),
            psi_term<C>(uzh, p.psiH[2][1], p.psiH1[2][1], 1, p.slab[1], sy, i, j, k, p.Ny, p.Nzp, p.bH[1], p.cH[1], p.rkH[1], j)};
        C* const d[6] = {&x1, &x2, &y1, &y2, &z1, &z2};
        psi_apply<C, 6>(t, d);
      }
      nhx = uxh ? stored<T, C>(fmaC(-p.Dbs, x1 - x2, hx)) : hx;
      nhy = uyh ? stored<T, C>(fmaC(-p.Dbs, y1 - y2, hy)) : hy;
      nhz = uzh ? stored<T, C>(fmaC(-p.Dbs, z1 - z2, hz)) : hz;
      ex_.hr[par][0][row][lane] = nhz;
      ex_.hr[par][1][row][lane] = nhx;
    } else {
      // ---- H phase, halo warp: new Hz, Hx of cell (i, j0-1, k0+lane) of the row below the
      // tile, and new Hy, Hx of cell (i, j0+lane, k0-1) of the column before it (lane < kTY)
      const int jr = j0 - 1, cx = lane + XO;
      const bool rowv = jr >= 0 && k < p.Nz;
      const bool uzr = rowv && i < p.Nx - 1 && jr < p.Ny - 1, uxr = rowv && jr < p.Ny - 1 && k < p.Nz - 1;
      const int jc = j0 + lane, kh = k0 - 1, ch = XO - 1;
      const bool colv = lane < kTY && kh >= 0 && jc < p.Ny;
      const bool uyc = colv && i < p.Nx - 1, uxc = colv && jc < p.Ny - 1;
      const int rc = min(lane, kTY - 1) + 1;  // in-tile row of the column cell (clamped for lanes >= kTY)
      const C eyr = tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 1, 0, cx);
      const C ezh = tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 2, rc, ch);
      // row cell: Hz (m: x, y parts), Hx (n: y, z parts); column cell: Hy (u: z, x), Hx (v: y, z)
      C m1 = diff<C, UNI>(tile_at<T, C>(sc, L::E_OFF, L::E_STRIDE, 1, 0, cx), eyr, p.rd[0]);
      C m2 = diff<C, UNI>(tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 0, 1, cx), tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 0, 0, cx), p.rd[1]);
      C n1 = diff<C, UNI>(tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 2, 1, cx), tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 2, 0, cx), p.rd[1]);
      C n2 = diff<C, UNI>(tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 1, 0, cx + 1), eyr, p.rd[2]);
      C u1 = diff<C, UNI>(tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 0, rc, XO), tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 0, rc, ch), p.rd[2]);
      C u2 = diff<C, UNI>(tile_at<T, C>(sc, L::E_OFF, L::E_STRIDE, 2, rc, ch), ezh, p.rd[0]);
      C v1 = diff<C, UNI>(tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 2, rc + 1, ch), ezh, p.rd[1]);
      C v2 = diff<C, UNI>(tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 1, rc, XO), tile_at<T, C>(sp, L::E_OFF, L::E_STRIDE, 1, rc, ch), p.rd[2]);
      if (tf) {
        if (tf & (1u << 0)) { tfsf_apply<C>(p.setsH[0][0], p.tab, i, jr, k, n1); tfsf_apply<C>(p.setsH[0][0], p.tab, i, jc, kh, v1); }
        if (tf & (1u << 1)) { tfsf_apply<C>(p.setsH[0][1], p.tab, i, jr, k, n2); tfsf_apply<C>(p.setsH[0][1], p.tab, i, jc, kh, v2); }
        if (tf & (1u << 2)) tfsf_apply<C>(p.setsH[1][0], p.tab, i, jc, kh, u1);
        if (tf & (1u << 3)) tfsf_apply<C>(p.setsH[1][1], p.tab, i, jc, kh, u2);
        if (tf & (1u << 4)) tfsf_apply<C>(p.setsH[2][0], p.tab, i, jr, k, m1);
        if (tf & (1u << 5)) tfsf_apply<C>(p.setsH[2][1], p.tab, i, jr, k, m2);
      }
      if (psi) {
        const int syr = slab_index(p.slab[1], jr), syc = slab_index(p.slab[1], jc), szh = slab_index(p.slab[2], kh);
        const Psi<C> t[8] = {
            psi_term<C>(uzr, p.psiH[2][0], nullptr, 0, p.slab[0], sx, i, jr, k, p.Ny, p.Nzp, p.bH[0], p.cH[0], p.rkH[0], i),
            psi_term<C>(uzr, p.psiH[2][1], nullptr, 1, p.slab[1], syr, i, jr, k, p.Ny, p.Nzp, p.bH[1], p.cH[1], p.rkH[1], jr),
            psi_term<C>(uxr, p.psiH[0][0], nullptr, 1, p.slab[1], syr, i, jr, k, p.Ny, p.Nzp, p.bH[1], p.cH[1], p.rkH[1], jr),
            psi_term<C>(uxr, p.psiH[0][1], nullptr, 2, p.slab[2], sz, i, jr, k, p.Ny, p.Nzp, p.bH[2], p.cH[2], p.rkH[2], k),
            psi_term<C>(uyc, p.psiH[1][0], nullptr, 2, p.slab[2], szh, i, jc, kh, p.Ny, p.Nzp, p.bH[2], p.cH[2], p.rkH[2], kh),
            psi_term<C>(uyc, p.psiH[1][1], nullptr, 0, p.slab[0], sx, i, jc, kh, p.Ny, p.Nzp, p.bH[0], p.cH[0], p.rkH[0], i),
            psi_term<C>(uxc, p.psiH[0][0], nullptr, 1, p.slab[1], syc, i, jc, kh, p.Ny, p.Nzp, p.bH[1], p.cH[1], p.rkH[1], jc),
            psi_term<C>(uxc, p.psiH[0][1], nullptr, 2, p.slab[2], szh, i, jc, kh, p.Ny, p.Nzp, p.bH[2], p.cH[2], p.rkH[2], kh)};
        C* const d[8] = {&m1, &m2, &n1, &n2, &u1, &u2, &v1, &v2};
        psi_apply<C, 8>(t, d);
      }
      if (rowv) {
        const C hzo = tile_at<T, C>(sc, L::H_OFF, L::H_STRIDE, 2, 0, cx), hxo = tile_at<T, C>(sc, L::H_OFF, L::H_STRIDE, 0, 0, cx);
        ex_.hr[par][0][0][lane] = uzr ? stored<T, C>(fmaC(-p.Dbs, m1 - m2, hzo)) : hzo;
        ex_.hr[par][1][0][lane] = uxr ? stored<T, C>(fmaC(-p.Dbs, n1 - n2, hxo)) : hxo;
      }
      if (colv) {
        const C hyo = tile_at<T, C>(sc, L::H_OFF, L::H_STRIDE, 1, rc, ch), hxo = tile_at<T, C>(sc, L::H_OFF, L::H_STRIDE, 0, rc, ch);
        ex_.hc[par][0][lane] = uyc ? stored<T, C>(fmaC(-p.Dbs, u1 - u2, hyo)) : hyo;
        ex_.hc[par][1][lane] = uxc ? stored<T, C>(fmaC(-p.Dbs, v1 - v2, hxo)) : hxo;
      }
    }
    __syncthreads();
    // stage i-1 is read no more: the producer refills it with plane i-1+kStages
    if (producer && i - 1 + kStages < i1) stage_plane<T>(maps, smem + prv * L::BYTES, &ex_.full[prv], i - 1 + kStages, j0, k0);
    if (w < kTY) {
      // ---- E phase, row warp: new E(i) of cell (i, j, k)
      const int row = w + 1;
      const C hz_j = ex_.hr[par][0][row - 1][lane], hx_j = ex_.hr[par][1][row - 1][lane];
      C hy_k = __shfl_up_sync(0xffffffffu, nhy, 1), hx_k = __shfl_up_sync(0xffffffffu, nhx, 1);
      if (lane == 0) {
        hy_k = k0 >= 1 ? ex_.hc[par][0][w] : C(0);
        hx_k = k0 >= 1 ? ex_.hc[par][1][w] : C(0);
      }
      const bool ii = !edge || (i >= 1 && i < p.Nx - 1), jj = !edge || (j >= 1 && j < p.Ny - 1),
                 kk = !edge || (k >= 1 && k < p.Nz - 1);
      const bool uxe = !edge || (act && i < p.Nx - 1 && jj && kk);
      const bool uye = !edge || (act && ii && j < p.Ny - 1 && kk);
      const bool uze = !edge || (act && ii && jj && k < p.Nz - 1);
      C a1 = diff<C, UNI>(nhz, hz_j, p.rd[1]), a2 = diff<C, UNI>(nhy, hy_k, p.rd[2]);  // dHz/dy, dHy/dz
      C b1 = diff<C, UNI>(nhx, hx_k, p.rd[2]), b2 = diff<C, UNI>(nhz, hzm, p.rd[0]);   // dHx/dz, dHz/dx
      C g1 = diff<C, UNI>(nhy, hym, p.rd[0]), g2 = diff<C, UNI>(nhx, hx_j, p.rd[1]);   // dHy/dx, dHx/dy
      if (tf) {
        if (tf & (1u << 6)) tfsf_apply<C>(p.setsE[0][0], p.tab, i, j, k, a1);
        if (tf & (1u << 7)) tfsf_apply<C>(p.setsE[0][1], p.tab, i, j, k, a2);
        if (tf & (1u << 8)) tfsf_apply<C>(p.setsE[1][0], p.tab, i, j, k, b1);
        if (tf & (1u << 9)) tfsf_apply<C>(p.setsE[1][1], p.tab, i, j, k, b2);
        if (tf & (1u << 10)) tfsf_apply<C>(p.setsE[2][0], p.tab, i, j, k, g1);
        if (tf & (1u << 11)) tfsf_apply<C>(p.setsE[2][1], p.tab, i, j, k, g2);
      }
      if (psi) {
        const Psi<C> t[6] = {
            psi_term<C>(uxe, p.psiE[0][0], p.psiE1[0][0], 1, p.slab[1], sy, i, j, k, p.Ny, p.Nzp, p.bE[1], p.cE[1], p.rkE[1], j),
            psi_term<C>(uxe, p.psiE[0][1], p.psiE1[0][1], 2, p.slab[2], sz, i, j, k, p.Ny, p.Nzp, p.bE[2], p.cE[2], p.rkE[2], k),
            psi_term<C>(uye, p.psiE[1][0], p.psiE1[1][0], 2, p.slab[2], sz, i, j, k, p.Ny, p.Nzp, p.bE[2], p.cE[2], p.rkE[2], k),
            psi_term<C>(uye, p.psiE[1][1], p.psiE1[1][1], 0, p.slab[0], sx, i, j, k, p.Ny, p.Nzp, p.bE[0], p.cE[0], p.rkE[0], i),
            psi_term<C>(uze, p.psiE[2][0], p.psiE1[2][0], 0, p.slab[0], sx, i, j, k, p.Ny, p.Nzp, p.bE[0], p.cE[0], p.rkE[0], i),
            psi_term<C>(uze, p.psiE[2][1], p.psiE1[2][1], 1, p.slab[1], sy, i, j, k, p.Ny, p.Nzp, p.bE[1], p.cE[1], p.rkE[1], j)};
        C* const d[6] = {&a1, &a2, &b1, &b2, &g1, &g2};
        psi_apply<C, 6>(t, d);
      }
      const float* cbt = reinterpret_cast<const float*>(sc + L::CB_OFF);
      const C cbx = cbt[0 * (L::CB_STRIDE / 4) + w * 32 + lane], cby = cbt[1 * (L::CB_STRIDE / 4) + w * 32 + lane],
              cbz = cbt[2 * (L::CB_STRIDE / 4) + w * 32 + lane];
      const C exn = uxe ? fmaC(cbx, a1 - a2, ex) : ex;
      const C eyn = uye ? fmaC(cby, b1 - b2, ey) : ey;
      const C ezn = uze ? fmaC(cbz, g1 - g2, ez) : ez;
      if (act && !fault) {
        st<T, C>(p.E1[0] + c, exn);
        st<T, C>(p.E1[1] + c, eyn);
        st<T, C>(p.E1[2] + c, ezn);
        st<T, C>(p.H1[0] + c, nhx);
        st<T, C>(p.H1[1] + c, nhy);
        st<T, C>(p.H1[2] + c, nhz);
        if (MON && (!edge || (i < p.Nx - 1 && j < p.Ny - 1 && k < p.Nz - 1))) {
          // Etotal = Ez*Ez + Ey*Ey + Ex*Ex (three_dim_pml.cc:270), as e_apply forms it
          const C e2 = fmaC(exn, exn, fmaC(eyn, eyn, ezn * ezn));
          if (p.etotal) p.etotal[c] = e2;
          const typename MaxBits<C>::type b = MaxBits<C>::of(e2);
          mbits = b > mbits ? b : mbits;
        }
      }
      hzm = nhz;
      hym = nhy;
    }
  }
  if (fault && p.fault) atomicOr(p.fault, 1u);
  if (MON && p.max_slot) block_max_atomic(mbits, p.max_slot);
}

namespace {

// cuTensorMapEncodeTiled, taken from the driver at first use (no link against libcuda).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

// A 3-D map over one padded array (Nz, Ny, Nx; rows of Nzp elements) with a box of bx x by x 1.
bool encode(CUtensorMap* m, const void* base, CUtensorMapDataType dt, size_t esize, int Nx, int Ny, int Nz, int Nzp, int bx,
            int by) {
  const PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)Nz, (cuuint64_t)Ny, (cuuint64_t)Nx};
  const cuuint64_t strides[2] = {(cuuint64_t)Nzp * esize, (cuuint64_t)Ny * Nzp * esize};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(m, dt, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

// Tensor maps of the buffers a launch reads, cached by their arrays and shape: a handle steps
// from its two buffers in turn, so two entries per handle serve every step.
struct MapKey {
  const void* a[9];
  int Nx, Ny, Nz, Nzp, esize;
  bool operator==(const MapKey& o) const {
    for (int q = 0; q < 9; ++q)
      if (a[q] != o.a[q]) return false;
    return Nx == o.Nx && Ny == o.Ny && Nz == o.Nz && Nzp == o.Nzp && esize == o.esize;
  }
};
std::mutex g_maps_mu;
std::vector<std::pair<MapKey, Sweep3Maps>> g_maps;

template <class T, class C>
bool maps_for(const StepParams<T, C>& p, Sweep3Maps* out) {
  MapKey key;
  for (int c = 0; c < 3; ++c) {
    key.a[c] = p.E[c];
    key.a[3 + c] = p.H[c];
    key.a[6 + c] = p.Cbs[c];
  }
  key.Nx = p.Nx;
  key.Ny = p.Ny;
  key.Nz = p.Nz;
  key.Nzp = p.Nzp;
  key.esize = (int)sizeof(T);
  {
    std::lock_guard<std::mutex> lk(g_maps_mu);
    for (auto& e : g_maps)
      if (e.first == key) {
        *out = e.second;
        return true;
      }
  }
  Sweep3Maps m;
  const CUtensorMapDataType dt = sizeof(T) == 2 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  constexpr int W = TileCols<T>::W;
  for (int c = 0; c < 3; ++c) {
    if (!encode(&m.e[c], p.E[c], dt, sizeof(T), p.Nx, p.Ny, p.Nz, p.Nzp, W, kTY + 2)) return false;
    if (!encode(&m.h[c], p.H[c], dt, sizeof(T), p.Nx, p.Ny, p.Nz, p.Nzp, W, kTY + 1)) return false;
    if (!encode(&m.cb[c], p.Cbs[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, p.Nx, p.Ny, p.Nz, p.Nzp, 32, kTY)) return false;
  }
  std::lock_guard<std::mutex> lk(g_maps_mu);
  if (g_maps.size() >= 256) g_maps.erase(g_maps.begin());
  g_maps.emplace_back(key, m);
  *out = m;
  return true;
}

}  // namespace

template <class T, class C>
cudaError_t launch_step_sweep3(const StepParams<T, C>& p, bool uniform, cudaStream_t s) {
  Sweep3Maps maps;
  if (!maps_for(p, &maps)) return cudaErrorInvalidValue;
  // planes per block: 16 where that still gives every SM 8 blocks, fewer on small grids
  const long long tiles = (long long)((p.Nz + 31) / 32) * ((p.Ny + kTY - 1) / kTY);
  int R = 16;
  while (R > 2 && tiles * ((p.Nx + R - 1) / R) < 152LL * 8) R /= 2;
  const dim3 block(32, kTY + 1), grid((unsigned)((p.Nz + 31) / 32), (unsigned)((p.Ny + kTY - 1) / kTY),
                                      (unsigned)((p.Nx + R - 1) / R));
  const size_t smem = (size_t)kStages * StageLayout<T>::BYTES + sizeof(Exchange<C>);
  const bool mon = p.max_slot || p.etotal;
  auto go = [&](auto kernel) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kernel<<<grid, block, smem, s>>>(p, maps, R);
    return cudaGetLastError();
  };
  if (uniform) return mon ? go(step_kernel_3d<T, C, true, true>) : go(step_kernel_3d<T, C, true, false>);
  return mon ? go(step_kernel_3d<T, C, false, true>) : go(step_kernel_3d<T, C, false, false>);
}

template cudaError_t launch_step_sweep3<float, float>(const StepParams<float, float>&, bool, cudaStream_t);
template cudaError_t launch_step_sweep3<__half, float>(const StepParams<__half, float>&, bool, cudaStream_t);

}  // namespace lx
