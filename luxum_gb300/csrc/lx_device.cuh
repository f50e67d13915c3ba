// lx_device.cuh -- device helpers shared by the update kernels (lx_kernels.cu, lx_sweep3d.cu):
// storage access in the three precision forms, the CPML psi recursion, TF/SF increments and
// the max|E|^2 block reduction.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lx_internal.h"

namespace lx {

// ------------------------------------------------------------------ storage access

template <class T, class C>
__device__ __forceinline__ C ld(const T* p) {
  return static_cast<C>(*p);
}
template <>
__device__ __forceinline__ float ld<__half, float>(const __half* p) {
  return __half2float(*p);
}
template <class T, class C>
__device__ __forceinline__ void st(T* p, C v) {
  *p = static_cast<T>(v);
}
template <>
__device__ __forceinline__ void st<__half, float>(__half* p, float v) {
  *p = __float2half_rn(v);
}

__device__ __forceinline__ double fmaC(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmaC(float a, float b, float c) { return fmaf(a, b, c); }
// A rounded product that is never contracted into a neighbouring add: the 1/d factors of
// non-uniform spacing.  Contraction decisions differ between kernels, and the single-sweep
// and two-sweep planar kernels must give the same bits (the oracle does not contract).
__device__ __forceinline__ double mulC(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mulC(float a, float b) { return __fmul_rn(a, b); }

// ------------------------------------------------------------------ TF/SF

// Adds the increments of the planes of `ps` that cell (i,j,k) lies on to d (reference:
// curl = curl +/- exp(...) * dir / d..., one line of plane_wave_execute per plane).
template <class C>
__device__ __forceinline__ void tfsf_apply(const PatchSet& ps, const C* tab, int i, int j, int k, C& d) {
  if (!ps.active) return;
  const int a = ps.axis;
  const int n = a == 0 ? i : (a == 1 ? j : k);
  const bool h0 = (n == ps.plane[0]);
  const bool h1 = (n == ps.plane[1]);
  if (!(h0 || h1)) return;
  // in-plane ranges and table offset (the normal axis has lo = hi = 0 and stride 0 in the
  // checks below, so it is excluded by selecting 0 for it)
  const int ui = a == 0 ? 0 : i - ps.lo[0], uj = a == 1 ? 0 : j - ps.lo[1], uk = a == 2 ? 0 : k - ps.lo[2];
  const int wi = a == 0 ? 0 : ps.hi[0] - ps.lo[0], wj = a == 1 ? 0 : ps.hi[1] - ps.lo[1], wk = a == 2 ? 0 : ps.hi[2] - ps.lo[2];
  if (ui < 0 || uj < 0 || uk < 0 || ui > wi || uj > wj || uk > wk) return;
  const int off = ui * ps.stride[0] + uj * ps.stride[1] + uk * ps.stride[2];
  if (h0) d = d + tab[ps.tab + off];
  if (h1) d = d + tab[ps.tab + ps.plane_len + off];
}

// psi = b*psi + c*curl; returns curl/kappa + psi (reference: three_dim_pml.cc:186-188).
template <class C>
__device__ __forceinline__ C pml_term(C d, C* psi, C b, C cc, C rk) {
  C ps = fmaC(b, *psi, cc * d);
  *psi = ps;
  return fmaC(d, rk, ps);
}

__device__ __forceinline__ long long psi_index(int axis, const Slab& s, int si_, int i, int j, int k, int Ny,
                                               int Nzp) {
  if (axis == 0) return ((long long)si_ * Ny + j) * Nzp + k;
  if (axis == 1) return ((long long)i * s.n + si_) * Nzp + k;
  return ((long long)i * Ny + j) * s.n + si_;
}

// ------------------------------------------------------------------ monitor

// max|E|^2 is reduced on bit patterns: squares are non-negative, so their IEEE patterns
// order like their values, and NaN/inf sort above every finite value (blow-up detection).
// FP32 members reduce 32-bit float patterns and widen only the block's winner to the
// double pattern the monitor slot holds.
template <class C>
struct MaxBits;
template <>
struct MaxBits<double> {
  using type = unsigned long long;
  static __device__ __forceinline__ type of(double v) { return (unsigned long long)__double_as_longlong(v); }
};
template <>
struct MaxBits<float> {
  using type = unsigned;
  static __device__ __forceinline__ type of(float v) { return __float_as_uint(v); }
};

__device__ __forceinline__ unsigned long long as_slot_bits(unsigned long long v) { return v; }
__device__ __forceinline__ unsigned long long as_slot_bits(unsigned v) {
  return (unsigned long long)__double_as_longlong((double)__uint_as_float(v));
}
__device__ __forceinline__ unsigned long long warp_max(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}
__device__ __forceinline__ unsigned warp_max(unsigned v) { return __reduce_max_sync(0xffffffffu, v); }

// Block maximum of the bit patterns, then one atomicMax on the 64-bit slot per block.
template <class B>
__device__ __forceinline__ void block_max_atomic(B v, unsigned long long* slot) {
  __shared__ B red[32];
  v = warp_max(v);
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int nw = (blockDim.x * blockDim.y + 31) / 32;
  if ((tid & 31) == 0) red[tid >> 5] = v;
  __syncthreads();
  if (tid < 32) {
    v = warp_max(tid < nw ? red[tid] : B(0));
    if (tid == 0 && v) atomicMax(slot, as_slot_bits(v));
  }
}

// A computed value as a later load of the stored value returns it.
template <class T, class C>
__device__ __forceinline__ C stored(C v) {
  return static_cast<C>(static_cast<T>(v));
}
template <>
__device__ __forceinline__ float stored<__half, float>(float v) {
  return __half2float(__float2half_rn(v));
}

}  // namespace lx
