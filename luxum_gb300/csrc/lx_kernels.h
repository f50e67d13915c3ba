// lx_kernels.h -- host-side launchers of the kernels in lx_kernels.cu.
#pragma once
#include <cuda_runtime.h>

#include "lx_internal.h"

namespace lx {

template <class C>
cudaError_t launch_prologue(const PrologueParams& p, cudaStream_t s);
template <class T, class C>
cudaError_t launch_step(const StepParams<T, C>& p, bool planar, bool uniform, bool h_half, cudaStream_t s);
template <class T>
cudaError_t launch_gather(const T* src, double* dst, const int ext[3], int Ny, int Nzp, cudaStream_t s);
template <class T>
cudaError_t launch_scatter(const double* src, T* dst, const int ext[3], int Ny, int Nzp, int mode, double a, double dt,
                           double eps0, double scale, cudaStream_t s);
template <class C>
cudaError_t launch_eps_box(C* dst, const int ext[3], int Ny, int Nzp, const int lo[3], const int hi[3], double val,
                           cudaStream_t s);
template <class T>
cudaError_t launch_probes(const ProbeParams& pp, T* const f[6], double* out, cudaStream_t s);

template <class T>
cudaError_t launch_dft(const DftParams& d, T* const f[4], cudaStream_t s);

template <class T, class C>
cudaError_t launch_batch_step(const StepParams<T, C>* ps, const Tile* tiles, int ntiles, bool planar, bool uniform,
                              bool h_half, cudaStream_t s);
template <class C>
cudaError_t launch_prologue_batch(const PrologueParams* pps, const int* ts, int nsims, int max_entries, cudaStream_t s);
cudaError_t launch_tick(int* ts, int n, cudaStream_t s);
template <class T>
cudaError_t launch_dft_batch(const DftParams* ds, int nplanes, long long max_cells4, const int* ts, cudaStream_t s);

}  // namespace lx
