// lx_kernels.h -- host-side launchers of the kernels in lx_kernels.cu.
#pragma once
#include <cuda_runtime.h>

#include "lx_internal.h"

namespace lx {

template <class C>
cudaError_t launch_prologue(const PrologueParams& p, cudaStream_t s);
template <class T, class C>
cudaError_t launch_step(const StepParams<T, C>& p, bool planar, bool uniform, bool h_half, cudaStream_t s);
// Single-sweep planar step (float compute, two state buffers): reads the buffers named in
// p.E, p.H, p.psiH, p.psiE and writes those in p.E1, p.H1, p.psiH1, p.psiE1.
template <class T, class C>
cudaError_t launch_step_sweep2(const StepParams<T, C>& p, bool uniform, cudaStream_t s);
// Single-sweep 3-D step (float compute, two state buffers), lx_sweep3d.cu: the same buffer
// convention as launch_step_sweep2.
template <class T, class C>
cudaError_t launch_step_sweep3(const StepParams<T, C>& p, bool uniform, cudaStream_t s);
template <class T>
cudaError_t launch_gather(const T* src, double* dst, const int ext[3], int Ny, int Nzp, double mul, cudaStream_t s);
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

// Batched updates: member m of a group owns blocks [first[m], first[m+1]) of each launch;
// launch_batch_tiles turns that prefix into the per-block tile map the update kernels read.
template <class T, class C>
cudaError_t launch_batch_tiles(const StepParams<T, C>* ps, const int* first, int n, int nblocks, bool planar, int march,
                               int4* tiles, cudaStream_t s);
template <class T, class C>
cudaError_t launch_batch_step(const StepParams<T, C>* ps, const int4* tiles, int nblocks, bool planar, bool uniform,
                              int march, bool h_half, cudaStream_t s);
// blocks one member occupies in a batched update launch; march = cells each thread walks
// along x (planar: rows 8 apart; 3-D: planes), one of 1, 2, 4, 8
int batch_blocks(int Nx, int Ny, int Nz, bool planar, int march);
// block -> {member, block within the member} for a prefix `first` of n members
cudaError_t launch_block_map(const int* first, int n, int nblocks, int2* map, cudaStream_t s);
template <class C>
// step k of a chunk runs at ts[sim] + k; launch_tick advances ts by the chunk's steps
cudaError_t launch_prologue_batch(const PrologueParams* pps, const int* ts, int k, int nsims, int max_entries,
                                  cudaStream_t s);
cudaError_t launch_tick(int* ts, int n, int steps, cudaStream_t s);
template <class T>
cudaError_t launch_dft_batch(const DftParams* ds, const int2* map, int nplanes, int nblocks, const int* ts, int k,
                             cudaStream_t s);
cudaError_t launch_dft_flux(const double* acc, int nfreq, long long ncell, double* part, double dA, double* out,
                            cudaStream_t s);

}  // namespace lx
