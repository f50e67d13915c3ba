// lx_noalloc.cu -- lx_sim_read_field_noalloc: reading a field without any device allocation.
//
// lx_sim_read_field compacts a component from the padded device layout into a staging
// buffer that the library allocates with cudaMalloc on first use (sized for the largest
// component), then copies it to the host.  Some callers cannot let the library allocate at
// that point: processes whose device memory is owned by another allocator (a framework's
// caching allocator that has reserved most of the GPU, so a fresh cudaMalloc fails or
// fragments its pool), and loops with latency budgets, where cudaMalloc/cudaFree may
// synchronise the whole device.  This entry point does the same compaction into a fixed
// staging array that lives in the library's own static device memory instead.
//
// The staging array below is a file-scope __device__ array of kLxNoAllocMaxElems doubles
// (8 MiB).  Every GPU that loads the library holds it until the process exits, whether or
// not the entry point is ever called.  Its host-side name is only a stand-in for the symbol:
// the device address is looked up once per device with cudaGetSymbolAddress, on the first
// call for a handle of that device (with that device made current for the call), and cached.
// Because that first call performs the lookup, it should be made before any stream capture
// begins.
//
// Every call on a device shares the one array and leaves the last call's data in it.  Calls
// whose device work overlaps (two handles read on different streams at once, or two host
// threads) race on it; callers must order them, e.g. by using one stream.  Nothing in the
// array needs to start at zero: each call writes every element it later copies out.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "luxum.h"
#include "lx_sim.h"

namespace lx {
lx_status set_thread_error(const char* msg, lx_status st);
}

namespace {

constexpr size_t kLxNoAllocMaxElems = size_t(1) << 20;  // 8 MiB of doubles
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_noalloc_staging[kLxNoAllocMaxElems];

std::mutex g_mu;
double* g_staging_ptr[kMaxDevices] = {};

// Device address of the staging array on device `dev`, which the caller has made current
// (looked up once per device).
cudaError_t staging_address(int dev, double** out) {
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  cudaError_t e;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_staging_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_staging);
    if (e != cudaSuccess) return e;
    g_staging_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_staging_ptr[dev];
  return cudaSuccess;
}

// padded (Nx,Ny,Nzp) storage -> dense doubles of extent (n0,n1,n2) in the static array
template <class T>
__global__ void gather_to_staging(const T* __restrict__ src, double* __restrict__ dst, int n0, int n1, int n2, int Ny,
                                  int Nzp, double mul) {
  const long long total = (long long)n0 * n1 * n2;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(q % n2);
    const long long r = q / n2;
    const int j = (int)(r % n1);
    const int i = (int)(r / n1);
    const T v = src[((long long)i * Ny + j) * Nzp + k];
    double w;
    if constexpr (sizeof(T) == 2) w = (double)__half2float(v);
    else w = (double)v;
    dst[q] = mul == 1.0 ? w : w * mul;  // H stored scaled (FP16 storage)
  }
}

template <class T>
void launch(const void* src, double* dst, const int ext[3], int Ny, int Nzp, double mul, cudaStream_t s) {
  const long long n = (long long)ext[0] * ext[1] * ext[2];
  long long g = (n + 255) / 256;
  if (g > 152LL * 64) g = 152LL * 64;
  gather_to_staging<T><<<(unsigned)(g < 1 ? 1 : g), 256, 0, s>>>((const T*)src, dst, ext[0], ext[1], ext[2], Ny, Nzp, mul);
}

}  // namespace

extern "C" LX_API lx_status lx_sim_read_field_noalloc(lx_sim* s, int comp, double* host, size_t n) {
  if (!s || !host) return lx::set_thread_error("null argument", LX_ERR_INVALID);
  lx::DeviceGuard dg_(s->device);  // the handle's device, for the lookup and the launch
  auto bad = [&](lx_status st, const std::string& m) {
    s->err = m;
    return lx::set_thread_error(m.c_str(), st);
  };
  if (comp < LX_EX || comp > LX_ETOTAL) return bad(LX_ERR_INVALID, "bad component");
  const size_t m = (size_t)s->ext[comp][0] * s->ext[comp][1] * s->ext[comp][2];
  if (n != m) return bad(LX_ERR_INVALID, "buffer size does not match the component's staggered extent");
  if (m > kLxNoAllocMaxElems)
    return bad(LX_ERR_INVALID, "component has " + std::to_string(m) + " values; lx_sim_read_field_noalloc handles at most " +
                                   std::to_string(kLxNoAllocMaxElems) + " (8 MiB of static staging); use lx_sim_read_field");
  if (m == 0) return LX_OK;
  if (s->batch) {  // a batch chunk in flight writes this handle's fields
    const lx_status st = lx_batch_wait(s->batch);
    if (st && st != LX_ERR_BLOWUP) return st;
  }
  const void* src = lx::comp_ptr(s, comp);  // the buffer holding the state after t steps
  if (!src) return bad(LX_ERR_STATE, comp == LX_ETOTAL ? "|E|^2 is only kept when a snapshot asks for it" : "component absent");
  double* staging = nullptr;
  cudaError_t e = staging_address(s->device, &staging);
  if (e != cudaSuccess) return bad(LX_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  const bool compute_prec = comp == LX_ETOTAL;
  const double mul = (comp >= LX_HX && comp <= LX_HZ) ? 1.0 / s->hscale : 1.0;
  if ((compute_prec ? s->csize == 8 : s->prec == LX_PREC_FP64)) launch<double>(src, staging, s->ext[comp], s->Ny, s->Nzp, mul, s->stream);
  else if (compute_prec || s->prec == LX_PREC_FP32) launch<float>(src, staging, s->ext[comp], s->Ny, s->Nzp, mul, s->stream);
  else launch<__half>(src, staging, s->ext[comp], s->Ny, s->Nzp, mul, s->stream);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, staging, m * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return bad(LX_ERR_CUDA, std::string("lx_sim_read_field_noalloc: ") + cudaGetErrorString(e));
  s->n_kernels++;
  s->n_d2h += m * sizeof(double);
  return LX_OK;
}
