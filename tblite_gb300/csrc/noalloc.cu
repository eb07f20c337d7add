// Density matrix P = C diag(f) C^T without any device allocation.
//
// The engine's own density step (density_matrix in eigen.cu) scales the occupied columns of C
// into a workspace buffer that the calculator allocates with the rest of its device memory,
// then runs one GEMM.  Some callers cannot allocate device memory at the moment they need a
// density matrix: a caller that has already handed the whole device to its own pool
// allocator (a further cudaMalloc would fail or fragment it), or a caller on a latency-bound
// loop where cudaMalloc/cudaFree would synchronise the device and stall its other streams.
// This variant takes the workspace from a fixed array of device memory that belongs to the
// library image itself, so a call performs no cudaMalloc/cudaFree and uses no allocating
// library.
//
// Limits and rules:
//   * n * k must not exceed TBLITE_GB300_NOALLOC_DENSITY_MAX (2^19 doubles = 4 MiB); larger
//     problems are rejected before anything is launched.
//   * Every call looks up the device address of the array with the caller's device current
//     (cudaGetSymbolAddress); the first call on a device can load the module there.  Make that
//     first call before any stream capture is started on the device.
//   * The array is shared by every call on a device: two calls that can run at the same time
//     (different streams, or different host threads) race on it.  Serialise them.
//   * Nothing in the array has to start at zero: the scale kernel writes all n*k entries that
//     the GEMM reads, on the same stream, before the GEMM runs.
#include <cuda_runtime.h>

#include <mutex>

#include "engine.h"

#define TBLITE_GB300_NOALLOC_DENSITY_MAX (1u << 19)

namespace tb {
namespace {

__device__ __align__(256) double g_density_scratch[TBLITE_GB300_NOALLOC_DENSITY_MAX];

// The device address of the fixed scratch array in the current device's context.  It is looked
// up on every call (cheap once the module is loaded), so a context that was torn down and
// created again (cudaDeviceReset) never sees a stale address.  The first lookup on a device can
// load the module; the mutex keeps concurrent first calls from different host threads apart.
std::mutex g_setup_mutex;
cudaError_t scratch_for_current_device(double** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  void* p = nullptr;
  const cudaError_t rc = cudaGetSymbolAddress(&p, g_density_scratch);
  if (rc != cudaSuccess) return rc;
  *out = static_cast<double*>(p);
  return cudaSuccess;
}

__global__ void k_scale_cols_fixed(int n, int k, const double* __restrict__ C,
                                   const double* __restrict__ f, double* __restrict__ out) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)n * k) return;
  out[t] = C[t] * f[t / n];
}

__global__ void k_zero(size_t count, double* __restrict__ out) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t < count) out[t] = 0.0;
}

}  // namespace
}  // namespace tb

extern "C" int tblite_gb300_density_matrix_noalloc(int n, int k, const double* C, const double* f,
                                                   double* P, void* stream) {
  using namespace tb;
  if (n <= 0 || k < 0 || k > n || !C || !f || !P) return -1;
  if ((size_t)n * (size_t)k > (size_t)TBLITE_GB300_NOALLOC_DENSITY_MAX) return -2;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* work = nullptr;
  if (scratch_for_current_device(&work) != cudaSuccess) return -3;
  // every launch is checked through its own return code, so an error left behind by an
  // earlier, unrelated launch is not reported as this call's failure
  if (k == 0) {  // no occupied orbital: P = 0
    size_t nn = (size_t)n * n;
    void* args[] = {&nn, &P};
    ++g_kernel_launches;
    if (cudaLaunchKernel((const void*)k_zero, dim3((unsigned)((nn + 255) / 256)), dim3(256), args,
                         0, s) != cudaSuccess)
      return -3;
  } else {
    const size_t tot = (size_t)n * k;
    void* args[] = {&n, &k, (void*)&C, (void*)&f, &work};
    ++g_kernel_launches;
    if (cudaLaunchKernel((const void*)k_scale_cols_fixed, dim3((unsigned)((tot + 255) / 256)),
                         dim3(256), args, 0, s) != cudaSuccess)
      return -3;
    if (gemm64(false, true, n, n, k, 1.0, work, n, C, n, 0.0, P, n, KM_SYM, s) != cudaSuccess)
      return -3;
  }
  return 0;
}

extern "C" int tblite_gb300_density_matrix_noalloc_max(void) {
  return (int)TBLITE_GB300_NOALLOC_DENSITY_MAX;
}
