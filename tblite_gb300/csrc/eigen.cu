// Generalised symmetric eigenproblem  F C = S C e  (reference src/tblite/lapack/sygvd.f90:125-151,
// LAPACK dsygvd itype 1, jobz V).
//
// Cholesky reduction: S = L L^T is factorised once per geometry (the reference refactorises S
// on every SCF iteration; the factor is the same).  Per iteration
//   A = L^-1 F L^-T  (two triangular solves),  A Y = Y e,  C = L^-T Y.
// The triangular solves and the dense tridiagonal eigensolver run on cuBLAS / cuSOLVER;
// the density matrix GEMM uses cuBLAS.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <cstdio>
#include <stdexcept>

#include "engine.h"

namespace tb {

struct EigenSolver {
  int n = 0;
  cudaStream_t stream = nullptr;
  cusolverDnHandle_t sol = nullptr;
  cublasHandle_t blas = nullptr;
  double* L = nullptr;     // Cholesky factor (lower, column-major == upper of row-major)
  double* work = nullptr;  // cuSOLVER workspace
  int lwork = 0;
  int* info = nullptr;     // device
  int* hinfo = nullptr;    // pinned host
};

static void check_cusolver(cusolverStatus_t st, const char* what) {
  if (st != CUSOLVER_STATUS_SUCCESS) {
    char buf[160];
    snprintf(buf, sizeof(buf), "cuSOLVER error %d in %s", (int)st, what);
    throw std::runtime_error(buf);
  }
}
static void check_cublas(cublasStatus_t st, const char* what) {
  if (st != CUBLAS_STATUS_SUCCESS) {
    char buf[160];
    snprintf(buf, sizeof(buf), "cuBLAS error %d in %s", (int)st, what);
    throw std::runtime_error(buf);
  }
}
static void check_cuda(cudaError_t st, const char* what) {
  if (st != cudaSuccess) {
    char buf[200];
    snprintf(buf, sizeof(buf), "CUDA error '%s' in %s", cudaGetErrorString(st), what);
    throw std::runtime_error(buf);
  }
}

EigenSolver* eigen_create(int n, cudaStream_t s) {
  auto* e = new EigenSolver();
  e->n = n;
  e->stream = s;
  check_cusolver(cusolverDnCreate(&e->sol), "create");
  check_cusolver(cusolverDnSetStream(e->sol, s), "set stream");
  check_cublas(cublasCreate(&e->blas), "cublas create");
  check_cublas(cublasSetStream(e->blas, s), "cublas stream");
  check_cuda(cudaMalloc(&e->L, sizeof(double) * (size_t)n * n), "alloc L");
  check_cuda(cudaMalloc(&e->info, sizeof(int)), "alloc info");
  check_cuda(cudaMallocHost(&e->hinfo, sizeof(int)), "alloc hinfo");
  int lw1 = 0, lw2 = 0;
  check_cusolver(cusolverDnDpotrf_bufferSize(e->sol, CUBLAS_FILL_MODE_LOWER, n, e->L, n, &lw1),
                 "potrf ws");
  check_cusolver(cusolverDnDsyevd_bufferSize(e->sol, CUSOLVER_EIG_MODE_VECTOR,
                                             CUBLAS_FILL_MODE_LOWER, n, e->L, n, nullptr, &lw2),
                 "syevd ws");
  e->lwork = lw1 > lw2 ? lw1 : lw2;
  check_cuda(cudaMalloc(&e->work, sizeof(double) * (size_t)e->lwork), "alloc work");
  return e;
}

void eigen_destroy(EigenSolver* e) {
  if (!e) return;
  cudaFree(e->L);
  cudaFree(e->work);
  cudaFree(e->info);
  cudaFreeHost(e->hinfo);
  cublasDestroy(e->blas);
  cusolverDnDestroy(e->sol);
  delete e;
}

int eigen_set_overlap(EigenSolver* e, const double* S) {
  const int n = e->n;
  check_cuda(cudaMemcpyAsync(e->L, S, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice,
                             e->stream),
             "copy S");
  check_cusolver(cusolverDnDpotrf(e->sol, CUBLAS_FILL_MODE_LOWER, n, e->L, n, e->work, e->lwork,
                                  e->info),
                 "potrf");
  check_cuda(cudaMemcpyAsync(e->hinfo, e->info, sizeof(int), cudaMemcpyDeviceToHost, e->stream),
             "info");
  check_cuda(cudaStreamSynchronize(e->stream), "sync potrf");
  return *e->hinfo;
}

int eigen_solve(EigenSolver* e, double* F, double* C, double* w) {
  const int n = e->n;
  const double one = 1.0;
  // A = L^-1 F   (column-major view; F symmetric)
  check_cublas(cublasDtrsm(e->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                           CUBLAS_DIAG_NON_UNIT, n, n, &one, e->L, n, F, n),
               "trsm 1");
  // A = A L^-T
  check_cublas(cublasDtrsm(e->blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                           CUBLAS_DIAG_NON_UNIT, n, n, &one, e->L, n, F, n),
               "trsm 2");
  check_cusolver(cusolverDnDsyevd(e->sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, F,
                                  n, w, e->work, e->lwork, e->info),
                 "syevd");
  // C = L^-T Y
  check_cublas(cublasDtrsm(e->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                           CUBLAS_DIAG_NON_UNIT, n, n, &one, e->L, n, F, n),
               "trsm 3");
  if (C != F)
    check_cuda(cudaMemcpyAsync(C, F, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice,
                               e->stream),
               "copy C");
  check_cuda(cudaMemcpyAsync(e->hinfo, e->info, sizeof(int), cudaMemcpyDeviceToHost, e->stream),
             "info");
  check_cuda(cudaStreamSynchronize(e->stream), "sync syevd");
  return *e->hinfo;
}

// P = sum_{m<k} f_m C_m C_m^T  (C column-major): scale columns into work, then one GEMM
__global__ void k_scale_cols(int n, int k, const double* C, const double* f, double* out) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)n * k) return;
  out[t] = C[t] * f[t / n];
}

static cublasHandle_t g_blas = nullptr;
static cudaStream_t g_blas_stream = nullptr;

void density_matrix(int n, int k, const double* C, const double* f, double* P, double* work,
                    cudaStream_t s) {
  if (!g_blas) check_cublas(cublasCreate(&g_blas), "create");
  if (g_blas_stream != s) {
    check_cublas(cublasSetStream(g_blas, s), "stream");
    g_blas_stream = s;
  }
  if (k <= 0) {
    cudaMemsetAsync(P, 0, sizeof(double) * (size_t)n * n, s);
    return;
  }
  const size_t tot = (size_t)n * k;
  ++g_kernel_launches;
  k_scale_cols<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, k, C, f, work);
  const double one = 1.0, zero = 0.0;
  // P(n x n) = work(n x k) * C(n x k)^T
  check_cublas(cublasDgemm(g_blas, CUBLAS_OP_N, CUBLAS_OP_T, n, n, k, &one, work, n, C, n, &zero,
                           P, n),
               "gemm P");
}

}  // namespace tb
