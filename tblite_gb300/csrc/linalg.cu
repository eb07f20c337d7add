// Dense FP64 linear algebra kernels of the engine: tiled GEMM with triangle-aware k ranges,
// Cholesky factorisation and the inverse of its transpose (once per geometry).
//
// GB300 executes FP64 at ~2 FMA/clk/SM, so these kernels are arithmetic bound even from L2;
// the tiling only has to keep every SM busy (small tiles, many CTAs) and avoid wasted work on
// the zero triangles of triangular operands.  All matrices are column-major
// (element (i, j) at p[i + j*ld]) as in BLAS.
#include <cooperative_groups.h>
#include <stdexcept>
#include <string>
#include <cuda_runtime.h>

#include "engine.h"

namespace cg = cooperative_groups;

namespace tb {

// ------------------------------------------------------------------------------------------
// GEMM:  C = alpha op(A) op(B) + beta C ,  op(A): M x K,  op(B): K x N
// kmode restricts the summation range when an operand is triangular:
//   KM_NONE        0 <= k < K
//   KM_LT_COLEND   k <  column tile end   (op(B) upper triangular:  B(k,j) = 0 for k > j)
//   KM_LT_ROWEND   k <  row tile end      (op(A) lower triangular:  A(i,k) = 0 for k > i)
//   KM_GE_ROWBEG   k >= row tile begin    (op(A) upper triangular:  A(i,k) = 0 for k < i)
// KM_SYM marks a symmetric product (M == N, square tiles): tiles above the diagonal are not
// computed, the others (and the lower half of a diagonal tile) are written twice (C(i,j) and
// C(j,i)), so C is exactly symmetric.
// ------------------------------------------------------------------------------------------
template <int BM, int BN, int BK, int TM, int TN>
__device__ __forceinline__ void gemm_dev(int M, int N, int K, double alpha, const double* __restrict__ A, int lda, bool ta,
           const double* __restrict__ B, int ldb, bool tb, double beta, double* __restrict__ C,
           int ldc, int kmode) {
  constexpr int NT = (BM / TM) * (BN / TN);
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  static_assert(!(BM != BN), "square tiles");
  const int i0 = blockIdx.y * BM, j0 = blockIdx.x * BN;
  const bool sym = (kmode & KM_SYM) != 0;
  if (sym && i0 < j0) return;  // above the diagonal: written by the mirror tile
  kmode &= 7;
  const int tid = threadIdx.x;
  const int tr = tid / (BN / TN), tc = tid % (BN / TN);
  int kbeg = 0, kend = K;
  if (kmode == KM_LT_COLEND) kend = min(K, j0 + BN);
  else if (kmode == KM_LT_ROWEND) kend = min(K, i0 + BM);
  else if (kmode == KM_GE_ROWBEG) kbeg = (i0 / BK) * BK;
  double acc[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) acc[a][b] = 0.0;
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    for (int t = tid; t < BM * BK; t += NT) {
      const int ii = ta ? t / BK : t % BM, kk = ta ? t % BK : t / BM;
      const int gi = i0 + ii, gk = k0 + kk;
      double v = 0.0;
      if (gi < M && gk < kend) v = ta ? A[gk + (size_t)gi * lda] : A[gi + (size_t)gk * lda];
      As[kk][ii] = v;
    }
    for (int t = tid; t < BK * BN; t += NT) {
      const int kk = tb ? t / BN : t % BK, jj = tb ? t % BN : t / BK;
      const int gk = k0 + kk, gj = j0 + jj;
      double v = 0.0;
      if (gj < N && gk < kend) v = tb ? B[gj + (size_t)gk * ldb] : B[gk + (size_t)gj * ldb];
      Bs[kk][jj] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[TM], b[TN];
#pragma unroll
      for (int x = 0; x < TM; ++x) a[x] = As[kk][tr * TM + x];
#pragma unroll
      for (int y = 0; y < TN; ++y) b[y] = Bs[kk][tc * TN + y];
#pragma unroll
      for (int x = 0; x < TM; ++x)
#pragma unroll
        for (int y = 0; y < TN; ++y) acc[x][y] = fma(a[x], b[y], acc[x][y]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int x = 0; x < TM; ++x) {
    const int gi = i0 + tr * TM + x;
    if (gi >= M) continue;
#pragma unroll
    for (int y = 0; y < TN; ++y) {
      const int gj = j0 + tc * TN + y;
      if (gj >= N) continue;
      if (sym && gi < gj) continue;  // diagonal tile: the upper entries are mirrors too
      double* c = C + gi + (size_t)gj * ldc;
      const double v = beta == 0.0 ? alpha * acc[x][y] : alpha * acc[x][y] + beta * *c;
      *c = v;
      if (sym && gi != gj) C[gj + (size_t)gi * ldc] = v;
    }
  }
}
template <int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    k_gemm(int M, int N, int K, double alpha, const double* __restrict__ A, int lda, bool ta,
           const double* __restrict__ B, int ldb, bool tb, double beta, double* __restrict__ C,
           int ldc, int kmode) {
  gemm_dev<BM, BN, BK, TM, TN>(M, N, K, alpha, A, lda, ta, B, ldb, tb, beta, C, ldc, kmode);
}

int device_sm_count() {
  constexpr int kMaxDevices = 64;
  static std::atomic<int> cache[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 1;
  int nsm = cache[dev].load(std::memory_order_relaxed);
  if (nsm <= 0) {
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        nsm <= 0)
      nsm = 1;
    cache[dev].store(nsm, std::memory_order_relaxed);
  }
  return nsm;
}

cudaError_t gemm64(bool ta, bool tb, int M, int N, int K, double alpha, const double* A,
                   int lda, const double* B, int ldb, double beta, double* C, int ldc, int kmode,
                   cudaStream_t s) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  const int tk = prof_kbegin(s);
  void* args[] = {&M, &N, &K, &alpha, (void*)&A, &lda, &ta, (void*)&B, &ldb, &tb, &beta, &C,
                  &ldc, &kmode};
  cudaError_t e;
  // small problems: 16x16 tiles keep enough CTAs in flight (two 32x32 tiles per SM or fewer)
  if ((long long)((M + 31) / 32) * ((N + 31) / 32) < 2LL * device_sm_count()) {
    dim3 grid((N + 15) / 16, (M + 15) / 16);
    ++g_kernel_launches;
    e = cudaLaunchKernel((const void*)k_gemm<16, 16, 16, 2, 2>, grid, dim3(64), args, 0, s);
  } else {
    dim3 grid((N + 31) / 32, (M + 31) / 32);
    ++g_kernel_launches;
    e = cudaLaunchKernel((const void*)k_gemm<32, 32, 16, 4, 4>, grid, dim3(64), args, 0, s);
  }
  prof_kend(KS_GEMM, tk, s);
  return e;
}

// ------------------------------------------------------------------------------------------
// Cholesky S = L L^T (lower, in place, column-major), right looking, one grid barrier per
// column: warps own trailing columns and update them with the (not yet scaled) pivot column.
// status: 0 ok, j+1 if the j-th pivot is not positive.
// ------------------------------------------------------------------------------------------
__global__ void k_cholesky(int n, double* A, int* status) {
  cg::grid_group grid = cg::this_grid();
  const int lane = threadIdx.x & 31;
  const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarp = (gridDim.x * blockDim.x) >> 5;
  for (int j = 0; j < n; ++j) {
    const double piv = A[j + (size_t)j * n];
    if (!(piv > 0.0)) {
      if (gwarp == 0 && lane == 0) *status = j + 1;
      return;  // every thread reads the same pivot and leaves together
    }
    const double inv = 1.0 / piv;
    for (int c = j + 1 + gwarp; c < n; c += nwarp) {
      const double ljc = A[c + (size_t)j * n] * inv;
      double* col = A + (size_t)c * n;
      const double* pj = A + (size_t)j * n;
      for (int i = c + lane; i < n; i += 32) col[i] -= pj[i] * ljc;
    }
    grid.sync();
  }
  if (gwarp == 0 && lane == 0) *status = 0;
}

// scale columns: L(i,j) = A(i,j)/sqrt(A(j,j)), zero the strict upper triangle
__device__ __forceinline__ void chol_scale_dev(int n, double* A) {
  const int j = blockIdx.x;
  const double d = sqrt(A[j + (size_t)j * n]);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double* p = A + i + (size_t)j * n;
    if (i < j) *p = 0.0;
    else if (i > j) *p = *p / d;
  }
  __syncthreads();
  if (threadIdx.x == 0) A[j + (size_t)j * n] = d;
}
__global__ void k_chol_scale(int n, double* A) {
  chol_scale_dev(n, A);
}

// X = L^-T (upper triangular): column j solves L^T x = e_j by back substitution; the dot
// products read columns of L, which are contiguous.  One warp per column.
__device__ __forceinline__ void tri_inv_t_dev(int n, const double* __restrict__ L, double* X) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= n) return;
  double* x = X + (size_t)j * n;
  for (int i = lane; i < n; i += 32) x[i] = 0.0;
  __syncwarp();
  if (lane == 0) x[j] = 1.0 / L[j + (size_t)j * n];
  __syncwarp();
  for (int i = j - 1; i >= 0; --i) {
    const double* li = L + (size_t)i * n;  // column i of L
    double s = 0.0;
    for (int k = i + 1 + lane; k <= j; k += 32) s += li[k] * x[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[i] = -s / li[i];
    __syncwarp();
  }
}
__global__ void k_tri_inv_t(int n, const double* __restrict__ L, double* X) {
  tri_inv_t_dev(n, L, X);
}

// Shared-memory resident Cholesky: column j lives in block j % nb for the whole factorisation.
// Step j: the owner scales its column and publishes it (double-buffered by parity of j), one
// grid barrier, every block updates its own trailing columns from the published column.
constexpr size_t CHOL_SMEM_MAX = 200 * 1024;

__global__ void __launch_bounds__(256) k_cholesky_smem(int n, double* A, double* buf, int* status) {
  cg::grid_group grid = cg::this_grid();
  extern __shared__ double sm[];
  const int nb = gridDim.x, b = blockIdx.x;
  const int ncpb = (n + nb - 1) / nb;
  double* scol = sm;                   // [ncpb][n]
  double* sl = sm + (size_t)ncpb * n;  // [n] published column
  for (int s = 0; s < ncpb; ++s) {
    const int j = b + s * nb;
    if (j >= n) break;
    for (int r = threadIdx.x; r < n; r += blockDim.x) scol[(size_t)s * n + r] = A[r + (size_t)j * n];
  }
  if (b == 0 && threadIdx.x == 0) *status = 0;
  __syncthreads();
  grid.sync();
  for (int j = 0; j < n; ++j) {
    double* pub = buf + (size_t)(j & 1) * n;
    if (j % nb == b) {
      double* col = scol + (size_t)(j / nb) * n;
      const double piv = col[j];
      if (!(piv > 0.0)) {
        if (threadIdx.x == 0) *status = j + 1;
      } else {
        const double dd = sqrt(piv), inv = 1.0 / dd;
        for (int r = j + threadIdx.x; r < n; r += blockDim.x) {
          const double v = r == j ? dd : col[r] * inv;
          col[r] = v;
          pub[r] = v;
          A[r + (size_t)j * n] = v;
        }
        for (int r = threadIdx.x; r < j; r += blockDim.x) A[r + (size_t)j * n] = 0.0;
      }
    }
    grid.sync();
    if (*(volatile int*)status != 0) return;  // every block sees the same flag
    for (int r = j + 1 + threadIdx.x; r < n; r += blockDim.x) sl[r] = pub[r];
    __syncthreads();
    for (int s = 0; s < ncpb; ++s) {
      const int c = b + s * nb;
      if (c <= j || c >= n) continue;
      double* col = scol + (size_t)s * n;
      const double lcj = sl[c];
      for (int r = c + threadIdx.x; r < n; r += blockDim.x) col[r] -= sl[r] * lcj;
    }
    __syncthreads();
  }
}

int cholesky_inverse(int n, double* L, double* X, int* d_status, int* h_status, cudaStream_t s) {
  {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int nb = nsm;
    const int need = (n + 7) / 8;  // at least 8 columns per block
    if (nb > need) nb = need > 0 ? need : 1;
    const size_t ncpb = (n + nb - 1) / nb;
    const size_t smem = sizeof(double) * (ncpb + 1) * (size_t)n;
    if (smem <= CHOL_SMEM_MAX) {
      static bool attr = false;
      if (!attr) {
        cudaFuncSetAttribute(k_cholesky_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)CHOL_SMEM_MAX);
        attr = true;
      }
      double* buf = X;  // X is written after the factorisation; use it as the publish buffer
      void* args[] = {&n, &L, &buf, &d_status};
      ++g_kernel_launches;
      cudaError_t e = cudaLaunchCooperativeKernel((void*)k_cholesky_smem, nb, 256, args, smem, s);
      if (e != cudaSuccess) return -1;
      cudaMemcpyAsync(h_status, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
      stream_wait(s);
      if (*h_status != 0) return *h_status;
      ++g_kernel_launches;
      k_tri_inv_t<<<(n * 32 + 255) / 256, 256, 0, s>>>(n, L, X);
      return 0;
    }
  }
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cholesky, 256, 0);
  (void)per_sm;
  int blocks = nsm;  // one block per SM keeps the grid barrier cheap
  const int need = (n * 32 + 255) / 256;
  if (blocks > need) blocks = need > 0 ? need : 1;
  void* args[] = {&n, &L, &d_status};
  ++g_kernel_launches;
  cudaError_t e = cudaLaunchCooperativeKernel((void*)k_cholesky, blocks, 256, args, 0, s);
  if (e != cudaSuccess) return -1;
  cudaMemcpyAsync(h_status, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
  stream_wait(s);
  if (*h_status != 0) return *h_status;
  ++g_kernel_launches;
  k_chol_scale<<<n, 256, 0, s>>>(n, L);
  ++g_kernel_launches;
  k_tri_inv_t<<<(n * 32 + 255) / 256, 256, 0, s>>>(n, L, X);
  return 0;
}

// ------------------------------------------------------------------------------------------
// Batched launches (blockIdx.z walks the listed molecules)
// ------------------------------------------------------------------------------------------
#define BMOL const MolPtrs& q = mp[list[blockIdx.z]]
#define BARGS const MolPtrs* __restrict__ mp, const int* __restrict__ list

template <int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN)) kb_gemm(BARGS, int site) {
  BMOL;
  const int n = q.m.nao;
  const int k = *q.icount;
  int M = n, N = n, K = n, km = KM_NONE;
  double alpha = 1.0;
  const double *A = nullptr, *B = nullptr;
  double* C = nullptr;
  bool ta = false, tb = false;
  switch (site) {
    case GS_FX: A = q.F; B = q.X; C = q.T1; km = KM_LT_COLEND; break;
    case GS_XTT: A = q.X; ta = true; B = q.T1; C = q.A; km = KM_LT_ROWEND | KM_SYM; break;
    case GS_XY: A = q.X; B = q.Y; C = q.C; N = k; km = KM_GE_ROWBEG; break;
    case GS_DENS: A = q.scratch; B = q.C; tb = true; C = q.P; K = k; km = KM_SYM; break;
    case GS_WDENS: A = q.scratch; B = q.C; tb = true; C = q.F; K = k; km = KM_SYM; break;
    case GS_FS: A = q.F; B = q.S; C = q.scratch; break;
    case GS_PS: A = q.P; B = q.S; C = q.scratch; break;
    case GS_XD: A = q.X; B = q.Y; C = q.T1; km = KM_GE_ROWBEG; alpha = 2.0; break;
    case GS_PXT: A = q.T1; B = q.X; tb = true; C = q.P; km = KM_SYM; break;
    case GS_PF: A = q.P; B = q.F; C = q.T1; alpha = 0.5; break;
    default: A = q.T1; B = q.P; C = q.F; km = KM_SYM; break;  // GS_WPFP
  }
  if ((int)blockIdx.x * BN >= N || (int)blockIdx.y * BM >= M) return;  // tile outside
  if (*q.flag < 0) return;  // the molecule has left the batch
  gemm_dev<BM, BN, BK, TM, TN>(M, N, K, alpha, A, n, ta, B, n, tb, 0.0, C, n, km);
}

bool g_split_gemm = true;

void gemm_b(const BatchLaunch& b, int site) {
  if (!b.count) return;
  if (g_split_gemm && b.nao_max >= 128) {
    ogemm_b(b, site);
    return;
  }
  const int tk = prof_kbegin(b.s);
  ++g_kernel_launches;
  if (b.nao_max <= 128) {
    const unsigned t = (b.nao_max + 15) / 16;
    kb_gemm<16, 16, 16, 2, 2><<<dim3(t, t, b.count), 64, 0, b.s>>>(b.mp, b.list, site);
  } else {
    const unsigned t = (b.nao_max + 31) / 32;
    kb_gemm<32, 32, 16, 4, 4><<<dim3(t, t, b.count), 64, 0, b.s>>>(b.mp, b.list, site);
  }
  prof_kend(KS_GEMM, tk, b.s);
}

// Cholesky S = L L^T of one molecule per block, in T1 (column-major lower, L2 resident),
// blocked by panels of CHOL_NB columns.  The panel (rows j0..n-1) is factorised in shared
// memory (per column: scale by 1/sqrt(pivot), rank-1 update of the panel's later columns),
// written back, and the trailing lower triangle takes the panel's CHOL_NB rank-1 updates at
// once: 64 x 64 tiles, a 4 x 4 register block per thread, the panel rows from shared memory.
// Each trailing element is read and written once per panel instead of once per column, so the
// update runs on the FP64 pipe instead of waiting on L2.  A pivot that is not positive marks
// the molecule failed (flag -2); it is read after a barrier, so the whole block leaves together.
constexpr int CHOL_NB = 16;
__global__ void __launch_bounds__(256) kb_cholesky(BARGS) {
  BMOL;
  const int n = q.m.nao;
  double* A = q.T1;
  extern __shared__ double pan[];  // [CHOL_NB][m] panel, column-major (m = n - j0 rows)
  __shared__ int bad;
  const int tid = threadIdx.x;
  const size_t nn = (size_t)n * n;
  for (size_t t = tid; t < nn; t += blockDim.x) A[t] = q.S[t];  // S symmetric
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int j0 = 0; j0 < n; j0 += CHOL_NB) {
    const int nb = min(CHOL_NB, n - j0), m = n - j0;
    for (int t = tid; t < nb * m; t += blockDim.x) {
      const int c = t / m, r = t % m;
      pan[(size_t)c * m + r] = A[(size_t)(j0 + c) * n + j0 + r];
    }
    __syncthreads();
    for (int jj = 0; jj < nb; ++jj) {
      double* cj = pan + (size_t)jj * m;
      const double piv = cj[jj];
      if (!(piv > 0.0)) {
        if (tid == 0) bad = 1;
        break;
      }
      const double d = sqrt(piv), inv = 1.0 / d;
      for (int r = jj + 1 + tid; r < m; r += blockDim.x) cj[r] *= inv;
      __syncthreads();
      if (tid == 0) cj[jj] = d;
      for (int t = tid; t < (nb - jj - 1) * m; t += blockDim.x) {  // later panel columns
        const int c = jj + 1 + t / m, r = t % m;
        if (r >= c) pan[(size_t)c * m + r] -= cj[r] * cj[c];
      }
      __syncthreads();
    }
    __syncthreads();
    if (bad) {
      if (tid == 0) *q.flag = -2;
      return;
    }
    for (int t = tid; t < nb * m; t += blockDim.x) {
      const int c = t / m, r = t % m;
      if (r >= c) A[(size_t)(j0 + c) * n + j0 + r] = pan[(size_t)c * m + r];
    }
    // trailing update of rows and columns j0 + nb .. n-1 (lower triangle)
    const int m2 = m - nb, nt = (m2 + 63) / 64;
    const int tr = tid & 15, tc = tid >> 4;
    for (int tile = 0; tile < nt * (nt + 1) / 2; ++tile) {
      int ti = 0;
      while ((ti + 1) * (ti + 2) / 2 <= tile) ++ti;
      const int tj = tile - ti * (ti + 1) / 2;  // tile row ti >= tile column tj
      const int r0 = nb + 64 * ti, c0 = nb + 64 * tj;  // panel-relative rows / columns
      double acc[4][4];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
      for (int k = 0; k < nb; ++k) {
        const double* pk = pan + (size_t)k * m;
        double pr[4], pc[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const int r = r0 + tr + 16 * a, c = c0 + tc + 16 * a;
          pr[a] = r < m ? pk[r] : 0.0;
          pc[a] = c < m ? pk[c] : 0.0;
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] = fma(pr[a], pc[b], acc[a][b]);
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int r = r0 + tr + 16 * a, c = c0 + tc + 16 * b;
          if (r < m && c < m && r >= c) A[(size_t)(j0 + c) * n + j0 + r] -= acc[a][b];
        }
    }
    __syncthreads();
  }
  for (size_t t = tid; t < nn; t += blockDim.x) {
    const int i = (int)(t % n), j = (int)(t / n);
    if (i < j) A[t] = 0.0;
  }
}

// X = L^-T of the batch, one warp per column j of X (back substitution x_i = -(sum_{i<k<=j}
// L_ki x_k) / L_ii for i = j-1 .. 0).  The column stays in registers across the warp (element k
// on lane k % 32), so the chain of j steps waits only on a warp sum and a multiplication; the
// column of L that the next step needs is loaded one step ahead, the reciprocals of the
// diagonal are formed once per warp (spread over its lanes), and only the registers holding
// rows i+1 .. j take part in a step's sum.
// Orders beyond 32 TRI_INV_R take the general form.
constexpr int TRI_INV_R = 18;
__device__ __forceinline__ void tri_col_load(const double* __restrict__ L, int n, int i, int j,
                                             int lane, double (&v)[TRI_INV_R]) {
#pragma unroll
  for (int t = 0; t < TRI_INV_R; ++t) {
    const int k = lane + 32 * t;
    v[t] = (k > i && k <= j) ? L[k + (size_t)i * n] : 0.0;
  }
}
__global__ void kb_tri_inv_t(BARGS) {
  BMOL;
  if (*q.flag < 0) return;
  const int n = q.m.nao;
  if (n > 32 * TRI_INV_R) {
    tri_inv_t_dev(n, q.T1, q.X);
    return;
  }
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= n) return;
  const double* __restrict__ L = q.T1;
  double xr[TRI_INV_R];
  const double xjj = 1.0 / L[j + (size_t)j * n];
#pragma unroll
  for (int t = 0; t < TRI_INV_R; ++t) xr[t] = (lane + 32 * t == j) ? xjj : 0.0;
  // reciprocals of the diagonal elements L_kk, k < j, one per lane and register (a few
  // divisions per warp instead of one per step); step i takes its own by a shuffle
  double rd[TRI_INV_R];
#pragma unroll
  for (int t = 0; t < TRI_INV_R; ++t) {
    const int k = lane + 32 * t;
    rd[t] = k < j ? 1.0 / L[k + (size_t)k * n] : 1.0;
  }
  double cur[TRI_INV_R];
  if (j > 0) tri_col_load(L, n, j - 1, j, lane, cur);
  const int thi = j >> 5;
  for (int i = j - 1; i >= 0; --i) {
    double nxt[TRI_INV_R];
    if (i > 0) tri_col_load(L, n, i - 1, j, lane, nxt);
    double rsel = 1.0;
#pragma unroll
    for (int t = 0; t < TRI_INV_R; ++t)
      if (t == (i >> 5)) rsel = rd[t];
    const double rcur = __shfl_sync(0xffffffffu, rsel, i & 31);
    const int tlo = (i + 1) >> 5;  // registers that hold rows i+1 .. j (a warp-uniform range)
    double s = 0.0;
#pragma unroll
    for (int t = 0; t < TRI_INV_R; ++t)
      if (t >= tlo && t <= thi) s = fma(cur[t], xr[t], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const double xi = -s * rcur;
#pragma unroll
    for (int t = 0; t < TRI_INV_R; ++t)
      if (lane + 32 * t == i) xr[t] = xi;
    if (i > 0) {
#pragma unroll
      for (int t = 0; t < TRI_INV_R; ++t) cur[t] = nxt[t];
    }
  }
  double* x = q.X + (size_t)j * n;
#pragma unroll
  for (int t = 0; t < TRI_INV_R; ++t) {
    const int k = lane + 32 * t;
    if (k < n) x[k] = xr[t];
  }
}

void cholesky_inverse_b(const BatchLaunch& b) {
  if (!b.count) return;
  g_kernel_launches += 2;
  const size_t smem = (size_t)CHOL_NB * b.nao_max * sizeof(double);
  static size_t attr = 0;  // the kernel's static shared memory comes on top of smem
  if (smem > attr) {
    const cudaError_t e = cudaFuncSetAttribute(
        kb_cholesky, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
      throw std::runtime_error(std::string("CUDA error '") + cudaGetErrorString(e) +
                               "' in batched Cholesky shared memory");
    attr = smem;
  }
  kb_cholesky<<<dim3(1, 1, b.count), 256, smem, b.s>>>(b.mp, b.list);
  kb_tri_inv_t<<<dim3((b.nao_max * 32 + 255) / 256, 1, b.count), 256, 0, b.s>>>(b.mp, b.list);
}

#undef BMOL
#undef BARGS

}  // namespace tb
