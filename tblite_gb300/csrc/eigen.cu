// Generalised symmetric eigenproblem  F C = S C e  of the SCF (reference
// src/tblite/lapack/sygvd.f90:125-151, LAPACK dsygvd itype 1, jobz V), written for GB300.
//
//   once per geometry   S = L L^T (Cholesky), X = L^-T                      (linalg.cu)
//   every iteration     A = X^T F X            two triangle-aware GEMMs
//                       A = Q T Q^T            Householder tridiagonalisation, one cooperative
//                                              kernel, two grid barriers per column
//                       T y = y e              all eigenvalues by Sturm-count bisection
//   after Fermi filling eigenvectors only for the occupied orbitals: inverse iteration on T,
//                       clusters of close eigenvalues re-orthonormalised + Rayleigh-Ritz,
//                       back-transformation Z = Q Y (column blocks per CTA, reflectors
//                       staged in shared memory), C = X Z (triangular GEMM).
//
// The reference refactorises S on every call of dsygvd; the factor is identical, so it is
// computed once here.  Eigenvector signs are arbitrary in both codes; every quantity the
// engine derives (density, energy weighted density, charges) is sign invariant.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "engine.h"

namespace cg = cooperative_groups;

namespace tb {

static void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("CUDA error '") + cudaGetErrorString(e) + "' in " + what);
}

// GEMMs of the one-molecule path go to the tensor cores from 128 orbitals on
static inline bool split_gemm(int n) { return g_split_gemm && n >= 128; }

struct EigenSolver {
  int n = 0;
  cudaStream_t stream = nullptr;
  double *L = nullptr, *X = nullptr, *A = nullptr, *T1 = nullptr;
  double *d = nullptr, *e = nullptr, *tau = nullptr, *w = nullptr, *pv = nullptr, *scal = nullptr;
  double *lu = nullptr;   // inverse iteration scratch [5][n][n]
  double *tw = nullptr;   // eigenvalue scratch: e^2 [n] (double), d and e^2 [n] (float)
  double *Y = nullptr;    // eigenvectors of T, column-major [k][n]
  int* status = nullptr;  // device
  int* gstatus = nullptr; // device: 1 once a tensor-core GEMM did not answer
  int* hstatus = nullptr; // pinned
  int coop_blocks = 0;
  int cap = 0;  // buffers hold problems up to this order
};

int eigen_capacity(const EigenSolver* e) { return e ? e->cap : 0; }
void eigen_resize(EigenSolver* e, int n) {
  if (n > e->cap) throw std::runtime_error("eigen solver capacity exceeded");
  e->n = n;
}

// ------------------------------------------------------------------------------------------
// Householder tridiagonalisation of the symmetric A (column-major, full storage), lower form
// as LAPACK dsytd2('L'): for column i, v = [1; A(i+2:n, i)], tau_i, e_i = beta, d_i = A(i,i).
// Warp 0 of block 0 owns the column that becomes the next pivot column: it updates that column
// during the rank-2 update of step i and immediately builds reflector i+1 from it, so every
// step needs two grid barriers (after the reflector, after the symmetric matrix-vector product).
// ------------------------------------------------------------------------------------------
// 1/x from the hardware approximation refined by two Newton steps (relative error ~1e-16);
// used where x is bounded away from zero and denormals (pivots, Sturm quotients).
__device__ __forceinline__ double frcp(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

__device__ __forceinline__ double wred(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ double block_sum256(double v, double* red) {
  v = wred(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
  __syncthreads();
  return t;
}

// reflector for column i, built by all threads of one block; writes tau[i], e[i], scaled v
__device__ void make_reflector(int n, int i, double* A, double* tau, double* e, double* red) {
  double* col = A + (size_t)i * n;
  const double alpha = col[i + 1];
  double s = 0.0;
#pragma unroll 4
  for (int r = i + 2 + threadIdx.x; r < n; r += blockDim.x) s += col[r] * col[r];
  s = block_sum256(s, red);
  double t = 0.0, beta = alpha;
  if (s > 0.0) {
    beta = -copysign(sqrt(alpha * alpha + s), alpha);
    t = (beta - alpha) / beta;
    const double sc = 1.0 / (alpha - beta);
#pragma unroll 4
    for (int r = i + 2 + threadIdx.x; r < n; r += blockDim.x) col[r] *= sc;
  }
  if (threadIdx.x == 0) {
    tau[i] = t;
    e[i] = beta;
  }
}

__global__ void __launch_bounds__(256) k_tridiag(int n, double* A, double* d, double* e,
                                                 double* tau, double* pv, double* scal) {
  cg::grid_group grid = cg::this_grid();
  const int lane = threadIdx.x & 31;
  const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarp = (gridDim.x * blockDim.x) >> 5;
  const int bw = blockDim.x >> 5;  // warps per block
  // warps that update trailing columns 1..m-1 (block 0 owns column 0 and the next reflector)
  const bool solo = gridDim.x == 1;
  const int uw = solo ? gwarp : gwarp - bw, nuw = solo ? nwarp : nwarp - bw;
  __shared__ double red[32];
  __shared__ double sK;
  (void)scal;
  if (blockIdx.x == 0 && n > 1) make_reflector(n, 0, A, tau, e, red);
  grid.sync();
  for (int i = 0; i < n - 1; ++i) {
    const int m = n - i - 1;  // size of the trailing block A22 = A(i+1:n, i+1:n)
    const double* v = A + (size_t)i * n + (i + 1);  // v[0] is implicitly 1
    const double t = tau[i];
    // p = t * A22 v  (rows of A22 via its columns, symmetric), also p_r v_r
    for (int r = gwarp; r < m; r += nwarp) {
      const double* colr = A + (size_t)(i + 1 + r) * n + (i + 1);
      double s = 0.0;
      if (lane < m) s = lane == 0 ? colr[0] : colr[lane] * v[lane];
#pragma unroll 8
      for (int c = lane + 32; c < m; c += 32) s += colr[c] * v[c];
      s = wred(s) * t;
      if (lane == 0) {
        pv[r] = s;
        pv[n + r] = s * (r == 0 ? 1.0 : v[r]);
      }
    }
    grid.sync();
    // K = -1/2 t (p . v), reduced by every block in the same order
    {
      double s = 0.0;
      for (int r = threadIdx.x; r < m; r += blockDim.x) s += pv[n + r];
      s = block_sum256(s, red);
      if (threadIdx.x == 0) sK = -0.5 * t * s;
      __syncthreads();
    }
    const double K = sK;
    if (blockIdx.x == 0) {
      if (threadIdx.x == 0) d[i] = A[i + (size_t)i * n];
      // column 0 of A22 (global column i+1), then reflector i+1 from it
      if (t != 0.0) {
        const double wc = pv[0] + K;
        double* colc = A + (size_t)(i + 1) * n + (i + 1);
#pragma unroll 4
        for (int r = threadIdx.x; r < m; r += blockDim.x) {
          const double vr = r == 0 ? 1.0 : v[r];
          const double wr = pv[r] + K * vr;
          colc[r] -= vr * wc + wr;
        }
      }
      __syncthreads();
      if (i + 1 < n - 1) make_reflector(n, i + 1, A, tau, e, red);
      else if (threadIdx.x == 0) d[n - 1] = A[(n - 1) + (size_t)(n - 1) * n];
    }
    // rank-2 update of the remaining columns: A22 -= v w^T + w v^T, w = p + K v
    if (t != 0.0 && uw >= 0) {
      for (int c = 1 + uw; c < m; c += nuw) {
        const double vc = v[c];
        const double wc = pv[c] + K * vc;
        double* colc = A + (size_t)(i + 1 + c) * n + (i + 1);
        if (lane == 0) colc[0] -= wc + (pv[0] + K) * vc;
#pragma unroll 8
        for (int r = 1 + lane; r < m; r += 32) {
          const double vr = v[r];
          colc[r] -= vr * wc + (pv[r] + K * vr) * vc;
        }
      }
    }
    grid.sync();
  }
  if (n == 1 && gwarp == 0 && lane == 0) d[0] = A[0];
}

constexpr size_t TRIDIAG_SMEM_MAX = 200 * 1024;

// Shared-memory resident variant for n where every block can hold its columns: global column j
// lives in block j % nb (slot j / nb) for the whole reduction, so the symmetric matrix-vector
// product, the rank-2 update and the next reflector read and write shared memory only; just the
// reflector v and the product p travel through L2.  Two grid barriers per column.
template <class Sync>
__device__ __forceinline__ void tridiag_smem_body(int n, double* A, double* d, double* e, double* tau,
                                                  double* vbuf, double* pbuf, int nb, int b,
                                                  Sync sync) {
  // columns owned round-robin by the nb cooperating blocks; sync() is their common barrier
  extern __shared__ double sm[];

  const int ncpb = (n + nb - 1) / nb;
  double* scol = sm;                    // [ncpb][n]
  double* sv = sm + (size_t)ncpb * n;   // [n]  reflector of the current step
  double* sp = sv + n;                  // [n]  p of the current step
  __shared__ double red[32];
  __shared__ double sK;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  // load owned columns
  for (int s = 0; s < ncpb; ++s) {
    const int j = b + s * nb;
    if (j >= n) break;
    for (int r = threadIdx.x; r < n; r += blockDim.x) scol[(size_t)s * n + r] = A[r + (size_t)j * n];
  }
  __syncthreads();
  // owner of column i builds reflector i from its shared copy and publishes it
  auto reflector = [&](int i) {
    double* col = scol + (size_t)(i / nb) * n;
    const double alpha = col[i + 1];
    double s = 0.0;
    for (int r = i + 2 + threadIdx.x; r < n; r += blockDim.x) s += col[r] * col[r];
    s = block_sum256(s, red);
    double t = 0.0, beta = alpha;
    if (s > 0.0) {
      beta = -copysign(sqrt(alpha * alpha + s), alpha);
      t = (beta - alpha) / beta;
    }
    const double sc = s > 0.0 ? 1.0 / (alpha - beta) : 0.0;
    for (int r = i + 2 + threadIdx.x; r < n; r += blockDim.x) {
      const double v = col[r] * sc;
      col[r] = v;
      vbuf[r] = v;
      A[r + (size_t)i * n] = v;
    }
    if (threadIdx.x == 0) {
      vbuf[i + 1] = 1.0;
      tau[i] = t;
      e[i] = beta;
      d[i] = col[i];
    }
  };
  if (n > 1 && b == 0) reflector(0);
  if (n == 1 && b == 0 && threadIdx.x == 0) d[0] = scol[0];
  sync();
  for (int i = 0; i < n - 1; ++i) {
    const int m = n - i - 1;
    const double t = tau[i];
    // copy v (rows i+1..n-1) into shared memory
    for (int r = i + 1 + threadIdx.x; r < n; r += blockDim.x) sv[r] = vbuf[r];
    __syncthreads();
    // p_j = t * A(i+1:n, j) . v for owned columns j > i
    for (int s = wid; s < ncpb; s += nwb) {
      const int j = b + s * nb;
      if (j <= i || j >= n) continue;
      const double* col = scol + (size_t)s * n;
      double acc = 0.0;
      for (int r = i + 1 + lane; r < n; r += 32) acc += col[r] * sv[r];
      acc = wred(acc) * t;
      if (lane == 0) {
        pbuf[j] = acc;
        pbuf[n + j] = acc * sv[j];
      }
    }
    sync();
    // K = -1/2 t (p . v), same order in every block
    {
      double s = 0.0;
      for (int r = i + 1 + threadIdx.x; r < n; r += blockDim.x) {
        sp[r] = pbuf[r];
        s += pbuf[n + r];
      }
      s = block_sum256(s, red);
      if (threadIdx.x == 0) sK = -0.5 * t * s;
      __syncthreads();
    }
    const double K = sK;
    if (t != 0.0) {
      // w = p + K v once per row, then two FMAs per element: A -= v w^T + w v^T
      for (int r = i + 1 + threadIdx.x; r < n; r += blockDim.x) sp[r] = fma(K, sv[r], sp[r]);
      __syncthreads();
      for (int s = 0; s < ncpb; ++s) {
        const int j = b + s * nb;
        if (j <= i || j >= n) continue;
        double* col = scol + (size_t)s * n;
        const double vc = sv[j], wc = sp[j];
        for (int r = i + 1 + threadIdx.x; r < n; r += blockDim.x)
          col[r] = fma(-sv[r], wc, fma(-sp[r], vc, col[r]));
      }
    }
    __syncthreads();
    if ((i + 1) % nb == b) {
      if (i + 1 < n - 1) reflector(i + 1);
      else if (threadIdx.x == 0) d[n - 1] = scol[(size_t)((n - 1) / nb) * n + (n - 1)];
    }
    sync();
  }
}
__global__ void __launch_bounds__(256) k_tridiag_smem(int n, double* A, double* d, double* e,
                                                      double* tau, double* vbuf, double* pbuf) {
  cg::grid_group grid = cg::this_grid();
  tridiag_smem_body(n, A, d, e, tau, vbuf, pbuf, (int)gridDim.x, (int)blockIdx.x,
                    [&] { grid.sync(); });
}

// ------------------------------------------------------------------------------------------
// Eigenvalues of the tridiagonal T (one thread per eigenvalue, ascending order).
//
// GB300 executes FP32 about 60x faster than FP64, so each eigenvalue is found in three stages:
//   1. FP32 bisection on the Sturm count of fl32(T) down to a bracket of 2^-21 |T|;
//   2. the bracket is widened by 2^-16 |T| (the FP32 count is exact for a matrix within a few
//      FP32 ulps of T, i.e. within ~1e-6 |T| in its eigenvalues) and both ends are checked
//      with FP64 Sturm counts; a bracket that fails the check restarts from the Gershgorin
//      interval;
//   3. FP64: while the bracket holds exactly this eigenvalue, regula falsi with the Illinois
//      modification on det(T - x I) (superlinear; a point at a converged end is moved half a
//      tolerance inside); otherwise, and whenever three interpolation steps have not halved
//      the bracket, bisection.  About 7 FP64 counts per isolated eigenvalue instead of ~55.
// The stopping rule is the one of plain bisection (width <= 2 eps max(|lo|, |hi|) + 4 pivmin)
// and the result is the midpoint of the final bracket.  The FP64 sweep is the determinant
// recurrence p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2}: division free, the pair rescaled by
// a power of two every 8 steps (the exponent is carried, so det(T - x I) = p * 2^E), an exact
// zero takes the sign opposite to its predecessor; the number of sign changes is the number
// of eigenvalues below x.
// ------------------------------------------------------------------------------------------
// One step of the FP64 recurrence.  FP64 issue slots are scarce on this GPU: the sign tests,
// the zero test and the exponent test read the high word with integer instructions, so per
// step the FP64 pipe sees one subtraction, one multiplication and one FMA.
__device__ __forceinline__ void step64(double a, double ee, double& p0, double& p1, int& h1,
                                       int& cnt) {
  double p2 = fma(a, p1, -ee * p0);
  const bool z = ((__double2hiint(p2) << 1) | __double2loint(p2)) == 0;
  p2 = z ? (h1 < 0 ? 0x1p-900 : -0x1p-900) : p2;  // exact zero: opposite sign to p1
  const int h2 = __double2hiint(p2);
  cnt += (unsigned)(h2 ^ h1) >> 31;
  p0 = p1;
  p1 = p2;
  h1 = h2;
}
__device__ __forceinline__ void rescale64(double& p0, double& p1, int& h1, int& E) {
  const int be = (h1 >> 20) & 0x7ff;  // biased exponent of |p1|
  if (be > 1023 + 400 || be < 1023 - 400) {
    const double sc = __hiloint2double((2046 - be) << 20, 0);  // 2^-(be - 1023), exact
    p1 *= sc;
    p0 *= sc;
    h1 = __double2hiint(p1);
    E += be - 1023;
  }
}
// Sturm count below x and det(T - x I) = fm * 2^fe.  Blocks of 8 steps load their d and e^2
// together, so the loads of a block overlap and the FMA chain runs back to back.
__device__ __forceinline__ int sweep64(int n, const double* __restrict__ d,
                                       const double* __restrict__ e2, double x, double& fm,
                                       int& fe) {
  double p0 = 1.0, p1 = d[0] - x;
  if (p1 == 0.0) p1 = -0x1p-900;
  int h1 = __double2hiint(p1);
  int cnt = (unsigned)h1 >> 31, E = 0;
  int i = 1;
  for (; i + 8 <= n; i += 8) {
    double dv[8], ev[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      dv[k] = d[i + k];
      ev[k] = e2[i + k - 1];
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) step64(dv[k] - x, ev[k], p0, p1, h1, cnt);
    rescale64(p0, p1, h1, E);
  }
  for (; i < n; ++i) step64(d[i] - x, e2[i - 1], p0, p1, h1, cnt);
  fm = p1;
  fe = E;
  return cnt;
}

__device__ __forceinline__ void step32(float a, float ee, float& p0, float& p1, int& cnt) {
  float p2 = fmaf(a, p1, -ee * p0);
  p2 = p2 == 0.f ? -copysignf(0x1p-100f, p1) : p2;
  cnt += (unsigned)(__float_as_int(p2) ^ __float_as_int(p1)) >> 31;
  const float m = fabsf(p2);
  const float sc = m > 0x1p32f ? 0x1p-64f : (m < 0x1p-32f ? 0x1p64f : 1.f);
  p0 = p1 * sc;
  p1 = p2 * sc;
}
__device__ __forceinline__ int sweep32(int n, const float* __restrict__ d,
                                       const float* __restrict__ e2, float x) {
  float p0 = 1.f, p1 = d[0] - x;
  if (p1 == 0.f) p1 = -0x1p-100f;
  int cnt = p1 < 0.f;
  int i = 1;
  for (; i + 8 <= n; i += 8) {
    float dv[8], ev[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      dv[k] = d[i + k];
      ev[k] = e2[i + k - 1];
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) step32(dv[k] - x, ev[k], p0, p1, cnt);
  }
  for (; i < n; ++i) step32(d[i] - x, e2[i - 1], p0, p1, cnt);
  return cnt;
}

// Gershgorin interval [lo, hi] (widened by 4 ulps) and pivmin of T, for every thread of the block
struct TriBounds {
  double lo, hi, tnorm, pivmin;
};
__device__ TriBounds tri_bounds(int n, const double* __restrict__ d,
                                const double* __restrict__ e) {
  __shared__ double red[3][32];
  __shared__ TriBounds out;
  double lo = 1e300, hi = -1e300, emax = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < n - 1 ? fabs(e[i]) : 0.0);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    if (i < n - 1) emax = fmax(emax, e[i] * e[i]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) {
    red[0][w] = lo;
    red[1][w] = hi;
    red[2][w] = emax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < nw; ++k) {
      lo = fmin(lo, red[0][k]);
      hi = fmax(hi, red[1][k]);
      emax = fmax(emax, red[2][k]);
    }
    const double tnorm = fmax(fabs(lo), fabs(hi));
    out.lo = lo - 8.9e-16 * tnorm - 1e-300;
    out.hi = hi + 8.9e-16 * tnorm + 1e-300;
    out.tnorm = fmax(fabs(out.lo), fabs(out.hi));
    out.pivmin = fmax(2.2250738585072014e-308 * fmax(1.0, emax), 1e-300);
  }
  __syncthreads();
  return out;
}

// eigenvalue j of T; warp-collective (every lane of the warp calls it, inactive lanes too)
__device__ double tri_eigenvalue(int n, const double* __restrict__ d, const double* __restrict__ e2,
                                 const float* __restrict__ fd, const float* __restrict__ fe2,
                                 int j, bool active, const TriBounds& b) {
  // 1. FP32 bisection
  float flo = __double2float_rd(b.lo), fhi = __double2float_ru(b.hi);
  const float ftol = (float)(b.tnorm * 0x1p-21);
  for (int it = 0; it < 64; ++it) {
    const float x = 0.5f * (flo + fhi);
    const bool done = !active || fhi - flo <= ftol || x <= flo || x >= fhi;
    if (__all_sync(0xffffffffu, done)) break;
    if (done) continue;
    if (sweep32(n, fd, fe2, x) > j) fhi = x;
    else flo = x;
  }
  // 2. widened bracket, checked in FP64
  const double wid = b.tnorm * 0x1p-16;
  double lo = fmax(b.lo, (double)flo - wid), hi = fmin(b.hi, (double)fhi + wid);
  double flm = 0.0, fhm = 0.0;
  int fle = 0, fhe = 0, clo = 0, chi = n;
  bool kl = false, kh = false;
  if (active) {
    clo = sweep64(n, d, e2, lo, flm, fle);
    chi = sweep64(n, d, e2, hi, fhm, fhe);
    kl = kh = true;
    if (clo > j || chi <= j) {  // the FP32 stage missed: full interval
      lo = b.lo;
      hi = b.hi;
      clo = 0;
      chi = n;
      kl = kh = false;
    }
  }
  // 3. FP64 regula falsi (Illinois) / bisection
  int last = 0, since = 0;
  double wref = hi - lo;
  for (int it = 0; it < 400; ++it) {
    const double tol = 2.0 * 2.220446049250313e-16 * fmax(fabs(lo), fabs(hi)) + 4.0 * b.pivmin;
    const bool done = !active || hi - lo <= tol;
    if (__all_sync(0xffffffffu, done)) break;
    if (done) continue;
    double x = 0.5 * (lo + hi);
    const bool iso = kl && kh && clo == j && chi == j + 1;  // only eigenvalue j inside
    bool bis = !iso;
    if (iso && since >= 3) {  // three interpolation steps must halve the bracket
      if (hi - lo > 0.5 * wref) {
        bis = true;
      } else {
        since = 0;
        wref = hi - lo;
      }
    }
    if (!bis) {
      const int E = max(fle, fhe);
      const double a = scalbn(flm, fle - E), c = scalbn(fhm, fhe - E);
      double xr = lo + a / (a - c) * (hi - lo);
      // a point at the converged end moves half a tolerance inside, so that the next count
      // closes the bracket instead of leaving it to bisection
      xr = fmin(fmax(xr, lo + 0.5 * tol), hi - 0.5 * tol);
      if (xr > lo && xr < hi) x = xr;
      else bis = true;
    }
    if (!(x > lo && x < hi)) {  // no representable point inside: the bracket is final
      lo = hi = x;
      continue;
    }
    if (bis) {
      since = 0;
      wref = 0.5 * (hi - lo);
    } else {
      ++since;
    }
    double fm;
    int fe;
    const int c = sweep64(n, d, e2, x, fm, fe);
    if (c > j) {
      hi = x;
      chi = c;
      fhm = fm;
      fhe = fe;
      kh = true;
      if (last == 1) flm *= 0.5;  // Illinois: the stale end's value is halved
      last = 1;
    } else {
      lo = x;
      clo = c;
      flm = fm;
      fle = fe;
      kl = true;
      if (last == -1) fhm *= 0.5;
      last = -1;
    }
  }
  return 0.5 * (lo + hi);
}

// TRI_SENTINEL stands for eigenvalues above the computed range: (e - ef)/kT >= 50 for any
// Fermi level, so their occupation is exactly zero
constexpr double TRI_SENTINEL = 1e300;

// one-molecule path, stage 0: e^2, FP32 copies and the Gershgorin data into scratch
//   ws layout: e2[n] (double), then fd[n], fe2[n] (float)
__global__ void k_tri_prep(int n, const double* __restrict__ d, const double* __restrict__ e,
                           double* ws, double* scal) {
  float* fd = reinterpret_cast<float*>(ws + n);
  float* fe2 = fd + n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double ee = i < n - 1 ? e[i] * e[i] : 0.0;
    ws[i] = ee;
    fd[i] = (float)d[i];
    fe2[i] = (float)ee;
  }
  if (blockIdx.x == 0) {
    const TriBounds b = tri_bounds(n, d, e);
    if (threadIdx.x == 0) {
      scal[1] = b.tnorm;  // |T| estimate for the inverse iteration
      scal[2] = b.lo;
      scal[3] = b.hi;
      scal[4] = b.pivmin;
    }
  }
}
// one-molecule path: eigenvalues j0 <= j < j1; with fill, w[j1 .. n) = TRI_SENTINEL
__global__ void __launch_bounds__(32) k_eigvals(int n, int j0, int j1, int fill,
                                                 const double* __restrict__ d,
                                                 const double* __restrict__ ws,
                                                 const double* __restrict__ scal, double* w) {
  const int j = j0 + blockIdx.x * blockDim.x + threadIdx.x;
  if ((int)(blockIdx.x * blockDim.x) + j0 >= n) return;  // whole warp beyond n
  const float* fd = reinterpret_cast<const float*>(ws + n);
  const float* fe2 = fd + n;
  TriBounds b;
  b.tnorm = scal[1];
  b.lo = scal[2];
  b.hi = scal[3];
  b.pivmin = scal[4];
  const bool active = j < j1;
  const double v = tri_eigenvalue(n, d, ws, fd, fe2, j, active, b);
  if (active) w[j] = v;
  else if (fill && j < n) w[j] = TRI_SENTINEL;
}

// ------------------------------------------------------------------------------------------
// inverse iteration: one thread per eigenvector (column j < k), Gaussian elimination with
// partial pivoting of the tridiagonal T - w_j I, three solves from a pseudo-random start.
// scratch layout [array][row][j] keeps the per-row accesses of a warp contiguous.
// Y is written column-major [j][n].
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ double hash_uniform(unsigned a, unsigned b) {
  unsigned h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return (double)h / 4294967296.0 * 2.0 - 1.0;
}

__device__ __forceinline__ void invit_dev(int n, int k0, int k, const double* __restrict__ d,
                        const double* __restrict__ e, const double* __restrict__ w,
                        const double* __restrict__ scal, double* lu, double* Y) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;  // vector k0 + j of the spectrum
  if (j >= k) return;
  const size_t nk = (size_t)n * k;
  double* U0 = lu;
  double* U1 = lu + nk;
  double* U2 = lu + 2 * nk;
  double* Lm = lu + 3 * nk;
  double* PV = lu + 4 * nk;  // pivot flag stored as double
#define AT(arr, r) arr[(size_t)(r) * k + j]
  const double lam = w[k0 + j];
  const double tnorm = scal[1] > 0 ? scal[1] : 1.0;
  const double tiny = 2.220446049250313e-16 * tnorm;
  // factorise T - lam I
  double u0 = d[0] - lam, u1 = n > 1 ? e[0] : 0.0, u2 = 0.0;
  for (int r = 0; r < n - 1; ++r) {
    const double c = e[r];                                  // sub-diagonal of row r+1
    const double a1 = d[r + 1] - lam, b1 = r + 1 < n - 1 ? e[r + 1] : 0.0;
    if (fabs(u0) >= fabs(c)) {
      if (fabs(u0) < tiny) u0 = copysign(tiny, u0 == 0.0 ? 1.0 : u0);
      const double l = c / u0;
      AT(U0, r) = u0; AT(U1, r) = u1; AT(U2, r) = u2; AT(Lm, r) = l; AT(PV, r) = 0.0;
      u0 = a1 - l * u1;
      u1 = b1 - l * u2;
      u2 = 0.0;
    } else {
      const double l = u0 / c;
      AT(U0, r) = c; AT(U1, r) = a1; AT(U2, r) = b1; AT(Lm, r) = l; AT(PV, r) = 1.0;
      const double n0 = u1 - l * a1, n1 = u2 - l * b1;
      u0 = n0;
      u1 = n1;
      u2 = 0.0;
    }
  }
  if (fabs(u0) < tiny) u0 = copysign(tiny, u0 == 0.0 ? 1.0 : u0);
  AT(U0, n - 1) = u0; AT(U1, n - 1) = 0.0; AT(U2, n - 1) = 0.0;
  double* y = Y + (size_t)(k0 + j) * n;
  for (int r = 0; r < n; ++r) y[r] = hash_uniform(k0 + j + 1, r + 1);
  for (int iter = 0; iter < 2; ++iter) {
    // forward: apply row operations to the right-hand side
    for (int r = 0; r < n - 1; ++r) {
      const double l = AT(Lm, r);
      if (AT(PV, r) == 0.0) {
        y[r + 1] -= l * y[r];
      } else {
        const double t = y[r];
        y[r] = y[r + 1];
        y[r + 1] = t - l * y[r];
      }
    }
    // backward: U x = y
    double x1 = 0.0, x2 = 0.0;
    for (int r = n - 1; r >= 0; --r) {
      const double v = (y[r] - AT(U1, r) * x1 - AT(U2, r) * x2) * frcp(AT(U0, r));
      y[r] = v;
      x2 = x1;
      x1 = v;
    }
    double nrm = 0.0;
    for (int r = 0; r < n; ++r) nrm += y[r] * y[r];
    nrm = 1.0 / sqrt(nrm);
    for (int r = 0; r < n; ++r) y[r] *= nrm;
  }
#undef AT
}
__global__ void k_invit(int n, int k0, int k, const double* __restrict__ d,
                        const double* __restrict__ e, const double* __restrict__ w,
                        const double* __restrict__ scal, double* lu, double* Y) {
  invit_dev(n, k0, k, d, e, w, scal, lu, Y);
}

// Clusters of close eigenvalues (gap < tol |T|): modified Gram-Schmidt, then Rayleigh-Ritz
// with T inside the cluster (Jacobi on the small projected matrix).  One block per cluster
// start; vectors of a cluster are consecutive columns of Y.
constexpr int MAXCL = 32;
__device__ __forceinline__ void clusters_dev(int n, int k0, int k, const double* __restrict__ d,
                           const double* __restrict__ e, const double* __restrict__ w,
                           const double* __restrict__ scal, double tolrel, double* Y) {
  const int j0 = k0 + blockIdx.x;  // clusters are looked for among vectors k0 .. k-1
  if (j0 >= k) return;
  const double tol = tolrel * (scal[1] > 0 ? scal[1] : 1.0);
  if (j0 > k0 && w[j0] - w[j0 - 1] < tol) return;  // not a cluster start
  int c = 1;
  while (j0 + c < k && w[j0 + c] - w[j0 + c - 1] < tol) ++c;
  if (c == 1) return;
  __shared__ double red[32];
  __shared__ double H[MAXCL][MAXCL], V[MAXCL][MAXCL];
  auto bsum = [&](double v) {
    v = wred(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
      t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
      t = wred(t);
      if (threadIdx.x == 0) red[0] = t;
    }
    __syncthreads();
    t = red[0];
    __syncthreads();
    return t;
  };
  // MGS
  for (int a = 0; a < c; ++a) {
    double* ya = Y + (size_t)(j0 + a) * n;
    for (int b = 0; b < a; ++b) {
      const double* yb = Y + (size_t)(j0 + b) * n;
      double s = 0.0;
      for (int r = threadIdx.x; r < n; r += blockDim.x) s += ya[r] * yb[r];
      s = bsum(s);
      for (int r = threadIdx.x; r < n; r += blockDim.x) ya[r] -= s * yb[r];
      __syncthreads();
    }
    double s = 0.0;
    for (int r = threadIdx.x; r < n; r += blockDim.x) s += ya[r] * ya[r];
    s = 1.0 / sqrt(bsum(s));
    for (int r = threadIdx.x; r < n; r += blockDim.x) ya[r] *= s;
    __syncthreads();
  }
  if (c > MAXCL) return;
  // H = Y_c^T T Y_c
  for (int a = 0; a < c; ++a)
    for (int b = a; b < c; ++b) {
      const double* ya = Y + (size_t)(j0 + a) * n;
      const double* yb = Y + (size_t)(j0 + b) * n;
      double s = 0.0;
      for (int r = threadIdx.x; r < n; r += blockDim.x) {
        double ty = d[r] * yb[r];
        if (r > 0) ty += e[r - 1] * yb[r - 1];
        if (r < n - 1) ty += e[r] * yb[r + 1];
        s += ya[r] * ty;
      }
      s = bsum(s);
      if (threadIdx.x == 0) {
        H[a][b] = s;
        H[b][a] = s;
      }
    }
  __syncthreads();
  // cyclic Jacobi on H (thread 0), V accumulates rotations
  if (threadIdx.x == 0) {
    for (int a = 0; a < c; ++a)
      for (int b = 0; b < c; ++b) V[a][b] = a == b ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 30; ++sweep) {
      double off = 0.0;
      for (int a = 0; a < c; ++a)
        for (int b = a + 1; b < c; ++b) off += H[a][b] * H[a][b];
      if (off < 1e-60) break;
      for (int p = 0; p < c; ++p)
        for (int q = p + 1; q < c; ++q) {
          if (H[p][q] == 0.0) continue;
          const double th = (H[q][q] - H[p][p]) / (2.0 * H[p][q]);
          const double t = copysign(1.0, th) / (fabs(th) + sqrt(th * th + 1.0));
          const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
          for (int r = 0; r < c; ++r) {
            const double hp = H[r][p], hq = H[r][q];
            H[r][p] = cs * hp - sn * hq;
            H[r][q] = sn * hp + cs * hq;
          }
          for (int r = 0; r < c; ++r) {
            const double hp = H[p][r], hq = H[q][r];
            H[p][r] = cs * hp - sn * hq;
            H[q][r] = sn * hp + cs * hq;
          }
          for (int r = 0; r < c; ++r) {
            const double vp = V[r][p], vq = V[r][q];
            V[r][p] = cs * vp - sn * vq;
            V[r][q] = sn * vp + cs * vq;
          }
        }
    }
    // sort by Ritz value (ascending) -- columns of V
    for (int a = 0; a < c; ++a) {
      int mn = a;
      for (int b = a + 1; b < c; ++b)
        if (H[b][b] < H[mn][mn]) mn = b;
      if (mn != a) {
        const double t = H[a][a];
        H[a][a] = H[mn][mn];
        H[mn][mn] = t;
        for (int r = 0; r < c; ++r) {
          const double v = V[r][a];
          V[r][a] = V[r][mn];
          V[r][mn] = v;
        }
      }
    }
  }
  __syncthreads();
  // Y_c <- Y_c V (row by row through registers)
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    double row[MAXCL];
    for (int a = 0; a < c; ++a) row[a] = Y[(size_t)(j0 + a) * n + r];
    for (int b = 0; b < c; ++b) {
      double s = 0.0;
      for (int a = 0; a < c; ++a) s += row[a] * V[a][b];
      Y[(size_t)(j0 + b) * n + r] = s;
    }
  }
}
__global__ void k_clusters(int n, int k0, int k, const double* __restrict__ d,
                           const double* __restrict__ e, const double* __restrict__ w,
                           const double* __restrict__ scal, double tolrel, double* Y) {
  clusters_dev(n, k0, k, d, e, w, scal, tolrel, Y);
}

// ------------------------------------------------------------------------------------------
// back-transformation Z = Q Y = H_0 H_1 ... H_{n-2} Y  (apply H_{n-2} first).  Each block owns
// a set of columns (one warp per column); reflectors are staged in shared memory in chunks.
// ------------------------------------------------------------------------------------------
// Back-transformation Z = Q Y of the eigenvectors of T.  The reflectors are taken in blocks of
// four, [4g, 4g+3], from the top block down, each block as one compact-WY update
//     y <- y - V (T (V^T y))      (V = the block's four reflectors, T upper triangular 4 x 4)
// so that a column makes one pass for the four dot products and one for the update, and the
// four warp reductions are independent.  T (LAPACK dlarft, forward, column-wise) is formed
// once per block by k_bt_tmat.  One warp per column; the block's reflectors are staged in
// shared memory (zero above each reflector's first row), the column too when it fits.
// warps (columns) per block: 4 on the one-molecule path (more blocks for small k), 8 in the batch
// (the reflectors staged per block serve twice the columns; measured 2131 -> 2104 ms on the
// 4096-molecule ensemble, while 8 slowed the 192-orbital single point)
constexpr int BT_WARPS = 4, BT_WARPS_B = 8;
constexpr int BT_CHUNK_MAX = 16;  // reflectors staged per round (a multiple of 4)
constexpr size_t BT_SMEM_MAX = 200 * 1024;
// the columns live in shared memory too when at least one block of reflectors fits beside them
__host__ __device__ static inline bool bt_ysmem(int n, int w = BT_WARPS) {
  return (int)(BT_SMEM_MAX / (sizeof(double) * (size_t)n)) - w >= 4;
}
__host__ __device__ static inline int bt_chunk(int n, int w = BT_WARPS) {
  int c = (int)(BT_SMEM_MAX / (sizeof(double) * (size_t)n)) - (bt_ysmem(n, w) ? w : 0);
  c = c < 4 ? 4 : (c > BT_CHUNK_MAX ? BT_CHUNK_MAX : c);
  return c & ~3;
}
__host__ __device__ static inline size_t bt_smem(int n, int w = BT_WARPS) {
  return sizeof(double) * (size_t)n * (bt_chunk(n, w) + (bt_ysmem(n, w) ? w : 0));
}
// reflector j: v[j+1] = 1, v[r] = A[r + j n] for r > j+1; j > n-2 does not exist (zero)
__device__ __forceinline__ double bt_v(int n, const double* __restrict__ A, int j, int r) {
  if (j > n - 2 || r <= j) return 0.0;
  return r == j + 1 ? 1.0 : A[r + (size_t)j * n];
}
// T of block g (reflectors 4g .. 4g+3), one warp: Tm[16 g + a + 4 b], upper triangular
__device__ __forceinline__ void bt_tmat_dev(int n, const double* __restrict__ A,
                                            const double* __restrict__ tau, double* Tm, int g,
                                            int lane) {
  const int j0 = 4 * g;
  double dd[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) dd[a][b] = 0.0;
#pragma unroll
  for (int b = 1; b < 4; ++b) {
    const int rb = j0 + b + 1;  // first row of reflector b (v = 1 there)
#pragma unroll
    for (int a = 0; a < b; ++a) {
      double acc = 0.0;
      for (int r = rb + lane; r < n; r += 32) acc += bt_v(n, A, j0 + a, r) * bt_v(n, A, j0 + b, r);
      dd[a][b] = wred(acc);
    }
  }
  if (lane != 0) return;
  double t[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int j = j0 + a;
#pragma unroll
    for (int b = 0; b < 4; ++b) t[a][b] = 0.0;
    t[a][a] = j <= n - 2 ? tau[j] : 0.0;
  }
#pragma unroll
  for (int b = 1; b < 4; ++b)
#pragma unroll
    for (int a = 0; a < b; ++a) {
      double acc = 0.0;
#pragma unroll
      for (int c = a; c < b; ++c) acc += t[a][c] * dd[c][b];
      t[a][b] = -t[b][b] * acc;
    }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) Tm[16 * g + a + 4 * b] = t[a][b];
}
__global__ void k_bt_tmat(int n, const double* __restrict__ A, const double* __restrict__ tau,
                          double* Tm) {
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (g * 4 > n - 2) return;
  bt_tmat_dev(n, A, tau, Tm, g, threadIdx.x & 31);
}

template <int W>
__device__ __forceinline__ void backtransform_dev(int n, int k, int chunk, bool ysmem,
                                                  const double* __restrict__ A,
                                                  const double* __restrict__ Tm, double* Y) {
  extern __shared__ double smem[];  // [chunk][n] reflectors, then [W][n] columns
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int col = blockIdx.x * W + wid;
  double* yg = col < k ? Y + (size_t)col * n : nullptr;
  double* y = !yg ? nullptr : (ysmem ? smem + (size_t)chunk * n + (size_t)wid * n : yg);
  if (y && ysmem)
    for (int r = lane; r < n; r += 32) y[r] = yg[r];
  const int cb = chunk / 4;  // blocks per round
  for (int gtop = (n - 2) / 4; gtop >= 0; gtop -= cb) {
    const int gbot = max(0, gtop - cb + 1);
    __syncthreads();
    for (int g = gtop; g >= gbot; --g)
      for (int a = 0; a < 4; ++a) {
        double* sv = smem + (size_t)((gtop - g) * 4 + a) * n;
        for (int r = 4 * g + 1 + threadIdx.x; r < n; r += blockDim.x)
          sv[r] = bt_v(n, A, 4 * g + a, r);
      }
    __syncthreads();
    if (y) {
      for (int g = gtop; g >= gbot; --g) {
        const double* v0 = smem + (size_t)((gtop - g) * 4) * n;
        const double* v1 = v0 + n;
        const double* v2 = v1 + n;
        const double* v3 = v2 + n;
        double w0 = 0.0, w1 = 0.0, w2 = 0.0, w3 = 0.0;
        for (int r = 4 * g + 1 + lane; r < n; r += 32) {
          const double yr = y[r];
          w0 = fma(v0[r], yr, w0);
          w1 = fma(v1[r], yr, w1);
          w2 = fma(v2[r], yr, w2);
          w3 = fma(v3[r], yr, w3);
        }
        w0 = wred(w0);
        w1 = wred(w1);
        w2 = wred(w2);
        w3 = wred(w3);
        const double* T = Tm + 16 * g;  // z = T w (upper triangular, column-major)
        const double z0 = T[0] * w0 + T[4] * w1 + T[8] * w2 + T[12] * w3;
        const double z1 = T[5] * w1 + T[9] * w2 + T[13] * w3;
        const double z2 = T[10] * w2 + T[14] * w3;
        const double z3 = T[15] * w3;
        for (int r = 4 * g + 1 + lane; r < n; r += 32)
          y[r] -= fma(v0[r], z0, fma(v1[r], z1, fma(v2[r], z2, v3[r] * z3)));
        __syncwarp();
      }
    }
  }
  if (y && ysmem)
    for (int r = lane; r < n; r += 32) yg[r] = y[r];
}
__global__ void __launch_bounds__(BT_WARPS * 32) k_backtransform(int n, int k, int chunk, bool ysmem,
                                                                 const double* __restrict__ A,
                                                                 const double* __restrict__ Tm,
                                                                 double* Y) {
  backtransform_dev<BT_WARPS>(n, k, chunk, ysmem, A, Tm, Y);
}

// ------------------------------------------------------------------------------------------
EigenSolver* eigen_create(int n, cudaStream_t s) {
  auto* e = new EigenSolver();
  e->n = n;
  e->cap = n;
  e->stream = s;
  const size_t nn = (size_t)n * n;
  ck(cudaMalloc(&e->L, sizeof(double) * nn), "L");
  ck(cudaMalloc(&e->X, sizeof(double) * nn), "X");
  ck(cudaMalloc(&e->A, sizeof(double) * nn), "A");
  ck(cudaMalloc(&e->T1, sizeof(double) * nn), "T1");
  ck(cudaMalloc(&e->Y, sizeof(double) * nn), "Y");
  ck(cudaMalloc(&e->lu, sizeof(double) * 5 * nn), "lu");
  ck(cudaMalloc(&e->d, sizeof(double) * (n + 1)), "d");
  ck(cudaMalloc(&e->e, sizeof(double) * (n + 1)), "e");
  ck(cudaMalloc(&e->tau, sizeof(double) * (n + 1)), "tau");
  ck(cudaMalloc(&e->w, sizeof(double) * (n + 1)), "w");
  ck(cudaMalloc(&e->pv, sizeof(double) * 4 * (n + 1)), "pv");
  ck(cudaMalloc(&e->tw, sizeof(double) * 2 * (n + 1)), "tw");
  ck(cudaMalloc(&e->scal, sizeof(double) * 8), "scal");
  ck(cudaMalloc(&e->status, sizeof(int)), "status");
  ck(cudaMalloc(&e->gstatus, sizeof(int)), "gstatus");
  ck(cudaMemsetAsync(e->gstatus, 0, sizeof(int), s), "gstatus");
  ck(cudaMallocHost(&e->hstatus, sizeof(int)), "hstatus");
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tridiag, 256, 0);
  (void)per_sm;
  e->coop_blocks = nsm;  // one block per SM keeps the grid barrier cheap
  // shared memory of the back-transformation
  ck(cudaFuncSetAttribute(k_tridiag_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)TRIDIAG_SMEM_MAX),
     "smem attr tridiag");
  ck(cudaFuncSetAttribute(k_backtransform, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)BT_SMEM_MAX + (int)(BT_WARPS * sizeof(double) * 64)),
     "smem attr");
  return e;
}

void eigen_destroy(EigenSolver* e) {
  if (!e) return;
  for (double* p : {e->L, e->X, e->A, e->T1, e->Y, e->lu, e->d, e->e, e->tau, e->w, e->pv, e->tw,
                    e->scal})
    cudaFree(p);
  cudaFree(e->status);
  cudaFree(e->gstatus);
  cudaFreeHost(e->hstatus);
  delete e;
}

int cholesky_inverse(int n, double* L, double* X, int* d_status, int* h_status, cudaStream_t s);

int eigen_set_overlap(EigenSolver* e, const double* S) {
  const int n = e->n;
  // a new geometry: the tensor-core status word starts clear
  ck(cudaMemsetAsync(e->gstatus, 0, sizeof(int), e->stream), "gstatus");
  ck(cudaMemcpyAsync(e->L, S, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, e->stream),
     "copy S");
  return cholesky_inverse(n, e->L, e->X, e->status, e->hstatus, e->stream);
}

int eigen_values(EigenSolver* es, const double* F, double* w_out, int nev) {
  const int n = es->n;
  cudaStream_t s = es->stream;
  // A = X^T (F X): X upper triangular
  if (split_gemm(n)) {  // BF16 tensor cores, FP64-accurate splitting (exponents in tw)
    int* ex = reinterpret_cast<int*>(es->tw);
    ogemm(false, false, n, n, n, F, es->X, es->T1, n, KM_LT_COLEND, ex, es->gstatus, s);
    ogemm(true, false, n, n, n, es->X, es->T1, es->A, n, KM_LT_ROWEND | KM_SYM, ex, es->gstatus, s);
  } else {
    gemm64(false, false, n, n, n, 1.0, F, n, es->X, n, 0.0, es->T1, n, KM_LT_COLEND, s);
    gemm64(true, false, n, n, n, 1.0, es->X, n, es->T1, n, 0.0, es->A, n, KM_LT_ROWEND | KM_SYM, s);
  }
  // tridiagonalise
  {
    int nn = n;
    int blocks = es->coop_blocks;
    const int need = (n * 32 + 255) / 256;
    if (blocks > need) blocks = need > 0 ? need : 1;
    // shared-memory resident path when every block can hold its columns
    int nb = blocks;
    const size_t ncpb = (n + nb - 1) / nb;
    const size_t smem = sizeof(double) * (ncpb * n + 2 * (size_t)n);
    if (smem <= TRIDIAG_SMEM_MAX) {
      double* vbuf = es->pv;
      double* pbuf = es->pv + (n + 1);
      void* args[] = {&nn, &es->A, &es->d, &es->e, &es->tau, &vbuf, &pbuf};
      ++g_kernel_launches;
      const int tk = prof_kbegin(s);
      ck(cudaLaunchCooperativeKernel((void*)k_tridiag_smem, nb, 256, args, smem, s), "tridiag_smem");
      prof_kend(KS_TRIDIAG, tk, s);
    } else {
      void* args[] = {&nn, &es->A, &es->d, &es->e, &es->tau, &es->pv, &es->scal};
      ++g_kernel_launches;
      const int tk = prof_kbegin(s);
      ck(cudaLaunchCooperativeKernel((void*)k_tridiag, blocks, 256, args, 0, s), "tridiag");
      prof_kend(KS_TRIDIAG, tk, s);
    }
  }
  if (nev <= 0 || nev > n) nev = n;
  g_kernel_launches += 2;
  const int tm = prof_kbegin(s);
  k_tri_prep<<<(n + 255) / 256, 256, 0, s>>>(n, es->d, es->e, es->tw, es->scal);
  // one warp per block: the warps of a single molecule spread over as many SMs as possible
  k_eigvals<<<(n + 31) / 32, 32, 0, s>>>(n, 0, nev, 1, es->d, es->tw, es->scal, es->w);
  prof_kend(KS_MULTISECT, tm, s);
  ck(cudaMemcpyAsync(w_out, es->w, sizeof(double) * n, cudaMemcpyDeviceToDevice, s), "w");
  return 0;
}

void eigen_values_rest(EigenSolver* es, int nev, double* w_out) {
  const int n = es->n;
  if (nev >= n) return;
  cudaStream_t s = es->stream;
  g_kernel_launches += 2;
  const int tm = prof_kbegin(s);
  k_tri_prep<<<(n + 255) / 256, 256, 0, s>>>(n, es->d, es->e, es->tw, es->scal);
  k_eigvals<<<(n - nev + 31) / 32, 32, 0, s>>>(n, nev, n, 0, es->d, es->tw, es->scal, es->w);
  prof_kend(KS_MULTISECT, tm, s);
  ck(cudaMemcpyAsync(w_out + nev, es->w + nev, sizeof(double) * (n - nev), cudaMemcpyDeviceToDevice, s),
     "w");
}

void eigen_vectors_range(EigenSolver* es, int k0, int k1, double* C) {
  const int n = es->n;
  cudaStream_t s = es->stream;
  const int k = k1 - k0;
  if (k <= 0) return;
  ++g_kernel_launches;
  const int ti = prof_kbegin(s);
  k_invit<<<(k + 15) / 16, 16, 0, s>>>(n, k0, k, es->d, es->e, es->w, es->scal, es->lu, es->Y);
  prof_kend(KS_INVIT, ti, s);
  ++g_kernel_launches;
  k_clusters<<<k, 256, 0, s>>>(n, k0, k1, es->d, es->e, es->w, es->scal, 1e-5, es->Y);
  const int chunk = bt_chunk(n);
  double* Yk = es->Y + (size_t)k0 * n;
  ++g_kernel_launches;
  const int tb_ = prof_kbegin(s);
  ++g_kernel_launches;  // T of the blocks of four reflectors, into lu (free after the solves)
  k_bt_tmat<<<(((n - 2) / 4 + 1) * 32 + 127) / 128, 128, 0, s>>>(n, es->A, es->tau, es->lu);
  k_backtransform<<<(k + BT_WARPS - 1) / BT_WARPS, BT_WARPS * 32, bt_smem(n), s>>>(
      n, k, chunk, bt_ysmem(n), es->A, es->lu, Yk);
  prof_kend(KS_BACKTRANSFORM, tb_, s);
  // C = X Y (X upper triangular)
  if (split_gemm(n))
    ogemm(false, false, n, k, n, es->X, Yk, C + (size_t)k0 * n, n, KM_GE_ROWBEG,
          reinterpret_cast<int*>(es->tw), es->gstatus, s);
  else
    gemm64(false, false, n, k, n, 1.0, es->X, n, Yk, n, 0.0, C + (size_t)k0 * n, n, KM_GE_ROWBEG,
           s);
}

void eigen_vectors(EigenSolver* es, int k, double* C) { eigen_vectors_range(es, 0, k, C); }

// P = sum_{m<k} f_m C_m C_m^T: scale columns into work, then one GEMM
__device__ __forceinline__ void scale_cols_dev(int n, int k, const double* C, const double* f, double* out) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= (size_t)n * k) return;
  out[t] = C[t] * f[t / n];
}
__global__ void k_scale_cols(int n, int k, const double* C, const double* f, double* out) {
  scale_cols_dev(n, k, C, f, out);
}

void density_matrix(int n, int k, const double* C, const double* f, double* P, double* work,
                    cudaStream_t s, int* status) {
  if (k <= 0) {
    cudaMemsetAsync(P, 0, sizeof(double) * (size_t)n * n, s);
    return;
  }
  const size_t tot = (size_t)n * k;
  ++g_kernel_launches;
  k_scale_cols<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, k, C, f, work);
  // the split GEMM keeps its 2n exponents behind the scaled columns (needs k < n)
  if (status && split_gemm(n) && k < n)
    ogemm(false, true, n, n, k, work, C, P, n, KM_NONE | KM_SYM,
          reinterpret_cast<int*>(work + tot), status, s);
  else
    gemm64(false, true, n, n, k, 1.0, work, n, C, n, 0.0, P, n, KM_NONE | KM_SYM, s);
}

int* eigen_gemm_status(EigenSolver* es) { return es->gstatus; }
bool eigen_gemm_failed(EigenSolver* es) {
  int h = 0;
  ck(cudaMemcpyAsync(&h, es->gstatus, sizeof(int), cudaMemcpyDeviceToHost, es->stream), "gstatus");
  stream_wait(es->stream);
  return h != 0;
}

// ------------------------------------------------------------------------------------------
// Batched eigensolver: one thread-block cluster per molecule for the tridiagonalisation (the
// columns stay in the cluster's shared memory, the barrier is the cluster's hardware barrier
// instead of a grid barrier), blockIdx.z over molecules for the other steps.  The eigenvalues
// are written straight into emo; icount (from the Fermi filling) bounds the vectors.
// ------------------------------------------------------------------------------------------
#define BMOL const MolPtrs& q = mp[list[blockIdx.z]]
#define BARGS const MolPtrs* __restrict__ mp, const int* __restrict__ list

// Householder tridiagonalisation of one molecule per thread-block cluster, lower-triangle
// storage.  Column j lives in CTA j % nb of the cluster, packed (rows j .. n-1 only), so the
// cluster holds n^2/2 doubles instead of n^2 and each element costs four FMAs per step
// instead of six:
//   p = A v   a column's dot product covers its rows r >= c; the rows above the diagonal are
//             the same elements seen from their own columns, so every CTA also scatters
//             A(r, c) v_c into a partial vector (one thread per row, no atomics), and each CTA
//             sums the nb partial vectors through distributed shared memory;
//   A -= v w^T + w v^T on the stored lower part only, w = t p + K v formed once per row.
// Two cluster barriers per column, as in the full-storage form; v and tau of a step are read
// from the owner CTA's shared memory.  The reflectors also go to global A (column-major, below
// the subdiagonal) for the back-transformation.
__device__ __forceinline__ size_t sym_off(int s, int n, int b, int nb) {
  return (size_t)s * n - (size_t)s * b - (size_t)nb * s * (s - 1) / 2;
}
constexpr int TRI_WARPS = 8;  // warps of a kb_tridiag CTA (256 threads)
__host__ __device__ inline size_t sym_tridiag_doubles(int n, int nb) {
  const size_t ncpb = (size_t)(n + nb - 1) / nb;  // CTA 0 owns the most columns
  // packed columns, four vectors (+1) and one row accumulator per warp
  return ncpb * n - (size_t)nb * ncpb * (ncpb - 1) / 2 + (4 + TRI_WARPS) * (size_t)n + 1;
}
__global__ void __launch_bounds__(256) kb_tridiag(BARGS) {
  cg::cluster_group cl = cg::this_cluster();
  BMOL;
  const int n = q.m.nao;
  const int nb = (int)cl.num_blocks(), b = (int)cl.block_rank();
  double* Ag = q.A;
  double* d = q.ed;
  double* e = q.ee;
  double* tau = q.etau;
  extern __shared__ double sm[];
  const int ncpb = b < n ? (n - b + nb - 1) / nb : 0;
  // the vectors first: other CTAs address spart and svpub at the same offset in their view
  double* sv = sm;             // [n] v of the current step
  double* sw = sv + n;         // [n] w = t p + K v
  double* spart = sw + n;      // [n] this CTA's part of p (read by the others)
  double* svpub = spart + n;   // [n + 1] v and tau published by the owner
  double* wrow = svpub + n + 1;  // [TRI_WARPS][n] per-warp row accumulators of p, kept zero
  double* scol = wrow + (size_t)TRI_WARPS * n;  // packed columns (their total differs by CTA)
  __shared__ double red[32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nwb = blockDim.x >> 5;
  for (int s = 0; s < ncpb; ++s) {
    const int j = b + s * nb;
    double* col = scol + sym_off(s, n, b, nb) - j;
    for (int r = j + tid; r < n; r += blockDim.x) col[r] = Ag[r + (size_t)j * n];
  }
  for (size_t u = tid; u < (size_t)TRI_WARPS * n; u += blockDim.x) wrow[u] = 0.0;
  __syncthreads();
  auto column = [&](int s) { return scol + sym_off(s, n, b, nb) - (b + s * nb); };  // col[r], r >= c
  // owner of column i builds reflector i from its stored column and publishes v, tau
  auto reflector = [&](int i) {
    double* col = column(i / nb);
    const double alpha = col[i + 1];
    double ss = 0.0;
    for (int r = i + 2 + tid; r < n; r += blockDim.x) ss += col[r] * col[r];
    ss = block_sum256(ss, red);
    double t = 0.0, beta = alpha;
    if (ss > 0.0) {
      beta = -copysign(sqrt(alpha * alpha + ss), alpha);
      t = (beta - alpha) / beta;
    }
    const double sc = ss > 0.0 ? 1.0 / (alpha - beta) : 0.0;
    for (int r = i + 2 + tid; r < n; r += blockDim.x) {
      const double v = col[r] * sc;
      col[r] = v;
      svpub[r] = v;
      Ag[r + (size_t)i * n] = v;
    }
    if (tid == 0) {
      svpub[i + 1] = 1.0;
      svpub[n] = t;
      tau[i] = t;
      e[i] = beta;
      d[i] = col[i];
    }
  };
  if (n == 1 && b == 0 && tid == 0) d[0] = scol[0];
  if (n > 1 && b == 0) reflector(0);
  cl.sync();
  for (int i = 0; i < n - 1; ++i) {
    // v_i and tau_i from the owner of column i
    const double* pv = cl.map_shared_rank(svpub, i % nb);
    for (int r = i + 1 + tid; r < n; r += blockDim.x) sv[r] = pv[r];
    const double t = pv[n];
    const int s0 = i < b ? 0 : (i - b) / nb + 1;  // first owned column > i
    if (t != 0.0) {
      __syncthreads();
      // p from the owned columns c > i, one warp per column and one pass over its stored rows
      // r >= c: the column's dot product sum_r A(r, c) v_r goes to p_c, and A(r, c) v_c (r > c,
      // the elements above the diagonal seen from their rows) into the warp's row accumulator
      double* acc = wrow + (size_t)wid * n;
      for (int s2 = s0 + wid; s2 < ncpb; s2 += nwb) {
        const int c = b + s2 * nb;
        const double* col = column(s2);
        const double vc = sv[c];
        double dot = 0.0;
        int r = c + lane;
        if (r == c) {  // the diagonal: dot only
          dot = col[r] * sv[r];
          r += 32;
        }
        for (; r < n; r += 32) {
          const double a = col[r];
          dot = fma(a, sv[r], dot);
          acc[r] = fma(a, vc, acc[r]);
        }
        dot = wred(dot);
        if (lane == 0) acc[c] += dot;
        __syncwarp();
      }
      __syncthreads();
      // this CTA's part of p: the sum of the warp accumulators, which are zeroed again
      for (int r = i + 1 + tid; r < n; r += blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < TRI_WARPS; ++w) {
          s += wrow[(size_t)w * n + r];
          wrow[(size_t)w * n + r] = 0.0;
        }
        spart[r] = s;
      }
    }
    cl.sync();
    if (t != 0.0) {
      // p = t * (sum of the nb partial vectors), K = -t/2 p.v (same order in every CTA)
      double kk = 0.0;
      for (int r = i + 1 + tid; r < n; r += blockDim.x) {
        double p = 0.0;
        for (int q2 = 0; q2 < nb; ++q2) p += cl.map_shared_rank(spart, q2)[r];
        p *= t;
        sw[r] = p;
        kk = fma(p, sv[r], kk);
      }
      kk = block_sum256(kk, red);
      const double K = -0.5 * t * kk;
      for (int r = i + 1 + tid; r < n; r += blockDim.x) sw[r] = fma(K, sv[r], sw[r]);
      __syncthreads();
      // rank-2 update of the owned columns c > i, one warp per column
      for (int s2 = s0 + wid; s2 < ncpb; s2 += nwb) {
        const int c = b + s2 * nb;
        double* col = column(s2);
        const double vc = sv[c], wc = sw[c];
        for (int r = c + lane; r < n; r += 32) col[r] = fma(-sv[r], wc, fma(-sw[r], vc, col[r]));
      }
    }
    __syncthreads();
    if ((i + 1) % nb == b) {
      if (i + 1 < n - 1) reflector(i + 1);
      else if (tid == 0) d[n - 1] = column((n - 1) / nb)[n - 1];
    }
    cl.sync();
  }
}
// Small molecules (the whole n x n matrix in one CTA's shared memory): the same Householder
// reduction with everything on chip.  Per column: warp 0 builds the reflector (no block
// reduction), the warps form p = t A22 v column by column, every warp reduces K = -t/2 p.v
// for itself, w = p + K v is formed once per row, and all threads apply the symmetric rank-2
// update to the lower triangle only (two FMAs per stored element, half the elements of the
// full block).  p_j then reads column j from the diagonal down and the rest of it, above the
// diagonal, as row j of the lower triangle (the same elements by symmetry); the columns are
// ld = n | 1 doubles apart, so those row reads hit distinct banks.  Five block barriers per
// column.  The reflectors and the diagonal go to global memory at the end in the layout the
// back-transformation reads (column-major A, v below the subdiagonal).
constexpr int TRI_SMALL_MAX = 156;  // n (n | 1) + 2n doubles <= 200 KB
__host__ __device__ constexpr size_t tri_small_doubles(int n) {
  return (size_t)n * (size_t)(n | 1) + 2 * (size_t)n;
}
static_assert(sizeof(double) * tri_small_doubles(TRI_SMALL_MAX) <= TRIDIAG_SMEM_MAX,
              "the largest small tridiagonalisation fits the shared-memory attribute");
__global__ void __launch_bounds__(256) kb_tridiag_small(BARGS) {
  BMOL;
  const int n = q.m.nao, ld = n | 1;
  extern __shared__ double sm[];
  double* a = sm;                    // [n][ld] column-major; the lower triangle is kept current
  double* sv = sm + (size_t)n * ld;  // [n] reflector (sv[i+1] = 1)
  double* sp = sv + n;               // [n] p, then w
  __shared__ double s_t;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  const double* A0 = q.A;
  for (int t = tid; t < n * n; t += blockDim.x) a[(size_t)(t / n) * ld + t % n] = A0[t];
  __syncthreads();
  for (int i = 0; i < n - 1; ++i) {
    const int r0 = i + 1;  // trailing block rows/cols r0 .. n-1
    if (wid == 0) {        // reflector of column i
      double* col = a + (size_t)i * ld;
      const double alpha = col[r0];
      double s = 0.0;
      for (int r = r0 + 1 + lane; r < n; r += 32) s += col[r] * col[r];
      s = wred(s);
      double t = 0.0, beta = alpha;
      if (s > 0.0) {
        beta = -copysign(sqrt(alpha * alpha + s), alpha);
        t = (beta - alpha) / beta;
      }
      const double sc = s > 0.0 ? 1.0 / (alpha - beta) : 0.0;
      for (int r = r0 + 1 + lane; r < n; r += 32) {
        const double v = col[r] * sc;
        col[r] = v;
        sv[r] = v;
      }
      if (lane == 0) {
        sv[r0] = 1.0;
        s_t = t;
        q.etau[i] = t;
        q.ee[i] = beta;
        q.ed[i] = col[i];
      }
    }
    __syncthreads();
    const double t = s_t;
    if (t != 0.0) {
      // p_j = t * A22(:, j) . v  (warp per column): rows j .. n-1 from column j, rows
      // r0 .. j-1 from row j
      for (int j = r0 + wid; j < n; j += nw) {
        const double* col = a + (size_t)j * ld;
        double acc = 0.0;
        for (int r = j + lane; r < n; r += 32) acc += col[r] * sv[r];
        for (int r = r0 + lane; r < j; r += 32) acc += a[(size_t)r * ld + j] * sv[r];
        acc = wred(acc) * t;
        if (lane == 0) sp[j] = acc;
      }
      __syncthreads();
      // K = -1/2 t (p . v), each warp for itself
      double kk = 0.0;
      for (int r = r0 + lane; r < n; r += 32) kk += sp[r] * sv[r];
      const double K = -0.5 * t * wred(kk);
      __syncthreads();  // every warp has read p
      // w = p + K v once per row, then two FMAs per element: A -= v w^T + w v^T (lower part)
      for (int r = r0 + tid; r < n; r += blockDim.x) sp[r] = fma(K, sv[r], sp[r]);
      __syncthreads();
      for (int c = r0 + wid; c < n; c += nw) {  // warp per column, v_c and w_c in registers
        double* col = a + (size_t)c * ld;
        const double vc = sv[c], wc = sp[c];
        for (int r = c + lane; r < n; r += 32) col[r] = fma(-sv[r], wc, fma(-sp[r], vc, col[r]));
      }
    }
    __syncthreads();
  }
  if (tid == 0) q.ed[n - 1] = a[(size_t)(n - 1) * ld + (n - 1)];
  // reflectors (strictly below the subdiagonal of each column) for the back-transformation
  double* Ag = q.A;
  for (int t2 = tid; t2 < n * n; t2 += blockDim.x) Ag[t2] = a[(size_t)(t2 / n) * ld + t2 % n];
}

// Eigenvalues for the batch, one thread per eigenvalue (tri_eigenvalue: FP32 bisection, FP64
// check, FP64 Illinois / bisection).  d, e^2 and their FP32 copies are staged in shared memory
// (every thread reads the same element at the same step).  rest = 0: eigenvalues j < nev and
// the sentinel above them; rest = 1 (after the SCF): the eigenvalues nev <= j < n.
constexpr int BIS_MAXN = 1024;
// one warp per block: the Sturm counts are FP64-bound (a division per element), so spreading a
// molecule's eigenvalues over more SMs shortens the kernel; each block stages d and e^2 again
constexpr int EIG_BLOCK = 32;
__global__ void __launch_bounds__(128) kb_eigvals(BARGS, int rest) {
  BMOL;
  const int n = q.m.nao;
  const int j0 = rest ? q.nev : 0, j1 = rest ? n : q.nev;
  if ((int)blockIdx.x * (int)blockDim.x + j0 >= n) return;
  __shared__ double sd[BIS_MAXN], se2[BIS_MAXN];
  __shared__ float fd[BIS_MAXN], fe2[BIS_MAXN];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double ee = i < n - 1 ? q.ee[i] * q.ee[i] : 0.0;
    sd[i] = q.ed[i];
    se2[i] = ee;
    fd[i] = (float)q.ed[i];
    fe2[i] = (float)ee;
  }
  const TriBounds b = tri_bounds(n, q.ed, q.ee);  // ends with a block barrier
  if (blockIdx.x == 0 && threadIdx.x == 0 && !rest) q.escal[1] = b.tnorm;
  const int j = j0 + blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = j < j1;
  const double v = tri_eigenvalue(n, sd, se2, fd, fe2, j, active, b);
  if (active) q.emo[j] = v;
  else if (!rest && j < n) q.emo[j] = TRI_SENTINEL;
}

__global__ void kb_invit(BARGS) {
  BMOL;
  invit_dev(q.m.nao, 0, *q.icount, q.ed, q.ee, q.emo, q.escal, q.lu, q.Y);
}
__global__ void kb_clusters(BARGS) {
  BMOL;
  clusters_dev(q.m.nao, 0, *q.icount, q.ed, q.ee, q.emo, q.escal, 1e-5, q.Y);
}
__global__ void __launch_bounds__(BT_WARPS_B * 32) kb_backtransform(BARGS) {
  BMOL;
  const int n = q.m.nao, k = *q.icount;
  if ((int)blockIdx.x * BT_WARPS_B >= k) return;  // no column of this molecule here
  backtransform_dev<BT_WARPS_B>(n, k, bt_chunk(n, BT_WARPS_B), bt_ysmem(n, BT_WARPS_B), q.A, q.lu,
                                q.Y);
}
__global__ void kb_bt_tmat(BARGS) {
  BMOL;
  const int n = q.m.nao;
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (g * 4 > n - 2) return;
  bt_tmat_dev(n, q.A, q.etau, q.lu, g, threadIdx.x & 31);
}
// mode 0: occupations (total), 1: occupations x energies (vec_out), 2 + c: spin channel c of
// the bond orders (a closed shell's channel 0 is the total occupation)
__global__ void kb_scale_cols(BARGS, int mode) {
  BMOL;
  const int n = q.m.nao;
  const double* f = mode == 0 ? q.focc : mode == 1 ? q.vec_out
                  : q.wbo_ch == 2 ? q.focc + (size_t)(mode - 1) * n : q.focc;
  scale_cols_dev(n, *q.icount, q.C, f, q.scratch);
}

// CTAs of the batched tridiagonalisation that should fit on one SM (1 or 2): with 2 the
// clusters are made wide enough that each CTA holds at most ~110 KB, so a second molecule's CTA
// computes while the first waits at a cluster barrier
static int g_tridiag_ctas_per_sm = 2;
// smallest cluster (1, 2, 4, 8 blocks) whose shared memory holds the lower triangle, within the
// per-CTA budget of the chosen residency when possible
static int tridiag_cluster(int n, size_t* smem) {
  const size_t caps[2] = {g_tridiag_ctas_per_sm >= 2 ? (size_t)110 * 1024 : TRIDIAG_SMEM_MAX,
                          TRIDIAG_SMEM_MAX};
  for (size_t cap : caps)
    for (int nb = 1; nb <= 8; nb *= 2) {
      const size_t need = sizeof(double) * sym_tridiag_doubles(n, nb);
      if (need <= cap) {
        *smem = need;
        return nb;
      }
    }
  return 0;
}
void set_tridiag_ctas_per_sm(int k) { g_tridiag_ctas_per_sm = k >= 2 ? 2 : 1; }
int get_tridiag_ctas_per_sm() { return g_tridiag_ctas_per_sm; }
// buckets of at most TRI_SMALL_MAX orbitals: the one-CTA full-storage kernel (1, default) or the
// packed lower-triangle kernel as a cluster of one CTA (0: two thirds of the FMAs, half the
// shared memory, but row accumulators summed per column)
static int g_tridiag_small = 1;
void set_tridiag_small(int k) { g_tridiag_small = k ? 1 : 0; }
int get_tridiag_small() { return g_tridiag_small; }
int batch_tridiag_max_n() {
  int n = 1;
  size_t sm = 0;
  while (tridiag_cluster(n + 1, &sm)) ++n;  // the second cap is the residency-independent one
  return n;
}

static void batch_attributes() {
  static bool done = false;
  if (done) return;
  ck(cudaFuncSetAttribute(kb_tridiag, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)TRIDIAG_SMEM_MAX),
     "smem attr batch tridiag");
  ck(cudaFuncSetAttribute(kb_tridiag_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)TRIDIAG_SMEM_MAX),
     "smem attr batch tridiag small");
  ck(cudaFuncSetAttribute(kb_backtransform, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)BT_SMEM_MAX + (int)(BT_WARPS_B * sizeof(double) * 64)),
     "smem attr batch backtransform");
  done = true;
}

static void tridiag_cluster_b(const BatchLaunch& b);

void eigen_values_b(const BatchLaunch& b) {
  if (!b.count) return;
  batch_attributes();
  gemm_b(b, GS_FX);
  gemm_b(b, GS_XTT);
  if (b.nao_max <= TRI_SMALL_MAX && g_tridiag_small) {
    const size_t sm_small = sizeof(double) * tri_small_doubles(b.nao_max);
    ++g_kernel_launches;
    const int tk = prof_kbegin(b.s);
    kb_tridiag_small<<<dim3(1, 1, b.count), 256, sm_small, b.s>>>(b.mp, b.list);
    prof_kend(KS_TRIDIAG, tk, b.s);
  } else {
    tridiag_cluster_b(b);
  }
  ++g_kernel_launches;
  const int tm = prof_kbegin(b.s);
  if (b.nao_max > BIS_MAXN) throw std::runtime_error("batched eigenvalues: molecule too large");
  kb_eigvals<<<dim3((b.nao_max + EIG_BLOCK - 1) / EIG_BLOCK, 1, b.count), EIG_BLOCK, 0, b.s>>>(
      b.mp, b.list, 0);
  prof_kend(KS_MULTISECT, tm, b.s);
}

void eigen_values_rest_b(const BatchLaunch& b) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_eigvals<<<dim3((b.nao_max + EIG_BLOCK - 1) / EIG_BLOCK, 1, b.count), EIG_BLOCK, 0, b.s>>>(
      b.mp, b.list, 1);
}

static void tridiag_cluster_b(const BatchLaunch& b) {
  size_t smem = 0;
  const int nb = tridiag_cluster(b.nao_max, &smem);
  if (!nb) throw std::runtime_error("batched tridiagonalisation: molecule too large");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nb, 1, b.count);
  cfg.blockDim = dim3(256, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = b.s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = nb;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  ++g_kernel_launches;
  const int tk = prof_kbegin(b.s);
  ck(cudaLaunchKernelEx(&cfg, kb_tridiag, b.mp, b.list), "batch tridiag");
  prof_kend(KS_TRIDIAG, tk, b.s);
}

void eigen_vectors_b(const BatchLaunch& b) {
  if (!b.count) return;
  batch_attributes();
  g_kernel_launches += 3;
  const int ti = prof_kbegin(b.s);
  // one thread per vector; full warps (the one-molecule path keeps 16-thread blocks so that a
  // single molecule's vectors spread over more SMs)
  kb_invit<<<dim3((b.nao_max + 31) / 32, 1, b.count), 32, 0, b.s>>>(b.mp, b.list);
  prof_kend(KS_INVIT, ti, b.s);
  kb_clusters<<<dim3(b.nao_max, 1, b.count), 256, 0, b.s>>>(b.mp, b.list);
  const int tb_ = prof_kbegin(b.s);
  ++g_kernel_launches;
  kb_bt_tmat<<<dim3((((b.nao_max - 2) / 4 + 1) * 32 + 127) / 128, 1, b.count), 128, 0, b.s>>>(
      b.mp, b.list);
  kb_backtransform<<<dim3((b.nao_max + BT_WARPS_B - 1) / BT_WARPS_B, 1, b.count),
                     BT_WARPS_B * 32, bt_smem(b.nao_max, BT_WARPS_B), b.s>>>(b.mp, b.list);
  prof_kend(KS_BACKTRANSFORM, tb_, b.s);
  gemm_b(b, GS_XY);
}

void density_b(const BatchLaunch& b, bool weighted) {
  if (!b.count) return;
  const size_t tot = (size_t)b.nao_max * b.nao_max;
  ++g_kernel_launches;
  kb_scale_cols<<<dim3((unsigned)((tot + 255) / 256), 1, b.count), 256, 0, b.s>>>(
      b.mp, b.list, weighted ? 1 : 0);
  gemm_b(b, weighted ? GS_WDENS : GS_DENS);
}

void wbo_b(const BatchLaunch& b, int channel) {
  if (!b.count) return;
  if (b.sp2) {  // closed shells without orbitals: P S directly
    pipe_site_b(b, GS_PS);
    launch_wbo_b(b, channel);
    return;
  }
  const size_t tot = (size_t)b.nao_max * b.nao_max;
  ++g_kernel_launches;
  kb_scale_cols<<<dim3((unsigned)((tot + 255) / 256), 1, b.count), 256, 0, b.s>>>(
      b.mp, b.list, 2 + channel);
  gemm_b(b, GS_WDENS);  // the channel's density into F (W is no longer needed)
  gemm_b(b, GS_FS);
  launch_wbo_b(b, channel);
}

#undef BMOL
#undef BARGS

}  // namespace tb
