// Density matrix by spectral projection (closed shell, gapped systems): a second density solver
// for large orbital counts, beside the eigen solver (eigen.cu).
//
// The reference obtains the density through its solver interface (src/tblite/scf/solver.f90:
// 28-45, get_density / get_wdensity), implemented by diagonalisation (scf/diag.f90:62-143:
// sygvd, Fermi filling, P = C f C^T, W = C f e C^T).  For n in the thousands the one-stage
// Householder reduction streams the trailing matrix from HBM once per column.  A closed-shell
// system whose HOMO-LUMO gap spans many kT has Fermi occupations that are 0 or 1 to machine
// precision, so P is twice the spectral projector onto the occupied orbitals, and a polynomial
// recursion in the Fock matrix gives that projector from matrix products alone:
//
//   1. Loewdin orthogonaliser Z = S^-1/2 (once per geometry), coupled Newton-Schulz iteration
//      (Higham, Numer. Algorithms 15, 227 (1997)): Y = S/c, Z = I, M = (3I - Z Y)/2,
//      Y <- Y M, Z <- M Z, with c a power of four above the Gershgorin bound of S, so that the
//      scalings by c and sqrt(c) are exact;
//   2. per SCF iteration A = Z F Z, Gershgorin bounds [emin, emax], X = (emax I - A)/(emax - emin)
//      and the second-order spectral projection (SP2; Niklasson, Phys. Rev. B 66, 155115
//      (2002)): X <- X^2 or 2X - X^2, whichever brings the trace closer to the number of
//      occupied orbitals, until the idempotency error tr(X - X^2) stops decreasing
//      (Kruchinin, Rubensson, Niklasson, J. Chem. Phys. 145, 204106 (2016));
//   3. P = 2 Z X Z (the reference's P = C f C^T) and W = P F P / 2 (its C f e C^T);
//   4. a gap certificate on the converged Fock matrix: Lanczos with full reorthogonalisation on
//      X (A - emin) X and (I - X)(emax I - A)(I - X) gives the HOMO and the LUMO with residual
//      bounds; a gap below 80 kT is an error (the Fermi occupations would not be 0/1 to
//      ~1e-17), and so is an open shell or a fractional electron count.
//
// Every matrix product runs on the FP64-accurate split GEMM of the tensor cores (ozaki.cu); the
// symmetric ones compute the tiles on and below the diagonal and mirror them.
#include <cuda_runtime.h>

#include <cmath>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "engine.h"

namespace tb {

namespace {

constexpr int PU_LZ_M = 48;          // Lanczos steps of the gap certificate
constexpr int PU_NS_MAX = 60;        // Newton-Schulz iterations before giving up
constexpr int PU_SP2_MAX = 120;      // SP2 iterations before giving up
constexpr double PU_GAP_KT = 80.0;   // smallest certified gap, in kT

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("CUDA error '") + cudaGetErrorString(e) + "' in " + what);
}

int ew_blocks(size_t count) {
  const size_t b = (count + 255) / 256, cap = 16 * (size_t)device_sm_count();
  return (int)(b < cap ? b : cap);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// block-wide sum (blockDim.x a multiple of 32, at most 1024); the result is valid in thread 0
__device__ double block_sum(double v) {
  __shared__ double part[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) part[wid] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
  if (wid == 0) v = warp_sum(v);
  return v;
}

// Gershgorin discs of a symmetric matrix, one warp per column: lo[j], hi[j]
__global__ void k_gersh(int n, const double* __restrict__ A, double* lo, double* hi) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= n) return;
  const double* col = A + (size_t)j * n;
  double r = 0.0;
  for (int i = lane; i < n; i += 32)
    if (i != j) r += fabs(col[i]);
  r = warp_sum(r);
  if (lane == 0) {
    lo[j] = col[j] - r;
    hi[j] = col[j] + r;
  }
}
// out[0] = min lo, out[1] = max hi (one block)
__global__ void k_bounds(int n, const double* __restrict__ lo, const double* __restrict__ hi,
                         double* out) {
  __shared__ double smin[32], smax[32];
  double a = 1e300, b = -1e300;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    a = fmin(a, lo[j]);
    b = fmax(b, hi[j]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a = fmin(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    smin[wid] = a;
    smax[wid] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      a = fmin(a, smin[w]);
      b = fmax(b, smax[w]);
    }
    out[0] = fmin(a, smin[0]);
    out[1] = fmax(b, smax[0]);
  }
}

// Newton-Schulz start: Y = S 4^-k, Z = I with 4^k >= the Gershgorin bound sc[1]; sc[2] = 2^-k
__global__ void k_ns_init(int n, const double* __restrict__ S, const double* sc, double* Y,
                          double* Z, double* scal_out) {
  int e2 = 0;
  frexp(sc[1], &e2);  // sc[1] < 2^e2
  const int k = (e2 + 1) / 2;
  const size_t nn = (size_t)n * n;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nn;
       t += (size_t)gridDim.x * blockDim.x) {
    Y[t] = ldexp(S[t], -2 * k);
    Z[t] = (t % (n + 1) == 0) ? 1.0 : 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) scal_out[2] = ldexp(1.0, -k);
}
// M = (3I - T)/2 in place, err += ||I - T||_F^2
__global__ void k_ns_mid(int n, double* T, double* err) {
  const size_t nn = (size_t)n * n;
  double acc = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nn;
       t += (size_t)gridDim.x * blockDim.x) {
    const double d = ((t % (n + 1) == 0) ? 1.0 : 0.0) - T[t];
    acc += d * d;
    T[t] = 0.5 * (((t % (n + 1) == 0) ? 3.0 : 0.0) - T[t]);
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) atomicAdd(err, acc);
}
// x *= scale (device scalar)
__global__ void k_scale_dev(size_t count, double* x, const double* scale) {
  const double f = *scale;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count;
       t += (size_t)gridDim.x * blockDim.x)
    x[t] *= f;
}
// y = a x (host scalar)
__global__ void k_scale_to(size_t count, const double* __restrict__ x, double a, double* y) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count;
       t += (size_t)gridDim.x * blockDim.x)
    y[t] = a * x[t];
}
// X = (emax I - A)/(emax - emin)
__global__ void k_sp2_init(int n, const double* __restrict__ A, const double* sc, double* X) {
  const double emin = sc[0], emax = sc[1];
  const double f = 1.0 / (emax - emin);
  const size_t nn = (size_t)n * n;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nn;
       t += (size_t)gridDim.x * blockDim.x)
    X[t] = (((t % (n + 1) == 0) ? emax : 0.0) - A[t]) * f;
}
// tr X, tr X^2 into out[0], out[1] (one block)
__global__ void k_sp2_traces(int n, const double* __restrict__ X, const double* __restrict__ X2,
                             double* out) {
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    a += X[i + (size_t)i * n];
    b += X2[i + (size_t)i * n];
  }
  a = block_sum(a);
  __syncthreads();
  b = block_sum(b);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
  }
}
// X <- X^2 (square != 0) or 2X - X^2
__global__ void k_sp2_update(size_t count, double* X, const double* __restrict__ X2, int square) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count;
       t += (size_t)gridDim.x * blockDim.x)
    X[t] = square ? X2[t] : 2.0 * X[t] - X2[t];
}

// ---- Lanczos (gap certificate) ----------------------------------------------------------
// y = M x for a symmetric M, one warp per column (coalesced column reads)
__global__ void k_symv(int n, const double* __restrict__ M, const double* __restrict__ x,
                       double* y) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (j >= n) return;
  const double* col = M + (size_t)j * n;
  double s = 0.0;
  for (int i = lane; i < n; i += 32) s += col[i] * x[i];
  s = warp_sum(s);
  if (lane == 0) y[j] = s;
}
// z = a x + b y (host scalars; sc index < 0: none), optionally plus c * sc[ic] * y
__global__ void k_axpby(int n, double a, const double* x, double b, const double* y,
                        const double* sc, int ic, double c, double* z) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double f = b;
  if (ic >= 0) f += c * sc[ic];
  z[i] = a * x[i] + f * y[i];
}
// h[r] = V_r . w for r < cnt, one block per r
__global__ void k_dots(int n, int cnt, const double* __restrict__ V, const double* __restrict__ w,
                       double* h) {
  const int r = blockIdx.x;
  if (r >= cnt) return;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += V[(size_t)r * n + i] * w[i];
  s = block_sum(s);
  if (threadIdx.x == 0) h[r] = s;
}
// w -= sum_r h[r] V_r; alpha[j] += h[j] when j >= 0 (the projection on the newest vector)
__global__ void k_orth(int n, int cnt, const double* __restrict__ V, const double* __restrict__ h,
                       double* w, double* alpha, int j) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    double s = w[i];
    for (int r = 0; r < cnt; ++r) s -= h[r] * V[(size_t)r * n + i];
    w[i] = s;
  }
  if (j >= 0 && blockIdx.x == 0 && threadIdx.x == 0) alpha[j] += h[j];
}
// beta[j] = ||w||; V_{j+1} = w / beta[j] (zero vector once the Krylov space is exhausted)
__global__ void k_normalize(int n, const double* __restrict__ w, double* beta, int j,
                            double* vnext, double scale) {
  __shared__ double nrm;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += w[i] * w[i];
  s = block_sum(s);
  if (threadIdx.x == 0) {
    nrm = sqrt(s);
    if (j >= 0) beta[j] = nrm;
  }
  __syncthreads();
  const double b = nrm;
  const double f = b > 1e-13 * scale ? 1.0 / b : 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) vnext[i] = w[i] * f;
}
// Sturm count: eigenvalues of the m x m tridiagonal (a, b) below x
__device__ int sturm_below(int m, const double* a, const double* b, double x) {
  int c = 0;
  double q = a[0] - x;
  if (q < 0.0) ++c;
  for (int k = 1; k < m; ++k) {
    if (fabs(q) < 1e-300) q = 1e-300;
    q = a[k] - x - b[k - 1] * b[k - 1] / q;
    if (q < 0.0) ++c;
  }
  return c;
}
// largest eigenvalue theta of T_m (bisection) and the residual bound beta_m |s_m| of its Ritz
// vector (inverse iteration with partial pivoting); out[0] = theta, out[1] = bound
__global__ void k_ritz(int m, const double* __restrict__ a, const double* __restrict__ b,
                       double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double lo = a[0], hi = a[0];
  for (int k = 0; k < m; ++k) {
    const double r = (k > 0 ? fabs(b[k - 1]) : 0.0) + (k < m - 1 ? fabs(b[k]) : 0.0);
    lo = fmin(lo, a[k] - r);
    hi = fmax(hi, a[k] + r);
  }
  const double span = fmax(hi - lo, 1e-300);
  for (int it = 0; it < 200 && hi - lo > 1e-15 * span; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (sturm_below(m, a, b, mid) < m) lo = mid;  // some eigenvalue above mid
    else hi = mid;
  }
  const double th = hi;
  // inverse iteration on (T - (th + d) I), d a tiny shift off the eigenvalue
  double s[PU_LZ_M], dl[PU_LZ_M], dd[PU_LZ_M], du[PU_LZ_M], du2[PU_LZ_M];
  int piv[PU_LZ_M];
  const double shift = th + 1e-12 * span;
  for (int k = 0; k < m; ++k) {
    dd[k] = a[k] - shift;
    if (k < m - 1) dl[k] = du[k] = b[k];
    s[k] = 1.0;
  }
  // LU with partial pivoting of a tridiagonal matrix (rows k, k+1 swapped when needed)
  for (int k = 0; k < m; ++k) du2[k] = 0.0;
  for (int k = 0; k < m - 1; ++k) {
    if (fabs(dd[k]) >= fabs(dl[k])) {
      piv[k] = 0;
      const double f = dd[k] != 0.0 ? dl[k] / dd[k] : 0.0;
      dl[k] = f;
      dd[k + 1] -= f * du[k];
    } else {
      piv[k] = 1;
      const double f = dd[k] / dl[k];
      dd[k] = dl[k];
      dl[k] = f;
      const double t = du[k];
      du[k] = dd[k + 1];
      dd[k + 1] = t - f * dd[k + 1];
      if (k < m - 2) {
        du2[k] = du[k + 1];
        du[k + 1] = -f * du[k + 1];
      }
    }
  }
  for (int it = 0; it < 3; ++it) {
    for (int k = 0; k < m - 1; ++k) {  // L solve with the row swaps
      if (piv[k]) {
        const double t = s[k];
        s[k] = s[k + 1];
        s[k + 1] = t - dl[k] * s[k + 1];
      } else {
        s[k + 1] -= dl[k] * s[k];
      }
    }
    for (int k = m - 1; k >= 0; --k) {  // U solve
      double v = s[k];
      if (k < m - 1) v -= du[k] * s[k + 1];
      if (k < m - 2) v -= du2[k] * s[k + 2];
      const double d = dd[k] != 0.0 ? dd[k] : 1e-300;
      s[k] = v / d;
    }
    double nrm = 0.0;
    for (int k = 0; k < m; ++k) nrm += s[k] * s[k];
    nrm = sqrt(nrm);
    for (int k = 0; k < m; ++k) s[k] /= nrm;
  }
  out[0] = th;
  out[1] = fabs(b[m - 1] * s[m - 1]);
}

}  // namespace

struct Purifier {
  int n = 0;
  cudaStream_t s = nullptr;
  double *Z = nullptr, *A = nullptr, *X = nullptr, *X2 = nullptr, *T = nullptr;
  double* sc = nullptr;   // device scalars: [0] emin [1] emax [2] 2^-k [3] err [4] trX [5] trX2
  double* gl = nullptr;   // Gershgorin lo/hi [2n]
  double* V = nullptr;    // Lanczos basis [PU_LZ_M + 1][n]
  double* lz = nullptr;   // u, w [2n], h [PU_LZ_M + 1], alpha, beta [PU_LZ_M + 1], ritz [4]
  int* ex = nullptr;      // split-GEMM exponents [2n]
  int* status = nullptr;  // split-GEMM wait limit
  double* hsc = nullptr;  // pinned copy of sc
  PImage img[3];          // slice images: 0, 1 operands; 2 the orthogonaliser Z
  int last_iterations = 0;
};

// the products of the projection run on the pipelined split GEMM (ozaki_pipe.cu); switched off,
// on the per-tile split GEMM (ozaki.cu)
bool g_pipe_gemm = true;

Purifier* purify_create(int n, cudaStream_t s) {
  auto* p = new Purifier();
  p->n = n;
  p->s = s;
  const size_t nn = (size_t)n * n;
  for (double** b : {&p->Z, &p->A, &p->X, &p->X2, &p->T}) ck(cudaMalloc(b, sizeof(double) * nn), "purify");
  ck(cudaMalloc(&p->sc, sizeof(double) * 16), "purify sc");
  ck(cudaMalloc(&p->gl, sizeof(double) * 2 * n), "purify gl");
  ck(cudaMalloc(&p->V, sizeof(double) * (PU_LZ_M + 1) * (size_t)n), "purify V");
  ck(cudaMalloc(&p->lz, sizeof(double) * (2 * (size_t)n + 3 * (PU_LZ_M + 1) + 4)), "purify lz");
  ck(cudaMalloc(&p->ex, sizeof(int) * 2 * n), "purify ex");
  ck(cudaMalloc(&p->status, sizeof(int)), "purify status");
  ck(cudaMemsetAsync(p->status, 0, sizeof(int), s), "purify status");
  ck(cudaMallocHost(&p->hsc, sizeof(double) * 16), "purify hsc");
  for (PImage& im : p->img) {
    ck(cudaMalloc(&im.data, pimage_bytes(n, n)), "purify image");
    ck(cudaMalloc(&im.e, sizeof(int) * pimage_lines(n)), "purify image e");
  }
  return p;
}

void purify_destroy(Purifier* p) {
  if (!p) return;
  for (double* b : {p->Z, p->A, p->X, p->X2, p->T, p->sc, p->gl, p->V, p->lz}) cudaFree(b);
  cudaFree(p->ex);
  cudaFree(p->status);
  cudaFreeHost(p->hsc);
  for (PImage& im : p->img) {
    cudaFree(im.data);
    cudaFree(im.e);
  }
  delete p;
}

int purify_capacity(const Purifier* p) { return p ? p->n : 0; }
int purify_iterations(const Purifier* p) { return p ? p->last_iterations : 0; }

static void read_scalars(Purifier* p, int count) {
  ck(cudaMemcpyAsync(p->hsc, p->sc, sizeof(double) * count, cudaMemcpyDeviceToHost, p->s), "sc");
  stream_wait(p->s);
}
// C = A B (n x n, column-major; sym: C is symmetric, the tiles on and below the diagonal are
// computed and mirrored).  The pipelined GEMM first splits A into image slot sa (its rows) and
// B into slot sb (its columns), unless keep_a / keep_b say the slot already holds that image.
static void product(Purifier* p, const double* A, int sa, bool keep_a, const double* B, int sb,
                    bool keep_b, double* C, bool sym) {
  const int n = p->n;
  if (!g_pipe_gemm) {
    ogemm(false, false, n, n, n, A, B, C, n, KM_NONE | (sym ? KM_SYM : 0), p->ex, p->status,
          p->s);
    return;
  }
  if (!keep_a) psplit(A, n, 0, n, n, p->img[sa], p->s);
  if (!keep_b && !(sb == sa && B == A)) psplit(B, n, 1, n, n, p->img[sb], p->s);
  pgemm(p->img[sa], p->img[sb], C, n, sym, p->status, p->s);
}
static void bounds(Purifier* p, const double* M) {
  const int n = p->n;
  g_kernel_launches += 2;
  k_gersh<<<(n * 32 + 255) / 256, 256, 0, p->s>>>(n, M, p->gl, p->gl + n);
  k_bounds<<<1, 1024, 0, p->s>>>(n, p->gl, p->gl + n, p->sc);
}

// Z = S^-1/2; returns the Newton-Schulz iterations, -1 if they did not converge
int purify_set_overlap(Purifier* p, const double* S) {
  const int n = p->n;
  const size_t nn = (size_t)n * n;
  const int eb = ew_blocks(nn);
  // a new geometry: the status word of the split GEMMs starts clear (a wait that ran out in an
  // earlier single point was reported there)
  ck(cudaMemsetAsync(p->status, 0, sizeof(int), p->s), "purify status");
  bounds(p, S);
  double *Y = p->A, *Z = p->Z, *Yn = p->X, *Zn = p->X2;
  ++g_kernel_launches;
  k_ns_init<<<eb, 256, 0, p->s>>>(n, S, p->sc, Y, Z, p->sc);
  int it = 0;
  bool done = false;
  for (; it < PU_NS_MAX && !done; ++it) {
    product(p, Z, 0, false, Y, 1, false, p->T, true);
    ck(cudaMemsetAsync(p->sc + 3, 0, sizeof(double), p->s), "err");
    ++g_kernel_launches;
    k_ns_mid<<<eb, 256, 0, p->s>>>(n, p->T, p->sc + 3);
    read_scalars(p, 4);
    const double err = p->hsc[3];
    if (!(err == err)) return -1;
    if (err < 1e-26 * n) {  // converged before this update
      done = true;
      break;
    }
    // quadratic convergence (||I - T'||_F^2 <= 0.6 ||I - T||_F^4): one more update after 1e-12
    done = err < 1e-12;
    product(p, Y, 1, true, p->T, 2, false, Yn, true);   // M = T into slot 2
    product(p, p->T, 2, true, Z, 0, true, Zn, true);
    std::swap(Y, Yn);
    std::swap(Z, Zn);
  }
  if (!done) return -1;
  ++g_kernel_launches;
  k_scale_dev<<<eb, 256, 0, p->s>>>(nn, Z, p->sc + 2);
  if (Z != p->Z) ck(cudaMemcpyAsync(p->Z, Z, sizeof(double) * nn, cudaMemcpyDeviceToDevice, p->s), "Z");
  if (g_pipe_gemm) psplit(p->Z, n, 0, n, n, p->img[2], p->s);  // Z stays split (symmetric)
  return it;
}

// P = 2 Z X Z from the Fock matrix F; nocc occupied orbitals per spin.  Returns the SP2
// iterations, -1 if they did not converge.  A = Z F Z and X stay for the gap certificate and
// the energy-weighted density.
int purify_density(Purifier* p, const double* F, int nocc, double* P) {
  const int n = p->n;
  const size_t nn = (size_t)n * n;
  const int eb = ew_blocks(nn);
  product(p, F, 0, false, p->Z, 2, true, p->T, false);
  product(p, p->Z, 2, true, p->T, 1, false, p->A, true);
  bounds(p, p->A);
  ++g_kernel_launches;
  k_sp2_init<<<eb, 256, 0, p->s>>>(n, p->A, p->sc, p->X);
  std::vector<double> err;
  int it = 0;
  bool done = false;
  for (; it < PU_SP2_MAX; ++it) {
    product(p, p->X, 0, false, p->X, 0, true, p->X2, true);
    ++g_kernel_launches;
    k_sp2_traces<<<1, 1024, 0, p->s>>>(n, p->X, p->X2, p->sc + 4);
    read_scalars(p, 6);
    const double tx = p->hsc[4], tx2 = p->hsc[5];
    const double e = tx - tx2;
    if (!(e == e)) return -1;
    err.push_back(e);
    const size_t k = err.size() - 1;
    // noise floor reached: the error no longer falls over two steps (one of each kind)
    if (k >= 2 && err[k - 2] < 1e-4 * n && e >= err[k - 2]) {
      done = true;
      break;
    }
    if (e <= 1e-15 * n) {
      done = true;
      break;
    }
    const bool square = fabs(tx2 - nocc) <= fabs(2.0 * tx - tx2 - nocc);
    ++g_kernel_launches;
    k_sp2_update<<<eb, 256, 0, p->s>>>(nn, p->X, p->X2, square ? 1 : 0);
  }
  p->last_iterations = it + 1;
  if (!done) return -1;
  if (g_pipe_gemm) {  // T = 2 X Z: slot 0 holds X, the factor 2 goes into its exponents
    pgemm(p->img[0], p->img[2], p->T, n, false, p->status, p->s, 1);
  } else {
    ++g_kernel_launches;
    k_scale_to<<<eb, 256, 0, p->s>>>(nn, p->X, 2.0, p->X2);
    product(p, p->X2, 0, false, p->Z, 2, true, p->T, false);
  }
  product(p, p->Z, 2, true, p->T, 1, false, P, true);
  return it + 1;
}

void purify_product(Purifier* p, const double* A, const double* B, double* C) {
  product(p, A, 0, false, B, 1, false, C, false);
}

// W = P F P / 2 (the energy-weighted density of the last purify_density call)
void purify_weighted(Purifier* p, const double* F, const double* P, double* W) {
  const size_t nn = (size_t)p->n * p->n;
  product(p, F, 0, false, P, 1, false, p->T, false);
  product(p, P, 1, true, p->T, 0, false, W, true);  // slot 1 holds P (symmetric)
  ++g_kernel_launches;
  k_scale_to<<<ew_blocks(nn), 256, 0, p->s>>>(nn, W, 0.5, W);
}

// largest eigenvalue (out[0]) and residual bound (out[1]) of B = Q (sign (A - shift I)) Q with
// Q = X (occupied: sign +1, shift emin) or I - X (virtual: sign -1, shift emax)
static void lanczos(Purifier* p, bool occupied, double* out_host) {
  const int n = p->n, m = PU_LZ_M;
  cudaStream_t s = p->s;
  double* u = p->lz;
  double* w = p->lz + n;
  double* h = p->lz + 2 * (size_t)n;
  double* alpha = h + (m + 1);
  double* beta = alpha + (m + 1);
  double* ritz = beta + (m + 1);
  const int vb = (n + 255) / 256, sb = (n * 32 + 255) / 256;
  ck(cudaMemsetAsync(alpha, 0, sizeof(double) * 2 * (m + 1), s), "lz");
  // start: a fixed pseudo-random vector, projected on the subspace
  std::vector<double> v0(n);
  uint64_t st = 0x9E3779B97F4A7C15ull;
  for (int i = 0; i < n; ++i) {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    v0[i] = (double)(st >> 11) * 0x1.0p-53 - 0.5;
  }
  ck(cudaMemcpyAsync(u, v0.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s), "lz v0");
  // Q u: X u, or u - X u
  auto project = [&](const double* in, double* out) {
    ++g_kernel_launches;
    k_symv<<<sb, 256, 0, s>>>(n, p->X, in, out);
    if (!occupied) {
      ++g_kernel_launches;
      k_axpby<<<vb, 256, 0, s>>>(n, 1.0, in, -1.0, out, nullptr, -1, 0.0, out);
    }
  };
  project(u, w);
  ++g_kernel_launches;
  k_normalize<<<1, 1024, 0, s>>>(n, w, beta, -1, p->V, 1.0);
  // scale of the operator for the breakdown test
  const double scale = p->hsc[1] - p->hsc[0];
  for (int j = 0; j < m; ++j) {
    const double* vj = p->V + (size_t)j * n;
    project(vj, u);
    ++g_kernel_launches;
    k_symv<<<sb, 256, 0, s>>>(n, p->A, u, w);
    // occupied: w = A u - emin u;  virtual: w = emax u - A u
    ++g_kernel_launches;
    if (occupied) k_axpby<<<vb, 256, 0, s>>>(n, 1.0, w, 0.0, u, p->sc, 0, -1.0, w);
    else k_axpby<<<vb, 256, 0, s>>>(n, -1.0, w, 0.0, u, p->sc, 1, 1.0, w);
    project(w, u);
    // two passes of classical Gram-Schmidt against V_0..V_j (alpha_j from the first)
    for (int pass = 0; pass < 2; ++pass) {
      g_kernel_launches += 2;
      k_dots<<<j + 1, 256, 0, s>>>(n, j + 1, p->V, u, h);
      k_orth<<<vb, 256, 0, s>>>(n, j + 1, p->V, h, u, alpha, j);
    }
    ++g_kernel_launches;
    k_normalize<<<1, 1024, 0, s>>>(n, u, beta, j, p->V + (size_t)(j + 1) * n, scale);
  }
  ++g_kernel_launches;
  k_ritz<<<1, 32, 0, s>>>(m, alpha, beta, ritz);
  ck(cudaMemcpyAsync(out_host, ritz, sizeof(double) * 2, cudaMemcpyDeviceToHost, s), "ritz");
  stream_wait(s);
}

// HOMO and LUMO of the last purify_density call with their residual bounds: gap[0] HOMO,
// gap[1] LUMO, gap[2] bound on |HOMO error| + |LUMO error|
void purify_gap(Purifier* p, double* gap) {
  read_scalars(p, 2);
  double ro[2], rv[2];
  lanczos(p, true, ro);
  lanczos(p, false, rv);
  gap[0] = p->hsc[0] + ro[0];
  gap[1] = p->hsc[1] - rv[0];
  gap[2] = ro[1] + rv[1];
}

double purify_gap_kt() { return PU_GAP_KT; }

int* purify_status(Purifier* p) { return p->status; }

}  // namespace tb
