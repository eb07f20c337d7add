// Density matrix by spectral projection for the batched ensemble path (closed shells with a
// gap), beside the batched eigensolver.
//
// The reference reaches the density through its solver slot (src/tblite/scf/solver.f90:28-45),
// filled by diagonalisation (scf/diag.f90:62-143: sygvd, Fermi filling, P = C f C^T).  For a
// closed shell whose HOMO-LUMO gap spans many kT the Fermi occupations are 0 or 2 to ~e^-80, so
// P = 2 X D X^T with X = L^-T (the Cholesky factor of S, X^T S X = I) and D the spectral
// projector onto the lowest nocc eigenvectors of A = X^T F X.  D comes from matrix squarings
// alone (SP2, Niklasson, Phys. Rev. B 66, 155115 (2002)):
//
//   D0 = (emax I - A) / (emax - emin) with Gershgorin bounds [emin, emax] of A,
//   D <- D^2 or 2D - D^2, whichever brings tr D closer to nocc,
//   until the idempotency error tr(D - D^2) stops falling over two steps (Kruchinin, Rubensson,
//   Niklasson, J. Chem. Phys. 145, 204106 (2016)) or reaches the rounding floor.
//
// Per molecule and SCF iteration the eigensolver's tridiagonalisation, eigenvalues, inverse
// iteration and back-transformation (FP64 cores) become ~25 symmetric squarings on the BF16
// tensor cores with FP64-accurate operand splitting (ozaki_pipe.cu: kb_opipe_sq squares the
// iterate from its slice image and writes the next iterate over it in the epilogue; kb_sp2_slice
// writes the new iterate's slice image with one exponent for every line, sums its trace and,
// exactly in integers, tr D^2 = sum of its squared elements, and its last block per molecule
// takes the next decision, so a step is two launches and the decision needs no product).  Every
// molecule of a size bucket iterates in lockstep; each decides its own step on the device and
// stops on its own (its later launches return at once).  The host launches a step budget per
// bucket (the most steps any of its molecules took in the previous SCF iteration plus a margin);
// a molecule that has not converged within it, or whose final gap is below 80 kT (checked after
// the SCF with all eigenvalues of the last Fock matrix), leaves the batch for the one-molecule
// path, which reproduces the reference's diagonalisation exactly.
//
// The energy-weighted density of the gradient is W = P F P / 2 (the reference's C f e C^T for
// 0/2 occupations); bond orders use P S.
#include <cuda_runtime.h>

#include "engine.h"

namespace tb {

namespace {

#define BMOL const MolPtrs& q = mp[list[blockIdx.z]]
#define BARGS const MolPtrs* __restrict__ mp, const int* __restrict__ list

constexpr double SP2_GAP_KT = 80.0;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Gershgorin bounds of A and a fresh projection state: one block per 8 columns (a warp per
// column) writes its columns' lowest and highest bound into its partial-sum slot (the slots of
// the later slice passes, free here); the last block of the molecule to finish (a fence and the
// block count sp2i[5], zero between passes) takes the minimum and maximum over the slots in a
// fixed order and resets the state
__global__ void __launch_bounds__(256) kb_sp2_start(BARGS) {
  BMOL;
  const int n = q.m.nao, lp = ((n + 127) / 128) * 128, nblk = lp / 8;
  if ((int)blockIdx.x >= nblk || *q.flag < 0) return;  // uniform over the block
  __shared__ double smin[8], smax[8];
  __shared__ int last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int j = (int)blockIdx.x * 8 + wid;
  double lo = 1e300, hi = -1e300;
  if (j < n) {
    const double* col = q.A + (size_t)j * n;
    double r = 0.0;
    for (int i = lane; i < n; i += 32)
      if (i != j) r += fabs(col[i]);
    r = warp_sum(r);
    lo = col[j] - r;
    hi = col[j] + r;
  }
  if (lane == 0) {
    smin[wid] = lo;
    smax[wid] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) {
      lo = fmin(lo, smin[w]);
      hi = fmax(hi, smax[w]);
    }
    unsigned long long* pt = q.sp2p + 3 * blockIdx.x;
    pt[0] = (unsigned long long)__double_as_longlong(lo);
    pt[1] = (unsigned long long)__double_as_longlong(hi);
    __threadfence();
    last = atomicAdd(q.sp2i + 5, 1) == nblk - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  lo = 1e300;
  hi = -1e300;
  for (int t = 0; t < nblk; ++t) {
    lo = fmin(lo, __longlong_as_double((long long)__ldcg(q.sp2p + 3 * t)));
    hi = fmax(hi, __longlong_as_double((long long)__ldcg(q.sp2p + 3 * t + 1)));
  }
  if (!(hi > lo)) hi = lo + 1.0;  // a 1 x 1 or scalar A: any positive width
  q.sp2s[0] = lo;
  q.sp2s[1] = hi;
  q.sp2s[2] = q.sp2s[3] = q.sp2s[4] = 1e300;  // idempotency errors e(k-2), e(k-1), e(k)
  q.sp2i[0] = 0;   // converged
  q.sp2i[1] = 0;   // steps taken
  q.sp2i[2] = -1;  // update of the current step: 1 square, 0 2D - D^2, -1 none
  q.sp2i[4] = 0;   // an element outside the fixed-point range
  q.sp2i[5] = 0;   // blocks of the current pass finished (the last one decides)
  // sp2i[3]: tensor-core pipeline status, set by any pipelined product of the molecule; it
  // starts zeroed with the batch and is never cleared (a failure sends the molecule away)
  q.scal[0] = 0.0;  // no Fermi entropy: the occupations are 0/2 (checked after the SCF)
}

// after the step budget: a projection that has not converged sends the molecule to the
// one-molecule path; the steps taken go to the host (budget of the next SCF iteration)
__global__ void kb_sp2_finish(BARGS) {
  BMOL;
  if (threadIdx.x != 0) return;
  *q.sp2steps = q.sp2i[1];
  if (*q.flag < 0) return;
  if (q.sp2i[0] == 0) *q.flag = -6;
}

// after the SCF, with every eigenvalue of the last Fock matrix: the occupations are 0/2 only
// if the HOMO-LUMO gap spans at least 80 kT; otherwise the molecule leaves the batch
__global__ void kb_sp2_gap(BARGS) {
  BMOL;
  if (threadIdx.x != 0 || *q.flag < 0) return;
  const int nocc = (int)q.nalp, n = q.m.nao;
  if (nocc <= 0 || nocc >= n) return;  // no gap to speak of: all levels empty or full
  if (q.emo[nocc] - q.emo[nocc - 1] < SP2_GAP_KT * q.kt) *q.flag = -7;
}

}  // namespace

void sp2_density_b(const BatchLaunch& b, int steps) {
  if (!b.count) return;
  pipe_site_b(b, GS_FX);   // T1 = F X
  pipe_site_b(b, GS_XTT);  // A = X^T T1
  ++g_kernel_launches;
  kb_sp2_start<<<dim3(pimage_lines(b.nao_max) / 8, 1, b.count), 256, 0, b.s>>>(b.mp, b.list);
  sp2_slice_b(b, true);  // D0, its slice image and the first decision
  for (int k = 0; k < steps; ++k) {
    sp2_square_b(b);         // D^2 and the next iterate over D
    sp2_slice_b(b, false);  // its slice image and the next decision
  }
  ++g_kernel_launches;
  kb_sp2_finish<<<dim3(1, 1, b.count), 32, 0, b.s>>>(b.mp, b.list);
  sp2_unfix_b(b);          // D from fixed point to FP64
  pipe_site_b(b, GS_XD);   // T1 = 2 X D
  pipe_site_b(b, GS_PXT);  // P = T1 X^T
}

// a pipelined product after the SCF (W, bond orders) whose wait ran out: the molecule leaves
__global__ void kb_pipe_check(BARGS) {
  BMOL;
  if (threadIdx.x == 0 && *q.flag >= 0 && q.sp2i[3] != 0) *q.flag = -5;
}

void sp2_pipe_check_b(const BatchLaunch& b) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_pipe_check<<<dim3(1, 1, b.count), 32, 0, b.s>>>(b.mp, b.list);
}

void sp2_gap_b(const BatchLaunch& b) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_sp2_gap<<<dim3(1, 1, b.count), 32, 0, b.s>>>(b.mp, b.list);
}

void sp2_weighted_b(const BatchLaunch& b) {
  if (!b.count) return;
  pipe_site_b(b, GS_PF);    // T1 = P F / 2
  pipe_site_b(b, GS_WPFP);  // W = T1 P, into F
}

#undef BMOL
#undef BARGS

}  // namespace tb
