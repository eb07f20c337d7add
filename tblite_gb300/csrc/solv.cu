// Implicit solvation: generalized Born reaction field (P16 or Still kernel, GBOBC Born radii,
// optional ALPB shape term), CDS surface term with hydrogen-bond correction, free-energy shift:
// ALPB(water), GBSA(water) and the dielectric-constant GB models.
//
// Restated from the reference:
//   Born radii           src/tblite/solvation/born.f90:135-454 (compute_bornr, compute_psi)
//   ALPB matrix/energy   src/tblite/solvation/alpb.f90:218-365, 426-535 (P16 kernel), 562-684
//                        (Still kernel), 656-787 (shape term)
//   CDS and SASA         src/tblite/solvation/cds.f90:247-365, surface.f90:80-387
//   shift                src/tblite/solvation/shift.f90:185-241
//
// GPU formulation.  The reference stores the ALPB matrix J (N x N) and the derivative tensors
// dR_born/dx and dSASA/dx (3 x N x N).  Here none of them is stored: J q is evaluated on the fly
// (one warp per atom, like the Coulomb kernels), and the gradient re-walks the same pair and
// grid loops with the final charges folded into per-atom weights, so the memory stays O(N)
// plus a neighbour list for the surface grid.
#include <cuda_runtime.h>

#include "engine.h"

namespace tb {

constexpr double ZETA_P16 = 1.028;
constexpr double OBC0 = 1.0, OBC1 = 0.8, OBC2 = 4.85;

__device__ __forceinline__ double wsum_s(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// contribution of partner j to psi_i (j's descreening sphere rho_j seen from i's radius
// rvdw_i) and the factor dg with d g / d x_i = dg (x_i - x_j)
__device__ __forceinline__ void psi_term(double r, double rhoj, double rvdwi, double& g,
                                         double& dg) {
  if (r >= rvdwi + rhoj) {
    const double r1 = 1.0 / r;
    const double ap = r + rhoj, am = r - rhoj, ab = ap * am;
    const double rhab = rhoj / ab;
    const double lnab = 0.5 * log(am / ap) * r1;
    g = rhab + lnab;
    dg = -2.0 * rhab / ab + (rhab - lnab) * r1 * r1;
  } else if (r + rhoj > rvdwi) {
    const double r1 = 1.0 / r, r12 = 0.5 * r1, r24 = r12 * r12;
    const double ap = r + rhoj, am = r - rhoj;
    const double rh1 = 1.0 / rvdwi, rhr1 = 1.0 / ap, aprh1 = ap * rh1;
    const double lnab = log(aprh1);
    g = rh1 - rhr1 + r12 * (0.5 * am * (rhr1 - rh1 * aprh1) - lnab);
    dg = (rhr1 * rhr1 * (1.0 - 0.25 * am * r1 * (1.0 + aprh1 * aprh1)) +
          rhoj * r24 * (rhr1 - rh1 * aprh1) + r12 * (r1 * lnab - rhr1)) *
         r1;
  } else {
    g = 0.0;
    dg = 0.0;
  }
}

// Born radii: psi_i summed over partners within the cutoff, then the OBC transform
__global__ void k_born(DevSolv v, const double* __restrict__ xyz) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= v.nat) return;
  const double cut2 = v.lrcut * v.lrcut;
  double psi = 0.0;
  for (int j = lane; j < v.nat; j += 32) {
    if (j == i) continue;
    double d[3], r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      d[k] = xyz[3 * i + k] - xyz[3 * j + k];
      r2 += d[k] * d[k];
    }
    if (r2 > cut2) continue;
    double g, dg;
    psi_term(sqrt(r2), v.rho[j], v.vdwr[i], g, dg);
    psi += g;
  }
  psi = wsum_s(psi);
  if (lane == 0) {
    const double s1 = 1.0 / v.svdw[i], v1 = 1.0 / v.vdwr[i], s2 = 0.5 * v.svdw[i];
    const double br = psi * s2;
    double arg2 = br * (OBC2 * br - OBC1);
    const double arg = br * (OBC0 + arg2);
    arg2 = 2.0 * arg2 + OBC0 + OBC2 * br * br;
    const double th = tanh(arg), ch = cosh(arg);
    v.brad[i] = v.born_scale / (s1 - v1 * th);
    double dp = ch * (s1 - v1 * th);
    v.dscale[i] = v.born_scale * s2 * v1 * arg2 / (dp * dp);
  }
}

// neighbour list of the surface grid (partners within srcut), one warp per atom
__global__ void k_sasa_nbl(DevSolv v, const double* __restrict__ xyz) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= v.nat) return;
  const double cut2 = v.srcut * v.srcut;
  int count = 0;
  for (int j0 = 0; j0 < v.nat; j0 += 32) {
    const int j = j0 + lane;
    bool in = false;
    if (j < v.nat && j != i) {
      double r2 = 0.0;
      for (int k = 0; k < 3; ++k) {
        const double d = xyz[3 * i + k] - xyz[3 * j + k];
        r2 += d * d;
      }
      in = r2 <= cut2;
    }
    const unsigned mask = __ballot_sync(0xffffffffu, in);
    const int pos = count + __popc(mask & ((1u << lane) - 1u));
    if (in && pos < SOLV_MAXNB) v.nbl[(size_t)i * SOLV_MAXNB + pos] = j;
    count += __popc(mask);
  }
  if (lane == 0) {
    v.nnb[i] = count < SOLV_MAXNB ? count : SOLV_MAXNB;
    if (count > SOLV_MAXNB) *v.status = 1;  // list overflow: reported to the host
  }
}

// smoothed exposure of grid point xp of atom i; with grads, the derivative factors of every
// partner in the smoothing shell (d sasap / d x_j = -sasap * fac_j * t_j)
template <bool GRAD>
__device__ __forceinline__ double point_exposure(const DevSolv& v, const double* __restrict__ xyz,
                                                 int i, const double xp[3], int* gj, double* gt,
                                                 int& ng) {
  double sasap = 1.0;
  ng = 0;
  const int nn = v.nnb[i];
  const int* nb = v.nbl + (size_t)i * SOLV_MAXNB;
  for (int q = 0; q < nn; ++q) {
    const int j = nb[q];
    const double t0 = xp[0] - xyz[3 * j], t1 = xp[1] - xyz[3 * j + 1], t2 = xp[2] - xyz[3 * j + 2];
    const double tj2 = t0 * t0 + t1 * t1 + t2 * t2;
    if (tj2 < v.trj2_hi[j]) {
      if (tj2 <= v.trj2_lo[j]) return 0.0;
      const double sq = sqrt(tj2);
      const double uj = sq - v.vdwsa[j];
      const double a3 = v.ah3 * uj * uj;
      const double sij = v.ah0 + (v.ah1 + a3) * uj;
      sasap *= sij;
      if (GRAD) {
        const double ds = (v.ah1 + 3.0 * a3) / (sij * sq);
        gj[ng] = j;
        gt[3 * ng] = ds * t0;
        gt[3 * ng + 1] = ds * t1;
        gt[3 * ng + 2] = ds * t2;
        ++ng;
      }
    }
  }
  return sasap;
}

__device__ __forceinline__ double block_sum_s(double x, double* red) {
  x = wsum_s(x);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  double t = 0.0;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
  __syncthreads();
  return t;
}

// solvent accessible surface of atom i: one block, one thread per grid point
__global__ void __launch_bounds__(256) k_sasa(DevSolv v, const double* __restrict__ xyz) {
  const int i = blockIdx.x;
  __shared__ double red[8];
  double s = 0.0;
  const int p = threadIdx.x;
  if (p < SOLV_NGRID) {
    const double r = v.vdwsa[i];
    const double xp[3] = {xyz[3 * i] + r * v.grid[4 * p], xyz[3 * i + 1] + r * v.grid[4 * p + 1],
                          xyz[3 * i + 2] + r * v.grid[4 * p + 2]};
    int ng;
    const double sasap = point_exposure<false>(v, xyz, i, xp, nullptr, nullptr, ng);
    if (sasap > 1.0e-6) s = v.grid[4 * p + 3] * v.wrp[i] * sasap;
  }
  s = block_sum_s(s, red);
  if (threadIdx.x == 0) v.surface[i] = s;
}

// geometry-only energy per atom: surface tension + the free-energy shift (added to eat)
__global__ void k_solv_nonsc(DevSolv v, double* eat) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.nat) return;
  eat[i] += v.surface[i] * v.tension[i] + v.shift / v.nat;
}

__device__ __forceinline__ double p16(double r, double bi, double bj, double keps) {
  const double ab = sqrt(bi * bj);
  double arg = ab / (ab + ZETA_P16 / 16.0 * r);
  arg *= arg;
  arg *= arg;
  arg *= arg;
  arg *= arg;
  return keps / (r + ab * arg);
}

// Still kernel (alpb.f90:562-601): keps / sqrt(r^2 + a exp(-r^2 / (4 a))), a = R_i R_j
__device__ __forceinline__ double still(double r2, double bi, double bj, double keps) {
  const double aa = bi * bj;
  return keps / sqrt(r2 + aa * exp(-0.25 * r2 / aa));
}

// MODE 0: vat += J q + 2 hbond S q ;  MODE 1: eat += 1/2 q (J q) + hbond S q^2
template <int MODE>
__global__ void k_solv_jq(DevSolv v, const double* __restrict__ xyz, const double* __restrict__ q,
                          double* out) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= v.nat) return;
  const double kconst = v.keps * v.alpbet / v.adet;  // shape term, every matrix element
  double s = 0.0;
  for (int j = lane; j < v.nat; j += 32) {
    double jij;
    if (j == i) {
      jij = v.keps / v.brad[i];
    } else {
      double r2 = 0.0;
      for (int k = 0; k < 3; ++k) {
        const double d = xyz[3 * i + k] - xyz[3 * j + k];
        r2 += d * d;
      }
      jij = v.kernel == 1 ? still(r2, v.brad[i], v.brad[j], v.keps)
                          : p16(sqrt(r2), v.brad[i], v.brad[j], v.keps);
    }
    s += (jij + kconst) * q[j];
  }
  s = wsum_s(s);
  if (lane == 0) {
    const double qi = q[i];
    if (MODE == 0) out[i] += s + 2.0 * v.hbond[i] * v.surface[i] * qi;
    else out[i] += 0.5 * qi * s + v.hbond[i] * v.surface[i] * qi * qi;
  }
}

// Born pair gradient (explicit part) and dE/dR_born, one warp per atom: P16 kernel
// (alpb.f90:470-535) or Still kernel (alpb.f90:604-684)
__global__ void k_solv_pair_grad(DevSolv v, const double* __restrict__ xyz,
                                 const double* __restrict__ q, double* grad) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= v.nat) return;
  const double keps = v.keps, bi = v.brad[i], qi = q[i];
  double g[3] = {0, 0, 0}, dedbr = 0.0;
  for (int j = lane; j < v.nat; j += 32) {
    if (j == i) continue;
    double d[3], r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      d[k] = xyz[3 * i + k] - xyz[3 * j + k];
      r2 += d[k] * d[k];
    }
    const double bj = v.brad[j], qq = qi * q[j];
    if (v.kernel == 1) {
      const double aa = bi * bj, dd = 0.25 * r2 / aa, expd = exp(-dd);
      const double dfgb2 = 1.0 / (r2 + aa * expd);
      const double dfgb3 = dfgb2 * sqrt(dfgb2) * keps;
      const double f = (1.0 - 0.25 * expd) * dfgb3 * qq;
      for (int k = 0; k < 3; ++k) g[k] -= f * d[k];
      dedbr += bj * (-0.5 * expd * (1.0 + dd) * dfgb3) * qq;
      continue;
    }
    const double r1 = sqrt(r2);
    const double ab = sqrt(bi * bj);
    const double arg1 = ab / (ab + ZETA_P16 / 16.0 * r1);
    double a16 = arg1 * arg1;
    a16 *= a16;
    a16 *= a16;
    a16 *= a16;
    const double fgb = r1 + ab * a16;
    const double dfgb2 = 1.0 / (fgb * fgb);
    const double ap = (1.0 - ZETA_P16 * arg1 * a16) * dfgb2;
    const double f = ap * keps / r1 * qq;
    for (int k = 0; k < 3; ++k) g[k] -= f * d[k];
    const double bp = -0.5 * (r1 * ZETA_P16 / ab * arg1 + 1.0) / ab * a16 * dfgb2;
    dedbr += bj * bp * keps * qq;
  }
  for (int k = 0; k < 3; ++k) g[k] = wsum_s(g[k]);
  dedbr = wsum_s(dedbr);
  if (lane == 0) {
    dedbr += -0.5 * keps * qi * qi / (bi * bi);
    for (int k = 0; k < 3; ++k) grad[3 * i + k] += g[k];
    v.wbr[i] = dedbr * v.dscale[i];  // weight of d psi_i in the chain rule
  }
}

// Born radius chain rule: grad_k += sum_j (w_k dg_k(j) + w_j dg_j(k)) (x_k - x_j)
__global__ void k_born_grad(DevSolv v, const double* __restrict__ xyz, double* grad) {
  const int k0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (k0 >= v.nat) return;
  const double cut2 = v.lrcut * v.lrcut;
  const double wk = v.wbr[k0];
  double g[3] = {0, 0, 0};
  for (int j = lane; j < v.nat; j += 32) {
    if (j == k0) continue;
    double d[3], r2 = 0.0;
    for (int c = 0; c < 3; ++c) {
      d[c] = xyz[3 * k0 + c] - xyz[3 * j + c];
      r2 += d[c] * d[c];
    }
    if (r2 > cut2) continue;
    const double r = sqrt(r2);
    double gk, dgk, gj, dgj;
    psi_term(r, v.rho[j], v.vdwr[k0], gk, dgk);   // j's sphere in psi_k
    psi_term(r, v.rho[k0], v.vdwr[j], gj, dgj);   // k's sphere in psi_j
    const double f = wk * dgk + v.wbr[j] * dgj;
    for (int c = 0; c < 3; ++c) g[c] += f * d[c];
  }
  for (int c = 0; c < 3; ++c) g[c] = wsum_s(g[c]);
  if (lane == 0)
    for (int c = 0; c < 3; ++c) grad[3 * k0 + c] += g[c];
}

// surface gradient weighted by c_i = tension_i + hbond_i q_i^2: block per atom i, thread per
// grid point; atom i's own share is block-reduced, the partners' shares go through atomics
__global__ void __launch_bounds__(256) k_sasa_grad(DevSolv v, const double* __restrict__ xyz,
                                                   const double* __restrict__ q, double* grad) {
  const int i = blockIdx.x;
  __shared__ double red[8];
  double gi[3] = {0, 0, 0};
  const int p = threadIdx.x;
  const double ci = v.tension[i] + v.hbond[i] * q[i] * q[i];
  if (p < SOLV_NGRID && ci != 0.0) {
    const double r = v.vdwsa[i];
    const double xp[3] = {xyz[3 * i] + r * v.grid[4 * p], xyz[3 * i + 1] + r * v.grid[4 * p + 1],
                          xyz[3 * i + 2] + r * v.grid[4 * p + 2]};
    int gj[SOLV_MAXSHELL];
    double gt[3 * SOLV_MAXSHELL];
    int ng = 0;
    // partners in the smoothing shell of one point: bounded by SOLV_MAXSHELL (checked)
    double sasap = 1.0;
    {
      const int nn = v.nnb[i];
      const int* nb = v.nbl + (size_t)i * SOLV_MAXNB;
      for (int qn = 0; qn < nn; ++qn) {
        const int j = nb[qn];
        const double t0 = xp[0] - xyz[3 * j], t1 = xp[1] - xyz[3 * j + 1],
                     t2 = xp[2] - xyz[3 * j + 2];
        const double tj2 = t0 * t0 + t1 * t1 + t2 * t2;
        if (tj2 < v.trj2_hi[j]) {
          if (tj2 <= v.trj2_lo[j]) {
            sasap = 0.0;
            break;
          }
          const double sq = sqrt(tj2);
          const double uj = sq - v.vdwsa[j];
          const double a3 = v.ah3 * uj * uj;
          const double sij = v.ah0 + (v.ah1 + a3) * uj;
          sasap *= sij;
          if (ng < SOLV_MAXSHELL) {
            const double ds = (v.ah1 + 3.0 * a3) / (sij * sq);
            gj[ng] = j;
            gt[3 * ng] = ds * t0;
            gt[3 * ng + 1] = ds * t1;
            gt[3 * ng + 2] = ds * t2;
          } else {
            *v.status = 2;  // more partners in one smoothing shell than the kernel holds
          }
          ++ng;
        }
      }
    }
    if (sasap > 1.0e-6) {
      const double wsa = v.grid[4 * p + 3] * v.wrp[i] * sasap * ci;
      const int nk = ng < SOLV_MAXSHELL ? ng : SOLV_MAXSHELL;
      for (int a = 0; a < nk; ++a) {
        const int j = gj[a];
        for (int c = 0; c < 3; ++c) {
          const double t = wsa * gt[3 * a + c];
          gi[c] += t;
          atomicAdd(&grad[3 * j + c], -t);
        }
      }
    }
  }
  for (int c = 0; c < 3; ++c) gi[c] = block_sum_s(gi[c], red);
  if (threadIdx.x == 0)
    for (int c = 0; c < 3; ++c) atomicAdd(&grad[3 * i + c], gi[c]);
}

static inline unsigned warps(int nat) { return (unsigned)((nat * 32 + 127) / 128); }

void solv_setup(const DevSolv& v, const double* xyz, double* eat, cudaStream_t s) {
  ++g_kernel_launches;
  k_born<<<warps(v.nat), 128, 0, s>>>(v, xyz);
  if (!v.cds) {  // no surface term: zero surfaces (read by the potential kernels), no shift
    cudaMemsetAsync(v.surface, 0, sizeof(double) * v.nat, s);
    return;
  }
  g_kernel_launches += 3;
  k_sasa_nbl<<<warps(v.nat), 128, 0, s>>>(v, xyz);
  k_sasa<<<v.nat, 256, 0, s>>>(v, xyz);
  k_solv_nonsc<<<(v.nat + 127) / 128, 128, 0, s>>>(v, eat);
}
void solv_potential(const DevSolv& v, const double* xyz, const double* qat, double* vat,
                    cudaStream_t s) {
  ++g_kernel_launches;
  k_solv_jq<0><<<warps(v.nat), 128, 0, s>>>(v, xyz, qat, vat);
}
void solv_energy(const DevSolv& v, const double* xyz, const double* qat, double* eat,
                 cudaStream_t s) {
  ++g_kernel_launches;
  k_solv_jq<1><<<warps(v.nat), 128, 0, s>>>(v, xyz, qat, eat);
}
void solv_gradient(const DevSolv& v, const double* xyz, const double* qat, double* grad,
                   cudaStream_t s) {
  g_kernel_launches += 2;
  k_solv_pair_grad<<<warps(v.nat), 128, 0, s>>>(v, xyz, qat, grad);
  k_born_grad<<<warps(v.nat), 128, 0, s>>>(v, xyz, grad);
  if (!v.cds) return;
  ++g_kernel_launches;
  k_sasa_grad<<<v.nat, 256, 0, s>>>(v, xyz, qat, grad);
}

}  // namespace tb
