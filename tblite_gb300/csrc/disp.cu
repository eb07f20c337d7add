// Self-consistent D4 dispersion on the GPU (two-body, charge dependent) and the charge-free
// Axilrod-Teller-Muto three-body term.
//
// The reference calls dftd4 v4.2.0 through src/tblite/disp/d4.f90:105-474 (update:
// coordination number + dispersion matrix; get_engrad: three-body; get_energy /
// get_potential / get_gradient: two-body).  The D4 model is restated from its published
// form; its element data come from the element-data pack compiled into the library.
//
// GPU formulation: the (mref N)^2 dispersion matrix of the reference is never stored.  One
// warp per atom walks its partners and contracts the reference C6 table with the partner's
// weights on the fly; every per-atom kernel sums only its own atom's share of each pair or
// triple, so all reductions are deterministic (no atomics).
#include <cuda_runtime.h>

#include <stdexcept>

#include "engine.h"

namespace tb {

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// D4 coordination number, dcount/dr
__device__ __forceinline__ void d4_count(const DevD4& d, int i, int j, double r, double& c,
                                         double& dc) {
  const double rc = d.rcov[i] + d.rcov[j];
  const double den = d.k4 * exp(-(fabs(d.en[i] - d.en[j]) + d.k5) * (fabs(d.en[i] - d.en[j]) + d.k5) / d.k6);
  const double arg = -d.kn * (r - rc) / rc;
  c = den * 0.5 * (1.0 + erf(arg));
  dc = -den * d.kn / rc * exp(-arg * arg) * 0.5641895835477563;  // 1/sqrt(pi)
}

__device__ __forceinline__ void d4_cn_dev(DevMol m, DevD4 d, double* cn) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp;
  const double cut2 = d.cn_cutoff * d.cn_cutoff;
  double acc = 0.0;
  for (int j = lane; j < m.nat; j += 32) {
    if (j == i) continue;
    double r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double t = m.xyz[3 * i + k] - m.xyz[3 * j + k];
      r2 += t * t;
    }
    if (r2 > cut2 || r2 < 1e-12) continue;
    double c, dc;
    d4_count(d, i, j, sqrt(r2), c, dc);
    acc += c;
  }
  acc = wsum(acc);
  if (lane == 0) cn[i] = acc;
}
__global__ void k_d4_cn(DevMol m, DevD4 d, double* cn) {
  d4_cn_dev(m, d, cn);
}

// Gaussian reference weights in CN and their CN derivative (charge independent part)
__device__ __forceinline__ void d4_weights_dev(int nat, DevD4 d, const double* __restrict__ cn, double* gw,
                             double* dgw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  const int nr = d.nref[i];
  double num[D4_MREF], dnum[D4_MREF], norm = 0.0, dnorm = 0.0;
  for (int r = 0; r < D4_MREF; ++r) {
    num[r] = 0.0;
    dnum[r] = 0.0;
    if (r >= nr) continue;
    const double dcn = cn[i] - d.refcn[i * D4_MREF + r];
    for (int k = 1; k <= d.ngw[i * D4_MREF + r]; ++k) {
      const double w = exp(-d.wf * k * dcn * dcn);
      num[r] += w;
      dnum[r] += -2.0 * d.wf * k * dcn * w;
    }
    norm += num[r];
    dnorm += dnum[r];
  }
  for (int r = 0; r < D4_MREF; ++r) {
    gw[i * D4_MREF + r] = r < nr ? num[r] / norm : 0.0;
    dgw[i * D4_MREF + r] = r < nr ? dnum[r] / norm - num[r] * dnorm / (norm * norm) : 0.0;
  }
}
__global__ void k_d4_weights(int nat, DevD4 d, const double* __restrict__ cn, double* gw,
                             double* dgw) {
  d4_weights_dev(nat, d, cn, gw, dgw);
}

// charge scaling: gwv = gw zeta(q), dgwdq = gw dzeta/dq, dgwv_cn = dgw/dcn zeta(q)
__device__ __forceinline__ void d4_zeta_dev(int nat, DevD4 d, const double* __restrict__ q,
                          const double* __restrict__ gw, const double* __restrict__ dgw,
                          double* gwv, double* dgwdq, double* dgwv_cn) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  const double qi = q ? q[i] : 0.0;
  const double z = d.zeff[i] + qi;
  for (int r = 0; r < D4_MREF; ++r) {
    double zeta = 0.0, dzeta = 0.0;
    if (r < d.nref[i]) {
      const double zr = d.zeff[i] + d.refq[i * D4_MREF + r];
      if (z > 0.0) {
        const double t = exp(d.gc * d.gam[i] * (1.0 - zr / z));
        zeta = exp(d.ga * (1.0 - t));
        dzeta = zeta * (-d.ga * t) * d.gc * d.gam[i] * zr / (z * z);
      } else {
        zeta = exp(d.ga);
      }
    }
    const int k = i * D4_MREF + r;
    gwv[k] = gw[k] * zeta;
    if (dgwdq) dgwdq[k] = gw[k] * dzeta;
    if (dgwv_cn) dgwv_cn[k] = dgw[k] * zeta;
  }
}
__global__ void k_d4_zeta(int nat, DevD4 d, const double* __restrict__ q,
                          const double* __restrict__ gw, const double* __restrict__ dgw,
                          double* gwv, double* dgwdq, double* dgwv_cn) {
  d4_zeta_dev(nat, d, q, gw, dgw, gwv, dgwdq, dgwv_cn);
}

__device__ __forceinline__ double d4_de(double r2, double rrij, double r0, double s6, double s8,
                                        double& dd) {
  const double r6 = r2 * r2 * r2, r8 = r6 * r2;
  const double r02 = r0 * r0, r06 = r02 * r02 * r02, r08 = r06 * r02;
  const double t6 = 1.0 / (r6 + r06), t8 = 1.0 / (r8 + r08);
  const double r = sqrt(r2);
  dd = s6 * 6.0 * r6 / r * t6 * t6 + s8 * rrij * 8.0 * r8 / r * t8 * t8;
  return -(s6 * t6 + s8 * rrij * t8);
}

// MODE 0: vat += sum_r dgwdq_r u_r ; MODE 1: eat += 1/2 sum_r gwv_r u_r ;
// MODE 2: gradient at fixed weights + dEdcn (own atom share), per-atom sigma partials
// two-body damping kernel of every ordered pair (i, j), once per geometry: the pair kernels of
// the SCF iterations read it instead of evaluating the powers and divisions of d4_de
__device__ __forceinline__ void d4_de_table_dev(DevMol m, DevD4 d, double* tab) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int nat = m.nat;
  if (t >= (long long)nat * nat) return;
  const int i = (int)(t / nat), j = (int)(t % nat);
  double de = 0.0;
  if (i != j) {
    double r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double v = m.xyz[3 * i + k] - m.xyz[3 * j + k];
      r2 += v * v;
    }
    if (!(r2 > d.disp2_cutoff * d.disp2_cutoff || r2 < 1e-12)) {
      const double rrij = 3.0 * d.r4r2[i] * d.r4r2[j];
      const double r0 = d.a1 * sqrt(rrij) + d.a2;
      double dd;
      de = d4_de(r2, rrij, r0, d.s6, d.s8, dd);
    }
  }
  tab[t] = de;
}

// detab (MODE 0, 1): the table of d4_de_table_dev, or nullptr to evaluate the kernel here
template <int MODE>
__device__ __forceinline__ void d4_pair_dev(DevMol m, DevD4 d, const double* __restrict__ gwv,
                          const double* __restrict__ dgwdq, const double* __restrict__ dgwv_cn,
                          double* vat, double* eat, double* grad, double* sig_at, double* dEdcn,
                          const double* __restrict__ detab = nullptr) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp;
  const double cut2 = d.disp2_cutoff * d.disp2_cutoff;
  const int ld = d.nsp * D4_MREF;
  const double* tab_i = d.c6ref + (size_t)d.sp[i] * D4_MREF * ld;
  double gi[D4_MREF], dci[D4_MREF];
  const int nri = d.nref[i];
#pragma unroll
  for (int r = 0; r < D4_MREF; ++r) {
    gi[r] = gwv[i * D4_MREF + r];
    dci[r] = MODE == 2 ? dgwv_cn[i * D4_MREF + r] : 0.0;
  }
  double u[D4_MREF] = {0, 0, 0, 0, 0, 0, 0};
  double g[3] = {0, 0, 0}, sg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, dcn = 0.0;
  for (int j = lane; j < m.nat; j += 32) {
    if (j == i) continue;
    double v[3] = {0.0, 0.0, 0.0}, r2 = 0.0, dd = 0.0, de;
    if (MODE < 2 && detab) {
      de = detab[(size_t)i * m.nat + j];
      if (de == 0.0) continue;  // beyond the cutoff
    } else {
      for (int k = 0; k < 3; ++k) {
        v[k] = m.xyz[3 * i + k] - m.xyz[3 * j + k];
        r2 += v[k] * v[k];
      }
      if (r2 > cut2 || r2 < 1e-12) continue;
      const double rrij = 3.0 * d.r4r2[i] * d.r4r2[j];
      const double r0 = d.a1 * sqrt(rrij) + d.a2;
      de = d4_de(r2, rrij, r0, d.s6, d.s8, dd);
    }
    const double* tab = tab_i + d.sp[j] * D4_MREF;
    const double* gj = gwv + j * D4_MREF;
    // only the atoms' own reference points (weights and C6 entries beyond them are zero):
    // unrolled to the maximum with guards so the accumulators stay in registers
    const int nrj = d.nref[j];
    if (MODE < 2) {
#pragma unroll
      for (int r = 0; r < D4_MREF; ++r) {
        if (r >= nri) break;
        double acc = 0.0;
#pragma unroll
        for (int s = 0; s < D4_MREF; ++s)
          if (s < nrj) acc += tab[(size_t)r * ld + s] * gj[s];
        u[r] += de * acc;
      }
    } else {
      double c6 = 0.0, dc6 = 0.0;
#pragma unroll
      for (int r = 0; r < D4_MREF; ++r) {
        if (r >= nri) break;
        double acc = 0.0;
#pragma unroll
        for (int s = 0; s < D4_MREF; ++s)
          if (s < nrj) acc += tab[(size_t)r * ld + s] * gj[s];
        c6 += gi[r] * acc;
        dc6 += dci[r] * acc;
      }
      dcn += de * dc6;
      const double f = dd * c6 / sqrt(r2);
      for (int k = 0; k < 3; ++k) g[k] += f * v[k];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) sg[3 * a + b] += 0.5 * f * v[a] * v[b];
    }
  }
  if (MODE < 2) {
    for (int r = 0; r < D4_MREF; ++r) u[r] = wsum(u[r]);
    if (lane == 0) {
      double acc = 0.0;
      if (MODE == 0) {
        for (int r = 0; r < D4_MREF; ++r) acc += dgwdq[i * D4_MREF + r] * u[r];
        vat[i] += acc;
      } else {
        for (int r = 0; r < D4_MREF; ++r) acc += gi[r] * u[r];
        eat[i] += 0.5 * acc;
      }
    }
  } else {
    for (int k = 0; k < 3; ++k) g[k] = wsum(g[k]);
    for (int k = 0; k < 9; ++k) sg[k] = wsum(sg[k]);
    dcn = wsum(dcn);
    if (lane == 0) {
      for (int k = 0; k < 3; ++k) grad[3 * i + k] += g[k];
      for (int k = 0; k < 9; ++k) sig_at[9 * i + k] += sg[k];
      dEdcn[i] += dcn;
    }
  }
}
template <int MODE>
__global__ void k_d4_pair(DevMol m, DevD4 d, const double* __restrict__ gwv,
                          const double* __restrict__ dgwdq, const double* __restrict__ dgwv_cn,
                          double* vat, double* eat, double* grad, double* sig_at, double* dEdcn) {
  d4_pair_dev<MODE>(m, d, gwv, dgwdq, dgwv_cn, vat, eat, grad, sig_at, dEdcn);
}

// atomic C6 at the given weights and d c6_ij / d cn_i
__device__ __forceinline__ void d4_c6_dev(int nat, DevD4 d, const double* __restrict__ gwv,
                        const double* __restrict__ dgwv_cn, double* c6, double* dc6) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)nat * nat) return;
  const int i = (int)(t / nat), j = (int)(t % nat);
  const int ld = d.nsp * D4_MREF;
  const double* tab = d.c6ref + (size_t)d.sp[i] * D4_MREF * ld + d.sp[j] * D4_MREF;
  double c = 0.0, dc = 0.0;
  for (int r = 0; r < D4_MREF; ++r) {
    double acc = 0.0;
    for (int s = 0; s < D4_MREF; ++s) acc += tab[(size_t)r * ld + s] * gwv[j * D4_MREF + s];
    c += gwv[i * D4_MREF + r] * acc;
    dc += dgwv_cn[i * D4_MREF + r] * acc;
  }
  c6[t] = c;
  dc6[t] = dc;
}
__global__ void k_d4_c6(int nat, DevD4 d, const double* __restrict__ gwv,
                        const double* __restrict__ dgwv_cn, double* c6, double* dc6) {
  d4_c6_dev(nat, d, gwv, dgwv_cn, c6, dc6);
}

// Axilrod-Teller-Muto term (disp/d4.f90 three-body part, d4 get_atm_dispersion).  Every factor
// of a triple (i, j, l) that is a product over its three pairs is tabulated per pair first
// (k_d4_atm_pairs): r^2, 1/r, the damping ratio (r0/r)^(alpha/3), sqrt|C6| and
// dC6_ij/dCN_i / (2 C6_ij) in both index orders, so that no pow or sqrt and a single division
// remain per triple.  Each triple i < j < l is then evaluated once (k_d4_atm): its energy goes
// 1/3 to each atom, its CN derivatives to the three atoms, and its derivatives with respect to
// the three squared distances into a pair matrix Gamma (upper triangle); the forces and the
// virial follow from Gamma in one pass over the pairs (k_d4_atm_grad):
//   dE/dR_i = sum_j 2 Gamma_ij (R_i - R_j),  sigma = sum_{i<j} 2 Gamma_ij v_ij v_ij^T.
// tab layout [8][nat][nat]: r^2 (+inf beyond the cutoff), 1/r, ratio, sqrt|C6|, dq, dq^T,
// Gamma rows written by their owner atom, Gamma of the (j, l) pairs accumulated atomically.
constexpr int ATM_TABLES = 8;
__device__ __forceinline__ void d4_atm_pairs_dev(DevMol m, DevD4 d, const double* __restrict__ c6,
                                                 const double* __restrict__ dc6, double* tab,
                                                 double* eat) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int nat = m.nat;
  const size_t nn = (size_t)nat * nat;
  if (t >= (long long)nn) return;
  if (t < nat) eat[t] = 0.0;
  const int i = (int)(t / nat), j = (int)(t % nat);
  double r2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double v = m.xyz[3 * j + k] - m.xyz[3 * i + k];
    r2 += v * v;
  }
  const double cut2 = d.disp3_cutoff * d.disp3_cutoff;
  double ir = 0.0, w = 0.0, sc = 0.0, dq = 0.0, dqt = 0.0;
  if (i == j || r2 > cut2 || r2 < 1e-12) {
    r2 = __longlong_as_double(0x7ff0000000000000LL);  // +inf: never inside the cutoff
  } else {
    const double r = sqrt(r2);
    ir = 1.0 / r;
    const double r0 = d.a1 * sqrt(3.0 * d.r4r2[i] * d.r4r2[j]) + d.a2;
    w = pow(r0 * ir, d.atm_alpha / 3.0);
    const double c = c6[t];
    sc = sqrt(fabs(c));
    dq = c != 0.0 ? dc6[t] / (2.0 * c) : 0.0;
    dqt = c != 0.0 ? dc6[(size_t)j * nat + i] / (2.0 * c) : 0.0;
  }
  tab[t] = r2;
  tab[nn + t] = ir;
  tab[2 * nn + t] = w;
  tab[3 * nn + t] = sc;
  tab[4 * nn + t] = dq;
  tab[5 * nn + t] = dqt;
  tab[7 * nn + t] = 0.0;
}
__global__ void k_d4_atm_pairs(DevMol m, DevD4 d, const double* __restrict__ c6,
                               const double* __restrict__ dc6, double* tab, double* eat) {
  d4_atm_pairs_dev(m, d, c6, dc6, tab, eat);
}

// one warp per atom i, triples i < j < l: j warp-uniform, the lanes walk l > j.  The warp keeps
// three rows in shared memory (3 nat doubles): Gamma_i. (roles (i, j) and (i, l)), the energy
// thirds and the CN derivatives of the partners; Gamma of the (j, l) pairs goes to global memory
// with coalesced atomics.  eat and dEdcn are accumulated (eat is zeroed by the pairs kernel).
__device__ __forceinline__ void d4_atm_dev(DevMol m, DevD4 d, double* tab, double* eat,
                                           double* dEdcn, double* srow) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nat = m.nat;
  if (warp >= nat) return;
  const int i = warp;
  const size_t nn = (size_t)nat * nat;
  const double* R2 = tab;
  const double* IR = tab + nn;
  const double* W = tab + 2 * nn;
  const double* SC = tab + 3 * nn;
  const double* DQ = tab + 4 * nn;
  const double* DQT = tab + 5 * nn;
  double* GO = tab + 6 * nn;
  double* GB = tab + 7 * nn;
  double* sG = srow;
  double* sE = srow + nat;
  double* sD = srow + 2 * nat;
  for (int l = lane; l < nat; l += 32) {
    sG[l] = 0.0;
    sE[l] = 0.0;
    sD[l] = 0.0;
  }
  __syncwarp();
  const double cut2 = d.disp3_cutoff * d.disp3_cutoff;
  const double a6 = d.atm_alpha / 6.0;
  const size_t ri = (size_t)i * nat;
  double ei = 0.0, di = 0.0;
  for (int j = i + 1; j < nat; ++j) {
    const double a = R2[ri + j];
    if (!(a <= cut2)) continue;  // beyond the cutoff (warp uniform)
    const size_t rj = (size_t)j * nat;
    const double irij = IR[ri + j], wij = W[ri + j], scij = SC[ri + j];
    const double dqij = DQ[ri + j], dqji = DQT[ri + j];
    const double ia = irij * irij;
    double gA = 0.0, eJ = 0.0, dJ = 0.0;
    for (int l = j + 1 + lane; l < nat; l += 32) {
      const double c = R2[ri + l], b = R2[rj + l];
      if (!(c <= cut2) || !(b <= cut2)) continue;
      const double iril = IR[ri + l], irjl = IR[rj + l];
      const double c9 = -d.s9 * scij * SC[ri + l] * SC[rj + l];
      const double t = wij * W[ri + l] * W[rj + l];
      const double ir1 = irij * iril * irjl;
      const double ir2 = ir1 * ir1, ir3 = ir2 * ir1, ir5 = ir3 * ir2;
      const double fdmp = 1.0 / (1.0 + 6.0 * t);
      // angular factor in the squared distances a = r2ij, b = r2jl, c = r2il
      const double ib = irjl * irjl, ic = iril * iril;
      const double pa = a - b + c, pb = -a + b + c, pc = a + b - c;
      const double P = pc * pa * pb;
      const double ang = 0.375 * P * ir5 + ir3;
      const double E = ang * fdmp * c9;
      const double dPa = pa * pb + pc * pb - pc * pa;
      const double dPc = -pa * pb + pc * pb + pc * pa;
      const double dPb = pa * pb - pc * pb + pc * pa;
      const double g0 = ang * (-6.0 * fdmp * fdmp) * (-a6) * t;
      const double h = 0.375 * ir5, q = 2.5 * P * h, s = 1.5 * ir3;
      const double dEa = c9 * ((dPa * h - (q + s) * ia) * fdmp + g0 * ia);
      const double dEb = c9 * ((dPb * h - (q + s) * ib) * fdmp + g0 * ib);
      const double dEc = c9 * ((dPc * h - (q + s) * ic) * fdmp + g0 * ic);
      const double e3 = E * (1.0 / 3.0);
      ei += e3;
      eJ += e3;
      sE[l] += e3;
      gA += dEa;
      sG[l] += dEc;
      atomicAdd(GB + rj + l, dEb);
      // dE/dCN through C6_pq = sqrt: E dC6_pq/dCN_p / (2 C6_pq)
      di += E * (dqij + DQ[ri + l]);
      dJ += E * (dqji + DQ[rj + l]);
      sD[l] += E * (DQT[ri + l] + DQT[rj + l]);
    }
    gA = wsum(gA);
    eJ = wsum(eJ);
    dJ = wsum(dJ);
    if (lane == 0) {
      sG[j] += gA;
      sE[j] += eJ;
      sD[j] += dJ;
    }
    __syncwarp();
  }
  ei = wsum(ei);
  di = wsum(di);
  for (int l = lane; l < nat; l += 32) {
    if (l > i) GO[ri + l] = sG[l];
    if (l != i) {
      if (sE[l] != 0.0) atomicAdd(eat + l, sE[l]);
      if (sD[l] != 0.0) atomicAdd(dEdcn + l, sD[l]);
    }
  }
  if (lane == 0) {
    atomicAdd(eat + i, ei);
    atomicAdd(dEdcn + i, di);
  }
}
__global__ void k_d4_atm(DevMol m, DevD4 d, double* tab, double* eat, double* dEdcn) {
  extern __shared__ double atm_rows[];
  d4_atm_dev(m, d, tab, eat, dEdcn, atm_rows + (size_t)(threadIdx.x >> 5) * 3 * m.nat);
}

// forces and virial from Gamma: one warp per atom, half of each pair's virial to each atom
__device__ __forceinline__ void d4_atm_grad_dev(DevMol m, const double* __restrict__ tab,
                                                double* grad, double* sig_at) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nat = m.nat;
  if (warp >= nat) return;
  const int i = warp;
  const size_t nn = (size_t)nat * nat;
  const double* GO = tab + 6 * nn;
  const double* GB = tab + 7 * nn;
  double g[3] = {0, 0, 0}, sg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int j = lane; j < nat; j += 32) {
    if (j == i) continue;
    const size_t u = i < j ? (size_t)i * nat + j : (size_t)j * nat + i;
    const double G = GO[u] + GB[u];
    if (G == 0.0) continue;
    double v[3];
    for (int k = 0; k < 3; ++k) v[k] = m.xyz[3 * j + k] - m.xyz[3 * i + k];
    for (int k = 0; k < 3; ++k) g[k] += -2.0 * G * v[k];
    for (int p = 0; p < 3; ++p)
      for (int q = 0; q < 3; ++q) sg[3 * p + q] += G * v[p] * v[q];
  }
  for (int k = 0; k < 3; ++k) g[k] = wsum(g[k]);
  for (int k = 0; k < 9; ++k) sg[k] = wsum(sg[k]);
  if (lane == 0) {
    for (int k = 0; k < 3; ++k) grad[3 * i + k] += g[k];
    for (int k = 0; k < 9; ++k) sig_at[9 * i + k] += sg[k];
  }
}
__global__ void k_d4_atm_grad(DevMol m, const double* __restrict__ tab, double* grad,
                              double* sig_at) {
  d4_atm_grad_dev(m, tab, grad, sig_at);
}

// warps per block of k_d4_atm: its shared memory holds 3 nat doubles per warp
static inline int atm_warps(int nat) {
  const size_t per = (size_t)3 * nat * sizeof(double);
  if (per * 2 <= 200 * 1024) return 2;
  if (per <= 200 * 1024) return 1;
  return 0;
}
static void atm_attr(size_t smem) {
  static size_t set = 0;
  if (smem > 48 * 1024 && smem > set) {
    cudaFuncSetAttribute(k_d4_atm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    set = smem;
  }
}

__device__ __forceinline__ void d4_cn_grad_dev(DevMol m, DevD4 d, const double* __restrict__ dEdcn, double* grad,
                             double* sig_at) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp;
  const double cut2 = d.cn_cutoff * d.cn_cutoff;
  double g[3] = {0, 0, 0}, sg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int j = lane; j < m.nat; j += 32) {
    if (j == i) continue;
    double v[3], r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      v[k] = m.xyz[3 * i + k] - m.xyz[3 * j + k];
      r2 += v[k] * v[k];
    }
    if (r2 > cut2 || r2 < 1e-12) continue;
    const double r = sqrt(r2);
    double c, dc;
    d4_count(d, i, j, r, c, dc);
    const double f = (dEdcn[i] + dEdcn[j]) * dc / r;
    for (int k = 0; k < 3; ++k) g[k] += f * v[k];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) sg[3 * a + b] += 0.5 * f * v[a] * v[b];
  }
  for (int k = 0; k < 3; ++k) g[k] = wsum(g[k]);
  for (int k = 0; k < 9; ++k) sg[k] = wsum(sg[k]);
  if (lane == 0) {
    for (int k = 0; k < 3; ++k) grad[3 * i + k] += g[k];
    for (int k = 0; k < 9; ++k) sig_at[9 * i + k] += sg[k];
  }
}
__global__ void k_d4_cn_grad(DevMol m, DevD4 d, const double* __restrict__ dEdcn, double* grad,
                             double* sig_at) {
  d4_cn_grad_dev(m, d, dEdcn, grad, sig_at);
}

static inline unsigned warps_grid(int nat) { return (unsigned)((nat * 32 + 63) / 64); }

void d4_setup(const DevMol& m, const DevD4& d, D4Work& w, bool grad, double* grad_out,
              double* sig_at, cudaStream_t s) {
  ++g_kernel_launches;
  k_d4_cn<<<warps_grid(m.nat), 64, 0, s>>>(m, d, w.cn);
  ++g_kernel_launches;
  k_d4_weights<<<(m.nat + 127) / 128, 128, 0, s>>>(m.nat, d, w.cn, w.gw, w.dgw);
  // charge-free weights for the three-body term
  ++g_kernel_launches;
  k_d4_zeta<<<(m.nat + 127) / 128, 128, 0, s>>>(m.nat, d, nullptr, w.gw, w.dgw, w.gwv, nullptr,
                                                 w.dgwv_cn);
  const long long nn = (long long)m.nat * m.nat;
  ++g_kernel_launches;
  k_d4_c6<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(m.nat, d, w.gwv, w.dgwv_cn, w.c6, w.dc6);
  cudaMemsetAsync(w.dEdcn, 0, sizeof(double) * m.nat, s);
  g_kernel_launches += 2;
  k_d4_atm_pairs<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(m, d, w.c6, w.dc6, w.atm, w.e3);
  const int wpb = atm_warps(m.nat);
  if (!wpb) throw std::runtime_error("three-body dispersion: more atoms than the GPU kernel holds");
  const size_t smem = (size_t)wpb * 3 * m.nat * sizeof(double);
  atm_attr(smem);
  k_d4_atm<<<(m.nat + wpb - 1) / wpb, 32 * wpb, smem, s>>>(m, d, w.atm, w.e3, w.dEdcn);
  if (grad) {
    ++g_kernel_launches;
    k_d4_atm_grad<<<warps_grid(m.nat), 64, 0, s>>>(m, w.atm, grad_out, sig_at);
  }
}

void d4_potential(const DevMol& m, const DevD4& d, D4Work& w, const double* qat, double* vat,
                  cudaStream_t s) {
  ++g_kernel_launches;
  k_d4_zeta<<<(m.nat + 127) / 128, 128, 0, s>>>(m.nat, d, qat, w.gw, w.dgw, w.gwv, w.dgwdq,
                                                 nullptr);
  ++g_kernel_launches;
  k_d4_pair<0><<<warps_grid(m.nat), 64, 0, s>>>(m, d, w.gwv, w.dgwdq, nullptr, vat, nullptr,
                                                 nullptr, nullptr, nullptr);
}

void d4_energy(const DevMol& m, const DevD4& d, D4Work& w, const double* qat, double* eat,
               cudaStream_t s) {
  ++g_kernel_launches;
  k_d4_zeta<<<(m.nat + 127) / 128, 128, 0, s>>>(m.nat, d, qat, w.gw, w.dgw, w.gwv, nullptr,
                                                 nullptr);
  ++g_kernel_launches;
  k_d4_pair<1><<<warps_grid(m.nat), 64, 0, s>>>(m, d, w.gwv, nullptr, nullptr, nullptr, eat,
                                                 nullptr, nullptr, nullptr);
}

void d4_gradient(const DevMol& m, const DevD4& d, D4Work& w, const double* qat, double* grad,
                 double* sig_at, cudaStream_t s) {
  ++g_kernel_launches;
  k_d4_zeta<<<(m.nat + 127) / 128, 128, 0, s>>>(m.nat, d, qat, w.gw, w.dgw, w.gwv, nullptr,
                                                 w.dgwv_cn);
  ++g_kernel_launches;
  k_d4_pair<2><<<warps_grid(m.nat), 64, 0, s>>>(m, d, w.gwv, nullptr, w.dgwv_cn, nullptr, nullptr,
                                                 grad, sig_at, w.dEdcn);
  ++g_kernel_launches;
  k_d4_cn_grad<<<warps_grid(m.nat), 64, 0, s>>>(m, d, w.dEdcn, grad, sig_at);
}

// ------------------------------------------------------------------------------------
// D3(BJ) two-body dispersion of GFN1-xTB (reference src/tblite/disp/d3.f90, which calls
// s-dftd3 with s9 = 0): exponential coordination number over the covalent radii, normalised
// Gaussian reference weights w_ir in CN, C6_ij = sum_rs w_ir w_js C6ref(r, s, Z_i, Z_j) from the
// per-element-pair reference table, rational (BJ) damping.  Three kernels, one warp per atom
// each, every atom summing its own share of each pair (deterministic, no atomics):
//   setup:  CN_i, w_ir and dw_ir/dCN_i
//   pair:   E_i += 1/2 sum_j E_ij, the explicit pair gradient, dE/dCN_i
//   cn:     CN chain rule  grad_i += sum_j (dE/dCN_i + dE/dCN_j) dc_ij/dr (R_i - R_j)/r
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void d3_count(double r, double r0, double k1, double& c, double& dc) {
  const double e = exp(-k1 * (r0 / r - 1.0));
  c = 1.0 / (1.0 + e);
  dc = -c * c * e * k1 * r0 / (r * r);
}

__device__ __forceinline__ void d3_setup_dev(const DevMol& m, const DevD3& d) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp;
  const double cut2 = d.cn_cutoff * d.cn_cutoff;
  double acc = 0.0;
  for (int j = lane; j < m.nat; j += 32) {
    if (j == i) continue;
    double r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double t = m.xyz[3 * i + k] - m.xyz[3 * j + k];
      r2 += t * t;
    }
    if (r2 > cut2 || r2 < 1e-12) continue;
    double c, dc;
    d3_count(sqrt(r2), d.rcov[i] + d.rcov[j], d.k1, c, dc);
    acc += c;
  }
  acc = wsum(acc);
  if (lane != 0) return;
  d.cn[i] = acc;
  double w[D4_MREF], dw[D4_MREF], norm = 0.0, dnorm = 0.0;
  const int nr = d.nref[i];
  for (int r = 0; r < nr; ++r) {
    const double t = acc - d.refcn[i * D4_MREF + r];
    w[r] = exp(-d.k3 * t * t);
    dw[r] = -2.0 * d.k3 * t * w[r];
    norm += w[r];
    dnorm += dw[r];
  }
  for (int r = 0; r < D4_MREF; ++r) {
    d.w[i * D4_MREF + r] = r < nr ? w[r] / norm : 0.0;
    d.dw[i * D4_MREF + r] = r < nr ? (dw[r] * norm - w[r] * dnorm) / (norm * norm) : 0.0;
  }
}

// C6 of the pair (i, j) and its derivatives in CN_i and CN_j
__device__ __forceinline__ void d3_c6(const DevD3& d, int i, int j, double& c6, double& dc6i,
                                      double& dc6j) {
  const int ld = d.nsp * D4_MREF;
  const double* tab = d.c6ref + (size_t)d.sp[i] * D4_MREF * ld + d.sp[j] * D4_MREF;
  const double *wi = d.w + i * D4_MREF, *wj = d.w + j * D4_MREF;
  const double *dwi = d.dw + i * D4_MREF, *dwj = d.dw + j * D4_MREF;
  c6 = dc6i = dc6j = 0.0;
  for (int r = 0; r < d.nref[i]; ++r) {
    double s = 0.0, ds = 0.0;
    for (int q = 0; q < d.nref[j]; ++q) {
      const double c = tab[(size_t)r * ld + q];
      s += wj[q] * c;
      ds += dwj[q] * c;
    }
    c6 += wi[r] * s;
    dc6i += dwi[r] * s;
    dc6j += wi[r] * ds;
  }
}

__device__ __forceinline__ void d3_pair_dev(const DevMol& m, const DevD3& d, int grad, double* eat,
                                            double* grad_out, double* sig_at) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp;
  const double cut2 = d.cutoff * d.cutoff;
  const double ri = d.r4r2[i];
  double e = 0.0, dcn = 0.0, g[3] = {0, 0, 0}, sg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int j = lane; j < m.nat; j += 32) {
    if (j == i) continue;
    double v[3], r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      v[k] = m.xyz[3 * i + k] - m.xyz[3 * j + k];
      r2 += v[k] * v[k];
    }
    if (r2 > cut2) continue;
    const double r = sqrt(r2);
    const double qq = 3.0 * ri * d.r4r2[j];
    const double r0 = d.a1 * sqrt(qq) + d.a2;
    const double r02 = r0 * r0, r06 = r02 * r02 * r02, r08 = r06 * r02;
    const double r6 = r2 * r2 * r2, r8 = r6 * r2;
    const double t6 = 1.0 / (r6 + r06), t8 = 1.0 / (r8 + r08);
    double c6, dc6i, dc6j;
    d3_c6(d, i, j, c6, dc6i, dc6j);
    const double dedc6 = -(d.s6 * t6 + d.s8 * qq * t8);
    e += 0.5 * dedc6 * c6;
    if (grad) {
      const double de = c6 * (d.s6 * 6.0 * r6 / r * t6 * t6 + d.s8 * qq * 8.0 * r8 / r * t8 * t8);
      const double f = de / r;
      for (int k = 0; k < 3; ++k) g[k] += f * v[k];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) sg[3 * a + b] += 0.5 * f * v[a] * v[b];
      dcn += dedc6 * dc6i;
    }
  }
  e = wsum(e);
  if (grad) {
    dcn = wsum(dcn);
    for (int k = 0; k < 3; ++k) g[k] = wsum(g[k]);
    for (int k = 0; k < 9; ++k) sg[k] = wsum(sg[k]);
  }
  if (lane != 0) return;
  eat[i] += e;
  if (!grad) return;
  d.dEdcn[i] = dcn;
  for (int k = 0; k < 3; ++k) grad_out[3 * i + k] += g[k];
  for (int k = 0; k < 9; ++k) sig_at[9 * i + k] += sg[k];
}

__device__ __forceinline__ void d3_cn_grad_dev(const DevMol& m, const DevD3& d, double* grad,
                                               double* sig_at) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp;
  const double cut2 = d.cn_cutoff * d.cn_cutoff;
  double g[3] = {0, 0, 0}, sg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int j = lane; j < m.nat; j += 32) {
    if (j == i) continue;
    double v[3], r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      v[k] = m.xyz[3 * i + k] - m.xyz[3 * j + k];
      r2 += v[k] * v[k];
    }
    if (r2 > cut2 || r2 < 1e-12) continue;
    const double r = sqrt(r2);
    double c, dc;
    d3_count(r, d.rcov[i] + d.rcov[j], d.k1, c, dc);
    const double f = (d.dEdcn[i] + d.dEdcn[j]) * dc / r;
    for (int k = 0; k < 3; ++k) g[k] += f * v[k];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) sg[3 * a + b] += 0.5 * f * v[a] * v[b];
  }
  for (int k = 0; k < 3; ++k) g[k] = wsum(g[k]);
  for (int k = 0; k < 9; ++k) sg[k] = wsum(sg[k]);
  if (lane == 0) {
    for (int k = 0; k < 3; ++k) grad[3 * i + k] += g[k];
    for (int k = 0; k < 9; ++k) sig_at[9 * i + k] += sg[k];
  }
}

__global__ void k_d3_setup(DevMol m, DevD3 d) { d3_setup_dev(m, d); }
__global__ void k_d3_pair(DevMol m, DevD3 d, int grad, double* eat, double* grad_out,
                          double* sig_at) {
  d3_pair_dev(m, d, grad, eat, grad_out, sig_at);
}
__global__ void k_d3_cn_grad(DevMol m, DevD3 d, double* grad, double* sig_at) {
  d3_cn_grad_dev(m, d, grad, sig_at);
}

void d3_energy_gradient(const DevMol& m, const DevD3& d, bool grad, double* eat, double* grad_out,
                        double* sig_at, cudaStream_t s) {
  ++g_kernel_launches;
  k_d3_setup<<<warps_grid(m.nat), 64, 0, s>>>(m, d);
  ++g_kernel_launches;
  k_d3_pair<<<warps_grid(m.nat), 64, 0, s>>>(m, d, grad ? 1 : 0, eat, grad_out, sig_at);
  if (!grad) return;
  ++g_kernel_launches;
  k_d3_cn_grad<<<warps_grid(m.nat), 64, 0, s>>>(m, d, grad_out, sig_at);
}

// ------------------------------------------------------------------------------------
// batched launches: blockIdx.z walks the listed molecules (molecules without dispersion,
// i.e. single atoms, leave at once); the D4 dEdcn accumulators start zeroed
// ------------------------------------------------------------------------------------
#define BMOL                                  \
  const MolPtrs& q = mp[list[blockIdx.z]];    \
  if (!q.has_d4) return
#define BARGS const MolPtrs* __restrict__ mp, const int* __restrict__ list

__global__ void kb_d4_cn(BARGS) {
  BMOL;
  d4_cn_dev(q.m, q.d4, q.d4w.cn);
}
__global__ void kb_d4_weights(BARGS) {
  BMOL;
  d4_weights_dev(q.m.nat, q.d4, q.d4w.cn, q.d4w.gw, q.d4w.dgw);
}
// mode 0: charge-free (setup), 1: potential, 2: energy, 3: gradient
__global__ void kb_d4_zeta(BARGS, int mode) {
  BMOL;
  const D4Work& w = q.d4w;
  if (mode == 0)
    d4_zeta_dev(q.m.nat, q.d4, nullptr, w.gw, w.dgw, w.gwv, nullptr, w.dgwv_cn);
  else if (mode == 1)
    d4_zeta_dev(q.m.nat, q.d4, q.qat, w.gw, w.dgw, w.gwv, w.dgwdq, nullptr);
  else if (mode == 2)
    d4_zeta_dev(q.m.nat, q.d4, q.qat_o, w.gw, w.dgw, w.gwv, nullptr, nullptr);
  else
    d4_zeta_dev(q.m.nat, q.d4, q.qat_o, w.gw, w.dgw, w.gwv, nullptr, w.dgwv_cn);
}
__global__ void kb_d4_de(BARGS) {
  BMOL;
  d4_de_table_dev(q.m, q.d4, q.d4w.de);
}
__global__ void kb_d4_c6(BARGS) {
  BMOL;
  d4_c6_dev(q.m.nat, q.d4, q.d4w.gwv, q.d4w.dgwv_cn, q.d4w.c6, q.d4w.dc6);
}
__global__ void kb_d4_atm_pairs(BARGS) {
  BMOL;
  d4_atm_pairs_dev(q.m, q.d4, q.d4w.c6, q.d4w.dc6, q.d4w.atm, q.d4w.e3);
}
__global__ void kb_d4_atm(BARGS) {
  BMOL;
  extern __shared__ double atm_rows_b[];
  d4_atm_dev(q.m, q.d4, q.d4w.atm, q.d4w.e3, q.d4w.dEdcn,
             atm_rows_b + (size_t)(threadIdx.x >> 5) * 3 * q.m.nat);
}
__global__ void kb_d4_atm_grad(BARGS) {
  BMOL;
  d4_atm_grad_dev(q.m, q.d4w.atm, q.grad, q.sig_at);
}
__global__ void kb_d4_pair_pot(BARGS) {
  BMOL;
  d4_pair_dev<0>(q.m, q.d4, q.d4w.gwv, q.d4w.dgwdq, nullptr, q.vat, nullptr, nullptr, nullptr,
                 nullptr, q.d4w.de);
}
__global__ void kb_d4_pair_energy(BARGS) {
  BMOL;
  d4_pair_dev<1>(q.m, q.d4, q.d4w.gwv, nullptr, nullptr, nullptr, q.eelec, nullptr, nullptr,
                 nullptr, q.d4w.de);
}
__global__ void kb_d4_pair_grad(BARGS) {
  BMOL;
  d4_pair_dev<2>(q.m, q.d4, q.d4w.gwv, nullptr, q.d4w.dgwv_cn, nullptr, nullptr, q.grad,
                 q.sig_at, q.d4w.dEdcn);
}
__global__ void kb_d4_cn_grad(BARGS) {
  BMOL;
  d4_cn_grad_dev(q.m, q.d4, q.d4w.dEdcn, q.grad, q.sig_at);
}

// D3 (GFN1-xTB): energy into erep, explicit and CN chain-rule gradient, all at setup
#define BMOL3                                 \
  const MolPtrs& q = mp[list[blockIdx.z]];    \
  if (!q.has_d3) return
__global__ void kb_d3_setup(BARGS) {
  BMOL3;
  d3_setup_dev(q.m, q.d3);
}
__global__ void kb_d3_pair(BARGS) {
  BMOL3;
  d3_pair_dev(q.m, q.d3, 1, q.erep, q.grad, q.sig_at);
}
__global__ void kb_d3_cn_grad(BARGS) {
  BMOL3;
  d3_cn_grad_dev(q.m, q.d3, q.grad, q.sig_at);
}
#undef BMOL3

static inline dim3 bwarps(const BatchLaunch& b) { return dim3(warps_grid(b.nat_max), 1, b.count); }
static inline dim3 batoms(const BatchLaunch& b) {
  return dim3((b.nat_max + 127) / 128, 1, b.count);
}

void d4_setup_b(const BatchLaunch& b) {
  if (!b.count) return;
  g_kernel_launches += 7;
  kb_d4_cn<<<bwarps(b), 64, 0, b.s>>>(b.mp, b.list);
  kb_d4_weights<<<batoms(b), 128, 0, b.s>>>(b.mp, b.list);
  kb_d4_zeta<<<batoms(b), 128, 0, b.s>>>(b.mp, b.list, 0);
  const long long nn = (long long)b.nat_max * b.nat_max;
  kb_d4_c6<<<dim3((unsigned)((nn + 255) / 256), 1, b.count), 256, 0, b.s>>>(b.mp, b.list);
  ++g_kernel_launches;
  kb_d4_de<<<dim3((unsigned)((nn + 255) / 256), 1, b.count), 256, 0, b.s>>>(b.mp, b.list);
  kb_d4_atm_pairs<<<dim3((unsigned)((nn + 255) / 256), 1, b.count), 256, 0, b.s>>>(b.mp, b.list);
  kb_d4_atm<<<bwarps(b), 64, (size_t)2 * 3 * b.nat_max * sizeof(double), b.s>>>(b.mp, b.list);
  kb_d4_atm_grad<<<bwarps(b), 64, 0, b.s>>>(b.mp, b.list);
}
void d3_setup_b(const BatchLaunch& b) {
  if (!b.count) return;
  g_kernel_launches += 3;
  kb_d3_setup<<<bwarps(b), 64, 0, b.s>>>(b.mp, b.list);
  kb_d3_pair<<<bwarps(b), 64, 0, b.s>>>(b.mp, b.list);
  kb_d3_cn_grad<<<bwarps(b), 64, 0, b.s>>>(b.mp, b.list);
}
void d4_potential_b(const BatchLaunch& b) {
  if (!b.count) return;
  g_kernel_launches += 2;
  kb_d4_zeta<<<batoms(b), 128, 0, b.s>>>(b.mp, b.list, 1);
  kb_d4_pair_pot<<<bwarps(b), 64, 0, b.s>>>(b.mp, b.list);
}
void d4_energy_b(const BatchLaunch& b) {
  if (!b.count) return;
  g_kernel_launches += 2;
  kb_d4_zeta<<<batoms(b), 128, 0, b.s>>>(b.mp, b.list, 2);
  kb_d4_pair_energy<<<bwarps(b), 64, 0, b.s>>>(b.mp, b.list);
}
void d4_gradient_b(const BatchLaunch& b) {
  if (!b.count) return;
  g_kernel_launches += 3;
  kb_d4_zeta<<<batoms(b), 128, 0, b.s>>>(b.mp, b.list, 3);
  kb_d4_pair_grad<<<bwarps(b), 64, 0, b.s>>>(b.mp, b.list);
  kb_d4_cn_grad<<<bwarps(b), 64, 0, b.s>>>(b.mp, b.list);
}

#undef BMOL
#undef BARGS

}  // namespace tb
