// Shell-pair overlap / dipole / quadrupole integrals, H0 assembly and the H0 gradient.
//
// Restates reference src/tblite/integral/native/integrals.f90:91-1391 (multipole_cgto,
// multipole_grad_cgto), src/tblite/xtb/h0.f90:220-666 (get_hamiltonian,
// get_hamiltonian_gradient) and src/tblite/xtb/gfn2.f90:767-797 (get_hscale).
//
// GPU formulation.  For one primitive pair all 1-d integrals follow from the six Gaussian
// moments  m_p = int (x-A)^p exp(-eta (x-P)^2) dx / sqrt(pi/eta),  p = 0..5, A the ket
// centre.  With (x-B) = (x-A) + (A-B) every overlap, dipole and quadrupole factor, and the
// derivative of the ket function, is a short polynomial in those moments.  Moments about B
// (the operator on the bra atom) follow from the same binomial shift.  For s and p shells
// the cartesian -> spherical transform is a permutation (p -> y, z, x), so a thread can own
// one (shell pair, ket orbital) and keep all accumulators in registers.
#include <cuda_runtime.h>

#include "engine.h"

namespace tb {

__device__ __forceinline__ int sph_of_cart_p(int c) { return c == 0 ? 2 : c - 1; }  // x->2,y->0,z->1
__device__ __forceinline__ int cart_of_sph_p(int m) { return m == 2 ? 0 : m + 1; }

struct Moments {  // per direction: m[0..6]
  double m[3][7];
};

__device__ __forceinline__ void gauss_moments(const double pa[3], double eta, Moments& M) {
  const double s2 = 0.5 / eta;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double a = pa[k], a2 = a * a, a3 = a2 * a;
    M.m[k][0] = 1.0;
    M.m[k][1] = a;
    M.m[k][2] = a2 + s2;
    M.m[k][3] = a3 + 3.0 * a * s2;
    M.m[k][4] = a2 * a2 + 6.0 * a2 * s2 + 3.0 * s2 * s2;
    M.m[k][5] = a3 * a2 + 10.0 * a3 * s2 + 15.0 * a * s2 * s2;
    M.m[k][6] = a3 * a3 + 15.0 * a2 * a2 * s2 + 45.0 * a2 * s2 * s2 + 15.0 * s2 * s2 * s2;
  }
}

// O(p, b) = int (x-A)^p (x-B)^b G_P ;  b in {0,1}
__device__ __forceinline__ double O1(const Moments& M, int k, int p, int b, double vk) {
  return b == 0 ? M.m[k][p] : M.m[k][p + 1] + vk * M.m[k][p];
}

// cartesian exponent of component c (0=x,1=y,2=z) in direction k for an l<=1 function
__device__ __forceinline__ int cexp(int l, int c, int k) { return (l == 1 && c == k) ? 1 : 0; }

// ---------------------------------------------------------------------------------------
// H0 build: one thread per (shell pair ish >= jsh, ket orbital mi)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void tri_index(long long t, int& i, int& j) {
  // t = i*(i+1)/2 + j, 0 <= j <= i
  double d = sqrt(8.0 * (double)t + 1.0);
  i = (int)((d - 1.0) * 0.5);
  while ((long long)i * (i + 1) / 2 > t) --i;
  while ((long long)(i + 1) * (i + 2) / 2 <= t) ++i;
  j = (int)(t - (long long)i * (i + 1) / 2);
}

// GFN1 element-pair factor of the H0 scale (xtb/gfn1.f90:734-785)
__device__ __forceinline__ int dblock_row(int z) {
  return (z > 20 && z < 30) ? 1 : (z > 38 && z < 48) ? 2 : (z > 56 && z < 80) ? 3 : 0;
}
__device__ __forceinline__ double gfn1_pair(int zi, int zj, int mode) {
  const int a = zi < zj ? zi : zj, b = zi < zj ? zj : zi;
  if (mode == 1) {  // mode 0 (IPEA1-xTB): only the d-block rule below
  if (a == 1 && b == 1) return 0.96;
  if (a == 1 && b == 5) return 0.95;
  if (a == 1 && b == 7) return 1.04;
  if (a == 1 && b == 28) return 0.90;
  if (a == 1 && (b == 75 || b == 78)) return 0.80;
  if (a == 5 && b == 15) return 0.97;
  if (a == 7 && b == 14) return 1.01;
  }
  const int ti = dblock_row(zi), tj = dblock_row(zj);
  if (ti > 0 && tj > 0) {
    const double kp[3] = {1.1, 1.2, 1.2};
    return 0.5 * (kp[ti - 1] + kp[tj - 1]);
  }
  return 1.0;
}

__device__ __forceinline__ double hscale_of(const DevMol& m, const Gfn2Scalars& p, int ish,
                                            int jsh, int iat, int jat) {
  if (p.method == 1) {  // GFN1: valence / polarisation shells (xtb/gfn1.f90:797-828)
    const int li = m.sh_l[ish], lj = m.sh_l[jsh];
    const bool vi = m.sh_valence[ish] != 0, vj = m.sh_valence[jsh] != 0;
    if (vi && vj) {
      const double den = (m.at_en[iat] - m.at_en[jat]) * (m.at_en[iat] - m.at_en[jat]);
      return gfn1_pair(m.at_z[iat], m.at_z[jat], p.pair_mode) * p.kshell[lj][li] *
             (1.0 + p.enscale * den);
    }
    if (vi) return 0.5 * (p.kshell[li][li] + p.kdiff);
    if (vj) return 0.5 * (p.kshell[lj][lj] + p.kdiff);
    return p.kdiff;
  }
  const double zi = m.sh_zeta[ish], zj = m.sh_zeta[jsh];
  const double zij = pow(2.0 * sqrt(zi * zj) / (zi + zj), p.wexp);
  const double den = (m.at_en[iat] - m.at_en[jat]) * (m.at_en[iat] - m.at_en[jat]);
  return zij * p.kshell[m.sh_l[jsh]][m.sh_l[ish]] * (1.0 + p.enscale * den);
}

__device__ __forceinline__ void build_h0_dev(DevMol m, Gfn2Scalars p, const double* __restrict__ se, double* S,
                           double* H, double* D, double* Q, long long npair) {
  const long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long t = gid / 3;
  const int mi = (int)(gid % 3);
  if (t >= npair) return;
  int ish, jsh;
  tri_index(t, ish, jsh);
  const int li = m.sh_l[ish], lj = m.sh_l[jsh];
  if (mi > 2 * li) return;
  const int iat = m.sh_atom[ish], jat = m.sh_atom[jsh];
  double vec[3];
  double r2 = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    vec[k] = m.xyz[3 * iat + k] - m.xyz[3 * jat + k];
    r2 += vec[k] * vec[k];
  }
  const bool onsite = iat == jat;
  if (!onsite && (r2 > p.h0_cutoff * p.h0_cutoff || r2 < 2.220446049250313e-16)) return;
  const int ci = li == 1 ? cart_of_sph_p(mi) : 0;
  const int ncj = 2 * lj + 1;
  // accumulators per bra cartesian component: S, M1[3], M2[6] about A
  double aS[3] = {0, 0, 0}, aM1[3][3] = {{0}}, aM2[3][6] = {{0}};
  const int npi = m.sh_nprim[ish], npj = m.sh_nprim[jsh];
  const double pi3 = 5.568327996831708;  // pi^(3/2)
  for (int ip = 0; ip < npi; ++ip) {
    const double ai = m.sh_alpha[ish * MAXG + ip];
    const double ci_ = m.sh_coeff[ish * MAXG + ip];
    for (int jp = 0; jp < npj; ++jp) {
      const double aj = m.sh_alpha[jsh * MAXG + jp];
      const double eta = ai + aj, oeta = 1.0 / eta;
      const double est = ai * aj * r2 * oeta;
      if (est > INTCUT) continue;
      const double cc = ci_ * m.sh_coeff[jsh * MAXG + jp] * exp(-est) * pi3 * oeta * sqrt(oeta);
      double pa[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) pa[k] = -vec[k] * aj * oeta;
      Moments M;
      gauss_moments(pa, eta, M);
      for (int cj = 0; cj < ncj; ++cj) {
        double V[3][3];  // [dir][e] = O(a+e, b)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const int a = cexp(li, ci, k), b = cexp(lj, cj, k);
#pragma unroll
          for (int e = 0; e < 3; ++e) V[k][e] = O1(M, k, a + e, b, vec[k]);
        }
        aS[cj] += cc * V[0][0] * V[1][0] * V[2][0];
        aM1[cj][0] += cc * V[0][1] * V[1][0] * V[2][0];
        aM1[cj][1] += cc * V[0][0] * V[1][1] * V[2][0];
        aM1[cj][2] += cc * V[0][0] * V[1][0] * V[2][1];
        aM2[cj][0] += cc * V[0][2] * V[1][0] * V[2][0];  // xx
        aM2[cj][1] += cc * V[0][1] * V[1][1] * V[2][0];  // xy
        aM2[cj][2] += cc * V[0][0] * V[1][2] * V[2][0];  // yy
        aM2[cj][3] += cc * V[0][1] * V[1][0] * V[2][1];  // xz
        aM2[cj][4] += cc * V[0][0] * V[1][1] * V[2][1];  // yz
        aM2[cj][5] += cc * V[0][0] * V[1][0] * V[2][2];  // zz
      }
    }
  }
  double hij;
  if (!onsite) {
    const double rr = sqrt(sqrt(r2) / (m.at_rad[iat] + m.at_rad[jat]));
    const double poly = (1.0 + m.sh_shpoly[ish] * rr) * (1.0 + m.sh_shpoly[jsh] * rr);
    hij = 0.5 * (se[ish] + se[jsh]) * hscale_of(m, p, ish, jsh, iat, jat) * poly;
  } else {
    hij = 0.5 * (se[ish] + se[jsh]);
  }
  const int n = m.nao;
  const size_t nn = (size_t)n * n;
  const int io = m.sh_ao[ish] + mi, jo0 = m.sh_ao[jsh];
  const bool write_t = ish != jsh;
  for (int cj = 0; cj < ncj; ++cj) {
    const int mj = lj == 1 ? sph_of_cart_p(cj) : 0;
    const int jo = jo0 + mj;
    const double s = aS[cj];
    double dA[3], dB[3], qA[6], qB[6];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      dA[k] = aM1[cj][k];
      dB[k] = aM1[cj][k] + vec[k] * s;  // (r-B) = (r-A) + vec
    }
    const int qa[6] = {0, 0, 1, 0, 1, 2}, qb[6] = {0, 1, 1, 2, 2, 2};
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      qA[q] = aM2[cj][q];
      qB[q] = aM2[cj][q] + vec[qa[q]] * aM1[cj][qb[q]] + vec[qb[q]] * aM1[cj][qa[q]]
              + vec[qa[q]] * vec[qb[q]] * s;
    }
    // traceless
    {
      double tr = 0.5 * (qA[0] + qA[2] + qA[5]);
      qA[0] = 1.5 * qA[0] - tr; qA[1] *= 1.5; qA[2] = 1.5 * qA[2] - tr;
      qA[3] *= 1.5; qA[4] *= 1.5; qA[5] = 1.5 * qA[5] - tr;
      tr = 0.5 * (qB[0] + qB[2] + qB[5]);
      qB[0] = 1.5 * qB[0] - tr; qB[1] *= 1.5; qB[2] = 1.5 * qB[2] - tr;
      qB[3] *= 1.5; qB[4] *= 1.5; qB[5] = 1.5 * qB[5] - tr;
    }
    const size_t ji = (size_t)jo * n + io;  // row j (bra), column i (ket): operator on A
    S[ji] = s;
    H[ji] = s * hij;
#pragma unroll
    for (int k = 0; k < 3; ++k) D[k * nn + ji] = dA[k];
#pragma unroll
    for (int q = 0; q < 6; ++q) Q[q * nn + ji] = qA[q];
    if (write_t) {
      const size_t ij = (size_t)io * n + jo;  // row i, column j: operator on B
      S[ij] = s;
      H[ij] = s * hij;
#pragma unroll
      for (int k = 0; k < 3; ++k) D[k * nn + ij] = dB[k];
#pragma unroll
      for (int q = 0; q < 6; ++q) Q[q * nn + ij] = qB[q];
    }
  }
}
__global__ void k_build_h0(DevMol m, Gfn2Scalars p, const double* __restrict__ se, double* S,
                           double* H, double* D, double* Q, long long npair) {
  build_h0_dev(m, p, se, S, H, D, Q, npair);
}

void launch_build_h0(const DevMol& m, const Gfn2Scalars& p, const double* se, double* S,
                     double* H, double* D, double* Q, cudaStream_t s) {
  const size_t nn = (size_t)m.nao * m.nao;
  cudaMemsetAsync(S, 0, nn * sizeof(double), s);
  cudaMemsetAsync(H, 0, nn * sizeof(double), s);
  cudaMemsetAsync(D, 0, 3 * nn * sizeof(double), s);
  cudaMemsetAsync(Q, 0, 6 * nn * sizeof(double), s);
  const long long npair = (long long)m.nsh * (m.nsh + 1) / 2;
  const long long nthr = npair * 3;
  const int bs = 128;
  ++g_kernel_launches;
  k_build_h0<<<(unsigned)((nthr + bs - 1) / bs), bs, 0, s>>>(m, p, se, S, H, D, Q, npair);
}

// One primitive pair of the H0 gradient for shells of angular momenta LI (bra, A) and LJ
// (ket, B): for every component pair the overlap, the dipole moments about A (PS, PD) and the
// derivative of the multipole-potential integral and of the overlap with respect to A.  The
// 1-d factors O(p, b) come from one table per direction; the derivative of the product along
// c is written as sum_e G_c[e] T_c(e), with T_c(e) the polynomial's coefficients times the
// products of the other two directions' factors (fewer FP64 operations than expanding the ten
// monomials per direction).
template <int LI, int LJ>
__device__ __forceinline__ void h0g_prim(const Moments& M, const double (&vec)[3], double ai,
                                         double cc, const double (&wp)[3][3],
                                         const double (&ws)[3][3], double c0,
                                         const double (&c1)[3], const double (&c2)[6],
                                         double (&dG)[3], double& PS, double (&PD)[3]) {
  double T[3][2][5];  // O(p, b) of direction k, p = 0..4
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int p = 0; p < 5; ++p) {
      T[k][0][p] = M.m[k][p];
      T[k][1][p] = LJ ? M.m[k][p + 1] + vec[k] * M.m[k][p] : 0.0;
    }
  const double a2 = 2.0 * ai;
#pragma unroll
  for (int cj = 0; cj < 2 * LJ + 1; ++cj)
#pragma unroll
    for (int ci = 0; ci < 2 * LI + 1; ++ci) {
      double V[3][3], G[3][3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int a = (LI == 1 && ci == k) ? 1 : 0, b = (LJ == 1 && cj == k) ? 1 : 0;
#pragma unroll
        for (int e = 0; e < 3; ++e) {
          V[k][e] = T[k][b][a + e];
          G[k][e] = a ? a2 * T[k][b][a + 1 + e] - T[k][b][a - 1 + e] : a2 * T[k][b][1 + e];
        }
      }
      const double w_p = wp[cj][ci] * cc, w_s = ws[cj][ci] * cc;
      // products of the two other directions' factors, (e1, e2) = 00, 10, 01, 20, 11, 02
      const double p12[6] = {V[1][0] * V[2][0], V[1][1] * V[2][0], V[1][0] * V[2][1],
                             V[1][2] * V[2][0], V[1][1] * V[2][1], V[1][0] * V[2][2]};
      const double p02[6] = {V[0][0] * V[2][0], V[0][1] * V[2][0], V[0][0] * V[2][1],
                             V[0][2] * V[2][0], V[0][1] * V[2][1], V[0][0] * V[2][2]};
      const double p01[6] = {V[0][0] * V[1][0], V[0][1] * V[1][0], V[0][0] * V[1][1],
                             V[0][2] * V[1][0], V[0][1] * V[1][1], V[0][0] * V[1][2]};
      PS += w_p * (V[0][0] * p12[0]);
      PD[0] += w_p * (V[0][1] * p12[0]);
      PD[1] += w_p * (V[0][0] * p12[1]);
      PD[2] += w_p * (V[0][0] * p12[2]);
      // monomial coefficients: 1 c0; x, y, z c1[0..2]; xx, xy, yy, xz, yz, zz c2[0..5]
      {  // derivative along x: the other directions are y (first) and z (second)
        const double t0 = c0 * p12[0] + c1[1] * p12[1] + c1[2] * p12[2] + c2[2] * p12[3] +
                          c2[4] * p12[4] + c2[5] * p12[5];
        const double t1 = c1[0] * p12[0] + c2[1] * p12[1] + c2[3] * p12[2];
        const double t2 = c2[0] * p12[0];
        dG[0] += w_s * (G[0][0] * p12[0]) - w_p * (G[0][0] * t0 + G[0][1] * t1 + G[0][2] * t2);
      }
      {  // along y: the others are x and z
        const double t0 = c0 * p02[0] + c1[0] * p02[1] + c1[2] * p02[2] + c2[0] * p02[3] +
                          c2[3] * p02[4] + c2[5] * p02[5];
        const double t1 = c1[1] * p02[0] + c2[1] * p02[1] + c2[4] * p02[2];
        const double t2 = c2[2] * p02[0];
        dG[1] += w_s * (G[1][0] * p02[0]) - w_p * (G[1][0] * t0 + G[1][1] * t1 + G[1][2] * t2);
      }
      {  // along z: the others are x and y
        const double t0 = c0 * p01[0] + c1[0] * p01[1] + c1[1] * p01[2] + c2[0] * p01[3] +
                          c2[1] * p01[4] + c2[2] * p01[5];
        const double t1 = c1[2] * p01[0] + c2[3] * p01[1] + c2[4] * p01[2];
        const double t2 = c2[5] * p01[0];
        dG[2] += w_s * (G[2][0] * p01[0]) - w_p * (G[2][0] * t0 + G[2][1] * t1 + G[2][2] * t2);
      }
    }
}

// ---------------------------------------------------------------------------------------
// H0 gradient: one thread per cross-atom shell pair (ish > jsh).  The reference formula
// (h0.f90:528-560) is contracted on the fly:
//   dG = sum_ji [ sval dS + 2 P hij S dsv - P d<j|O|i>/dR_A ] ,
//   sval = -P (v_j + v_i) + 2 P hij - 2 W,
// where O is the multipole potential operator of atoms A and B written as a polynomial in
// (r - A).  The operator on A moves with A, which adds  P (vA_c S + sum_b (1+d_cb) wA_cb D_b).
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void h0_gradient_dev(DevMol m, Gfn2Scalars p, const double* __restrict__ se,
                              const double* __restrict__ P, const double* __restrict__ W,
                              const double* __restrict__ vao, const double* __restrict__ vdp,
                              const double* __restrict__ vqp, double* grad, double* sigma,
                              double* dEdcn, long long npair) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  // every thread reaches the warp-wide virial sum at the end: pairs that contribute nothing
  // (outside the list, on one atom, beyond the cutoff) skip the work, not the sum
  double vec[3] = {0.0, 0.0, 0.0}, dG[3] = {0.0, 0.0, 0.0};
  do {
  if (t >= npair) break;
  int ish, jsh;
  tri_index(t, ish, jsh);
  const int iat = m.sh_atom[ish], jat = m.sh_atom[jsh];
  if (iat == jat) break;
  double r2 = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    vec[k] = m.xyz[3 * iat + k] - m.xyz[3 * jat + k];
    r2 += vec[k] * vec[k];
  }
  if (r2 > p.h0_cutoff * p.h0_cutoff || r2 < 2.220446049250313e-16) {
    vec[0] = vec[1] = vec[2] = 0.0;
    break;
  }
  const int li = m.sh_l[ish], lj = m.sh_l[jsh];
  const int nci = 2 * li + 1, ncj = 2 * lj + 1;
  const double rr = sqrt(sqrt(r2) / (m.at_rad[iat] + m.at_rad[jat]));
  const double polyi = 1.0 + m.sh_shpoly[ish] * rr, polyj = 1.0 + m.sh_shpoly[jsh] * rr;
  const double poly = polyi * polyj;
  const double dpoly = (polyi * m.sh_shpoly[jsh] + polyj * m.sh_shpoly[ish]) * 0.5 * rr / r2;
  const double hs = hscale_of(m, p, ish, jsh, iat, jat) * poly;
  const double hij = 0.5 * (se[ish] + se[jsh]) * hs;
  // potential operator coefficients in (r-A) monomials
  double vA[3], vB[3], wA[6], wB[6];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    vA[k] = vdp[3 * iat + k];
    vB[k] = vdp[3 * jat + k];
  }
  {
    const double* qa_ = vqp + 6 * iat;
    const double* qb_ = vqp + 6 * jat;
    const double tra = qa_[0] + qa_[2] + qa_[5], trb = qb_[0] + qb_[2] + qb_[5];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const bool diag = q == 0 || q == 2 || q == 5;
      wA[q] = 1.5 * qa_[q] - (diag ? 0.5 * tra : 0.0);
      wB[q] = 1.5 * qb_[q] - (diag ? 0.5 * trb : 0.0);
    }
  }
  const int qa[6] = {0, 0, 1, 0, 1, 2}, qb[6] = {0, 1, 1, 2, 2, 2};
  double c0 = 0.0, c1[3], c2[6];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    c1[k] = vA[k] + vB[k];
    c0 += vB[k] * vec[k];
  }
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    c2[q] = wA[q] + wB[q];
    c1[qa[q]] += wB[q] * vec[qb[q]];
    c1[qb[q]] += wB[q] * vec[qa[q]];
    c0 += wB[q] * vec[qa[q]] * vec[qb[q]];
  }
  // contraction weights in the cartesian basis (l<=1: permutation of spherical)
  const int n = m.nao;
  const int io0 = m.sh_ao[ish], jo0 = m.sh_ao[jsh];
  double ws[3][3], wp[3][3];
  for (int cj = 0; cj < ncj; ++cj) {
    const int ja = jo0 + (lj == 1 ? sph_of_cart_p(cj) : 0);
    for (int ci = 0; ci < nci; ++ci) {
      const int ia = io0 + (li == 1 ? sph_of_cart_p(ci) : 0);
      const double pij = P[(size_t)ja * n + ia];
      const double wij = W[(size_t)ja * n + ia];
      wp[cj][ci] = pij;
      ws[cj][ci] = -pij * (vao[ja] + vao[ia]) + 2.0 * pij * hij - 2.0 * wij;
    }
  }
  double PS = 0.0, PD[3] = {0, 0, 0};
  const int npi = m.sh_nprim[ish], npj = m.sh_nprim[jsh];
  const double pi3 = 5.568327996831708;
  for (int ip = 0; ip < npi; ++ip) {
    const double ai = m.sh_alpha[ish * MAXG + ip];
    const double ci_ = m.sh_coeff[ish * MAXG + ip];
    for (int jp = 0; jp < npj; ++jp) {
      const double aj = m.sh_alpha[jsh * MAXG + jp];
      const double eta = ai + aj, oeta = 1.0 / eta;
      const double est = ai * aj * r2 * oeta;
      if (est > INTCUT) continue;
      const double cc = ci_ * m.sh_coeff[jsh * MAXG + jp] * exp(-est) * pi3 * oeta * sqrt(oeta);
      double pa[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) pa[k] = -vec[k] * aj * oeta;
      Moments M;
      gauss_moments(pa, eta, M);
      switch (2 * li + lj) {  // shell kinds as template arguments: the 1-d factors of all
        case 0:               // angular components are shared by the compiler
          h0g_prim<0, 0>(M, vec, ai, cc, wp, ws, c0, c1, c2, dG, PS, PD);
          break;
        case 1:
          h0g_prim<0, 1>(M, vec, ai, cc, wp, ws, c0, c1, c2, dG, PS, PD);
          break;
        case 2:
          h0g_prim<1, 0>(M, vec, ai, cc, wp, ws, c0, c1, c2, dG, PS, PD);
          break;
        default:
          h0g_prim<1, 1>(M, vec, ai, cc, wp, ws, c0, c1, c2, dG, PS, PD);
          break;
      }
    }
  }
  // operator on A moves with A;  symmetric quadrupole weight matrix of atom A
  const double wAm[3][3] = {{wA[0], wA[1], wA[3]}, {wA[1], wA[2], wA[4]}, {wA[3], wA[4], wA[5]}};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double mv = vA[c] * PS;
#pragma unroll
    for (int b = 0; b < 3; ++b) mv += (b == c ? 2.0 : 1.0) * wAm[c][b] * PD[b];
    dG[c] += mv + 2.0 * hij * PS * dpoly / poly * vec[c];
  }
  const double dcni = m.sh_kcn[ish] * (-1.0) * hs * PS;
  const double dcnj = m.sh_kcn[jsh] * (-1.0) * hs * PS;
  atomicAdd(dEdcn + iat, dcni);
  atomicAdd(dEdcn + jat, dcnj);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    atomicAdd(grad + 3 * iat + c, dG[c]);
    atomicAdd(grad + 3 * jat + c, -dG[c]);
  }
  } while (false);
  // virial: the six distinct elements of the symmetric 3 x 3 summed over the warp, then one
  // atomic per element and warp (every pair of a molecule adds to the same nine numbers)
  const int va[6] = {0, 0, 1, 0, 1, 2}, vb[6] = {0, 1, 1, 2, 2, 2};
#pragma unroll
  for (int e = 0; e < 6; ++e) {
    double v = 0.5 * (vec[va[e]] * dG[vb[e]] + dG[va[e]] * vec[vb[e]]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v != 0.0) {
      atomicAdd(sigma + 3 * va[e] + vb[e], v);
      if (va[e] != vb[e]) atomicAdd(sigma + 3 * vb[e] + va[e], v);
    }
  }
}
__global__ void k_h0_gradient(DevMol m, Gfn2Scalars p, const double* __restrict__ se,
                              const double* __restrict__ P, const double* __restrict__ W,
                              const double* __restrict__ vao, const double* __restrict__ vdp,
                              const double* __restrict__ vqp, double* grad, double* sigma,
                              double* dEdcn, long long npair) {
  h0_gradient_dev(m, p, se, P, W, vao, vdp, vqp, grad, sigma, dEdcn, npair);
}

// on-site CN derivative of the diagonal levels: dEdcn_A += sum_{mu in A} dse/dcn P_mumu
__device__ __forceinline__ void h0_onsite_dcn_dev(DevMol m, const double* __restrict__ P, double* dEdcn) {
  const int iat = blockIdx.x * blockDim.x + threadIdx.x;
  if (iat >= m.nat) return;
  double acc = 0.0;
  for (int ish = m.at_sh[iat]; ish < m.at_sh[iat + 1]; ++ish) {
    const int io = m.sh_ao[ish];
    for (int mi = 0; mi < 2 * m.sh_l[ish] + 1; ++mi)
      acc += -m.sh_kcn[ish] * P[(size_t)(io + mi) * m.nao + io + mi];
  }
  dEdcn[iat] += acc;
}
__global__ void k_h0_onsite_dcn(DevMol m, const double* __restrict__ P, double* dEdcn) {
  h0_onsite_dcn_dev(m, P, dEdcn);
}

void launch_h0_gradient(const DevMol& m, const Gfn2Scalars& p, const double* se, const double* P,
                        const double* W, const double* vao, const double* vdp, const double* vqp,
                        double* grad, double* sigma, double* dEdcn, cudaStream_t s) {
  const long long npair = (long long)m.nsh * (m.nsh + 1) / 2;
  const int bs = 128;
  ++g_kernel_launches;
  k_h0_gradient<<<(unsigned)((npair + bs - 1) / bs), bs, 0, s>>>(m, p, se, P, W, vao, vdp, vqp,
                                                                   grad, sigma, dEdcn, npair);
  ++g_kernel_launches;
  k_h0_onsite_dcn<<<(m.nat + 127) / 128, 128, 0, s>>>(m, P, dEdcn);
}

// ---------------------------------------------------------------------------------------
// dE/dzeta of the Slater exponents (GFN2-xTB), one thread per ordered shell pair (i, j): the
// derivative acts on the i function only; pair (j, i) carries the one of zeta_j.  A primitive
// of exponent alpha = alpha0 zeta^2 with its normalisation (2 alpha/pi)^(3/4) (4 alpha)^(l/2)
// gives  d phi / d zeta = (2 / zeta) sum_k c_k [(3/4 + l/2) - alpha_k |r - A|^2] g_k ,  so the
// derivative integrals are the pair's ordinary ones with (r - A)^2 inserted.  The SCF energy is
// stationary, so (as for the nuclear gradient, h0.f90:528-560)
//   dE/dzeta_i = sum_{mu in i, nu in j} [ (2 P h_ij - P (v_mu + v_nu) - 2 W) dS/dzeta_i
//                                         + 2 P S dh_ij/dzeta_i - P dO/dzeta_i ],
// O the multipole potential operator of both atoms, h_ij = (e_i + e_j)/2 hscale poly with
// d ln hscale / d zeta_i = wexp (1/(2 zeta_i) - 1/(zeta_i + zeta_j)) off-site.  The same form
// holds for on-site pairs (no H0 scaling there) and for i == j (bra and ket derivatives equal).
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void zeta_grad_dev(const DevMol& m, const Gfn2Scalars& p,
                                              const double* __restrict__ se,
                                              const double* __restrict__ P,
                                              const double* __restrict__ W,
                                              const double* __restrict__ vao,
                                              const double* __restrict__ vdp,
                                              const double* __restrict__ vqp, double* dz,
                                              long long t) {
  if (t >= (long long)m.nsh * m.nsh) return;
  const int ish = (int)(t / m.nsh), jsh = (int)(t % m.nsh);
  const int iat = m.sh_atom[ish], jat = m.sh_atom[jsh];
  double vec[3];
  double r2 = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    vec[k] = m.xyz[3 * iat + k] - m.xyz[3 * jat + k];
    r2 += vec[k] * vec[k];
  }
  const bool onsite = iat == jat;
  if (!onsite && (r2 > p.h0_cutoff * p.h0_cutoff || r2 < 2.220446049250313e-16)) return;
  const int li = m.sh_l[ish], lj = m.sh_l[jsh];
  const int nci = 2 * li + 1, ncj = 2 * lj + 1;
  double hij, dhij = 0.0;
  if (onsite) {
    hij = 0.5 * (se[ish] + se[jsh]);
  } else {
    const double rr = sqrt(sqrt(r2) / (m.at_rad[iat] + m.at_rad[jat]));
    const double poly = (1.0 + m.sh_shpoly[ish] * rr) * (1.0 + m.sh_shpoly[jsh] * rr);
    const double hs = hscale_of(m, p, ish, jsh, iat, jat);
    const double zi = m.sh_zeta[ish], zj = m.sh_zeta[jsh];
    hij = 0.5 * (se[ish] + se[jsh]) * hs * poly;
    dhij = hij * p.wexp * (0.5 / zi - 1.0 / (zi + zj));
  }
  // potential operator of both atoms in (r - A) monomials (as in the nuclear gradient)
  double c0 = 0.0, c1[3], c2[6];
  {
    double wA[6], wB[6];
    const double* qa_ = vqp + 6 * iat;
    const double* qb_ = vqp + 6 * jat;
    const double tra = qa_[0] + qa_[2] + qa_[5], trb = qb_[0] + qb_[2] + qb_[5];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const bool diag = q == 0 || q == 2 || q == 5;
      wA[q] = 1.5 * qa_[q] - (diag ? 0.5 * tra : 0.0);
      wB[q] = 1.5 * qb_[q] - (diag ? 0.5 * trb : 0.0);
    }
    const int qa[6] = {0, 0, 1, 0, 1, 2}, qb[6] = {0, 1, 1, 2, 2, 2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      c1[k] = vdp[3 * iat + k] + vdp[3 * jat + k];
      c0 += vdp[3 * jat + k] * vec[k];
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      c2[q] = wA[q] + wB[q];
      c1[qa[q]] += wB[q] * vec[qb[q]];
      c1[qb[q]] += wB[q] * vec[qa[q]];
      c0 += wB[q] * vec[qa[q]] * vec[qb[q]];
    }
  }
  const int n = m.nao;
  const int io0 = m.sh_ao[ish], jo0 = m.sh_ao[jsh];
  double ws[3][3], wp[3][3];
  for (int cj = 0; cj < ncj; ++cj) {
    const int ja = jo0 + (lj == 1 ? sph_of_cart_p(cj) : 0);
    for (int ci = 0; ci < nci; ++ci) {
      const int ia = io0 + (li == 1 ? sph_of_cart_p(ci) : 0);
      const double pij = P[(size_t)ja * n + ia];
      wp[cj][ci] = pij;
      ws[cj][ci] = -pij * (vao[ja] + vao[ia]) + 2.0 * pij * hij - 2.0 * W[(size_t)ja * n + ia];
    }
  }
  const double gl = 0.75 + 0.5 * li;
  double accd = 0.0, accs = 0.0;
  const int npi = m.sh_nprim[ish], npj = m.sh_nprim[jsh];
  const double pi3 = 5.568327996831708;
  for (int ip = 0; ip < npi; ++ip) {
    const double ai = m.sh_alpha[ish * MAXG + ip];
    const double ci_ = m.sh_coeff[ish * MAXG + ip];
    for (int jp = 0; jp < npj; ++jp) {
      const double aj = m.sh_alpha[jsh * MAXG + jp];
      const double eta = ai + aj, oeta = 1.0 / eta;
      const double est = ai * aj * r2 * oeta;
      if (est > INTCUT) continue;
      const double cc = ci_ * m.sh_coeff[jsh * MAXG + jp] * exp(-est) * pi3 * oeta * sqrt(oeta);
      double pa[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) pa[k] = -vec[k] * aj * oeta;
      Moments M;
      gauss_moments(pa, eta, M);
      for (int cj = 0; cj < ncj; ++cj) {
        for (int ci = 0; ci < nci; ++ci) {
          double V[3][5];  // (x-A)^(a+e) (x-B)^b, e = 0..4
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const int a = cexp(li, ci, k), b = cexp(lj, cj, k);
#pragma unroll
            for (int e = 0; e < 5; ++e) V[k][e] = O1(M, k, a + e, b, vec[k]);
          }
          auto f = [&](int ex, int ey, int ez) { return V[0][ex] * V[1][ey] * V[2][ez]; };
          // operator polynomial with the monomial (dx, dy, dz) multiplied in
          auto op = [&](int dx, int dy, int dz) {
            return c0 * f(dx, dy, dz) + c1[0] * f(dx + 1, dy, dz) + c1[1] * f(dx, dy + 1, dz) +
                   c1[2] * f(dx, dy, dz + 1) + c2[0] * f(dx + 2, dy, dz) +
                   c2[1] * f(dx + 1, dy + 1, dz) + c2[2] * f(dx, dy + 2, dz) +
                   c2[3] * f(dx + 1, dy, dz + 1) + c2[4] * f(dx, dy + 1, dz + 1) +
                   c2[5] * f(dx, dy, dz + 2);
          };
          const double s0 = f(0, 0, 0);
          const double sd = gl * s0 - ai * (f(2, 0, 0) + f(0, 2, 0) + f(0, 0, 2));
          const double od = gl * op(0, 0, 0) - ai * (op(2, 0, 0) + op(0, 2, 0) + op(0, 0, 2));
          accd += cc * (ws[cj][ci] * sd - wp[cj][ci] * od);
          accs += cc * wp[cj][ci] * s0;
        }
      }
    }
  }
  const double val = 2.0 / m.sh_zeta[ish] * accd + 2.0 * dhij * accs;
  atomicAdd(dz + ish, val);
}
__global__ void k_zeta_grad(DevMol m, Gfn2Scalars p, const double* __restrict__ se,
                            const double* __restrict__ P, const double* __restrict__ W,
                            const double* __restrict__ vao, const double* __restrict__ vdp,
                            const double* __restrict__ vqp, double* dz) {
  zeta_grad_dev(m, p, se, P, W, vao, vdp, vqp, dz,
                blockIdx.x * (long long)blockDim.x + threadIdx.x);
}

void launch_zeta_grad(const DevMol& m, const Gfn2Scalars& p, const double* se, const double* P,
                      const double* W, const double* vao, const double* vdp, const double* vqp,
                      double* dz, cudaStream_t s) {
  cudaMemsetAsync(dz, 0, sizeof(double) * m.nsh, s);
  const long long np = (long long)m.nsh * m.nsh;
  ++g_kernel_launches;
  k_zeta_grad<<<(unsigned)((np + 127) / 128), 128, 0, s>>>(m, p, se, P, W, vao, vdp, vqp, dz);
}

// batched launches (blockIdx.z walks the listed molecules; S, H, D, Q start zeroed)
__global__ void kb_build_h0(const MolPtrs* __restrict__ mp, const int* __restrict__ list,
                            Gfn2Scalars p) {
  const MolPtrs& q = mp[list[blockIdx.z]];
  const long long npair = (long long)q.m.nsh * (q.m.nsh + 1) / 2;
  p.h0_cutoff = q.h0_cutoff;
  build_h0_dev(q.m, p, q.se, q.S, q.H, q.D, q.Q, npair);
}
void launch_build_h0_b(const BatchLaunch& b, const Gfn2Scalars& p) {
  if (!b.count) return;
  const long long nthr = (long long)b.nsh_max * (b.nsh_max + 1) / 2 * 3;
  ++g_kernel_launches;
  kb_build_h0<<<dim3((unsigned)((nthr + 127) / 128), 1, b.count), 128, 0, b.s>>>(b.mp, b.list, p);
}

// the energy-weighted density W sits in F once the SCF is done
__global__ void kb_h0_gradient(const MolPtrs* __restrict__ mp, const int* __restrict__ list,
                               Gfn2Scalars p) {
  const MolPtrs& q = mp[list[blockIdx.z]];
  const long long npair = (long long)q.m.nsh * (q.m.nsh + 1) / 2;
  p.h0_cutoff = q.h0_cutoff;
  h0_gradient_dev(q.m, p, q.se, q.P, q.F, q.vao, q.vdp, q.vqp, q.grad, q.sigma, q.dEdcn, npair);
}
__global__ void kb_h0_onsite_dcn(const MolPtrs* __restrict__ mp, const int* __restrict__ list) {
  const MolPtrs& q = mp[list[blockIdx.z]];
  h0_onsite_dcn_dev(q.m, q.P, q.dEdcn);
}
// W is in F after the gradient phase; zgrad was zeroed by kb_param_grad
__global__ void kb_zeta_grad(const MolPtrs* __restrict__ mp, const int* __restrict__ list,
                             Gfn2Scalars p) {
  const MolPtrs& q = mp[list[blockIdx.z]];
  if (!q.param_grad) return;
  p.h0_cutoff = q.h0_cutoff;
  zeta_grad_dev(q.m, p, q.se, q.P, q.F, q.vao, q.vdp, q.vqp, q.zgrad,
                blockIdx.x * (long long)blockDim.x + threadIdx.x);
}
void launch_zeta_grad_b(const BatchLaunch& b, const Gfn2Scalars& p) {
  if (!b.count) return;
  const long long np = (long long)b.nsh_max * b.nsh_max;
  ++g_kernel_launches;
  kb_zeta_grad<<<dim3((unsigned)((np + 127) / 128), 1, b.count), 128, 0, b.s>>>(b.mp, b.list, p);
}

void launch_h0_gradient_b(const BatchLaunch& b, const Gfn2Scalars& p) {
  if (!b.count) return;
  const long long npair = (long long)b.nsh_max * (b.nsh_max + 1) / 2;
  ++g_kernel_launches;
  kb_h0_gradient<<<dim3((unsigned)((npair + 127) / 128), 1, b.count), 128, 0, b.s>>>(b.mp, b.list,
                                                                                     p);
  ++g_kernel_launches;
  kb_h0_onsite_dcn<<<dim3((b.nat_max + 127) / 128, 1, b.count), 128, 0, b.s>>>(b.mp, b.list);
}

}  // namespace tb
