// SCF kernels: coordination number, self energies, electrostatics (isotropic, third order,
// anisotropic multipoles), repulsion, Fock assembly, Mulliken analysis, Fermi filling,
// Broyden mixing, and the pair gradients.
//
// Restated from the reference:
//   self energies            src/tblite/xtb/h0.f90:113-217
//   AES radii                src/tblite/coulomb/multipole.f90:389-420
//   isotropic Coulomb        src/tblite/coulomb/charge/effective.f90:238-286, 487-556
//   third order              src/tblite/coulomb/thirdorder.f90:109-172
//   AES matrices/potential   src/tblite/coulomb/multipole.f90:197-350, 488-535, 746-852
//   repulsion                src/tblite/repulsion/effective.f90:187-247
//   Fock assembly            src/tblite/scf/potential.f90:122-255
//   Mulliken                 src/tblite/wavefunction/mulliken.f90:37-100
//   Fermi filling            src/tblite/wavefunction/fermi.f90:31-106, scf/iterator.f90:347-353
//   Broyden                  src/tblite/scf/mixer/broyden.f90:148-278
// Interaction matrices (gamma, AES) are evaluated on the fly inside the potential kernels
// instead of being stored: one warp per atom walks all partners.
#include <cuda_runtime.h>

#include "engine.h"

namespace tb {

std::atomic<unsigned long long> g_kernel_launches{0};
std::atomic<unsigned long long> g_split_flops{0};

void stream_wait(cudaStream_t s) {
  thread_local cudaEvent_t ev = nullptr;
  if (!ev) cudaEventCreateWithFlags(&ev, cudaEventBlockingSync | cudaEventDisableTiming);
  cudaEventRecord(ev, s);
  cudaEventSynchronize(ev);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// x^e for the small integer exponents of the damping functions, pow() otherwise
__device__ __forceinline__ double powe(double x, double e) {
  if (e == 2.0) return x * x;
  if (e == 3.0) return x * x * x;
  if (e == 4.0) { const double x2 = x * x; return x2 * x2; }
  return pow(x, e);
}

// average hardness of a shell pair: arithmetic (GFN2) or harmonic (GFN1) mean
__device__ __forceinline__ double eta_avg(double a, double b, int harmonic) {
  return harmonic ? 2.0 / (1.0 / a + 1.0 / b) : 0.5 * (a + b);
}

// isotropic kernel 1/(r^g + eta^-g)^(1/g); g = 2 is the GFN2 case
__device__ __forceinline__ double gam_kernel(double r1, double eta, double g) {
  if (g == 2.0) return rsqrt(r1 * r1 + 1.0 / (eta * eta));
  return 1.0 / pow(pow(r1, g) + pow(eta, -g), 1.0 / g);
}

// ------------------------------------------------------------------------------------
// coordination number (double exponential counting function, see oracle for the form)
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void dexp_count(double r, double r0, const Gfn2Scalars& p, double& c,
                                           double& dc) {
  if (p.method == 1) {  // GFN1: single exponential 1/(1 + exp(-k (r0/r - 1)))
    const double e = exp(-p.cn_exp_k * (r0 / r - 1.0));
    c = 1.0 / (1.0 + e);
    dc = -c * c * e * p.cn_exp_k * r0 / (r * r);
    return;
  }
  const double e1 = exp(-p.cn_ka * (r0 / r - 1.0));
  const double e2 = exp(-p.cn_kb * ((r0 + p.cn_rshift) / r - 1.0));
  const double f1 = 1.0 / (1.0 + e1), f2 = 1.0 / (1.0 + e2);
  c = f1 * f2;
  const double d1 = -f1 * f1 * e1 * p.cn_ka * r0 / (r * r);
  const double d2 = -f2 * f2 * e2 * p.cn_kb * (r0 + p.cn_rshift) / (r * r);
  dc = d1 * f2 + f1 * d2;
}

__device__ __forceinline__ void cn_dev(DevMol m, Gfn2Scalars p, double* cn) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp;
  const double xi = m.xyz[3 * i], yi = m.xyz[3 * i + 1], zi = m.xyz[3 * i + 2];
  const double cut2 = p.cn_cutoff * p.cn_cutoff;
  double acc = 0.0;
  for (int j = lane; j < m.nat; j += 32) {
    if (j == i) continue;
    const double dx = xi - m.xyz[3 * j], dy = yi - m.xyz[3 * j + 1], dz = zi - m.xyz[3 * j + 2];
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 > cut2 || r2 < 1e-12) continue;
    double c, dc;
    dexp_count(sqrt(r2), m.at_rcov[i] + m.at_rcov[j], p, c, dc);
    acc += c;
  }
  acc = warp_sum(acc);
  if (lane == 0) cn[i] = acc;
}
__global__ void k_cn(DevMol m, Gfn2Scalars p, double* cn) {
  cn_dev(m, p, cn);
}

void launch_cn(const DevMol& m, const Gfn2Scalars& p, double* cn, cudaStream_t s) {
  if (m.nat == 1) {
    cudaMemsetAsync(cn, 0, sizeof(double), s);
    return;
  }
  ++g_kernel_launches;
  k_cn<<<(m.nat * 32 + 63) / 64, 64, 0, s>>>(m, p, cn);
}

// grad_i += sum_j (dEdcn_i + dEdcn_j) dcount/dr (R_i - R_j)/r ; per-atom sigma partials
__device__ __forceinline__ void cn_grad_dev(DevMol m, Gfn2Scalars p, const double* __restrict__ dEdcn, double* grad,
                          double* sig_at) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp;
  const double cut2 = p.cn_cutoff * p.cn_cutoff;
  double g[3] = {0, 0, 0}, sg[9] = {0};
  for (int j = lane; j < m.nat; j += 32) {
    if (j == i) continue;
    double v[3], r2 = 0;
    for (int k = 0; k < 3; ++k) {
      v[k] = m.xyz[3 * i + k] - m.xyz[3 * j + k];
      r2 += v[k] * v[k];
    }
    if (r2 > cut2 || r2 < 1e-12) continue;
    const double r = sqrt(r2);
    double c, dc;
    dexp_count(r, m.at_rcov[i] + m.at_rcov[j], p, c, dc);
    const double f = (dEdcn[i] + dEdcn[j]) * dc / r;
    for (int k = 0; k < 3; ++k) g[k] += f * v[k];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) sg[3 * a + b] += 0.5 * f * v[a] * v[b];
  }
  for (int k = 0; k < 3; ++k) {
    g[k] = warp_sum(g[k]);
  }
  for (int k = 0; k < 9; ++k) sg[k] = warp_sum(sg[k]);
  if (lane == 0) {
    for (int k = 0; k < 3; ++k) grad[3 * i + k] += g[k];
    for (int k = 0; k < 9; ++k) sig_at[9 * i + k] += sg[k];
  }
}
__global__ void k_cn_grad(DevMol m, Gfn2Scalars p, const double* __restrict__ dEdcn, double* grad,
                          double* sig_at) {
  cn_grad_dev(m, p, dEdcn, grad, sig_at);
}

void launch_cn_grad(const DevMol& m, const Gfn2Scalars& p, const double* dEdcn, double* grad,
                    double* sig_at, cudaStream_t s) {
  if (m.nat == 1) return;
  ++g_kernel_launches;
  k_cn_grad<<<(m.nat * 32 + 63) / 64, 64, 0, s>>>(m, p, dEdcn, grad, sig_at);
}

// ------------------------------------------------------------------------------------
// self energies and AES damping radii
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void levels_dev(DevMol m, Gfn2Scalars p, const double* __restrict__ cn, double* se,
                         double* mrad, double* dmrdcn) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < m.nsh) se[t] = m.sh_se0[t] - m.sh_kcn[t] * cn[m.sh_atom[t]];
  if (t < m.nat) {
    const double arg = cn[t] - m.at_vcn[t] - p.mp_shift;
    const double t1 = exp(-p.mp_kexp * arg);
    const double t2 = (p.mp_rmax - m.at_mprad[t]) / (1.0 + t1);
    mrad[t] = m.at_mprad[t] + t2;
    dmrdcn[t] = -t2 * p.mp_kexp * t1 / (1.0 + t1);
  }
}
__global__ void k_levels(DevMol m, Gfn2Scalars p, const double* __restrict__ cn, double* se,
                         double* mrad, double* dmrdcn) {
  levels_dev(m, p, cn, se, mrad, dmrdcn);
}

void launch_setup_levels(const DevMol& m, const Gfn2Scalars& p, const double* cn, double* se,
                         double* mrad, double* dmrdcn, cudaStream_t s) {
  const int nt = m.nsh > m.nat ? m.nsh : m.nat;
  ++g_kernel_launches;
  k_levels<<<(nt + 127) / 128, 128, 0, s>>>(m, p, cn, se, mrad, dmrdcn);
}

// ------------------------------------------------------------------------------------
// homogeneous external electric field (external/field.f90:64-90): atomic and dipole
// potentials of the constant field, and its energy with the output moments
// ------------------------------------------------------------------------------------
struct Field3 {
  double e[3];
};
__global__ void k_field_potential(int nat, const double* __restrict__ xyz, Field3 f, double* vat,
                                  double* vdp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  vat[i] -= f.e[0] * xyz[3 * i] + f.e[1] * xyz[3 * i + 1] + f.e[2] * xyz[3 * i + 2];
  for (int k = 0; k < 3; ++k) vdp[3 * i + k] -= f.e[k];
}
__global__ void k_field_energy(int nat, const double* __restrict__ xyz, Field3 f,
                               const double* __restrict__ qat, const double* __restrict__ dpat,
                               double* eat) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  const double v = f.e[0] * xyz[3 * i] + f.e[1] * xyz[3 * i + 1] + f.e[2] * xyz[3 * i + 2];
  eat[i] -= v * qat[i] + f.e[0] * dpat[3 * i] + f.e[1] * dpat[3 * i + 1] + f.e[2] * dpat[3 * i + 2];
}
void launch_field_potential(int nat, const double* xyz, const double* efield, double* vat,
                            double* vdp, cudaStream_t s) {
  const Field3 f{{efield[0], efield[1], efield[2]}};
  ++g_kernel_launches;
  k_field_potential<<<(nat + 127) / 128, 128, 0, s>>>(nat, xyz, f, vat, vdp);
}
void launch_field_energy(int nat, const double* xyz, const double* efield, const double* qat,
                         const double* dpat, double* eat, cudaStream_t s) {
  const Field3 f{{efield[0], efield[1], efield[2]}};
  ++g_kernel_launches;
  k_field_energy<<<(nat + 127) / 128, 128, 0, s>>>(nat, xyz, f, qat, dpat, eat);
}

// ------------------------------------------------------------------------------------
// electrostatics: one warp per atom i, partners j strided over lanes
// MODE 0: potentials (vsh, vat, vdp, vqp);  MODE 1: per-atom energy (added to eat)
// ------------------------------------------------------------------------------------
constexpr int MAXSH = 3;

// AES pair scalars of atoms i, j at distance r1: g3 f3, g5 f5, g3 f5 with g = 1/r and the
// damping f_n = 1/(1 + 6 (rr)^dmp_n), rr = (mrad_i + mrad_j) / (2 r)
__device__ __forceinline__ void aes_pair(double r1, double mri, double mrj, const Gfn2Scalars& p,
                                         double& g3f3, double& g5f5, double& g3f5) {
  const double g1 = 1.0 / r1, g3 = g1 * g1 * g1, g5 = g3 * g1 * g1;
  const double rr = 0.5 * (mrj + mri) * g1;
  const double f3 = 1.0 / (1.0 + 6.0 * powe(rr, p.mp_dmp3));
  const double f5 = 1.0 / (1.0 + 6.0 * powe(rr, p.mp_dmp5));
  g3f3 = g3 * f3;
  g5f5 = g5 * f5;
  g3f5 = g3 * f5;
}

// Pair table of the electrostatics, once per geometry (one warp per atom i, partners over the
// lanes): gamma of every shell pair of different atoms and the AES pair scalars.  The kernels
// below then read instead of evaluating square roots, divisions and powers per pair in every
// SCF iteration (FP64 arithmetic is the scarce resource of this GPU; the table costs 8 bytes of
// HBM traffic per entry and iteration).
__device__ __forceinline__ void coulomb_table_dev(DevMol m, Gfn2Scalars p,
                                                  const double* __restrict__ mrad, double* tab) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp, nsh = m.nsh, nat = m.nat;
  const int is0 = m.at_sh[i], nsi = m.at_sh[i + 1] - is0;
  double* aes = tab + (size_t)nsh * nsh;
  const size_t plane = (size_t)nat * nat;
  for (int j = lane; j < nat; j += 32) {
    if (j == i) continue;
    double r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double d = m.xyz[3 * i + k] - m.xyz[3 * j + k];
      r2 += d * d;
    }
    const double r1 = sqrt(r2);
    const int js0 = m.at_sh[j], nsj = m.at_sh[j + 1] - js0;
    for (int a = 0; a < nsi; ++a)
      for (int b = 0; b < nsj; ++b)
        tab[(size_t)(is0 + a) * nsh + js0 + b] =
            gam_kernel(r1, eta_avg(m.sh_hub[is0 + a], m.sh_hub[js0 + b], p.harmonic), p.gexp);
    if (!p.aes) continue;
    double g3f3, g5f5, g3f5;
    aes_pair(r1, mrad[i], mrad[j], p, g3f3, g5f5, g3f5);
    const size_t ij = (size_t)i * nat + j;
    aes[ij] = g3f3;
    aes[plane + ij] = g5f5;
    aes[2 * plane + ij] = g3f5;
  }
}

// tab: the pair table of coulomb_table_dev, or nullptr to evaluate the pair terms here
template <int MODE>
__device__ __forceinline__ void coulomb_dev(DevMol m, Gfn2Scalars p, const double* __restrict__ mrad,
                          const double* __restrict__ qsh, const double* __restrict__ qat,
                          const double* __restrict__ dpat, const double* __restrict__ qpat,
                          double* vsh, double* vat, double* vdp, double* vqp, double* eat,
                          const double* __restrict__ tab = nullptr) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp;
  const int is0 = m.at_sh[i], nsi = m.at_sh[i + 1] - is0;
  double xi[3], di[3], qi[6];
  for (int k = 0; k < 3; ++k) {
    xi[k] = m.xyz[3 * i + k];
    di[k] = dpat[3 * i + k];
  }
  for (int k = 0; k < 6; ++k) qi[k] = qpat[6 * i + k];
  const double qa_i = qat[i], ri = mrad[i];
  double ush[MAXSH] = {0, 0, 0};     // sum_j gamma q_j for shells of i
  double uat = 0.0;                  // vat_i
  double ud[3] = {0, 0, 0};          // vdp_i: sd + dd parts
  double udd[3] = {0, 0, 0};         // dd part only (energy needs 1/2 of it)
  double uq[6] = {0, 0, 0, 0, 0, 0};  // vqp_i
  const int nsh = m.nsh, nat = m.nat;
  const double* aes = tab + (size_t)nsh * nsh;
  const size_t plane = (size_t)nat * nat;
  for (int j = lane; j < nat; j += 32) {
    if (j == i) continue;
    double v[3];
    for (int k = 0; k < 3; ++k) v[k] = xi[k] - m.xyz[3 * j + k];  // R_i - R_j
    const double r1 = tab ? 0.0 : sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    // isotropic: gamma = 1/sqrt(r^2 + eta^-2) for gexp = 2; general form kept
    const int js0 = m.at_sh[j], nsj = m.at_sh[j + 1] - js0;
    for (int a = 0; a < nsi; ++a) {
      const double hi = m.sh_hub[is0 + a];
      double acc = 0.0;
      for (int b = 0; b < nsj; ++b) {
        const double t = tab ? tab[(size_t)(is0 + a) * nsh + js0 + b]
                             : gam_kernel(r1, eta_avg(hi, m.sh_hub[js0 + b], p.harmonic), p.gexp);
        acc += t * qsh[js0 + b];
      }
      ush[a] += acc;
    }
    if (!p.aes) continue;
    // AES (multipole.f90:488-535), amat(:, jat, iat) with vec = R_iat - R_jat
    double g3f3, g5f5, g3f5;
    if (tab) {
      const size_t ij = (size_t)i * nat + j;
      g3f3 = aes[ij];
      g5f5 = aes[plane + ij];
      g3f5 = aes[2 * plane + ij];
    } else {
      aes_pair(r1, ri, mrad[j], p, g3f3, g5f5, g3f5);
    }
    const double* dj = dpat + 3 * j;
    const double* qj = qpat + 6 * j;
    const double qa_j = qat[j];
    // vat_i += sum_j amat_sd(:, j, i) . dpat_j + amat_sq(:, j, i) . qpat_j   (v = R_i - R_j)
    const double sq[6] = {v[0] * v[0] * g5f5, 2 * v[0] * v[1] * g5f5, v[1] * v[1] * g5f5,
                          2 * v[0] * v[2] * g5f5, 2 * v[1] * v[2] * g5f5, v[2] * v[2] * g5f5};
    uat += (v[0] * dj[0] + v[1] * dj[1] + v[2] * dj[2]) * g3f3;
    for (int k = 0; k < 6; ++k) uat += sq[k] * qj[k];
    // vdp_i += sum_j amat_sd(:, i, j) q_j + amat_dd(:, i, :, j) dpat_j ; amat_sd(:, i, j) = -v g3 f3
    const double vd = v[0] * dj[0] + v[1] * dj[1] + v[2] * dj[2];
    for (int k = 0; k < 3; ++k) {
      ud[k] += -v[k] * g3f3 * qa_j;
      const double dd = dj[k] * g3f5 - v[k] * vd * 3.0 * g5f5;
      udd[k] += dd;
    }
    for (int k = 0; k < 6; ++k) uq[k] += sq[k] * qa_j;
  }
  for (int a = 0; a < MAXSH; ++a) ush[a] = warp_sum(ush[a]);
  uat = warp_sum(uat);
  for (int k = 0; k < 3; ++k) {
    ud[k] = warp_sum(ud[k]);
    udd[k] = warp_sum(udd[k]);
  }
  for (int k = 0; k < 6; ++k) uq[k] = warp_sum(uq[k]);
  if (lane != 0) return;
  // on-site gamma block
  double gsh[MAXSH];
  for (int a = 0; a < nsi; ++a) {
    double acc = ush[a];
    for (int b = 0; b < nsi; ++b)
      acc += eta_avg(m.sh_hub[is0 + a], m.sh_hub[is0 + b], p.harmonic) * qsh[is0 + b];
    gsh[a] = acc;
  }
  const double mpscale[6] = {1, 2, 1, 2, 2, 1};
  if (MODE == 0) {
    for (int a = 0; a < nsi; ++a) {
      const double q = qsh[is0 + a];
      vsh[is0 + a] = gsh[a] + (p.third_atom ? 0.0 : q * q * m.sh_gam3[is0 + a]);
    }
    vat[i] = uat + (p.third_atom ? qa_i * qa_i * m.at_gam3[i] : 0.0);
    for (int k = 0; k < 3; ++k)
      vdp[3 * i + k] = p.aes ? ud[k] + udd[k] + 2.0 * m.at_dkern[i] * di[k] : 0.0;
    for (int k = 0; k < 6; ++k)
      vqp[6 * i + k] = p.aes ? uq[k] + 2.0 * m.at_qkern[i] * qi[k] * mpscale[k] : 0.0;
  } else {
    double e = 0.0;
    for (int a = 0; a < nsi; ++a) {
      const double q = qsh[is0 + a];
      e += 0.5 * gsh[a] * q + (p.third_atom ? 0.0 : q * q * q * m.sh_gam3[is0 + a] / 3.0);
    }
    if (p.third_atom) e += qa_i * qa_i * qa_i * m.at_gam3[i] / 3.0;
    if (!p.aes) {
      eat[i] += e;
      return;
    }
    for (int k = 0; k < 3; ++k) e += di[k] * (ud[k] + 0.5 * udd[k]);
    for (int k = 0; k < 6; ++k) e += qi[k] * uq[k];
    double d2 = 0.0, q2 = 0.0;
    for (int k = 0; k < 3; ++k) d2 += di[k] * di[k];
    for (int k = 0; k < 6; ++k) q2 += qi[k] * qi[k] * mpscale[k];
    e += m.at_dkern[i] * d2 + m.at_qkern[i] * q2;
    eat[i] += e;
  }
}
template <int MODE>
__global__ void k_coulomb(DevMol m, Gfn2Scalars p, const double* __restrict__ mrad,
                          const double* __restrict__ qsh, const double* __restrict__ qat,
                          const double* __restrict__ dpat, const double* __restrict__ qpat,
                          double* vsh, double* vat, double* vdp, double* vqp, double* eat) {
  coulomb_dev<MODE>(m, p, mrad, qsh, qat, dpat, qpat, vsh, vat, vdp, vqp, eat);
}

void launch_coulomb_potential(const DevMol& m, const Gfn2Scalars& p, const double* mrad,
                              const double* qsh, const double* qat, const double* dpat,
                              const double* qpat, double* vsh, double* vat, double* vdp,
                              double* vqp, cudaStream_t s) {
  ++g_kernel_launches;
  k_coulomb<0><<<(m.nat * 32 + 63) / 64, 64, 0, s>>>(m, p, mrad, qsh, qat, dpat, qpat, vsh, vat,
                                                         vdp, vqp, nullptr);
}

void launch_coulomb_energy(const DevMol& m, const Gfn2Scalars& p, const double* mrad,
                           const double* qsh, const double* qat, const double* dpat,
                           const double* qpat, double* eat, cudaStream_t s) {
  ++g_kernel_launches;
  k_coulomb<1><<<(m.nat * 32 + 63) / 64, 64, 0, s>>>(m, p, mrad, qsh, qat, dpat, qpat, nullptr,
                                                         nullptr, nullptr, nullptr, eat);
}

// ------------------------------------------------------------------------------------
// electrostatic gradient at fixed charges/moments (es2 + AES); dEdcn += dEdr dmrdcn
// per-atom formulation: atom i sums its own share of every pair (no atomics)
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void coulomb_grad_dev(DevMol m, Gfn2Scalars p, const double* __restrict__ mrad,
                               const double* __restrict__ dmrdcn, const double* __restrict__ qsh,
                               const double* __restrict__ qat, const double* __restrict__ dpat,
                               const double* __restrict__ qpat, double* grad, double* sig_at,
                               double* dEdcn) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp;
  const int is0 = m.at_sh[i], nsi = m.at_sh[i + 1] - is0;
  double g[3] = {0, 0, 0}, sg[9] = {0}, dEdr = 0.0;
  const double* di = dpat + 3 * i;
  const double* qi = qpat + 6 * i;
  for (int j = lane; j < m.nat; j += 32) {
    if (j == i) continue;
    double w[3];
    for (int k = 0; k < 3; ++k) w[k] = m.xyz[3 * i + k] - m.xyz[3 * j + k];  // R_i - R_j
    const double r2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2], r1 = sqrt(r2);
    // es2: d/dR_i of 1/2 sum q gamma q  (pair counted once per atom)
    const int js0 = m.at_sh[j], nsj = m.at_sh[j + 1] - js0;
    double f = 0.0;
    for (int a = 0; a < nsi; ++a)
      for (int b = 0; b < nsj; ++b) {
        const double gm = eta_avg(m.sh_hub[is0 + a], m.sh_hub[js0 + b], p.harmonic);
        double d;
        if (p.gexp == 2.0) {
          d = 1.0 / (r2 + 1.0 / (gm * gm));
          d = -d * sqrt(d);
        } else {
          d = 1.0 / (pow(r1, p.gexp) + pow(gm, -p.gexp));
          d = -pow(r1, p.gexp - 2.0) * d * pow(d, 1.0 / p.gexp);
        }
        f += d * qsh[is0 + a] * qsh[js0 + b];
      }
    double gp[3];
    for (int k = 0; k < 3; ++k) gp[k] = f * w[k];
    if (!p.aes) {  // no anisotropic electrostatics (GFN1)
      for (int k = 0; k < 3; ++k) g[k] += gp[k];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) sg[3 * a + b] += 0.5 * gp[a] * w[b];
      continue;
    }
    // AES pair term written as in the reference with (iat, jat) = (i, j), vec = R_j - R_i
    const double* dj = dpat + 3 * j;
    const double* qj = qpat + 6 * j;
    const double qai = qat[i], qaj = qat[j];
    double v[3] = {-w[0], -w[1], -w[2]};
    const double rr = 0.5 * (mrad[i] + mrad[j]);
    const double g1 = 1.0 / r1, g3 = g1 * g1 * g1, g5 = g3 * g1 * g1, g7 = g5 * g1 * g1;
    const double f3 = 1.0 / (1.0 + 6.0 * powe(rr * g1, p.mp_dmp3));
    const double d3 = -3 * g5 * f3 - p.mp_dmp3 * f3 * (f3 - 1.0) * g5;
    const double f5 = 1.0 / (1.0 + 6.0 * powe(rr * g1, p.mp_dmp5));
    const double d5 = -5 * f5 - p.mp_dmp5 * (f5 * f5 - f5);
    const double dpiqj = (v[0] * di[0] + v[1] * di[1] + v[2] * di[2]) * qaj;
    const double qidpj = (v[0] * dj[0] + v[1] * dj[1] + v[2] * dj[2]) * qai;
    double fddr = 3.0 * (dpiqj - qidpj) * p.mp_dmp3 * f3 * g3 * (f3 / rr) * powe(rr * g1, p.mp_dmp3);
    double ga[3];
    for (int k = 0; k < 3; ++k)
      ga[k] = -d3 * v[k] * (dpiqj - qidpj) + f3 * g3 * (qai * dj[k] - qaj * di[k]);
    const double dpidpj = di[0] * dj[0] + di[1] * dj[1] + di[2] * dj[2];
    const double dpiv = di[0] * v[0] + di[1] * v[1] + di[2] * v[2];
    const double dpjv = dj[0] * v[0] + dj[1] * v[1] + dj[2] * v[2];
    const double edd = dpidpj * r2 - 3 * dpjv * dpiv;
    fddr += 3.0 * edd * p.mp_dmp5 * f5 * g5 * (f5 / rr) * powe(rr * g1, p.mp_dmp5);
    for (int k = 0; k < 3; ++k)
      ga[k] += -2.0 * f5 * g5 * dpidpj * v[k] + 3.0 * f5 * g5 * (dpiv * dj[k] + dpjv * di[k])
               - edd * d5 * g7 * v[k];
    const double eq = 2 * (qaj * qi[1] + qj[1] * qai) * v[0] * v[1]
                      + 2 * (qaj * qi[3] + qj[3] * qai) * v[0] * v[2]
                      + 2 * (qaj * qi[4] + qj[4] * qai) * v[1] * v[2]
                      + (qaj * qi[0] + qj[0] * qai) * v[0] * v[0]
                      + (qaj * qi[2] + qj[2] * qai) * v[1] * v[1]
                      + (qaj * qi[5] + qj[5] * qai) * v[2] * v[2];
    fddr += eq * 3.0 * p.mp_dmp5 * f5 * g5 * f5 / rr * powe(rr * g1, p.mp_dmp5);
    const double qjv[3] = {v[0] * qj[0] + v[1] * qj[1] + v[2] * qj[3],
                           v[0] * qj[1] + v[1] * qj[2] + v[2] * qj[4],
                           v[0] * qj[3] + v[1] * qj[4] + v[2] * qj[5]};
    const double qiv[3] = {v[0] * qi[0] + v[1] * qi[1] + v[2] * qi[3],
                           v[0] * qi[1] + v[1] * qi[2] + v[2] * qi[4],
                           v[0] * qi[3] + v[1] * qi[4] + v[2] * qi[5]};
    for (int k = 0; k < 3; ++k)
      ga[k] += -eq * d5 * g7 * v[k] - 2.0 * f5 * g5 * qai * qjv[k] - 2.0 * f5 * g5 * qaj * qiv[k];
    dEdr += fddr;
    for (int k = 0; k < 3; ++k) g[k] += gp[k] + ga[k];
    // virial, half of each pair per atom
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        sg[3 * a + b] += 0.5 * gp[a] * w[b] - 0.25 * (v[a] * ga[b] + ga[a] * v[b]);
  }
  for (int k = 0; k < 3; ++k) g[k] = warp_sum(g[k]);
  for (int k = 0; k < 9; ++k) sg[k] = warp_sum(sg[k]);
  dEdr = warp_sum(dEdr);
  if (lane == 0) {
    for (int k = 0; k < 3; ++k) grad[3 * i + k] += g[k];
    for (int k = 0; k < 9; ++k) sig_at[9 * i + k] += sg[k];
    dEdcn[i] += dEdr * dmrdcn[i];
  }
}
__global__ void k_coulomb_grad(DevMol m, Gfn2Scalars p, const double* __restrict__ mrad,
                               const double* __restrict__ dmrdcn, const double* __restrict__ qsh,
                               const double* __restrict__ qat, const double* __restrict__ dpat,
                               const double* __restrict__ qpat, double* grad, double* sig_at,
                               double* dEdcn) {
  coulomb_grad_dev(m, p, mrad, dmrdcn, qsh, qat, dpat, qpat, grad, sig_at, dEdcn);
}

void launch_coulomb_gradient(const DevMol& m, const Gfn2Scalars& p, const double* mrad,
                             const double* dmrdcn, const double* qsh, const double* qat,
                             const double* dpat, const double* qpat, double* grad, double* sig_at,
                             double* dEdcn, cudaStream_t s) {
  if (m.nat == 1) return;
  ++g_kernel_launches;
  k_coulomb_grad<<<(m.nat * 32 + 63) / 64, 64, 0, s>>>(m, p, mrad, dmrdcn, qsh, qat, dpat, qpat,
                                                          grad, sig_at, dEdcn);
}

// ------------------------------------------------------------------------------------
// repulsion energy + gradient (per atom, each pair seen from both atoms)
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void repulsion_dev(DevMol m, Gfn2Scalars p, double* erep, double* grad, double* sig_at) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m.nat) return;
  const int i = warp;
  const double cut2 = p.rep_cutoff * p.rep_cutoff;
  double e = 0.0, g[3] = {0, 0, 0}, sg[9] = {0};
  for (int j = lane; j < m.nat; j += 32) {
    if (j == i) continue;
    double v[3], r2 = 0;
    for (int k = 0; k < 3; ++k) {
      v[k] = m.xyz[3 * i + k] - m.xyz[3 * j + k];
      r2 += v[k] * v[k];
    }
    if (r2 > cut2 || r2 < 1e-12) continue;
    const double r1 = sqrt(r2);
    const double ke = (m.at_z[i] > 2 || m.at_z[j] > 2) ? p.rep_kexp : p.rep_kexp_light;
    const double a = sqrt(m.at_repa[i] * m.at_repa[j]), z = m.at_repz[i] * m.at_repz[j];
    const double r1k = pow(r1, ke), exa = exp(-a * r1k), r1r = pow(r1, p.rep_rexp);
    const double dE = z * exa / r1r;
    e += 0.5 * dE;
    const double f = -(a * r1k * ke + p.rep_rexp) * dE / r2;
    for (int k = 0; k < 3; ++k) g[k] += f * v[k];
    for (int a2 = 0; a2 < 3; ++a2)
      for (int c = 0; c < 3; ++c) sg[3 * a2 + c] += 0.5 * f * v[a2] * v[c];
  }
  e = warp_sum(e);
  for (int k = 0; k < 3; ++k) g[k] = warp_sum(g[k]);
  for (int k = 0; k < 9; ++k) sg[k] = warp_sum(sg[k]);
  if (lane == 0) {
    erep[i] = e;
    if (grad) {
      for (int k = 0; k < 3; ++k) grad[3 * i + k] += g[k];
      for (int k = 0; k < 9; ++k) sig_at[9 * i + k] += sg[k];
    }
  }
}
__global__ void k_repulsion(DevMol m, Gfn2Scalars p, double* erep, double* grad, double* sig_at) {
  repulsion_dev(m, p, erep, grad, sig_at);
}

void launch_repulsion(const DevMol& m, const Gfn2Scalars& p, double* erep, double* grad,
                      double* sig_at, cudaStream_t s) {
  ++g_kernel_launches;
  k_repulsion<<<(m.nat * 32 + 63) / 64, 64, 0, s>>>(m, p, erep, grad, sig_at);
}

// ------------------------------------------------------------------------------------
// orbital potential: vao = vsh(ao) + vat(atom)
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void vao_dev(DevMol m, const double* vsh, const double* vat, double* vao) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m.nao) return;
  vao[t] = vsh[m.ao_sh[t]] + vat[m.ao_at[t]];
}
__global__ void k_vao(DevMol m, const double* vsh, const double* vat, double* vao) {
  vao_dev(m, vsh, vat, vao);
}

void launch_vao(const DevMol& m, const double* vsh, const double* vat, double* vao,
                cudaStream_t s) {
  ++g_kernel_launches;
  k_vao<<<(m.nao + 255) / 256, 256, 0, s>>>(m, vsh, vat, vao);
}

// ------------------------------------------------------------------------------------
// Fock assembly, tiles of 32x32; block (32, 8).  For a tile pair (I <= J) the block reads
// the (I,J) tiles of H, S, D, Q and the (J,I) tiles of D, Q (staged through shared memory),
// writes F(I,J) and its transpose F(J,I).  Every input element is read once.
//   F_rc = H_rc - 1/2 S_rc (v_r + v_c) - 1/2 sum_k (M_k,rc u_k,A(c) + M_k,cr u_k,A(r))
// The two multipole products are summed in an order that depends only on min/max(r,c),
// so F is exactly symmetric.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void fock_dev(int n, const int* __restrict__ ao_at,
                                              const double* __restrict__ H,
                                              const double* __restrict__ S,
                                              const double* __restrict__ D,
                                              const double* __restrict__ Q,
                                              const double* __restrict__ vao,
                                              const double* __restrict__ vdp,
                                              const double* __restrict__ vqp, double* F) {
  const int I = blockIdx.y, J = blockIdx.x;
  if (I > J) return;
  __shared__ double sh[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const size_t nn = (size_t)n * n;
  const int c = J * 32 + tx;
  const bool cin = c < n;
  double acc[4];
  int rows[4];
  const int atc = cin ? ao_at[c] : 0;
  const double vc = cin ? vao[c] : 0.0;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int r = I * 32 + ty + 8 * s;
    rows[s] = r;
    acc[s] = 0.0;
    if (r < n && cin) {
      const size_t rc = (size_t)r * n + c;
      acc[s] = H[rc] - 0.5 * S[rc] * (vao[r] + vc);
    }
  }
  // multipole terms (absent, D == nullptr, for a Hamiltonian without anisotropic electrostatics)
  for (int k = 0; D != nullptr && k < 9; ++k) {
    const double* M = k < 3 ? D + k * nn : Q + (k - 3) * nn;
    const double* u = k < 3 ? vdp : vqp;
    const int ku = k < 3 ? k : k - 3, su = k < 3 ? 3 : 6;
    // stage tile (J, I) of M: sh[a][b] = M[J*32 + a][I*32 + b]
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int a = ty + 8 * s;
      const int rr = J * 32 + a, cc = I * 32 + tx;
      sh[a][tx] = (rr < n && cc < n) ? M[(size_t)rr * n + cc] : 0.0;
    }
    __syncthreads();
    const double uc = cin ? u[su * atc + ku] : 0.0;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int r = rows[s];
      if (r < n && cin) {
        const double t1 = M[(size_t)r * n + c] * uc;          // M_rc u_A(c)
        const double t2 = sh[tx][ty + 8 * s] * u[su * ao_at[r] + ku];  // M_cr u_A(r)
        acc[s] -= 0.5 * (r <= c ? (t1 + t2) : (t2 + t1));
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int r = rows[s];
    if (r < n && cin) F[(size_t)r * n + c] = acc[s];
  }
  if (I == J) return;
  // transpose write of F(J,I)
#pragma unroll
  for (int s = 0; s < 4; ++s) sh[ty + 8 * s][tx] = acc[s];
  __syncthreads();
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int rr = J * 32 + ty + 8 * s, cc = I * 32 + tx;
    if (rr < n && cc < n) F[(size_t)rr * n + cc] = sh[tx][ty + 8 * s];
  }
}
__global__ void __launch_bounds__(256) k_fock(int n, const int* __restrict__ ao_at,
                                              const double* __restrict__ H,
                                              const double* __restrict__ S,
                                              const double* __restrict__ D,
                                              const double* __restrict__ Q,
                                              const double* __restrict__ vao,
                                              const double* __restrict__ vdp,
                                              const double* __restrict__ vqp, double* F) {
  fock_dev(n, ao_at, H, S, D, Q, vao, vdp, vqp, F);
}

void launch_fock(int n, const int* ao_at, const double* H, const double* S, const double* D,
                 const double* Q, const double* vao, const double* vdp, const double* vqp, double* F,
                 cudaStream_t s) {
  const int nt = (n + 31) / 32;
  ++g_kernel_launches;
  const int tk = prof_kbegin(s);
  k_fock<<<dim3(nt, nt), dim3(32, 8), 0, s>>>(n, ao_at, H, S, D, Q, vao, vdp, vqp, F);
  prof_kend(KS_FOCK, tk, s);
}

// ------------------------------------------------------------------------------------
// Mulliken: column sums over row chunks.  partial[chunk][11][n]:
//   0: sum_r P S, 1-3: sum_r P D_k, 4-9: sum_r P Q_q, 10: sum_r P H
// ------------------------------------------------------------------------------------
constexpr int MULL_ROWS = 64;

int mulliken_chunks(int n) { return (n + MULL_ROWS - 1) / MULL_ROWS; }

__device__ __forceinline__ void mull_partial_dev(int n, const double* __restrict__ P,
                                                      const double* __restrict__ S,
                                                      const double* __restrict__ H,
                                                      const double* __restrict__ D,
                                                      const double* __restrict__ Q,
                                                      double* partial) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int chunk = blockIdx.y;
  if (c >= n) return;
  const size_t nn = (size_t)n * n;
  double acc[11];
#pragma unroll
  for (int k = 0; k < 11; ++k) acc[k] = 0.0;
  const int r0 = chunk * MULL_ROWS, r1 = min(n, r0 + MULL_ROWS);
  for (int r = r0; r < r1; ++r) {
    const size_t rc = (size_t)r * n + c;
    const double pv = P[rc];
    acc[0] += pv * S[rc];
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[1 + k] += pv * D[k * nn + rc];
#pragma unroll
    for (int q = 0; q < 6; ++q) acc[4 + q] += pv * Q[q * nn + rc];
    acc[10] += pv * H[rc];
  }
#pragma unroll
  for (int k = 0; k < 11; ++k) partial[((size_t)chunk * 11 + k) * n + c] = acc[k];
}
__global__ void __launch_bounds__(128) k_mull_partial(int n, const double* __restrict__ P,
                                                      const double* __restrict__ S,
                                                      const double* __restrict__ H,
                                                      const double* __restrict__ D,
                                                      const double* __restrict__ Q,
                                                      double* partial) {
  mull_partial_dev(n, P, S, H, D, Q, partial);
}

// one thread per atom: reduce chunks for its orbitals, fill shells/atoms
__device__ __forceinline__ void mull_reduce_dev(DevMol m, const double* __restrict__ partial, int nchunk,
                              double* qsh, double* qat, double* dpat, double* qpat,
                              double* eband) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m.nat) return;
  const int n = m.nao;
  double d[3] = {0, 0, 0}, q[6] = {0, 0, 0, 0, 0, 0}, e = 0.0, qa = 0.0;
  for (int s = m.at_sh[i]; s < m.at_sh[i + 1]; ++s) {
    double ps = 0.0;
    const int o = m.sh_ao[s], no = 2 * m.sh_l[s] + 1;
    for (int mu = o; mu < o + no; ++mu) {
      for (int ch = 0; ch < nchunk; ++ch) {
        const double* pp = partial + (size_t)ch * 11 * n;
        ps += pp[mu];
        for (int k = 0; k < 3; ++k) d[k] += pp[(1 + k) * (size_t)n + mu];
        for (int k = 0; k < 6; ++k) q[k] += pp[(4 + k) * (size_t)n + mu];
        e += pp[10 * (size_t)n + mu];
      }
    }
    const double v = m.sh_refocc[s] - ps;
    qsh[s] = v;
    qa += v;
  }
  qat[i] = qa;
  for (int k = 0; k < 3; ++k) dpat[3 * i + k] = -d[k];
  for (int k = 0; k < 6; ++k) qpat[6 * i + k] = -q[k];
  eband[i] = e;
}
__global__ void k_mull_reduce(DevMol m, const double* __restrict__ partial, int nchunk,
                              double* qsh, double* qat, double* dpat, double* qpat,
                              double* eband) {
  mull_reduce_dev(m, partial, nchunk, qsh, qat, dpat, qpat, eband);
}

void launch_mulliken(const DevMol& m, const double* P, const double* S, const double* H,
                     const double* D, const double* Q, double* partial, int nchunk, double* qsh,
                     double* qat, double* dpat, double* qpat, double* eband, cudaStream_t s) {
  const int n = m.nao;
  ++g_kernel_launches;
  const int tk = prof_kbegin(s);
  k_mull_partial<<<dim3((n + 127) / 128, nchunk), 128, 0, s>>>(n, P, S, H, D, Q, partial);
  prof_kend(KS_MULLIKEN, tk, s);
  ++g_kernel_launches;
  k_mull_reduce<<<(m.nat + 127) / 128, 128, 0, s>>>(m, partial, nchunk, qsh, qat, dpat, qpat,
                                                    eband);
}

// ------------------------------------------------------------------------------------
// Fermi filling (one block).  Both spin channels share the eigenvalues.
// ------------------------------------------------------------------------------------
__device__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  double t = threadIdx.x < nw ? red[threadIdx.x] : 0.0;
  if (w == 0) t = warp_sum(t);
  __syncthreads();
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  return r;
}

// returns the highest Fermi level at which occupations were evaluated (-1e300 if none)
__device__ double fermi_channel(int n, const double* emo, double nel, double kt, double* occ,
                                double* red, double* ts) {
  double ef_max = -1e300;
  // Aufbau
  int homo = (int)floor(nel);
  const double frac = fmod(nel, 1.0);
  for (int k = threadIdx.x; k < n; k += blockDim.x)
    occ[k] = k < homo ? 1.0 : (k == homo ? frac : 0.0);
  __syncthreads();
  homo = frac > 0.5 ? homo + 1 : homo;
  if (homo > 0) {
    double ef = 0.5 * (emo[max(homo, 1) - 1] + emo[min(homo + 1, n) - 1]);
    const double occt = homo;
    const double thr = 1.4901161193847656e-08;      // sqrt(epsilon)
    const double sqrttiny = 1.4916681462400413e-154;  // sqrt(tiny)
    for (int cyc = 0; cyc < 200; ++cyc) {
      ef_max = fmax(ef_max, ef);
      double tn = 0.0, td = 0.0;
      for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double x = (emo[k] - ef) / kt;
        double f = 0.0, df = 0.0;
        if (x < 50.0) {
          const double ex = exp(x);
          f = 1.0 / (ex + 1.0);
          df = ex / (kt * (ex + 1.0) * (ex + 1.0));
        }
        occ[k] = f;
        tn += f;
        td += df;
      }
      tn = block_sum(tn, red);
      td = block_sum(td, red);
      const double change = td > sqrttiny ? (occt - tn) / td : 0.0;
      ef += change;
      if (fabs(occt - tn) <= thr) break;
    }
  }
  __syncthreads();
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double o = occ[k];
    s += log(pow(o, o) * pow(1.0 - o, 1.0 - o));
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0) *ts += s * kt;
  __syncthreads();
  return ef_max;
}

// emo[nev..n) may be placeholders (1e300) for levels that were not computed: valid as long as
// the highest computed level lies 51 kT above every Fermi level used (the occupation is then
// exactly zero above it, as for the true levels); otherwise ncols[1] = 1
__device__ __forceinline__ void fermi_dev(int n, const double* emo, double nalp, double nbet, double kt, double* fa,
                        double* fb, double* focc, double* ts, int* ncols, int nev) {
  __shared__ double red[32];
  if (threadIdx.x == 0) *ts = 0.0;
  __syncthreads();
  const double efa = fermi_channel(n, emo, nalp, kt, fa, red, ts);
  const double efb = fermi_channel(n, emo, nbet, kt, fb, red, ts);
  if (threadIdx.x == 0)
    ncols[1] = (nev < n && !(emo[nev - 1] >= fmax(efa, efb) + 51.0 * kt)) ? 1 : 0;
  int last = -1;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double f = fa[k] + fb[k];
    focc[k] = f;
    if (f != 0.0) last = max(last, k);
  }
  // block max
  __shared__ int mx;
  if (threadIdx.x == 0) mx = -1;
  __syncthreads();
  atomicMax(&mx, last);
  __syncthreads();
  if (threadIdx.x == 0) *ncols = mx + 1;
}
__global__ void k_fermi(int n, const double* emo, double nalp, double nbet, double kt, double* fa,
                        double* fb, double* focc, double* ts, int* ncols, int nev) {
  fermi_dev(n, emo, nalp, nbet, kt, fa, fb, focc, ts, ncols, nev);
}

void launch_fermi(int n, const double* emo, double nalp, double nbet, double kt, double* focc,
                  double* ts, int* ncols, cudaStream_t s, int nev) {
  // fa, fb scratch follow focc in memory: focc[n], fa[n], fb[n]
  ++g_kernel_launches;
  k_fermi<<<1, 1024, 0, s>>>(n, emo, nalp, nbet, kt, focc + n, focc + 2 * n, focc, ts, ncols,
                             nev > 0 ? nev : n);
}

// ------------------------------------------------------------------------------------
// mixer vector packing  [qsh | dpat | qpat]
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void pack_dev(int nsh, int nat, const double* qsh, const double* dpat, const double* qpat,
                       double* vec) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nd = nsh + 9 * nat;
  if (t >= nd) return;
  if (t < nsh) vec[t] = qsh[t];
  else if (t < nsh + 3 * nat) vec[t] = dpat[t - nsh];
  else vec[t] = qpat[t - nsh - 3 * nat];
}
__global__ void k_pack(int nsh, int nat, const double* qsh, const double* dpat, const double* qpat,
                       double* vec) {
  pack_dev(nsh, nat, qsh, dpat, qpat, vec);
}

void launch_pack(const DevMol& m, const double* qsh, const double* dpat, const double* qpat,
                 double* vec, cudaStream_t s, bool with_mp) {
  const int nmp = with_mp ? m.nat : 0;  // atoms whose multipoles enter the mixer
  const int nd = m.nsh + 9 * nmp;
  ++g_kernel_launches;
  k_pack<<<(nd + 255) / 256, 256, 0, s>>>(m.nsh, nmp, qsh, dpat, qpat, vec);
}

__device__ __forceinline__ void unpack_dev(DevMol m, const double* vec, double* qsh, double* qat, double* dpat,
                         double* qpat, int with_mp) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nsh = m.nsh, nat = m.nat;
  if (t < nsh) qsh[t] = vec[t];
  if (with_mp && t < 3 * nat) dpat[t] = vec[nsh + t];
  if (with_mp && t < 6 * nat) qpat[t] = vec[nsh + 3 * nat + t];
  if (t < nat) {
    double a = 0.0;
    for (int s = m.at_sh[t]; s < m.at_sh[t + 1]; ++s) a += vec[s];
    qat[t] = a;
  }
}
__global__ void k_unpack(DevMol m, const double* vec, double* qsh, double* qat, double* dpat,
                         double* qpat, int with_mp) {
  unpack_dev(m, vec, qsh, qat, dpat, qpat, with_mp);
}

void launch_unpack(const DevMol& m, const double* vec, double* qsh, double* qat, double* dpat,
                   double* qpat, cudaStream_t s, bool with_mp) {
  const int nt = m.nsh > 6 * m.nat ? m.nsh : 6 * m.nat;
  ++g_kernel_launches;
  k_unpack<<<(nt + 255) / 256, 256, 0, s>>>(m, vec, qsh, qat, dpat, qpat, with_mp ? 1 : 0);
}

__device__ __forceinline__ void diff_dev(int nd, const double* vout, const double* q, double* dq, double* err) {
  __shared__ double red[32];
  double s = 0.0;
  for (int t = threadIdx.x; t < nd; t += blockDim.x) {
    const double d = vout[t] - q[t];
    dq[t] = d;
    s += d * d / nd;
  }
  s = block_sum(s, red);
  if (threadIdx.x == 0) *err = sqrt(s);
}
__global__ void k_diff(int nd, const double* vout, const double* q, double* dq, double* err) {
  diff_dev(nd, vout, q, dq, err);
}

void launch_diff(int nd, const double* vout, const double* q, double* dq, double* err,
                 cudaStream_t s) {
  ++g_kernel_launches;
  k_diff<<<1, 1024, 0, s>>>(nd, vout, q, dq, err);
}

// ------------------------------------------------------------------------------------
// Broyden step (one block).  Same recurrences as the reference; the overlap matrix a(i,j)
// is kept between calls and only the row of the newest history vector is recomputed
// (the other rows are unchanged dot products).
// ------------------------------------------------------------------------------------
__device__ double block_dot(int nd, const double* x, const double* y, double* red) {
  double s = 0.0;
  for (int t = threadIdx.x; t < nd; t += blockDim.x) s += x[t] * y[t];
  return block_sum(s, red);
}

__device__ __forceinline__ void broyden_dev(int nd, int memory, int iter, double alpha, double* q, double* qlast,
                          const double* dq, double* dqlast, double* df, double* u, double* a,
                          double* omega, double* work, int* status) {
  __shared__ double red[32];
  if (iter == 1) {
    for (int t = threadIdx.x; t < nd; t += blockDim.x) {
      dqlast[t] = dq[t];
      qlast[t] = q[t];
      q[t] = q[t] + alpha * dq[t];
    }
    if (threadIdx.x == 0) *status = 0;
    return;
  }
  const int itn = iter - 1;
  const int it1 = (itn - 1) % memory;
  const int nhist = min(memory, itn);
  const int first = max(1, itn - memory + 1);
  const double omega0 = 0.01, minw = 1.0, maxw = 100000.0, wfac = 0.01;
  double w = sqrt(block_dot(nd, dq, dq, red));
  w = w > wfac / maxw ? wfac / w : maxw;
  if (w < minw) w = minw;
  if (threadIdx.x == 0) omega[it1] = w;
  double* dfn = df + (size_t)it1 * nd;
  for (int t = threadIdx.x; t < nd; t += blockDim.x) dfn[t] = dq[t] - dqlast[t];
  __syncthreads();
  double inv = sqrt(block_dot(nd, dfn, dfn, red));
  inv = inv > 2.220446049250313e-16 ? inv : 2.220446049250313e-16;
  inv = 1.0 / inv;
  for (int t = threadIdx.x; t < nd; t += blockDim.x) dfn[t] *= inv;
  __syncthreads();
  // history indices, c vector, a row
  double* beta = work;                      // [nhist][nhist]
  double* cvec = work + memory * memory;    // [nhist]
  for (int ih = 0; ih < nhist; ++ih) {
    const int i = (first + ih - 1) % memory;
    const double dfi_dq = block_dot(nd, df + (size_t)i * nd, dq, red);
    const double aij = block_dot(nd, df + (size_t)i * nd, dfn, red);
    if (threadIdx.x == 0) {
      cvec[ih] = omega[i] * dfi_dq;
      a[(size_t)i * memory + it1] = aij;
      a[(size_t)it1 * memory + i] = aij;
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nhist * nhist; t += blockDim.x) {
    const int ih = t / nhist, jh = t % nhist;
    const int i = (first + ih - 1) % memory, j = (first + jh - 1) % memory;
    beta[t] = omega[i] * omega[j] * a[(size_t)i * memory + j] + (ih == jh ? omega0 * omega0 : 0.0);
  }
  __syncthreads();
  // solve beta^T x = c by Gaussian elimination with partial pivoting (getrf + getrs 't')
  __shared__ int piv;
  __shared__ int fail;
  if (threadIdx.x == 0) fail = 0;
  __syncthreads();
  // transpose in place to solve beta^T
  for (int t = threadIdx.x; t < nhist * nhist; t += blockDim.x) {
    const int i = t / nhist, j = t % nhist;
    if (i < j) {
      const double x = beta[i * nhist + j];
      beta[i * nhist + j] = beta[j * nhist + i];
      beta[j * nhist + i] = x;
    }
  }
  __syncthreads();
  for (int k = 0; k < nhist; ++k) {
    if (threadIdx.x == 0) {
      int p = k;
      double best = fabs(beta[k * nhist + k]);
      for (int i = k + 1; i < nhist; ++i) {
        const double v = fabs(beta[i * nhist + k]);
        if (v > best) {
          best = v;
          p = i;
        }
      }
      piv = p;
      if (best == 0.0) fail = k + 1;
    }
    __syncthreads();
    if (fail) break;
    const int p = piv;
    if (p != k) {
      for (int j = threadIdx.x; j < nhist; j += blockDim.x) {
        const double x = beta[k * nhist + j];
        beta[k * nhist + j] = beta[p * nhist + j];
        beta[p * nhist + j] = x;
      }
      if (threadIdx.x == 0) {
        const double x = cvec[k];
        cvec[k] = cvec[p];
        cvec[p] = x;
      }
    }
    __syncthreads();
    const double pivv = beta[k * nhist + k];
    for (int t = threadIdx.x; t < (nhist - k - 1) * (nhist - k); t += blockDim.x) {
      const int i = k + 1 + t / (nhist - k), j = k + t % (nhist - k);
      const double f = beta[i * nhist + k] / pivv;
      if (j > k) beta[i * nhist + j] -= f * beta[k * nhist + j];
    }
    __syncthreads();
    for (int i = k + 1 + threadIdx.x; i < nhist; i += blockDim.x) {
      cvec[i] -= beta[i * nhist + k] / pivv * cvec[k];
    }
    __syncthreads();
  }
  if (fail) {
    if (threadIdx.x == 0) *status = fail;
    return;
  }
  if (threadIdx.x == 0) {
    for (int i = nhist - 1; i >= 0; --i) {
      double s = cvec[i];
      for (int j = i + 1; j < nhist; ++j) s -= beta[i * nhist + j] * cvec[j];
      cvec[i] = s / beta[i * nhist + i];
    }
    *status = 0;
  }
  __syncthreads();
  double* un = u + (size_t)it1 * nd;
  for (int t = threadIdx.x; t < nd; t += blockDim.x) {
    un[t] = alpha * dfn[t] + inv * (q[t] - qlast[t]);
    dqlast[t] = dq[t];
    qlast[t] = q[t];
    q[t] = q[t] + alpha * dq[t];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nd; t += blockDim.x) {
    double v = q[t];
    for (int ih = 0; ih < nhist; ++ih) {
      const int i = (first + ih - 1) % memory;
      v -= omega[i] * cvec[ih] * u[(size_t)i * nd + t];
    }
    q[t] = v;
  }
}
__global__ void k_broyden(int nd, int memory, int iter, double alpha, double* q, double* qlast,
                          const double* dq, double* dqlast, double* df, double* u, double* a,
                          double* omega, double* work, int* status) {
  broyden_dev(nd, memory, iter, alpha, q, qlast, dq, dqlast, df, u, a, omega, work, status);
}

__device__ __forceinline__ void eelec_init_dev(int nat, const double* ts, const double* eband, double* eelec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nat) eelec[i] = *ts / nat + eband[i];
}
__global__ void k_eelec_init(int nat, const double* ts, const double* eband, double* eelec) {
  eelec_init_dev(nat, ts, eband, eelec);
}

void launch_eelec_init(int nat, const double* ts, const double* eband, double* eelec,
                       cudaStream_t s) {
  ++g_kernel_launches;
  k_eelec_init<<<(nat + 127) / 128, 128, 0, s>>>(nat, ts, eband, eelec);
}

__device__ __forceinline__ void fe_dev(int n, const double* f, const double* e, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = f[i] * e[i];
}
__global__ void k_fe(int n, const double* f, const double* e, double* out) {
  fe_dev(n, f, e, out);
}

void launch_fe(int n, const double* f, const double* e, double* out, cudaStream_t s) {
  ++g_kernel_launches;
  k_fe<<<(n + 255) / 256, 256, 0, s>>>(n, f, e, out);
}

void launch_broyden_next(BroydenState& b, cudaStream_t s) {
  b.iter += 1;
  ++g_kernel_launches;
  k_broyden<<<1, 1024, 0, s>>>(b.ndim, b.memory, b.iter, b.damp, b.q, b.qlast, b.dq, b.dqlast,
                               b.df, b.u, b.a, b.omega, b.work, b.status);
}

// ------------------------------------------------------------------------------------
// Wiberg/Mayer bond orders (wavefunction/mulliken.f90:176-235): for atoms A != B
//   wbo(A, B) += scale * sum_{mu in A, nu in B} (PS)_{nu mu} (PS)_{mu nu}
// one thread per atom pair; the orbitals of an atom are contiguous
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void wbo_dev(DevMol m, const double* __restrict__ PS, double* wbo,
                                        double scale) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int nat = m.nat, n = m.nao;
  if (t >= (long long)nat * nat) return;
  const int a = (int)(t / nat), b = (int)(t % nat);
  if (a == b) return;
  const int a0 = m.sh_ao[m.at_sh[a]], a1 = m.sh_ao[m.at_sh[a + 1] - 1] + 2 * m.sh_l[m.at_sh[a + 1] - 1] + 1;
  const int b0 = m.sh_ao[m.at_sh[b]], b1 = m.sh_ao[m.at_sh[b + 1] - 1] + 2 * m.sh_l[m.at_sh[b + 1] - 1] + 1;
  double s = 0.0;
  for (int mu = a0; mu < a1; ++mu)
    for (int nu = b0; nu < b1; ++nu) s += PS[(size_t)nu * n + mu] * PS[(size_t)mu * n + nu];
  wbo[t] += scale * s;
}
__global__ void k_wbo(DevMol m, const double* __restrict__ PS, double* wbo, double scale) {
  wbo_dev(m, PS, wbo, scale);
}
void launch_wbo(const DevMol& m, const double* PS, double* wbo, double scale, cudaStream_t s) {
  const long long nn = (long long)m.nat * m.nat;
  ++g_kernel_launches;
  k_wbo<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(m, PS, wbo, scale);
}

// ------------------------------------------------------------------------------------
// Parameter gradient of the converged energy (the SCF energy is stationary in the density,
// so dE/dtheta is the explicit derivative at the final P and charges):
//   self energies   H0_{mu nu} = (e_i + e_j)/2 * G_{mu nu}  =>  dE/de_s = sum_{mu in s, nu} P G'
//                   with G' = H0 built with every self energy set to one (= 2 G)
//   hardness        E2 = 1/2 sum_st q_s q_t gamma_st, gamma = (R^2 + eta_st^-2)^-1/2,
//                   eta_st = (eta_s + eta_t)/2  =>  dgamma/deta_st = eta_st^-3 (R^2+eta_st^-2)^-3/2
//   third order     E3 = sum_s Gamma_s q_s^3 / 3
// one thread per shell
// ------------------------------------------------------------------------------------
// Hp: H0 built with unit self energies; or nullptr, and then the same elements come from H0
// and the self energies se, Hp = H0 / ((e_s + e_t) / 2) (H0 is linear in the pair's mean self
// energy, which is never zero).  cn != nullptr: also out[3 nsh + s] = dE/dkcn_s = -CN_A dE/de_s
__device__ __forceinline__ void param_grad_dev(const DevMol& m, const double* __restrict__ P,
                                               const double* __restrict__ Hp,
                                               const double* __restrict__ H,
                                               const double* __restrict__ se,
                                               const double* __restrict__ cn,
                                               const double* __restrict__ qsh, double* out,
                                               double* zgrad, int s) {
  const int n = m.nao, nsh = m.nsh;
  const int o = m.sh_ao[s], no = 2 * m.sh_l[s] + 1;
  double tr = 0.0;
  for (int mu = o; mu < o + no; ++mu) {
    const double* pr = P + (size_t)mu * n;
    if (Hp) {
      const double* hr = Hp + (size_t)mu * n;
      for (int nu = 0; nu < n; ++nu) tr += pr[nu] * hr[nu];
    } else {
      const double* hr = H + (size_t)mu * n;
      const double es = se[s];
      for (int nu = 0; nu < n; ++nu) tr += pr[nu] * hr[nu] * (2.0 / (es + se[m.ao_sh[nu]]));
    }
  }
  const double qs = qsh[s], es = m.sh_hub[s];
  const int ia = m.sh_atom[s];
  double dh = 0.5 * qs * qs;  // gamma_ss = eta_s
  for (int t = 0; t < nsh; ++t) {
    if (t == s) continue;
    const int ja = m.sh_atom[t];
    double r2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double d = m.xyz[3 * ia + k] - m.xyz[3 * ja + k];
      r2 += d * d;
    }
    const double eta = 0.5 * (es + m.sh_hub[t]);
    const double ie2 = 1.0 / (eta * eta);
    const double den = r2 + ie2;
    const double g = ie2 / eta / (den * sqrt(den));
    dh += qs * qsh[t] * 0.5 * g;
  }
  out[s] = tr;
  out[nsh + s] = dh;
  out[2 * nsh + s] = qs * qs * qs / 3.0;
  if (cn) out[3 * nsh + s] = -cn[ia] * tr;
  if (zgrad) zgrad[s] = 0.0;  // accumulated by the Slater-exponent kernel that follows
}
__global__ void k_param_grad(DevMol m, Gfn2Scalars p, const double* __restrict__ P,
                             const double* __restrict__ Hp, const double* __restrict__ qsh,
                             double* out /* [3][nsh]: dse, dhub, dgam3 */) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= m.nsh) return;
  param_grad_dev(m, P, Hp, nullptr, nullptr, nullptr, qsh, out, nullptr, s);
  (void)p;
}
void launch_param_grad(const DevMol& m, const Gfn2Scalars& p, const double* P, const double* Hp,
                       const double* qsh, double* out, cudaStream_t s) {
  ++g_kernel_launches;
  k_param_grad<<<(m.nsh + 127) / 128, 128, 0, s>>>(m, p, P, Hp, qsh, out);
}

// ------------------------------------------------------------------------------------
// Batched launches: blockIdx.z walks the listed molecules; each block runs the same body as
// the one-molecule kernel on that molecule's slices.  Blocks past a molecule's own size exit
// through the bodies' bounds checks (or the explicit tile checks below).
// ------------------------------------------------------------------------------------
#define BMOL const MolPtrs& q = mp[list[blockIdx.z]]
#define BARGS const MolPtrs* __restrict__ mp, const int* __restrict__ list

__global__ void kb_param_grad(BARGS) {
  BMOL;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (!q.param_grad || s >= q.m.nsh) return;
  param_grad_dev(q.m, q.P, nullptr, q.H, q.se, q.cn, q.qsh_o, q.pgrad, q.zgrad, s);
}
static inline dim3 bgrid(unsigned x, const BatchLaunch& b, unsigned y = 1);
void launch_param_grad_b(const BatchLaunch& b) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_param_grad<<<bgrid((b.nsh_max + 127) / 128, b), 128, 0, b.s>>>(b.mp, b.list);
}
static inline dim3 bgrid(unsigned x, const BatchLaunch& b, unsigned y) {
  return dim3(x > 0 ? x : 1, y, (unsigned)b.count);
}

__global__ void kb_cn(BARGS, Gfn2Scalars p) {
  BMOL;
  cn_dev(q.m, p, q.cn);
}
void launch_cn_b(const BatchLaunch& b, const Gfn2Scalars& p) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_cn<<<bgrid((b.nat_max * 32 + 63) / 64, b), 64, 0, b.s>>>(b.mp, b.list, p);
}

__global__ void kb_cn_grad(BARGS, Gfn2Scalars p) {
  BMOL;
  if (q.m.nat == 1) return;
  cn_grad_dev(q.m, p, q.dEdcn, q.grad, q.sig_at);
}
void launch_cn_grad_b(const BatchLaunch& b, const Gfn2Scalars& p) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_cn_grad<<<bgrid((b.nat_max * 32 + 63) / 64, b), 64, 0, b.s>>>(b.mp, b.list, p);
}

__global__ void kb_levels(BARGS, Gfn2Scalars p) {
  BMOL;
  levels_dev(q.m, p, q.cn, q.se, q.mrad, q.dmrdcn);
}
void launch_setup_levels_b(const BatchLaunch& b, const Gfn2Scalars& p) {
  if (!b.count) return;
  const int nt = b.nsh_max > b.nat_max ? b.nsh_max : b.nat_max;
  ++g_kernel_launches;
  kb_levels<<<bgrid((nt + 127) / 128, b), 128, 0, b.s>>>(b.mp, b.list, p);
}

__global__ void kb_coulomb_table(BARGS, Gfn2Scalars p) {
  BMOL;
  coulomb_table_dev(q.m, p, q.mrad, q.ctab);
}
void launch_coulomb_table_b(const BatchLaunch& b, const Gfn2Scalars& p) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_coulomb_table<<<bgrid((b.nat_max * 32 + 63) / 64, b), 64, 0, b.s>>>(b.mp, b.list, p);
}

template <int MODE>
__global__ void kb_coulomb(BARGS, Gfn2Scalars p) {
  BMOL;
  if (MODE == 0)
    coulomb_dev<0>(q.m, p, q.mrad, q.qsh, q.qat, q.dpat, q.qpat, q.vsh, q.vat, q.vdp, q.vqp,
                   nullptr, q.ctab);
  else
    coulomb_dev<1>(q.m, p, q.mrad, q.qsh_o, q.qat_o, q.dpat_o, q.qpat_o, nullptr, nullptr,
                   nullptr, nullptr, q.eelec, q.ctab);
}
void launch_coulomb_potential_b(const BatchLaunch& b, const Gfn2Scalars& p) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_coulomb<0><<<bgrid((b.nat_max * 32 + 63) / 64, b), 64, 0, b.s>>>(b.mp, b.list, p);
}
void launch_coulomb_energy_b(const BatchLaunch& b, const Gfn2Scalars& p) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_coulomb<1><<<bgrid((b.nat_max * 32 + 63) / 64, b), 64, 0, b.s>>>(b.mp, b.list, p);
}

__global__ void kb_coulomb_grad(BARGS, Gfn2Scalars p) {
  BMOL;
  if (q.m.nat == 1) return;
  coulomb_grad_dev(q.m, p, q.mrad, q.dmrdcn, q.qsh_o, q.qat_o, q.dpat_o, q.qpat_o, q.grad,
                   q.sig_at, q.dEdcn);
}
void launch_coulomb_gradient_b(const BatchLaunch& b, const Gfn2Scalars& p) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_coulomb_grad<<<bgrid((b.nat_max * 32 + 63) / 64, b), 64, 0, b.s>>>(b.mp, b.list, p);
}

__global__ void kb_repulsion(BARGS, Gfn2Scalars p) {
  BMOL;
  repulsion_dev(q.m, p, q.erep, q.grad, q.sig_at);
}
void launch_repulsion_b(const BatchLaunch& b, const Gfn2Scalars& p) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_repulsion<<<bgrid((b.nat_max * 32 + 63) / 64, b), 64, 0, b.s>>>(b.mp, b.list, p);
}

__global__ void kb_vao(BARGS) {
  BMOL;
  vao_dev(q.m, q.vsh, q.vat, q.vao);
}
void launch_vao_b(const BatchLaunch& b) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_vao<<<bgrid((b.nao_max + 255) / 256, b), 256, 0, b.s>>>(b.mp, b.list);
}

__global__ void __launch_bounds__(256) kb_fock(BARGS) {
  BMOL;
  const int n = q.m.nao;
  if ((int)blockIdx.x * 32 >= n || (int)blockIdx.y * 32 >= n) return;  // tile outside
  fock_dev(n, q.m.ao_at, q.H, q.S, q.with_mp ? q.D : nullptr, q.Q, q.vao, q.vdp, q.vqp, q.F);
}
void launch_fock_b(const BatchLaunch& b) {
  if (!b.count) return;
  const unsigned nt = (b.nao_max + 31) / 32;
  ++g_kernel_launches;
  kb_fock<<<bgrid(nt, b, nt), dim3(32, 8), 0, b.s>>>(b.mp, b.list);
}

__global__ void __launch_bounds__(128) kb_mull_partial(BARGS) {
  BMOL;
  if ((int)blockIdx.y >= q.mull_chunks) return;
  mull_partial_dev(q.m.nao, q.P, q.S, q.H, q.D, q.Q, q.mull);
}
__global__ void kb_mull_reduce(BARGS) {
  BMOL;
  mull_reduce_dev(q.m, q.mull, q.mull_chunks, q.qsh_o, q.qat_o, q.dpat_o, q.qpat_o, q.eband);
}
void launch_mulliken_b(const BatchLaunch& b) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_mull_partial<<<bgrid((b.nao_max + 127) / 128, b, mulliken_chunks(b.nao_max)), 128, 0,
                    b.s>>>(b.mp, b.list);
  ++g_kernel_launches;
  kb_mull_reduce<<<bgrid((b.nat_max + 127) / 128, b), 128, 0, b.s>>>(b.mp, b.list);
}

__global__ void kb_fermi(BARGS) {
  BMOL;
  const int n = q.m.nao;
  fermi_dev(n, q.emo, q.nalp, q.nbet, q.kt, q.focc + n, q.focc + 2 * n, q.focc, q.scal, q.icount,
            q.nev);
  // too few levels computed for this Fermi level: the molecule leaves for the one-molecule path
  if (threadIdx.x == 0 && q.icount[1] != 0) *q.flag = -3;
}
void launch_fermi_b(const BatchLaunch& b) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_fermi<<<bgrid(1, b), 1024, 0, b.s>>>(b.mp, b.list);
}

__global__ void kb_pack(BARGS, int output) {
  BMOL;
  const int nmp = q.with_mp ? q.m.nat : 0;
  if (output)
    pack_dev(q.m.nsh, nmp, q.qsh_o, q.dpat_o, q.qpat_o, q.vec_out);
  else
    pack_dev(q.m.nsh, nmp, q.qsh, q.dpat, q.qpat, q.bq);
}
void launch_pack_b(const BatchLaunch& b, bool output) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_pack<<<bgrid((b.nd_max + 255) / 256, b), 256, 0, b.s>>>(b.mp, b.list, output ? 1 : 0);
}

__global__ void kb_unpack(BARGS) {
  BMOL;
  unpack_dev(q.m, q.bq, q.qsh, q.qat, q.dpat, q.qpat, q.with_mp);
}
void launch_unpack_b(const BatchLaunch& b) {
  if (!b.count) return;
  const int nt = b.nsh_max > 6 * b.nat_max ? b.nsh_max : 6 * b.nat_max;
  ++g_kernel_launches;
  kb_unpack<<<bgrid((nt + 255) / 256, b), 256, 0, b.s>>>(b.mp, b.list);
}

__global__ void kb_diff(BARGS) {
  BMOL;
  diff_dev(q.nd, q.vec_out, q.bq, q.bdq, q.scal + 1);
}
void launch_diff_b(const BatchLaunch& b) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_diff<<<bgrid(1, b), 1024, 0, b.s>>>(b.mp, b.list);
}

__global__ void kb_broyden(BARGS, int iter) {
  BMOL;
  broyden_dev(q.nd, q.memory, iter, q.damp, q.bq, q.bqlast, q.bdq, q.bdqlast, q.bdf, q.bu, q.ba,
              q.bomega, q.bwork, q.bstatus);
}
void launch_broyden_b(const BatchLaunch& b, int iter) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_broyden<<<bgrid(1, b), 1024, 0, b.s>>>(b.mp, b.list, iter);
}

__global__ void kb_eelec_init(BARGS) {
  BMOL;
  eelec_init_dev(q.m.nat, q.scal, q.eband, q.eelec);
}
void launch_eelec_init_b(const BatchLaunch& b) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_eelec_init<<<bgrid((b.nat_max + 127) / 128, b), 128, 0, b.s>>>(b.mp, b.list);
}

// convergence test of the single-point driver (xtb/singlepoint.f90:300-304), one thread per
// molecule: the electronic energy is summed in atom order, as the one-molecule driver does
__global__ void kb_converge(BARGS) {
  BMOL;
  if (threadIdx.x != 0 || *q.flag < 0) return;
  double e = 0.0;
  for (int i = 0; i < q.m.nat; ++i) e += q.eelec[i];
  const double elast = q.conv[1];
  q.conv[0] = elast;
  q.conv[1] = e;
  q.conv[2] = q.scal[1];
  if (*q.bstatus != 0) {
    *q.flag = -1;
    return;
  }
  const bool ok = fabs(e - elast) < q.econv && q.scal[1] < q.pconv;
  *q.flag = ok ? 1 : 0;
}
void launch_converge_b(const BatchLaunch& b) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_converge<<<bgrid(1, b), 32, 0, b.s>>>(b.mp, b.list);
}

__global__ void kb_fe(BARGS) {
  BMOL;
  fe_dev(q.m.nao, q.focc, q.emo, q.vec_out);
}
__global__ void kb_wbo(BARGS, int channel) {
  BMOL;
  if (q.wbo_ch <= channel) return;
  wbo_dev(q.m, q.scratch, q.wbo + (size_t)channel * q.m.nat * q.m.nat, q.wbo_ch == 2 ? 2.0 : 1.0);
}
void launch_wbo_b(const BatchLaunch& b, int channel) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_wbo<<<bgrid((unsigned)(((long long)b.nat_max * b.nat_max + 255) / 256), b), 256, 0, b.s>>>(
      b.mp, b.list, channel);
}

void launch_fe_b(const BatchLaunch& b) {
  if (!b.count) return;
  ++g_kernel_launches;
  kb_fe<<<bgrid((b.nao_max + 255) / 256, b), 256, 0, b.s>>>(b.mp, b.list);
}

#undef BMOL
#undef BARGS

}  // namespace tb
