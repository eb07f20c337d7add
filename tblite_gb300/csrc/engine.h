// Internal interfaces of the GB300 GFN2-xTB engine (not part of the public C ABI).
//
// Layout conventions shared by all kernels (row-major, FP64):
//   S[n][n], H[n][n], F[n][n], P[n][n]   symmetric AO matrices
//   D[3][n][n], Q[6][n][n]              multipole integrals, operator on the atom of the
//                                       COLUMN index (the reference stores dpint(k, j, i)
//                                       with the operator on the atom of i)
//   C (eigenvectors) column-major: C[m*n + r] = coefficient of AO r in orbital m
//   Q components: xx, xy, yy, xz, yz, zz (traceless, 3/2 M - 1/2 tr M)
//   spherical p order (y, z, x); spherical d order (xy, yz, z2, xz, x2-y2)
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

namespace tb {

// number of engine kernels launched since library load (instrumentation)
extern std::atomic<unsigned long long> g_kernel_launches;
// algorithmic FP64 work (flop) issued to the one-molecule split GEMM since library load:
// 2 M N K per product, N (N + 1) K for a symmetric one (instrumentation)
extern std::atomic<unsigned long long> g_split_flops;

// wait for the stream with a blocking-sync event (the host thread sleeps instead of spinning)
void stream_wait(cudaStream_t s);

// streaming multiprocessors of the current device (cached per device)
int device_sm_count();

// per-kernel CUDA-event timing (only while profiling is enabled): prof_kbegin records an event
// on s and returns a token (-1 when disabled); prof_kend closes it for the given slot
enum { KS_TRIDIAG = 0, KS_MULTISECT, KS_INVIT, KS_BACKTRANSFORM, KS_GEMM, KS_FOCK, KS_MULLIKEN,
       KS_PIPE,       // batched products on the pipelined split GEMM (squarings and sites)
       KS_PIPE_PREP,  // their operands: projection steps, exponents and slice images
       KS_COUNT };
int prof_kbegin(cudaStream_t s);
void prof_kend(int slot, int token, cudaStream_t s);
void prof_reset();    // clear the kernel and phase records
bool prof_enabled();  // per-kernel events are being recorded
void prof_collect();  // after a stream wait: turn the recorded events into times

constexpr int MAXG = 12;    // max primitives per shell
constexpr int MAXL = 2;     // max angular momentum handled by the kernels
constexpr double INTCUT = 25.0;  // integral_cutoff(acc) is always 25 in the reference

// Device view of one molecule + GFN2 parameters (all pointers are device pointers).
struct DevMol {
  int nat, nsh, nao;
  const double* xyz;       // [nat][3]
  const int* at_z;         // [nat]
  const int* at_sh;        // [nat+1]
  const int* sh_atom;      // [nsh]
  const int* sh_l;         // [nsh]
  const int* sh_nprim;     // [nsh]
  const double* sh_alpha;  // [nsh][MAXG]
  const double* sh_coeff;  // [nsh][MAXG]
  const int* sh_ao;        // [nsh]
  const int* ao_sh;        // [nao]
  const int* ao_at;        // [nao]
  const double* sh_se0;    // base self energy
  const double* sh_kcn;    // CN shift (Hartree per CN)
  const double* sh_shpoly; // shell polynomial
  const double* sh_zeta;   // Slater exponent
  const double* sh_hub;    // shell hardness
  const double* sh_gam3;   // shell Hubbard derivative
  const double* sh_refocc; // reference occupation
  const double* at_en;     // Pauling EN (external data)
  const double* at_rad;    // atomic radius for the H0 polynomial (external data)
  const double* at_rcov;   // covalent radius for the CN (external data)
  const double* at_mprad;  // AES base radius
  const double* at_vcn;    // AES valence CN
  const double* at_dkern;  // AES dipole kernel
  const double* at_qkern;  // AES quadrupole kernel
  const double* at_repa;   // repulsion alpha
  const double* at_repz;   // repulsion zeff
  const int* sh_valence;   // GFN1: 1 for the first shell of its angular momentum on the atom
  const double* at_gam3;   // GFN1: atom-resolved third-order hardness derivative
};

// method constants of the tight-binding Hamiltonian (GFN2-xTB, or GFN1-xTB with method = 1)
struct Gfn2Scalars {
  int method;      // 2 GFN2-xTB, 1 GFN1-xTB
  int harmonic;    // hardness average of shell pairs: 0 arithmetic (GFN2), 1 harmonic (GFN1)
  int third_atom;  // third order on atomic charges (GFN1) instead of shell charges (GFN2)
  int aes;         // anisotropic electrostatics (GFN2 only)
  int pair_mode;   // GFN1 form: 1 the GFN1-xTB element-pair factors, 0 the d-block rule only
                   // (IPEA1-xTB)
  double kdiff;    // GFN1 H0 scale involving polarisation shells
  double cn_exp_k; // GFN1 coordination number: exponential counting steepness
  double wexp, enscale, gexp;
  double kshell[5][5];
  double mp_dmp3, mp_dmp5, mp_shift, mp_kexp, mp_rmax;
  double rep_kexp, rep_kexp_light, rep_rexp, rep_cutoff;
  double cn_ka, cn_kb, cn_rshift, cn_cutoff;
  double h0_cutoff;  // real-space cutoff of the integral pair list
};

// D4 dispersion data, per atom (device pointers) + model constants
constexpr int D4_MREF = 7;
struct DevD4 {
  int nsp;
  const int* sp;          // [nat] species index
  const int* nref;        // [nat]
  const int* ngw;         // [nat][MREF]
  const double* refcn;    // [nat][MREF]
  const double* refq;     // [nat][MREF]
  const double* zeff;     // [nat]
  const double* gam;      // [nat]
  const double* r4r2;     // [nat]
  const double* rcov;     // [nat]
  const double* en;       // [nat]
  const double* c6ref;    // [nsp][MREF][nsp][MREF]
  double ga, gc, wf, kn, k4, k5, k6, cn_cutoff, disp2_cutoff, disp3_cutoff, atm_alpha;
  double s6, s8, a1, a2, s9;
};
struct D4Work {  // device scratch
  double *cn, *gw, *dgw, *gwv, *dgwdq, *dgwv_cn, *c6, *dc6, *e3, *dEdcn;
  double* atm;  // [8][nat][nat] pair tables and pair derivatives of the three-body term
  double* de;   // [nat][nat] two-body damping kernel of each ordered pair (0 beyond the cutoff),
                // or nullptr: the pair kernels evaluate it
};
// geometry setup: CN, weights, atomic C6 at q = 0, three-body energy (e3) and, with grad,
// its gradient and dEdcn (w.dEdcn is reset here)
void d4_setup(const DevMol& m, const DevD4& d, D4Work& w, bool grad, double* grad_out,
              double* sig_at, cudaStream_t s);
void d4_potential(const DevMol& m, const DevD4& d, D4Work& w, const double* qat, double* vat,
                  cudaStream_t s);
void d4_energy(const DevMol& m, const DevD4& d, D4Work& w, const double* qat, double* eat,
               cudaStream_t s);
// two-body gradient at the final charges + the D4 CN chain rule (uses w.dEdcn from setup)
void d4_gradient(const DevMol& m, const DevD4& d, D4Work& w, const double* qat, double* grad,
                 double* sig_at, cudaStream_t s);

// D3(BJ) two-body dispersion of GFN1-xTB (no three-body term): per atom data, model
// constants and scratch (device pointers)
struct DevD3 {
  int nsp;
  const int* sp;        // [nat] species index
  const int* nref;      // [nat]
  const double* refcn;  // [nat][D4_MREF]
  const double* c6ref;  // [nsp][D4_MREF][nsp][D4_MREF] reference C6 per species pair
  const double* r4r2;   // [nat]
  const double* rcov;   // [nat]
  double k1, k3, cn_cutoff, cutoff, s6, s8, a1, a2;
  double *cn, *dEdcn;   // [nat] scratch
  double *w, *dw;       // [nat][D4_MREF] scratch: normalised weights and their CN derivatives
};
// energy (added to eat) and, with grad, gradient and per-atom virial partials
void d3_energy_gradient(const DevMol& m, const DevD3& d, bool grad, double* eat, double* grad_out,
                        double* sig_at, cudaStream_t s);

// Implicit solvation (ALPB + CDS + shift), per atom device data + model constants
constexpr int SOLV_MAXNB = 512;    // surface-grid neighbours per atom
constexpr int SOLV_NGRID = 230;    // Lebedev points per atom
constexpr int SOLV_MAXSHELL = 32;  // partners in the smoothing shell of one grid point
struct DevSolv {
  int nat;
  int kernel;  // Born interaction kernel: 1 Still, 2 P16
  int cds;     // surface term present (else the surface kernels do not run, surfaces are 0)
  double lrcut, srcut, keps, alpbet, adet, born_scale, ah0, ah1, ah3, shift;
  const double *vdwr, *rho, *svdw, *vdwsa, *wrp, *trj2_lo, *trj2_hi, *tension, *hbond;
  const double* grid;  // [230][4]: x, y, z, weight (x 4 pi)
  double *brad, *dscale, *wbr, *surface;
  int *nbl, *nnb;
  int* status;  // 0 ok; 1 neighbour list overflow; 2 smoothing shell overflow
};
// Born radii, surface neighbour list, surfaces; adds surface tension + shift energies to eat
void solv_setup(const DevSolv& v, const double* xyz, double* eat, cudaStream_t s);
void solv_potential(const DevSolv& v, const double* xyz, const double* qat, double* vat,
                    cudaStream_t s);
void solv_energy(const DevSolv& v, const double* xyz, const double* qat, double* eat,
                 cudaStream_t s);
// ALPB pair + Born-radius chain rule + surface terms (the shape term is added on the host)
void solv_gradient(const DevSolv& v, const double* xyz, const double* qat, double* grad,
                   cudaStream_t s);

// Kernel launchers (defined in the .cu files).  All run on `stream`.
void launch_cn(const DevMol& m, const Gfn2Scalars& p, double* cn, cudaStream_t s);
void launch_cn_grad(const DevMol& m, const Gfn2Scalars& p, const double* dEdcn, double* grad,
                    double* sigma, cudaStream_t s);
void launch_setup_levels(const DevMol& m, const Gfn2Scalars& p, const double* cn,
                         double* selfenergy, double* mrad, double* dmrdcn, cudaStream_t s);
void launch_build_h0(const DevMol& m, const Gfn2Scalars& p, const double* selfenergy, double* S,
                     double* H, double* D, double* Q, cudaStream_t s);
void launch_h0_gradient(const DevMol& m, const Gfn2Scalars& p, const double* selfenergy,
                        const double* P, const double* W, const double* vao, const double* vdp,
                        const double* vqp, double* grad, double* sigma, double* dEdcn,
                        cudaStream_t s);
void launch_repulsion(const DevMol& m, const Gfn2Scalars& p, double* erep, double* grad,
                      double* sigma, cudaStream_t s);
// electrostatics: potentials from (qsh, qat, dpat, qpat)
// homogeneous electric field E (host array of 3): vat -= E.R_A, vdp -= E; energies
// eat -= E.R_A q_A + E.mu_A (external/field.f90)
void launch_field_potential(int nat, const double* xyz, const double* efield, double* vat,
                            double* vdp, cudaStream_t s);
void launch_field_energy(int nat, const double* xyz, const double* efield, const double* qat,
                         const double* dpat, double* eat, cudaStream_t s);
void launch_coulomb_potential(const DevMol& m, const Gfn2Scalars& p, const double* mrad,
                              const double* qsh, const double* qat, const double* dpat,
                              const double* qpat, double* vsh, double* vat, double* vdp,
                              double* vqp, cudaStream_t s);
// per-atom electrostatic energy (es2 + es3 + AES incl. kernels), added into eat
void launch_coulomb_energy(const DevMol& m, const Gfn2Scalars& p, const double* mrad,
                           const double* qsh, const double* qat, const double* dpat,
                           const double* qpat, double* eat, cudaStream_t s);
void launch_coulomb_gradient(const DevMol& m, const Gfn2Scalars& p, const double* mrad,
                             const double* dmrdcn, const double* qsh, const double* qat,
                             const double* dpat, const double* qpat, double* grad, double* sigma,
                             double* dEdcn, cudaStream_t s);
void launch_vao(const DevMol& m, const double* vsh, const double* vat, double* vao, cudaStream_t s);
void launch_fock(int n, const int* ao_at, const double* H, const double* S, const double* D,
                 const double* Q, const double* vao, const double* vdp, const double* vqp,
                 double* F, cudaStream_t s);
// Mulliken analysis + band energy: column partial sums then per-shell/atom reduction
void launch_mulliken(const DevMol& m, const double* P, const double* S, const double* H,
                     const double* D, const double* Q, double* partial, int nchunk,
                     double* qsh, double* qat, double* dpat, double* qpat, double* eat_band,
                     cudaStream_t s);
int mulliken_chunks(int n);

// Fermi filling of both spin channels; writes focc (alpha+beta), ts (entropy term) to scal[0]
// nocc_cols[0]: orbitals with non-zero occupation; nocc_cols[1] = 1 when the nev computed
// eigenvalues do not reach 51 kT above the Fermi level (all n are then needed)
void launch_fermi(int n, const double* emo, double nalp, double nbet, double kt, double* focc,
                  double* ts, int* nocc_cols, cudaStream_t s, int nev = 0);

// Broyden mixer (reference scf/mixer/broyden.f90)
struct BroydenState {
  int ndim, memory, iter;
  double damp;
  double *q, *qlast, *dq, *dqlast, *df, *u, *a, *omega;  // device
  double* work;   // device scratch [memory*memory + 2*memory + 64]
  int* status;    // device status word (0 ok, !=0 singular)
};
void launch_broyden_next(BroydenState& b, cudaStream_t s);
// with_mp: the mixer vector holds the atomic multipoles too (GFN2); GFN1 mixes shell charges
void launch_pack(const DevMol& m, const double* qsh, const double* dpat, const double* qpat,
                 double* vec, cudaStream_t s, bool with_mp = true);
void launch_unpack(const DevMol& m, const double* vec, double* qsh, double* qat, double* dpat,
                   double* qpat, cudaStream_t s, bool with_mp = true);
// dq = vec_out - q ; err2 = sum(dq^2)/ndim (into *err)
void launch_diff(int ndim, const double* vec_out, const double* q, double* dq, double* err,
                 cudaStream_t s);

// eigen solver (generalised, Cholesky reduced)
struct EigenSolver;
EigenSolver* eigen_create(int n, cudaStream_t s);
void eigen_destroy(EigenSolver*);
// largest order the solver's buffers hold; eigen_resize switches to any order up to it
int eigen_capacity(const EigenSolver*);
void eigen_resize(EigenSolver*, int n);
// factorise S once per geometry; returns 0 on success, >0 if S is not positive definite
int eigen_set_overlap(EigenSolver*, const double* S);
// eigenvalues (ascending) of F C = S C e; keeps the tridiagonal form for eigen_vectors.
// Only the nev lowest are computed (nev <= 0: all); e[nev..n) = 1e300, which the Fermi
// filling treats as empty.  eigen_values_rest fills in e[nev..n) from the kept form.
int eigen_values(EigenSolver*, const double* F, double* e, int nev = 0);
void eigen_values_rest(EigenSolver*, int nev, double* e);
// eigenvalues needed during the SCF: all occupied levels, the first empty one and a margin
inline int scf_eigenvalue_count(int n, double nalp) {
  const int occ = (int)nalp + 1;  // ceil(nalp) or more
  const int m = occ + 1 + (n / 64 > 4 ? n / 64 : 4);
  return m < n ? m : n;
}
// the k lowest eigenvectors, C column-major [k][n] (S-orthonormal)
void eigen_vectors(EigenSolver*, int k, double* C);
// eigenvectors k0 .. k1-1 into columns k0 .. k1-1 of C (same tridiagonal form)
void eigen_vectors_range(EigenSolver*, int k0, int k1, double* C);

// pipelined split GEMM (ozaki_pipe.cu): a matrix is split once into a slice image (per line a
// power-of-two exponent and eight BF16 slices in the tensor cores' shared-memory layout), then
// C = op(A) op(B) runs from two images
struct PImage {
  int lines = 0, K = 0;
  uint16_t* data = nullptr;  // pimage_bytes(lines, K) bytes
  int* e = nullptr;          // pimage_lines(lines) ints
};
size_t pimage_bytes(int lines, int K);
int pimage_lines(int lines);
// line i, position k: M[i + k ld] (kcontig 0) or M[k + i ld] (kcontig 1)
void psplit(const double* M, int ld, int kcontig, int lines, int K, PImage& img, cudaStream_t s);
// C = 2^eshiftA op(A) op(B); sym: symmetric product (lower tiles computed, mirrored); status
// set to 1 if a wait of the tensor-core pipeline ran out
void pgemm(const PImage& A, const PImage& B, double* C, int ldc, bool sym, int* status,
           cudaStream_t s, int eshiftA = 0);

// density by spectral projection (purify.cu): closed-shell, gapped systems at large n
struct Purifier;
Purifier* purify_create(int n, cudaStream_t s);
void purify_destroy(Purifier*);
int purify_capacity(const Purifier*);
// Loewdin orthogonaliser S^-1/2 once per geometry: Newton-Schulz iterations, -1 on failure
int purify_set_overlap(Purifier*, const double* S);
// P = 2 (projector on the nocc lowest orbitals of F C = S C e): SP2 iterations, -1 on failure
int purify_density(Purifier*, const double* F, int nocc, double* P);
// W = P F P / 2 after purify_density
void purify_weighted(Purifier*, const double* F, const double* P, double* W);
// C = A B on the split GEMM (n x n, column-major)
void purify_product(Purifier*, const double* A, const double* B, double* C);
// HOMO, LUMO and the bound on their errors (Lanczos) of the last purify_density call
void purify_gap(Purifier*, double* gap3);
// smallest certified gap in kT; the purifier's tensor-core GEMM status word
double purify_gap_kt();
int* purify_status(Purifier*);
int purify_iterations(const Purifier*);

// dense FP64 GEMM (column-major, BLAS semantics); kmode skips zero triangles
// KM_SYM (or-ed with one of the others): the product is symmetric (M == N); only the tiles on
// and below the diagonal are computed and each is also written to its mirror position
// returns the status of its own launch (not an earlier error of another launch)
enum { KM_NONE = 0, KM_LT_COLEND = 1, KM_LT_ROWEND = 2, KM_GE_ROWBEG = 3, KM_SYM = 8 };
cudaError_t gemm64(bool ta, bool tb, int M, int N, int K, double alpha, const double* A, int lda,
            const double* B, int ldb, double beta, double* C, int ldc, int kmode, cudaStream_t s);

// eelec[i] = ts/nat + eband[i]
void launch_eelec_init(int nat, const double* ts, const double* eband, double* eelec,
                       cudaStream_t s);
// out[m] = f[m] * e[m]
void launch_fe(int n, const double* f, const double* e, double* out, cudaStream_t s);

// dense helpers
// P = C diag(f) C^T over k columns; with status (a device int of the eigensolver) the product
// may run on the tensor cores (split GEMM), which then keeps 2n ints behind the n*k scaled
// columns in work
void density_matrix(int n, int k, const double* C, const double* f, double* P, double* work,
                    cudaStream_t s, int* status = nullptr);
// split GEMM of the one-molecule path (ozaki.cu): C = op(A) op(B), column-major, leading
// dimension ld; ex: M + ld ints of device scratch; status set to 1 if it did not complete
void ogemm(bool ta, bool tb, int M, int N, int K, const double* A, const double* B, double* C,
           int ld, int kmode, int* ex, int* status, cudaStream_t s);
// the eigensolver's tensor-core GEMM status word, and its check (synchronises the stream)
int* eigen_gemm_status(EigenSolver*);
bool eigen_gemm_failed(EigenSolver*);
// wbo[A][B] += scale * sum (PS)_{nu mu} (PS)_{mu nu} over the orbitals of atoms A != B
void launch_wbo(const DevMol& m, const double* PS, double* wbo, double scale, cudaStream_t s);
// dE/d(shell self energy, hardness, hardness derivative) into out[3][nsh]; Hp is H0 built
// with all self energies equal to one, qsh the output shell charges
void launch_param_grad(const DevMol& m, const Gfn2Scalars& p, const double* P, const double* Hp,
                       const double* qsh, double* out, cudaStream_t s);
// dE/d(Slater exponent) per shell (GFN2-xTB) at the converged P, W and potentials (integrals.cu)
void launch_zeta_grad(const DevMol& m, const Gfn2Scalars& p, const double* se, const double* P,
                      const double* W, const double* vao, const double* vdp, const double* vqp,
                      double* dz, cudaStream_t s);

// ---------------------------------------------------------------------------------------------
// Batched ensemble path: many molecules in one launch per step.  Every molecule owns a slice of
// packed device arrays; MolPtrs (in device memory, one per molecule) holds the slice pointers.
// A batched kernel walks a list of molecule indices with blockIdx.z and runs the same device
// body as the one-molecule kernel, so both paths share their arithmetic.
// ---------------------------------------------------------------------------------------------
struct MolPtrs {
  DevMol m;
  DevD4 d4;
  D4Work d4w;
  DevD3 d3;
  int has_d4, nd, mull_chunks, memory, with_mp, has_d3;
  int nev;  // eigenvalues computed per SCF iteration (the rest after convergence)
  double nalp, nbet, kt, damp, econv, pconv;
  double h0_cutoff;  // depends on the basis of the molecule (smallest exponent)
  double *cn, *se, *mrad, *dmrdcn;
  // per-geometry pair table of the electrostatics: gamma of every shell pair (nsh x nsh, row
  // = shell of the potential's atom), then the AES pair scalars g3 f3, g5 f5, g3 f5 of every
  // ordered atom pair (three nat x nat planes)
  double* ctab;
  double *S, *H, *D, *Q, *F, *P, *C, *scratch;  // F doubles as W after the SCF
  double *emo, *focc;                            // focc [3][n]: total, alpha, beta
  double *qsh, *qat, *dpat, *qpat, *qsh_o, *qat_o, *dpat_o, *qpat_o;
  double *vsh, *vat, *vdp, *vqp, *vao;
  double *mull, *eband, *eelec, *erep, *vec_out, *scal;
  int* icount;  // [0] number of orbitals with non-zero occupation
  double *bq, *bqlast, *bdq, *bdqlast, *bdf, *bu, *ba, *bomega, *bwork;
  int* bstatus;
  double *grad, *sigma, *sig_at, *dEdcn;
  // eigensolver: X = L^-T (L is built in T1), A reduced matrix / reflectors, Y vectors of T
  double *X, *A, *T1, *Y, *lu, *ed, *ee, *etau, *ew, *epv, *escal;
  int* estatus;
  double* conv;  // [0] previous electronic energy, [1] current, [2] rms(dq)
  int* flag;     // 1 converged, 0 running, <0 failed (Broyden or Cholesky), set on device
  // parameter gradient (param_grad != 0): [4][nsh] dE/d(self energy, hardness, hardness
  // derivative, CN shift) and [nsh] dE/d(Slater exponent)
  int param_grad;
  double *pgrad, *zgrad;
  // Wiberg/Mayer bond orders: channels (0 none, 1 closed shell, 2 spin up/down for a restricted
  // open shell) and the output [channels][nat][nat]
  int wbo_ch;
  double* wbo;
  // density by spectral projection (closed shells of a projection bucket, sp2.cu): the slice
  // image of the iterate (in Y) and its line exponents, a second image (the columns of op(B) of
  // a pipelined GEMM site), state doubles [8] and ints [8], partial sums of the iterate
  // [3 sp2_slot_count(nao)] (trace and the 128-bit sum of squares per block of 8 lines), and the
  // steps of the last projection for the host
  uint16_t* img;
  int* iexp;
  uint16_t* img2;
  int* iexp2;
  double* sp2s;
  int* sp2i;
  unsigned long long* sp2p;
  int* sp2steps;
  // slice images of X = L^-T, split once per geometry (projection buckets): [0] its rows (the
  // lines of op(A) = X and of op(B) = X^T), [1] its columns (op(A) = X^T, op(B) = X)
  uint16_t* ximg[2];
  int* xexp[2];
};

// one launch of a batched step: the molecules list[0..count) of one size bucket
struct BatchLaunch {
  const MolPtrs* mp;
  const int* list;
  int count;
  int nat_max, nsh_max, nao_max, nd_max;
  int sp2;        // the bucket's density comes from the spectral projection (sp2.cu)
  int sp2_steps;  // its step budget in this SCF iteration
  cudaStream_t s;
};
// batched parameter gradient of the molecules that ask for it (after the gradient phase: P, W in
// F, the last potentials): self energies from H0 / ((e_s + e_t)/2), hardness, third order, CN
// shift, Slater exponents
void launch_param_grad_b(const BatchLaunch& b);
void launch_zeta_grad_b(const BatchLaunch& b, const Gfn2Scalars& p);


// batched counterparts of the launchers above (same arithmetic, per-molecule pointers)
void launch_cn_b(const BatchLaunch& b, const Gfn2Scalars& p);
void launch_setup_levels_b(const BatchLaunch& b, const Gfn2Scalars& p);
void launch_build_h0_b(const BatchLaunch& b, const Gfn2Scalars& p);
void launch_repulsion_b(const BatchLaunch& b, const Gfn2Scalars& p);
void launch_coulomb_potential_b(const BatchLaunch& b, const Gfn2Scalars& p);
void launch_coulomb_table_b(const BatchLaunch& b, const Gfn2Scalars& p);  // once per geometry
void launch_coulomb_energy_b(const BatchLaunch& b, const Gfn2Scalars& p);
void launch_coulomb_gradient_b(const BatchLaunch& b, const Gfn2Scalars& p);
void launch_vao_b(const BatchLaunch& b);
void launch_fock_b(const BatchLaunch& b);
void launch_mulliken_b(const BatchLaunch& b);
void launch_fermi_b(const BatchLaunch& b);  // temperature per molecule (no annealing)
void launch_pack_b(const BatchLaunch& b, bool output);  // output: *_o moments -> vec_out
void launch_unpack_b(const BatchLaunch& b);
void launch_diff_b(const BatchLaunch& b);
void launch_broyden_b(const BatchLaunch& b, int iter);
void launch_eelec_init_b(const BatchLaunch& b);
void launch_converge_b(const BatchLaunch& b);  // thresholds per molecule
void launch_fe_b(const BatchLaunch& b);
void launch_wbo_b(const BatchLaunch& b, int channel);  // atom-pair sums of scratch = P_c S
void launch_h0_gradient_b(const BatchLaunch& b, const Gfn2Scalars& p);
void launch_cn_grad_b(const BatchLaunch& b, const Gfn2Scalars& p);
void d4_setup_b(const BatchLaunch& b);
void d4_potential_b(const BatchLaunch& b);
void d4_energy_b(const BatchLaunch& b);
void d4_gradient_b(const BatchLaunch& b);
void d3_setup_b(const BatchLaunch& b);  // D3 energy + gradient of the GFN1-xTB molecules
// batched FP64 GEMM at one of the fixed call sites of the SCF (operands from MolPtrs)
enum { GS_FX = 0,  // T1 = F X            (X upper triangular)
       GS_XTT,     // A = X^T T1
       GS_XY,      // C = X Y, icount columns
       GS_DENS,    // P = (C f) C^T over icount orbitals (scaled copy in scratch)
       GS_WDENS,   // W (into F) = (C f e) C^T
       GS_FS,      // scratch = F S (bond orders: F holds a spin density after the gradient)
       GS_PS,      // scratch = P S (bond orders of a closed shell without orbitals)
       GS_XD,      // T1 = 2 X D (spectral projection: D, the occupied projector of A, in Y)
       GS_PXT,     // P = T1 X^T
       GS_PF,      // T1 = P F / 2
       GS_WPFP };  // W (into F) = T1 P
void gemm_b(const BatchLaunch& b, int site);

// one GEMM site of a molecule: C = alpha op(A) op(B), column-major, leading dimension ld (the
// orbital count); op(A)(i, k) = ta ? A[k + i ld] : A[i + k ld], op(B)(k, j) = tb ? B[j + k ld]
// : B[k + j ld]; km restricts k for a triangular operand, sym marks a symmetric product
struct Site {
  int M, N, K, ld;
  const double* A;
  bool ta;
  const double* B;
  bool tb;
  double* C;
  int km;
  bool sym;
  double alpha;  // power of two applied to the product (exact)
};
#ifdef __CUDACC__
__device__ __forceinline__ Site site_of(const MolPtrs& q, int site) {
  const int n = q.m.nao, k = *q.icount;
  Site s{n, n, n, n, nullptr, false, nullptr, false, nullptr, KM_NONE, false, 1.0};
  switch (site) {
    case GS_FX: s.A = q.F; s.B = q.X; s.C = q.T1; s.km = KM_LT_COLEND; break;
    case GS_XTT:
      s.A = q.X; s.ta = true; s.B = q.T1; s.C = q.A; s.km = KM_LT_ROWEND; s.sym = true;
      break;
    case GS_XY: s.A = q.X; s.B = q.Y; s.C = q.C; s.N = k; s.km = KM_GE_ROWBEG; break;
    case GS_DENS: s.A = q.scratch; s.B = q.C; s.tb = true; s.C = q.P; s.K = k; s.sym = true; break;
    case GS_WDENS: s.A = q.scratch; s.B = q.C; s.tb = true; s.C = q.F; s.K = k; s.sym = true; break;
    case GS_FS: s.A = q.F; s.B = q.S; s.C = q.scratch; break;
    case GS_PS: s.A = q.P; s.B = q.S; s.C = q.scratch; break;
    case GS_XD: s.A = q.X; s.B = q.Y; s.C = q.T1; s.km = KM_GE_ROWBEG; s.alpha = 2.0; break;
    case GS_PXT: s.A = q.T1; s.B = q.X; s.tb = true; s.C = q.P; s.sym = true; break;
    case GS_PF: s.A = q.P; s.B = q.F; s.C = q.T1; s.alpha = 0.5; break;
    default: s.A = q.T1; s.B = q.P; s.C = q.F; s.sym = true; break;  // GS_WPFP
  }
  return s;
}
#endif
// the same sites on the pipelined split GEMM (ozaki_pipe.cu; projection buckets: operands split
// into the molecule's two slice images, then one batched product), n x n sites only
void pipe_site_b(const BatchLaunch& b, int site);
// the two slice images of X (after cholesky_inverse_b), read by the sites F X, X^T T1, X D and
// T1 X^T instead of splitting X again
void pipe_x_images_b(const BatchLaunch& b);
// the same sites on the BF16 tensor cores with FP64-accurate splitting (ozaki.cu); gemm_b
// dispatches to it for buckets of at least 128 orbitals while split_gemm_enabled
void ogemm_b(const BatchLaunch& b, int site);
extern bool g_split_gemm;
// eigensolver steps for a bucket
void cholesky_inverse_b(const BatchLaunch& b);          // S -> X (status into flag)
void eigen_values_b(const BatchLaunch& b);              // F -> emo (tridiagonal form kept)
void eigen_values_rest_b(const BatchLaunch& b);         // emo[nev..n) after convergence
void eigen_vectors_b(const BatchLaunch& b);             // icount lowest vectors into C
void density_b(const BatchLaunch& b, bool weighted);   // P (or W into F) from C, focc (, emo)
// bond orders of one spin channel (0: closed shell or spin up, 1: spin down) into MolPtrs.wbo:
// the channel's density into F, F S into scratch, then the atom-pair sums (after the gradient)
void wbo_b(const BatchLaunch& b, int channel);
// batched spectral projection (sp2.cu): P = 2 X D X^T with D the SP2 projector of A = X^T F X
// after at most `steps` squarings; the gap check after the SCF (all eigenvalues of the last
// Fock matrix in emo); W = P F P / 2 into F
void sp2_density_b(const BatchLaunch& b, int steps);
void sp2_gap_b(const BatchLaunch& b);
void sp2_weighted_b(const BatchLaunch& b);
void sp2_pipe_check_b(const BatchLaunch& b);  // flag -5 for a molecule whose pipe wait ran out
// ozaki_pipe.cu: the squaring of a projection step of the iterating molecules (D^2 on the
// tensor cores from the slice image; the next iterate D^2 or 2D - D^2 over D in Y, as signed
// 64-bit fixed point in units of 2^-55 during the projection)
void sp2_square_b(const BatchLaunch& b);
// ozaki_pipe.cu: the slice image of the iterate in Y with its exact partial sums, and the next
// decision (init: D0 from A and the Gershgorin bounds into Y first)
void sp2_slice_b(const BatchLaunch& b, bool init);
// ozaki_pipe.cu: the converged iterate (fixed point during the projection) back to FP64 in Y
void sp2_unfix_b(const BatchLaunch& b);
int sp2_slot_count(int n);  // partial-sum slots of a molecule of n orbitals (3 words each)
constexpr int SP2_MIN_NAO = 96;    // smallest orbital count that takes the projection
constexpr int SP2_MAX_STEPS = 64;  // squarings per projection at most

}  // namespace tb
