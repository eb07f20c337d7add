// Internal object layout of the C ABI (error, context, structure, calculator, result) and the
// per-calculator device workspace; shared by the one-molecule driver (capi.cpp) and the batched
// ensemble driver (batch.cpp).  Not part of the public interface.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/tblite.h"
#include "engine.h"

using namespace tb;

// --------------------------------------------------------------------------------------
// objects
// --------------------------------------------------------------------------------------
struct _tblite_error {
  std::string msg;
  bool set = false;
};

struct _tblite_context {
  std::vector<std::string> errors;
  tblite_logger_callback logger = nullptr;
  void* userdata = nullptr;
  int verbosity = 1;
  int color = 0;
  void push(const std::string& m) { errors.push_back(m); }
  void message(const std::string& m) {
    if (logger) {
      std::string tmp = m;
      logger(nullptr, tmp.data(), (int)tmp.size(), userdata);
    } else if (verbosity > 0) {
      printf("%s\n", m.c_str());
    }
  }
};

struct _tblite_structure {
  int nat = 0;
  std::vector<int> num;
  std::vector<double> xyz;  // [nat][3] Bohr
  double charge = 0.0;
  int uhf = 0;
};

namespace {

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("CUDA error '") + cudaGetErrorString(e) + "' in " + what);
}

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  void alloc(size_t count) {
    if (count <= n && p) return;
    if (p) cudaFree(p);
    p = nullptr;
    cuda_check(cudaMalloc(&p, sizeof(T) * std::max<size_t>(count, 1)), "cudaMalloc");
    n = count;
  }
  void upload(const std::vector<T>& h, cudaStream_t s) {
    alloc(h.size());
    if (!h.empty())
      cuda_check(cudaMemcpyAsync(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s),
                 "upload");
  }
  void download(std::vector<T>& h, size_t count, cudaStream_t s) const {
    h.resize(count);
    if (count)
      cuda_check(cudaMemcpyAsync(h.data(), p, sizeof(T) * count, cudaMemcpyDeviceToHost, s),
                 "download");
  }
  ~DBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

struct Workspace {
  cudaStream_t stream = nullptr;
  int nat = -1, nsh = -1, nao = -1, memory = -1;
  // static molecule/basis data
  DBuf<double> xyz, sh_alpha, sh_coeff, sh_se0, sh_kcn, sh_shpoly, sh_zeta, sh_hub, sh_gam3,
      sh_refocc, at_en, at_rad, at_rcov, at_mprad, at_vcn, at_dkern, at_qkern, at_repa, at_repz;
  DBuf<int> at_z, at_sh, sh_atom, sh_l, sh_nprim, sh_ao, ao_sh, ao_at;
  // geometry dependent
  DBuf<double> cn, se, mrad, dmrdcn, S, H, D, Q, F, C, P, W, emo, focc, scratch;
  // SCF state
  DBuf<double> qsh, qat, dpat, qpat, qsh_o, qat_o, dpat_o, qpat_o, vsh, vat, vdp, vqp, vao;
  DBuf<double> mull, eband, eelec, erep, vec_out, scal;
  DBuf<int> icount;
  // Broyden
  DBuf<double> b_q, b_qlast, b_dq, b_dqlast, b_df, b_u, b_a, b_omega, b_work;
  DBuf<int> b_status;
  // gradient
  DBuf<double> grad, sigma, sig_at, dEdcn;
  DBuf<double> wbo, ones, pgrad, zgrad;
  // GFN1 per-shell/atom data and D3 dispersion (data and work)
  DBuf<int> sh_valence, d3_nref;
  DBuf<double> at_gam3, d3_refcn, d3_c6ref, d3_r4r2, d3_rcov, d3_cn, d3_w, d3_dw, d3_dEdcn;
  DBuf<int> d3_sp;
  // implicit solvation: per-atom model arrays [9][nat], grid [230][4], work [4][nat]
  DBuf<double> sv_atom, sv_grid, sv_work;
  DBuf<int> sv_nbl, sv_nnb, sv_status;
  int sv_nat = -1;
  // D4 dispersion
  DBuf<int> d4_sp, d4_nref, d4_ngw;
  DBuf<double> d4_refcn, d4_refq, d4_zeff, d4_gam, d4_r4r2, d4_rcov, d4_en, d4_c6ref;
  DBuf<double> d4_cn, d4_gw, d4_dgw, d4_gwv, d4_dgwdq, d4_dgwv_cn, d4_c6, d4_dc6, d4_e3, d4_dEdcn,
      d4_atm;
  EigenSolver* eig = nullptr;
  Purifier* pur = nullptr;
  ~Workspace() {
    if (eig) eigen_destroy(eig);
    if (pur) purify_destroy(pur);
    if (stream) cudaStreamDestroy(stream);
  }
};

// ALPB(water) + CDS + shift model for one molecule (reference solvation/alpb.f90, cds.f90,
// shift.f90 with the gfn2 water parameters), built by tblite_new_alpb_solvation_solvent
struct SolvModel {
  int nat = 0, state = 1;
  int kernel = 2;    // Born interaction kernel: 1 Still, 2 P16 (alpb.f90:45-51)
  bool cds = true;   // surface (CDS) term present; the dielectric-constant models have none
  double keps = 0, alpbet = 0, born_scale = 0, lrcut = 0, srcut = 0, ah0 = 0, ah1 = 0, ah3 = 0;
  double shift = 0;  // total free-energy shift (Hartree)
  std::vector<double> vdwr, rho, svdw, vdwsa, wrp, trj2_lo, trj2_hi, tension, hbond;
  std::vector<double> grid;  // [230][4]
};

struct _tblite_container {
  std::unique_ptr<SolvModel> solv;
  bool field = false;  // a homogeneous electric field (tblite_new_electric_field)
  double efield[3] = {0.0, 0.0, 0.0};
};

// global constants of the calculator's Hamiltonian, from its parametrisation record
struct ModelConstants {
  double wexp = 0.0, enscale = 0.0, kpol = 2.0;
  double ksh[5][5] = {};
  double gexp = 0.0;
  double rep_kexp = 0.0, rep_klight = 0.0;
  double dmp3 = 0.0, dmp5 = 0.0, mp_kexp = 0.0, mp_shift = 0.0, mp_rmax = 0.0;
  double s6 = 1.0, s8 = 0.0, a1 = 0.0, a2 = 0.0, s9 = 0.0;
  int pair_mode = 1;  // GFN1 form: 1 GFN1-xTB element-pair factors, 0 the d-block rule only
};

struct _tblite_calculator {
  // molecule-bound basis (built at construction)
  int nat = 0, nsh = 0, nao = 0;
  std::vector<int> at_z, at_sh, sh_atom, sh_l, sh_nprim, sh_ao, ao_sh, ao_at;
  // method form: 2 GFN2-xTB, 1 GFN1-xTB
  int method = 2;
  ModelConstants model;
  std::vector<int> sh_valence;   // GFN1: first shell of its angular momentum on the atom
  std::vector<double> at_gam3;   // GFN1: atom-resolved third-order hardness derivative
  // D3 data per atom (GFN1, molecules with pairs)
  bool has_d3 = false;
  std::vector<int> d3_nref;
  int d3_nsp = 0;
  std::vector<int> d3_sp;
  std::vector<double> d3_refcn, d3_c6ref, d3_r4r2, d3_rcov;
  // D4 data per atom (empty for a single atom: no pairs, no dispersion)
  bool has_d4 = false;
  int d4_nsp = 0;
  std::vector<int> d4_sp, d4_nref, d4_ngw;
  std::vector<double> d4_refcn, d4_refq, d4_zeff, d4_gam, d4_r4r2, d4_rcov, d4_en, d4_c6ref;
  std::vector<double> sh_alpha, sh_coeff, sh_se0, sh_kcn, sh_shpoly, sh_zeta, sh_hub, sh_gam3,
      sh_refocc, at_en, at_rad, at_rcov, at_mprad, at_vcn, at_dkern, at_qkern, at_repa, at_repz;
  double min_alpha = 1e300;
  std::vector<int> sh_pqn;  // principal quantum number of each shell (STO-nG expansion)
  // settings (reference api/calculator.f90:78-89, scf/mixer/input.f90:28-34)
  double accuracy = 1.0;
  double etemp = 300.0 * 3.166808578545117e-06;
  int max_iter = 250;
  double damping = 0.4;
  int memory = 0;
  int guess = TBLITE_GUESS_SAD;
  int save_integrals = 0;
  bool anneal = false;
  double anneal_kt = 0.0;
  int anneal_hold = 50, anneal_cycles = 50;
  // shell parameters changed through the extension API: re-upload before the next single point
  bool params_dirty = false;
  // evaluate dE/d(shell parameters) with the single point
  int param_grad = 0;
  // density solver: 0 diagonalisation (Fermi filling), 1 spectral projection (purify.cu)
  int density_solver = 0;
  // fault injected on the host for tests: 1 = the overlap factorisation reports a pivot that is
  // not positive (what a singular overlap, e.g. from coincident atoms, produces)
  int fault = 0;
  // post-processing of every single point, in order ("bond-orders", "molmom"); an empty list
  // becomes the reference's default (bond orders and molecular moments) at the first single
  // point (api/calculator.f90:668-675)
  std::vector<std::string> post_proc;
  bool wants(const char* name) const {
    return std::find(post_proc.begin(), post_proc.end(), name) != post_proc.end();
  }
  void default_post_processing() {
    if (post_proc.empty()) post_proc = {"bond-orders", "molmom"};
  }
  // implicit solvation container moved in by tblite_calculator_push_back
  std::unique_ptr<SolvModel> solv;
  // homogeneous electric field (atomic units) moved in by tblite_calculator_push_back
  bool has_field = false;
  double efield[3] = {0.0, 0.0, 0.0};
  std::unique_ptr<Workspace> ws;
};

struct _tblite_result {
  int nat = 0, nsh = 0, nao = 0;
  bool has_energy = false, has_wfn = false;
  double energy = 0.0;
  std::vector<double> energies, gradient, sigma, qat, qsh, dpat, qpat, emo, focc, P, C, S, H, wbo;
  int wbo_channels = 0;  // 1 closed shell; 2 (total, magnetisation) for open shell
  // labels of the post-processing dictionary of the last single point, in order
  // ("bond-orders" [nat][nat][channels], "molecular-dipole" [3], "molecular-quadrupole" [6])
  std::vector<std::string> pp;
  bool has_pp(const char* label) const {
    return std::find(pp.begin(), pp.end(), label) != pp.end();
  }
  // fill pp from the calculator's post-processing list
  void set_post_processing(const std::vector<std::string>& list) {
    pp.clear();
    for (const auto& e : list) {
      if (e == "bond-orders") pp.push_back("bond-orders");
      if (e == "molmom") {
        pp.push_back("molecular-dipole");
        pp.push_back("molecular-quadrupole");
      }
    }
  }
  // dE/d(per-shell parameters): self energy, its CN shift, hardness, hardness derivative
  std::vector<double> dse, dkcn, dhub, dgam3, dzeta;
  // spectral projection: HOMO, LUMO, bound on their errors (empty after diagonalisation)
  std::vector<double> gap;
  // wavefunction data of the restart file: reference occupations, electrons per spin, kT
  std::vector<double> n0at, n0sh;
  double nel[2] = {0.0, 0.0}, kt = 0.0;
  double dipole[3] = {0, 0, 0}, quadrupole[6] = {0, 0, 0, 0, 0, 0};
};


// D4 model constants (counting function, cutoffs of the element-data pack; damping parameters
// of the calculator)
void d4_model_constants(DevD4& d, const _tblite_calculator* c);
// D3 model constants (counting functions, cutoffs of the element-data pack; damping parameters
// of the calculator)
void d3_model_constants(DevD3& d, const _tblite_calculator* c);
// scalar parameters of a calculator's Hamiltonian (GFN2-xTB or GFN1-xTB)
Gfn2Scalars gfn2_scalars(const _tblite_calculator* c);
// electrons per spin channel (reference xtb/singlepoint.f90:140-156); throws on an impossible
// combination of charge and unpaired electrons
void electron_counts(const _tblite_calculator* c, const _tblite_structure* mol, double* nalp,
                     double* nbet);
// molecular dipole and traceless quadrupole from the atomic charges and multipoles
// (wavefunction/mulliken.f90 get_molecular_dipole_moment / get_molecular_quadrupole_moment)
void molecular_moments(const _tblite_structure* mol, _tblite_result* res);
// ALPB(water) or, with gbsa, GBSA(water) + CDS + shift model for the molecule (reference state
// 1 gsolv, 2 bar1mol, 3 reference); the generalized Born model with a dielectric constant
// (alpb: with the ALPB shape term; kernel 1 Still, 2 P16)
std::unique_ptr<SolvModel> build_solvation(const _tblite_structure* mol, int state, bool gbsa);
std::unique_ptr<SolvModel> build_gb_epsilon(const _tblite_structure* mol, double eps, bool alpb,
                                            int kernel);
// the one-molecule single point (energy + gradient) into res
void run_singlepoint(_tblite_context* ctx, const _tblite_structure* mol, _tblite_calculator* c,
                     _tblite_result* res);
