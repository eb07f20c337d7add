// C ABI of the GB300 engine: error / context / structure / calculator / result objects and the
// single-point driver (reference src/tblite/api/*.f90 for the object conventions and
// src/tblite/xtb/singlepoint.f90:73-433 for the driver).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/tblite.h"
#include "../../include/tblite_gb300_ext.h"
#include "element_data.inc"
#include "param.h"
#include "engine.h"
#include "params_gfn1.inc"
#include "params_gfn2.inc"
#include "params_solv.inc"

#include "api_internal.h"
#include "npz.h"

using namespace tb;

// --------------------------------------------------------------------------------------
// STO-nG expansion, reference src/tblite/basis/slater.f90:409-511
// --------------------------------------------------------------------------------------
static void slater_to_gauss(int ng, int n, int l, double zeta, double* alpha, double* coeff) {
  int ityp;
  if (l == 0) ityp = n;
  else if (l == 1) ityp = 4 + n;
  else if (l == 2) ityp = 7 + n;
  else throw std::runtime_error("angular momentum above d is not supported");
  const double* pa = nullptr;
  const double* pc = nullptr;
  if (ng == 1) {
    alpha[0] = STO_ALPHA1[ityp - 1] * zeta * zeta;
    coeff[0] = 1.0;
  } else {
    if (ng == 6 && n == 6) {
      pa = l == 0 ? STO_ALPHA6S : STO_ALPHA6P;
      pc = l == 0 ? STO_COEFF6S : STO_COEFF6P;
    } else {
      const double* A[] = {nullptr, nullptr, STO_ALPHA2, STO_ALPHA3, STO_ALPHA4, STO_ALPHA5, STO_ALPHA6};
      const double* Cc[] = {nullptr, nullptr, STO_COEFF2, STO_COEFF3, STO_COEFF4, STO_COEFF5, STO_COEFF6};
      pa = A[ng] + (ityp - 1) * ng;
      pc = Cc[ng] + (ityp - 1) * ng;
    }
    for (int k = 0; k < ng; ++k) {
      alpha[k] = pa[k] * zeta * zeta;
      coeff[k] = pc[k];
    }
  }
  static const double dfac[8] = {1, 1, 3, 15, 105, 945, 10395, 135135};  // (2l-1)!!
  const double top = 2.0 / M_PI;
  for (int k = 0; k < ng; ++k)
    coeff[k] = coeff[k] * pow(top * alpha[k], 0.75) * pow(sqrt(4 * alpha[k]), l) / sqrt(dfac[l]);
}

// reference C6 of reference r of element za with reference q of element zb, from the pack's
// per-pair table (stored once per unordered pair); NaN if the pack has no entry for the pair
static double pack_c6(int za, int r, int zb, int q) {
  if (za > zb) {
    std::swap(za, zb);
    std::swap(r, q);
  }
  const int off = EXT_D4_C6OFF[(za - 1) * 86 + zb - 1];
  return off < 0 ? NAN : EXT_D4_C6PAIR[off + r * EXT_D4_NREF[zb - 1] + q];
}

// the dispersion models' species tables: per-species-pair reference C6 [nsp][MREF][nsp][MREF]
// from the pack (zero outside the species' reference counts); throws if a pair is missing
static void species_c6(const std::vector<int>& species, std::vector<double>& c6ref) {
  const int nsp = (int)species.size(), ld = nsp * D4_MREF;
  c6ref.assign((size_t)ld * ld, 0.0);
  for (int a = 0; a < nsp; ++a)
    for (int b = 0; b < nsp; ++b)
      for (int r = 0; r < EXT_D4_NREF[species[a] - 1]; ++r)
        for (int q = 0; q < EXT_D4_NREF[species[b] - 1]; ++q) {
          const double v = pack_c6(species[a], r, species[b], q);
          if (std::isnan(v))
            throw std::runtime_error(std::string("element data pack '") + EXT_PACK_NAME +
                                     "' has no reference C6 for the element pair Z=" +
                                     std::to_string(species[a]) + ", Z=" +
                                     std::to_string(species[b]));
          c6ref[(size_t)(a * D4_MREF + r) * ld + b * D4_MREF + q] = v;
        }
}

// An element the element-data pack does not cover: the error names the library whose tables
// hold the real values (none of them ships with the reference's source tree)
[[noreturn]] static void pack_missing(const char* what, const char* origin, int z) {
  throw std::runtime_error(std::string("element data pack '") + EXT_PACK_NAME + "' has no " +
                           what + " for Z=" + std::to_string(z) + " (" + origin +
                           " data, not part of this build)");
}

// D4 model data of the molecule's species (element-data pack)
static void build_d4_data(_tblite_calculator* c, const _tblite_structure* mol) {
  // the reference builds its D4 model with the default smooth-cutoff widths of 0 (hard cutoffs,
  // disp/d4.f90:71-72); a pack asking for smooth cutoffs needs dftd4's switching function
  if (EXT_D4_WIDTH2 != 0.0 || EXT_D4_WIDTH3 != 0.0)
    throw std::runtime_error(std::string("element data pack '") + EXT_PACK_NAME +
                             "' asks for smooth dispersion cutoffs, which the GPU engine does "
                             "not provide");
  std::vector<int> species;
  for (int z : mol->num)
    if (std::find(species.begin(), species.end(), z) == species.end()) species.push_back(z);
  c->has_d4 = true;
  c->d4_nsp = (int)species.size();
  for (int z : species)
    if (EXT_D4_NREF[z - 1] <= 0 || std::isnan(EXT_D4_ZEFF[z - 1]))
      pack_missing("D4 reference data", "dftd4 v4.2.0", z);
  for (int i = 0; i < mol->nat; ++i) {
    const int z = mol->num[i];
    c->d4_sp.push_back((int)(std::find(species.begin(), species.end(), z) - species.begin()));
    c->d4_nref.push_back(EXT_D4_NREF[z - 1]);
    for (int r = 0; r < D4_MREF; ++r) {
      c->d4_ngw.push_back(EXT_D4_NGW[(z - 1) * D4_MREF + r]);
      c->d4_refcn.push_back(EXT_D4_REFCN[(z - 1) * D4_MREF + r]);
      c->d4_refq.push_back(EXT_D4_REFQ[(z - 1) * D4_MREF + r]);
    }
    c->d4_zeff.push_back(EXT_D4_ZEFF[z - 1]);
    c->d4_gam.push_back(EXT_D4_GAM[z - 1]);
    c->d4_r4r2.push_back(EXT_D4_R4R2[z - 1]);
    c->d4_rcov.push_back(EXT_D4_RCOV[z - 1]);
    c->d4_en.push_back(EXT_D4_EN[z - 1]);
  }
  species_c6(species, c->d4_c6ref);
}

// D3 data of the molecule's atoms (element-data pack)
static void build_d3_data(_tblite_calculator* c, const _tblite_structure* mol) {
  c->has_d3 = true;
  std::vector<int> species;
  for (int z : mol->num)
    if (std::find(species.begin(), species.end(), z) == species.end()) species.push_back(z);
  c->d3_nsp = (int)species.size();
  for (int i = 0; i < mol->nat; ++i) {
    const int z = mol->num[i];
    if (EXT_D4_NREF[z - 1] <= 0 || std::isnan(EXT_D4_R4R2[z - 1]) || std::isnan(EXT_D4_RCOV[z - 1]))
      pack_missing("D3 reference data", "s-dftd3 v1.4.0", z);
    c->d3_sp.push_back((int)(std::find(species.begin(), species.end(), z) - species.begin()));
    c->d3_nref.push_back(EXT_D4_NREF[z - 1]);
    for (int r = 0; r < D4_MREF; ++r) c->d3_refcn.push_back(EXT_D4_REFCN[(z - 1) * D4_MREF + r]);
    c->d3_r4r2.push_back(EXT_D4_R4R2[z - 1]);
    c->d3_rcov.push_back(EXT_D4_RCOV[z - 1]);
  }
  species_c6(species, c->d3_c6ref);
}

static void orthogonalize_s(int ni, const double* ai, const double* ci, int& nj, double* aj,
                            double* cj);

// The calculator of a molecule from a parametrisation record (reference
// xtb/calculator.f90:new_xtb_calculator with the records of param/*.f90; the built-in methods
// pass their exported records, xtb/gfn2.f90:914-1022 and xtb/gfn1.f90:931-1054).  Two model
// forms are available on the GPU: the GFN2-xTB form (CN "dexp", D4 dispersion, arithmetic
// hardness average, shell-resolved third order, damped multipoles) and the GFN1-xTB form (CN
// "exp", D3 dispersion, harmonic average, atom-resolved third order, no multipoles; valence and
// polarisation shells, the second shell of an angular momentum orthogonalised to the first).
// Within a form every element record entry and every global constant of the record is used;
// anything else (another form, d shells, the halogen-bond correction, element-pair factors
// other than the form's own) is refused with an error.
static void build_calculator(_tblite_calculator* c, const _tblite_structure* mol,
                             const ParamRecord& rec) {
  int method = 0;
  if (rec.cn == "dexp") method = 2;
  else if (rec.cn == "exp") method = 1;
  else throw std::runtime_error("coordination number '" + rec.cn + "' of the parameter set is "
                                "not available in the GPU engine (\"dexp\" or \"exp\")");
  const char* form = method == 2 ? "GFN2-xTB" : "GFN1-xTB";
  auto need = [&](bool ok, const std::string& what) {
    if (!ok)
      throw std::runtime_error(std::string("parameter set of the ") + form +
                               " form not supported by the GPU engine: " + what);
  };
  need(rec.has_repulsion && rec.has_charge && rec.has_thirdorder && rec.has_dispersion,
       "repulsion, charge, thirdorder and dispersion entries are required");
  if (method == 2) {
    need(!rec.d3 && rec.sc && !rec.smooth, "self-consistent D4 dispersion required");
    need(rec.average == "arithmetic", "arithmetic hardness average required");
    need(rec.third_shell, "shell-resolved third order required");
    need(rec.has_multipole, "damped multipole electrostatics required");
    need(rec.kpair.empty(), "element-pair scaling factors must be 1");
  } else {
    need(rec.d3, "D3 dispersion required");
    need(rec.average == "harmonic", "harmonic hardness average required");
    need(!rec.third_shell, "atom-resolved third order required");
    need(!rec.has_multipole, "no multipole electrostatics in this form");
    need(rec.wexp == 0.0, "Slater-exponent weighting must be 0");
  }
  ModelConstants& k = c->model;
  k.wexp = rec.wexp;
  k.enscale = rec.enscale;
  k.kpol = rec.kpol;
  for (int a = 0; a < 5; ++a)
    for (int b = 0; b < 5; ++b) k.ksh[a][b] = rec.ksh[a][b];
  k.gexp = rec.gexp;
  k.rep_kexp = rec.kexp;
  k.rep_klight = rec.klight;
  k.dmp3 = rec.dmp3;
  k.dmp5 = rec.dmp5;
  k.mp_kexp = rec.mp_kexp;
  k.mp_shift = rec.mp_shift;
  k.mp_rmax = rec.mp_rmax;
  k.s6 = rec.s6;
  k.s8 = rec.s8;
  k.a1 = rec.a1;
  k.a2 = rec.a2;
  k.s9 = rec.s9;
  c->method = method;
  c->nat = mol->nat;
  c->at_z = mol->num;
  c->at_sh.assign(1, 0);
  c->nsh = 0;
  c->nao = 0;
  bool pairs_gfn1 = true, pairs_dblock = true;  // which pair-factor rule the record follows
  for (int i = 0; i < mol->nat; ++i) {
    const int z = mol->num[i];
    if (z < 1 || z > 86) throw std::runtime_error("No support for elements with Z > 86.");
    const ElementRecord* e = rec.get(z);
    if (!e) throw std::runtime_error("No parameters for element " + element_symbol(z));
    if (method == 1 && e->xbond > 0.0)
      throw std::runtime_error("element Z=" + std::to_string(z) +
                               " needs the GFN1 halogen-bond correction, which the GPU engine "
                               "does not provide");
    if (method == 1)
      for (int j = 0; j <= i; ++j) {
        const double f = rec.pair(z, mol->num[j]);
        pairs_gfn1 = pairs_gfn1 && f == gfn1_pair_factor(z, mol->num[j]);
        pairs_dblock = pairs_dblock && f == dblock_pair_factor(z, mol->num[j]);
        need(pairs_gfn1 || pairs_dblock,
             "element-pair scaling factors other than GFN1-xTB's or IPEA1-xTB's");
      }
    const int ns = e->nsh;
    if (ns > 3 || (int)e->levels.size() != ns)
      throw std::runtime_error("element record of " + e->sym + " is inconsistent");
    double a[3][MAXG] = {{0}}, cc[3][MAXG] = {{0}};
    int np[3] = {0, 0, 0}, first[5] = {-1, -1, -1, -1, -1};
    bool val[3] = {true, true, true};
    for (int s = 0; s < ns; ++s) {
      const int l = e->lsh[s];
      if (l > 1)
        throw std::runtime_error("element Z=" + std::to_string(z) +
                                 " has d shells, which the CUDA integral kernels do not handle yet");
      np[s] = e->ngauss[s];
      if (np[s] < 1 || np[s] > 6) throw std::runtime_error("invalid number of primitives");
      slater_to_gauss(np[s], e->pqn[s], l, e->slater[s], a[s], cc[s]);
      if (method == 1) {  // valence: the first shell of its angular momentum
        val[s] = first[l] < 0;
        if (val[s]) first[l] = s;
      }
    }
    for (int s = 0; s < ns; ++s)
      if (!val[s]) {
        const int r = first[e->lsh[s]];
        if (np[s] + np[r] > MAXG) throw std::runtime_error("too many primitives");
        orthogonalize_s(np[r], a[r], cc[r], np[s], a[s], cc[s]);
      }
    for (int s = 0; s < ns; ++s) {
      const int l = e->lsh[s];
      for (int q = 0; q < MAXG; ++q) {
        c->sh_alpha.push_back(a[s][q]);
        c->sh_coeff.push_back(cc[s][q]);
        if (q < np[s]) c->min_alpha = std::min(c->min_alpha, a[s][q]);
      }
      c->sh_atom.push_back(i);
      c->sh_l.push_back(l);
      c->sh_nprim.push_back(np[s]);
      c->sh_ao.push_back(c->nao);
      c->sh_zeta.push_back(e->slater[s]);
      c->sh_pqn.push_back(e->pqn[s]);
      c->sh_se0.push_back(e->levels[s]);
      c->sh_kcn.push_back(e->kcn[s]);
      c->sh_shpoly.push_back(e->shpoly[s]);
      c->sh_hub.push_back(e->gam * e->lgam[s]);
      c->sh_gam3.push_back(method == 2 ? e->gam3 * rec.third_ksh[l] : 0.0);
      c->sh_refocc.push_back(val[s] ? e->refocc[s] : 0.0);
      c->sh_valence.push_back(val[s] ? 1 : 0);
      for (int m = 0; m < 2 * l + 1; ++m) {
        c->ao_sh.push_back(c->nsh);
        c->ao_at.push_back(i);
      }
      c->nao += 2 * l + 1;
      c->nsh += 1;
    }
    c->at_sh.push_back(c->nsh);
    // external element data: needed only when the molecule has pairs
    const bool pairs = mol->nat > 1;
    const double en = e->en, rad = EXT_RAD[z - 1], rcov = EXT_RCOV[z - 1];
    if (pairs && (std::isnan(en) || std::isnan(rad) || std::isnan(rcov)))
      pack_missing("covalent radius, electronegativity or atomic radius", "mctc-lib v0.5.2", z);
    c->at_en.push_back(pairs ? en : 0.0);
    c->at_rad.push_back(pairs ? rad : 1.0);
    c->at_rcov.push_back(pairs ? rcov : 1.0);
    c->at_mprad.push_back(method == 2 ? e->mprad : 1.0);  // no multipoles in the GFN1 form
    c->at_vcn.push_back(method == 2 ? e->mpvcn : 0.0);
    c->at_dkern.push_back(method == 2 ? e->dkernel : 0.0);
    c->at_qkern.push_back(method == 2 ? e->qkernel : 0.0);
    c->at_repa.push_back(e->arep);
    c->at_repz.push_back(e->zeff);
    c->at_gam3.push_back(method == 1 ? e->gam3 : 0.0);
  }
  c->model.pair_mode = pairs_gfn1 ? 1 : 0;
  if (mol->nat > 1) {
    if (method == 2) build_d4_data(c, mol);
    else build_d3_data(c, mol);
  }
}

// --------------------------------------------------------------------------------------
// GFN1-xTB calculator data (reference xtb/gfn1.f90:556-905): basis with the second s shell
// of hydrogen orthogonalised to the first (basis/ortho.f90:33-72), per-shell levels and CN
// shifts, valence flags, harmonic-mean hardness, atom-resolved third order, D3 data.
// --------------------------------------------------------------------------------------
static void orthogonalize_s(int ni, const double* ai, const double* ci, int& nj, double* aj,
                            double* cj) {
  double ov = 0.0;
  for (int p = 0; p < ni; ++p)
    for (int q = 0; q < nj; ++q) ov += ci[p] * cj[q] * pow(sqrt(M_PI / (ai[p] + aj[q])), 3);
  for (int p = 0; p < ni; ++p) {
    aj[nj + p] = ai[p];
    cj[nj + p] = -ov * ci[p];
  }
  nj += ni;
  double norm = 0.0;
  for (int p = 0; p < nj; ++p)
    for (int q = 0; q < nj; ++q) norm += cj[p] * cj[q] * pow(sqrt(M_PI / (aj[p] + aj[q])), 3);
  const double sc = 1.0 / sqrt(norm);
  for (int p = 0; p < nj; ++p) cj[p] *= sc;
}

Gfn2Scalars gfn2_scalars(const _tblite_calculator* c) {
  const ModelConstants& k = c->model;
  Gfn2Scalars p{};
  p.method = c->method;
  p.pair_mode = c->model.pair_mode;
  p.wexp = k.wexp;
  p.enscale = k.enscale;
  p.gexp = k.gexp;
  for (int a = 0; a < 5; ++a)
    for (int b = 0; b < 5; ++b) p.kshell[a][b] = k.ksh[a][b];
  p.rep_kexp = k.rep_kexp;
  p.rep_kexp_light = k.rep_klight;
  p.rep_rexp = 1.0;  // repulsion/effective.f90: 1/R
  p.rep_cutoff = 25.0;
  // get_cutoff, reference basis/type.f90:227-247
  p.h0_cutoff = std::min(sqrt(2.0 * INTCUT / c->min_alpha), 40.0);
  if (c->method == 1) {
    p.kdiff = k.kpol;
    p.harmonic = 1;
    p.third_atom = 1;
    p.aes = 0;
    p.cn_exp_k = EXT_CNEXP_K;
    p.cn_cutoff = EXT_CNEXP_CUTOFF;
    return p;
  }
  p.aes = 1;
  p.mp_dmp3 = k.dmp3;
  p.mp_dmp5 = k.dmp5;
  p.mp_shift = k.mp_shift;
  p.mp_kexp = k.mp_kexp;
  p.mp_rmax = k.mp_rmax;
  p.cn_ka = EXT_CN_KA;
  p.cn_kb = EXT_CN_KB;
  p.cn_rshift = EXT_CN_RSHIFT;
  p.cn_cutoff = EXT_CN_CUTOFF;
  return p;
}

// --------------------------------------------------------------------------------------
// single point driver
// --------------------------------------------------------------------------------------
// a failed projection step: report a tensor-core wait that ran out (the status word of the
// split GEMMs) before the numerical failure it caused
static void pipeline_check(Workspace& w) {
  if (!w.pur) return;
  stream_wait(w.stream);
  int st = 0;
  cuda_check(cudaMemcpy(&st, purify_status(w.pur), sizeof(int), cudaMemcpyDeviceToHost),
             "purify status");
  if (st != 0)
    throw std::runtime_error("tensor-core matrix product did not complete (wait limit reached)");
}

static void ensure_workspace(_tblite_calculator* c) {
  if (!c->ws) {
    c->ws.reset(new Workspace());
    cuda_check(cudaStreamCreateWithFlags(&c->ws->stream, cudaStreamNonBlocking), "stream");
  }
  Workspace& w = *c->ws;
  const int memory = c->memory > 0 ? std::min(c->memory, c->max_iter) : c->max_iter;
  cudaStream_t s = w.stream;
  if (c->params_dirty && w.nat == c->nat && w.nao == c->nao && w.nsh == c->nsh) {
    w.sh_alpha.upload(c->sh_alpha, s);
    w.sh_coeff.upload(c->sh_coeff, s);
    w.sh_zeta.upload(c->sh_zeta, s);
    w.sh_se0.upload(c->sh_se0, s);
    w.sh_kcn.upload(c->sh_kcn, s);
    w.sh_hub.upload(c->sh_hub, s);
    w.sh_gam3.upload(c->sh_gam3, s);
  }
  c->params_dirty = false;
  if (w.nat != c->nat || w.nao != c->nao || w.nsh != c->nsh) {
    const size_t n = c->nao, nn = n * n;
    w.sh_alpha.upload(c->sh_alpha, s);
    w.sh_coeff.upload(c->sh_coeff, s);
    w.sh_se0.upload(c->sh_se0, s);
    w.sh_kcn.upload(c->sh_kcn, s);
    w.sh_shpoly.upload(c->sh_shpoly, s);
    w.sh_zeta.upload(c->sh_zeta, s);
    w.sh_hub.upload(c->sh_hub, s);
    w.sh_gam3.upload(c->sh_gam3, s);
    w.sh_refocc.upload(c->sh_refocc, s);
    w.at_en.upload(c->at_en, s);
    w.at_rad.upload(c->at_rad, s);
    w.at_rcov.upload(c->at_rcov, s);
    w.at_mprad.upload(c->at_mprad, s);
    w.at_vcn.upload(c->at_vcn, s);
    w.at_dkern.upload(c->at_dkern, s);
    w.at_qkern.upload(c->at_qkern, s);
    w.at_repa.upload(c->at_repa, s);
    w.at_repz.upload(c->at_repz, s);
    w.sh_valence.upload(c->sh_valence, s);
    w.at_gam3.upload(c->at_gam3, s);
    if (c->has_d3) {
      w.d3_nref.upload(c->d3_nref, s);
      w.d3_refcn.upload(c->d3_refcn, s);
      w.d3_sp.upload(c->d3_sp, s);
      w.d3_c6ref.upload(c->d3_c6ref, s);
      w.d3_r4r2.upload(c->d3_r4r2, s);
      w.d3_rcov.upload(c->d3_rcov, s);
      for (auto* b : {&w.d3_cn, &w.d3_dEdcn}) b->alloc(c->nat);
      for (auto* b : {&w.d3_w, &w.d3_dw}) b->alloc((size_t)c->nat * D4_MREF);
    }
    if (c->has_d4) {
      w.d4_sp.upload(c->d4_sp, s);
      w.d4_nref.upload(c->d4_nref, s);
      w.d4_ngw.upload(c->d4_ngw, s);
      w.d4_refcn.upload(c->d4_refcn, s);
      w.d4_refq.upload(c->d4_refq, s);
      w.d4_zeff.upload(c->d4_zeff, s);
      w.d4_gam.upload(c->d4_gam, s);
      w.d4_r4r2.upload(c->d4_r4r2, s);
      w.d4_rcov.upload(c->d4_rcov, s);
      w.d4_en.upload(c->d4_en, s);
      w.d4_c6ref.upload(c->d4_c6ref, s);
      const size_t na = c->nat, nr = na * D4_MREF;
      for (auto* b : {&w.d4_gw, &w.d4_dgw, &w.d4_gwv, &w.d4_dgwdq, &w.d4_dgwv_cn}) b->alloc(nr);
      for (auto* b : {&w.d4_cn, &w.d4_e3, &w.d4_dEdcn}) b->alloc(na);
      w.d4_c6.alloc(na * na);
      w.d4_dc6.alloc(na * na);
      w.d4_atm.alloc(8 * na * na);
    }
    w.at_z.upload(c->at_z, s);
    w.at_sh.upload(c->at_sh, s);
    w.sh_atom.upload(c->sh_atom, s);
    w.sh_l.upload(c->sh_l, s);
    w.sh_nprim.upload(c->sh_nprim, s);
    w.sh_ao.upload(c->sh_ao, s);
    w.ao_sh.upload(c->ao_sh, s);
    w.ao_at.upload(c->ao_at, s);
    const size_t nat = c->nat, nsh = c->nsh;
    w.xyz.alloc(3 * nat);
    w.cn.alloc(nat);
    w.se.alloc(nsh);
    w.mrad.alloc(nat);
    w.dmrdcn.alloc(nat);
    w.S.alloc(nn);
    w.H.alloc(nn);
    w.D.alloc(3 * nn);
    w.Q.alloc(6 * nn);
    w.F.alloc(nn);
    w.C.alloc(nn);
    w.P.alloc(nn);
    w.W.alloc(nn);
    w.emo.alloc(n);
    w.focc.alloc(3 * n);
    w.scratch.alloc(nn);
    for (auto* b : {&w.qsh, &w.qsh_o, &w.vsh}) b->alloc(nsh);
    for (auto* b : {&w.qat, &w.qat_o, &w.vat, &w.eband, &w.eelec, &w.erep, &w.dEdcn}) b->alloc(nat);
    for (auto* b : {&w.dpat, &w.dpat_o, &w.vdp, &w.grad}) b->alloc(3 * nat);
    for (auto* b : {&w.qpat, &w.qpat_o, &w.vqp}) b->alloc(6 * nat);
    w.sig_at.alloc(9 * nat);
    w.sigma.alloc(9);
    w.vao.alloc(n);
    w.mull.alloc((size_t)mulliken_chunks((int)n) * 11 * n);
    w.scal.alloc(8);
    w.icount.alloc(4);
    const size_t nd = nsh + 9 * nat;
    w.vec_out.alloc(nd);
    if (w.eig && eigen_capacity(w.eig) >= (int)n) {
      eigen_resize(w.eig, (int)n);
    } else {
      if (w.eig) eigen_destroy(w.eig);
      w.eig = eigen_create((int)n, s);
    }
    w.nat = c->nat;
    w.nsh = c->nsh;
    w.nao = c->nao;
    w.memory = -1;
  }
  if (w.memory != memory) {
    const size_t nd = c->nsh + 9 * c->nat;
    for (auto* b : {&w.b_q, &w.b_qlast, &w.b_dq, &w.b_dqlast}) b->alloc(nd);
    w.b_df.alloc(nd * memory);
    w.b_u.alloc(nd * memory);
    w.b_a.alloc((size_t)memory * memory);
    w.b_omega.alloc(memory);
    w.b_work.alloc((size_t)memory * memory + 2 * memory + 64);
    w.b_status.alloc(1);
    w.memory = memory;
  }
}

void d4_model_constants(DevD4& d, const _tblite_calculator* c) {
  d.ga = EXT_D4_GA;
  d.gc = EXT_D4_GC;
  d.wf = EXT_D4_WF;
  d.kn = EXT_D4_CN_KN;
  d.k4 = EXT_D4_CN_K4;
  d.k5 = EXT_D4_CN_K5;
  d.k6 = EXT_D4_CN_K6;
  d.cn_cutoff = EXT_D4_CN_CUTOFF;
  d.disp2_cutoff = EXT_D4_DISP2_CUTOFF;
  d.disp3_cutoff = EXT_D4_DISP3_CUTOFF;
  d.atm_alpha = EXT_D4_ATM_ALPHA;
  d.s6 = c->model.s6;
  d.s8 = c->model.s8;
  d.a1 = c->model.a1;
  d.a2 = c->model.a2;
  d.s9 = c->model.s9;
}

static DevD4 dev_d4(const _tblite_calculator* c, D4Work& wk) {
  Workspace& w = *c->ws;
  DevD4 d{};
  d.nsp = c->d4_nsp;
  d.sp = w.d4_sp.p;
  d.nref = w.d4_nref.p;
  d.ngw = w.d4_ngw.p;
  d.refcn = w.d4_refcn.p;
  d.refq = w.d4_refq.p;
  d.zeff = w.d4_zeff.p;
  d.gam = w.d4_gam.p;
  d.r4r2 = w.d4_r4r2.p;
  d.rcov = w.d4_rcov.p;
  d.en = w.d4_en.p;
  d.c6ref = w.d4_c6ref.p;
  d4_model_constants(d, c);
  wk.cn = w.d4_cn.p;
  wk.gw = w.d4_gw.p;
  wk.dgw = w.d4_dgw.p;
  wk.gwv = w.d4_gwv.p;
  wk.dgwdq = w.d4_dgwdq.p;
  wk.dgwv_cn = w.d4_dgwv_cn.p;
  wk.c6 = w.d4_c6.p;
  wk.dc6 = w.d4_dc6.p;
  wk.e3 = w.d4_e3.p;
  wk.dEdcn = w.d4_dEdcn.p;
  wk.atm = w.d4_atm.p;
  return d;
}

static void alpb_shape(const SolvModel& sm, const double* xyz, double* adet, double cen[3],
                       double I[3][3], double* vol_out);
static void alpb_shape_gradient(const SolvModel& sm, const double* xyz, const double* qat,
                                double* grad);

// device view of the solvation model; uploads the per-atom arrays when the model is new
static DevSolv dev_solv(_tblite_calculator* c, const _tblite_structure* mol) {
  Workspace& w = *c->ws;
  const SolvModel& sm = *c->solv;
  const int nat = sm.nat;
  cudaStream_t s = w.stream;
  if (w.sv_nat != nat) {
    std::vector<double> atom;
    for (const auto* v : {&sm.vdwr, &sm.rho, &sm.svdw, &sm.vdwsa, &sm.wrp, &sm.trj2_lo,
                          &sm.trj2_hi, &sm.tension, &sm.hbond})
      atom.insert(atom.end(), v->begin(), v->end());
    w.sv_atom.upload(atom, s);
    w.sv_grid.upload(sm.grid, s);
    w.sv_work.alloc((size_t)4 * nat);
    w.sv_nbl.alloc((size_t)nat * SOLV_MAXNB);
    w.sv_nnb.alloc(nat);
    w.sv_status.alloc(1);
    w.sv_nat = nat;
  }
  cuda_check(cudaMemsetAsync(w.sv_status.p, 0, sizeof(int), s), "zero");
  DevSolv v{};
  v.nat = nat;
  v.kernel = sm.kernel;
  v.cds = sm.cds ? 1 : 0;
  v.lrcut = sm.lrcut;
  v.srcut = sm.srcut;
  v.keps = sm.keps;
  v.alpbet = sm.alpbet;
  v.born_scale = sm.born_scale;
  v.ah0 = sm.ah0;
  v.ah1 = sm.ah1;
  v.ah3 = sm.ah3;
  v.shift = sm.shift;
  double cen[3], I[3][3], vol;
  alpb_shape(sm, mol->xyz.data(), &v.adet, cen, I, &vol);
  const double* a = w.sv_atom.p;
  v.vdwr = a;
  v.rho = a + nat;
  v.svdw = a + 2 * nat;
  v.vdwsa = a + 3 * nat;
  v.wrp = a + 4 * nat;
  v.trj2_lo = a + 5 * nat;
  v.trj2_hi = a + 6 * nat;
  v.tension = a + 7 * nat;
  v.hbond = a + 8 * nat;
  v.grid = w.sv_grid.p;
  v.brad = w.sv_work.p;
  v.dscale = w.sv_work.p + nat;
  v.wbr = w.sv_work.p + 2 * nat;
  v.surface = w.sv_work.p + 3 * nat;
  v.nbl = w.sv_nbl.p;
  v.nnb = w.sv_nnb.p;
  v.status = w.sv_status.p;
  return v;
}

static DevMol dev_mol(const _tblite_calculator* c) {
  const Workspace& w = *c->ws;
  DevMol m{};
  m.nat = c->nat;
  m.nsh = c->nsh;
  m.nao = c->nao;
  m.xyz = w.xyz.p;
  m.at_z = w.at_z.p;
  m.at_sh = w.at_sh.p;
  m.sh_atom = w.sh_atom.p;
  m.sh_l = w.sh_l.p;
  m.sh_nprim = w.sh_nprim.p;
  m.sh_alpha = w.sh_alpha.p;
  m.sh_coeff = w.sh_coeff.p;
  m.sh_ao = w.sh_ao.p;
  m.ao_sh = w.ao_sh.p;
  m.ao_at = w.ao_at.p;
  m.sh_se0 = w.sh_se0.p;
  m.sh_kcn = w.sh_kcn.p;
  m.sh_shpoly = w.sh_shpoly.p;
  m.sh_zeta = w.sh_zeta.p;
  m.sh_hub = w.sh_hub.p;
  m.sh_gam3 = w.sh_gam3.p;
  m.sh_refocc = w.sh_refocc.p;
  m.at_en = w.at_en.p;
  m.at_rad = w.at_rad.p;
  m.at_rcov = w.at_rcov.p;
  m.at_mprad = w.at_mprad.p;
  m.at_vcn = w.at_vcn.p;
  m.at_dkern = w.at_dkern.p;
  m.at_qkern = w.at_qkern.p;
  m.at_repa = w.at_repa.p;
  m.at_repz = w.at_repz.p;
  m.sh_valence = w.sh_valence.p;
  m.at_gam3 = w.at_gam3.p;
  return m;
}

void d3_model_constants(DevD3& d, const _tblite_calculator* c) {
  d.k1 = EXT_D3_K1;
  d.k3 = EXT_D3_K3;
  d.cn_cutoff = EXT_D3_CN_CUTOFF;
  d.cutoff = EXT_D3_DISP2_CUTOFF;
  d.s6 = c->model.s6;
  d.s8 = c->model.s8;
  d.a1 = c->model.a1;
  d.a2 = c->model.a2;
}

static DevD3 dev_d3(const _tblite_calculator* c) {
  const Workspace& w = *c->ws;
  DevD3 d{};
  d3_model_constants(d, c);
  d.nsp = c->d3_nsp;
  d.sp = w.d3_sp.p;
  d.nref = w.d3_nref.p;
  d.refcn = w.d3_refcn.p;
  d.c6ref = w.d3_c6ref.p;
  d.r4r2 = w.d3_r4r2.p;
  d.rcov = w.d3_rcov.p;
  d.cn = w.d3_cn.p;
  d.w = w.d3_w.p;
  d.dw = w.d3_dw.p;
  d.dEdcn = w.d3_dEdcn.p;
  return d;
}

// --------------------------------------------------------------------------------------
// optional per-phase timing with CUDA events on the engine stream
// --------------------------------------------------------------------------------------
enum Phase { PH_SETUP, PH_POTENTIAL, PH_FOCK, PH_EIGEN, PH_DENSITY, PH_MULLIKEN, PH_MIXER,
             PH_GRADIENT, PH_TRANSFER, PH_COUNT };

struct Profiler {
  bool enabled = false;
  std::vector<cudaEvent_t> pool;
  std::vector<std::pair<int, std::pair<int, int>>> marks;  // phase, (event a, event b)
  int used = 0;
  double phase_ms[PH_COUNT] = {0};
  int phase_n[PH_COUNT] = {0};
  double total_ms = 0.0;
  int iterations = 0;
  int open_phase = -1, open_event = -1;
  std::vector<std::pair<int, std::pair<int, int>>> kmarks;  // kernel slot, (event a, event b)
  double kernel_ms[KS_COUNT] = {0};
  int kernel_n[KS_COUNT] = {0};
  cudaEvent_t ev() {
    if (used == (int)pool.size()) {
      cudaEvent_t e;
      cuda_check(cudaEventCreate(&e), "event");
      pool.push_back(e);
    }
    return pool[used++];
  }
  void reset() {
    used = 0;
    marks.clear();
    kmarks.clear();
    for (int k = 0; k < PH_COUNT; ++k) {
      phase_ms[k] = 0.0;
      phase_n[k] = 0;
    }
    for (int k = 0; k < KS_COUNT; ++k) {
      kernel_ms[k] = 0.0;
      kernel_n[k] = 0;
    }
    total_ms = 0.0;
  }
  void begin(int ph, cudaStream_t s) {
    if (!enabled) return;
    const int a = used;
    cuda_check(cudaEventRecord(ev(), s), "record");
    open_phase = ph;
    open_event = a;
  }
  void end(cudaStream_t s) {
    if (!enabled || open_phase < 0) return;
    const int b = used;
    cuda_check(cudaEventRecord(ev(), s), "record");
    marks.push_back({open_phase, {open_event, b}});
    open_phase = -1;
  }
  int kbegin(cudaStream_t s) {
    if (!enabled) return -1;
    const int a = used;
    cuda_check(cudaEventRecord(ev(), s), "record");
    return a;
  }
  void kend(int slot, int a, cudaStream_t s) {
    if (!enabled || a < 0) return;
    const int b = used;
    cuda_check(cudaEventRecord(ev(), s), "record");
    kmarks.push_back({slot, {a, b}});
  }
  void collect() {
    if (!enabled) return;
    for (auto& mk : kmarks) {
      float ms = 0.f;
      cuda_check(cudaEventElapsedTime(&ms, pool[mk.second.first], pool[mk.second.second]),
                 "elapsed");
      kernel_ms[mk.first] += ms;
      kernel_n[mk.first] += 1;
    }
    kmarks.clear();
    if (marks.empty()) return;
    for (auto& mk : marks) {
      float ms = 0.f;
      cuda_check(cudaEventElapsedTime(&ms, pool[mk.second.first], pool[mk.second.second]),
                 "elapsed");
      phase_ms[mk.first] += ms;
      phase_n[mk.first] += 1;
    }
    float tot = 0.f;
    cuda_check(cudaEventElapsedTime(&tot, pool[marks.front().second.first],
                                    pool[marks.back().second.second]),
               "elapsed");
    total_ms = tot;
  }
};
static Profiler g_prof;
namespace tb {
int prof_kbegin(cudaStream_t s) { return g_prof.kbegin(s); }
bool prof_enabled() { return g_prof.enabled; }
void prof_kend(int slot, int token, cudaStream_t s) { g_prof.kend(slot, token, s); }
void prof_reset() { g_prof.reset(); }
void prof_collect() { g_prof.collect(); }
}  // namespace tb

// occupation, reference xtb/singlepoint.f90:140-156
void electron_counts(const _tblite_calculator* c, const _tblite_structure* mol, double* nalp_out,
                     double* nbet_out) {
  const int nsh = c->nsh;
  double nocc = -mol->charge, nel_ref = 0.0;
  for (int i = 0; i < nsh; ++i) nocc += c->sh_refocc[i];
  nel_ref = nocc;
  int nuhf;
  const int nel_i = (int)lround(nel_ref);
  if ((mol->uhf % 2) == (nel_i % 2)) {
    nuhf = mol->uhf;
  } else {
    if (mol->uhf != 0)
      throw std::runtime_error("Total number of electrons (" + std::to_string(nel_i) +
                               ") and number unpaired electrons (" + std::to_string(mol->uhf) +
                               ") is not compatible");
    nuhf = nel_i % 2;
  }
  const double diff = std::min((double)nuhf, nocc);
  *nalp_out = (nocc - diff) / 2 + diff;
  *nbet_out = (nocc - diff) / 2;
}

static void singlepoint(_tblite_context* ctx, const _tblite_structure* mol,
                        _tblite_calculator* c, _tblite_result* res) {
  if (mol->nat != c->nat) throw std::runtime_error("structure does not match calculator");
  ensure_workspace(c);
  Workspace& w = *c->ws;
  cudaStream_t s = w.stream;
  const int nat = c->nat, nsh = c->nsh, n = c->nao;
  const Gfn2Scalars p = gfn2_scalars(c);
  // mixed quantities: shell charges, plus the atomic multipoles where they enter the
  // Hamiltonian (GFN2 anisotropic electrostatics)
  const bool with_mp = p.aes != 0;
  const size_t nd = nsh + (with_mp ? 9 * (size_t)nat : 0);
  cuda_check(cudaMemcpyAsync(w.xyz.p, mol->xyz.data(), sizeof(double) * 3 * nat,
                             cudaMemcpyHostToDevice, s),
             "xyz");
  DevMol m = dev_mol(c);
  double nalp = 0.0, nbet = 0.0;
  electron_counts(c, mol, &nalp, &nbet);
  // spectral projection (purify.cu): closed shells with whole electron pairs only
  const bool purify = c->density_solver == 1;
  const int nocc = (int)llround(nalp);
  if (purify) {
    if (nalp != nbet)
      throw std::runtime_error("the spectral-projection density solver needs a closed shell");
    if (fabs(nalp - nocc) > 1e-10)
      throw std::runtime_error("the spectral-projection density solver needs whole electron pairs");
    if (w.pur && purify_capacity(w.pur) != n) {
      purify_destroy(w.pur);
      w.pur = nullptr;
    }
    if (!w.pur) w.pur = purify_create(n, s);
  }

  g_prof.reset();
  // geometry-dependent setup
  g_prof.begin(PH_SETUP, s);
  launch_cn(m, p, w.cn.p, s);
  launch_setup_levels(m, p, w.cn.p, w.se.p, w.mrad.p, w.dmrdcn.p, s);
  launch_build_h0(m, p, w.se.p, w.S.p, w.H.p, w.D.p, w.Q.p, s);
  cuda_check(cudaMemsetAsync(w.grad.p, 0, sizeof(double) * 3 * nat, s), "zero");
  cuda_check(cudaMemsetAsync(w.sig_at.p, 0, sizeof(double) * 9 * nat, s), "zero");
  cuda_check(cudaMemsetAsync(w.sigma.p, 0, sizeof(double) * 9, s), "zero");
  cuda_check(cudaMemsetAsync(w.dEdcn.p, 0, sizeof(double) * nat, s), "zero");
  launch_repulsion(m, p, w.erep.p, w.grad.p, w.sig_at.p, s);
  D4Work d4w{};
  DevD4 d4 = c->has_d4 ? dev_d4(c, d4w) : DevD4{};
  if (c->has_d4) d4_setup(m, d4, d4w, true, w.grad.p, w.sig_at.p, s);
  if (c->has_d3) d3_energy_gradient(m, dev_d3(c), true, w.erep.p, w.grad.p, w.sig_at.p, s);
  // implicit solvation: Born radii, surfaces, geometry-only energies into erep
  DevSolv dsolv{};
  if (c->solv) {
    dsolv = dev_solv(c, mol);
    solv_setup(dsolv, w.xyz.p, w.erep.p, s);
  }
  int chol = 0;
  if (purify) chol = purify_set_overlap(w.pur, w.S.p) < 0 ? 1 : 0;
  else chol = eigen_set_overlap(w.eig, w.S.p);
  g_prof.end(s);
  if (c->fault == 1) chol = 1;  // injected: the first pivot is not positive
  if (chol != 0) {
    if (purify) {
      pipeline_check(w);
      throw std::runtime_error("overlap orthogonalisation (Newton-Schulz) did not converge");
    }
    // LAPACK's convention for sygvd (lapack/sygvd.f90:153-161): info = n + i when the leading
    // minor of order i of the overlap is not positive definite
    throw std::runtime_error("(sygvd) failed to solve eigenvalue problem. info=" +
                             std::to_string((long long)n + chol));
  }

  // initial guess: restart from a compatible result, else SAD (wavefunction/guess.f90:51-120)
  std::vector<double> qsh0(nsh), dp0(3 * nat, 0.0), qp0(6 * nat, 0.0), qat0(nat);
  if (res->has_wfn && res->nat == nat && res->nsh == nsh && res->nao == n) {
    qsh0 = res->qsh;
    dp0 = res->dpat;
    qp0 = res->qpat;
    qat0 = res->qat;
  } else {
    std::vector<double> n0at(nat, 0.0);
    for (int i = 0; i < nsh; ++i) n0at[c->sh_atom[i]] += c->sh_refocc[i];
    for (int i = 0; i < nat; ++i) qat0[i] = mol->charge / nat;
    for (int i = 0; i < nsh; ++i)
      qsh0[i] = c->sh_refocc[i] / n0at[c->sh_atom[i]] * qat0[c->sh_atom[i]];
  }
  w.qsh.upload(qsh0, s);
  w.dpat.upload(dp0, s);
  w.qpat.upload(qp0, s);
  w.qat.upload(qat0, s);

  BroydenState b{};
  b.ndim = (int)nd;
  b.memory = w.memory;
  b.iter = 0;
  b.damp = c->damping;
  b.q = w.b_q.p;
  b.qlast = w.b_qlast.p;
  b.dq = w.b_dq.p;
  b.dqlast = w.b_dqlast.p;
  b.df = w.b_df.p;
  b.u = w.b_u.p;
  b.a = w.b_a.p;
  b.omega = w.b_omega.p;
  b.work = w.b_work.p;
  b.status = w.b_status.p;

  const double econv = 1.0e-6 * c->accuracy, pconv = 2.0e-5 * c->accuracy;
  const double target_kt = c->etemp;
  double elevated_kt = target_kt;
  int anneal_hold = 50, anneal_steps = 50;
  if (c->anneal) {
    elevated_kt = c->anneal_kt;
    anneal_hold = std::max(0, c->anneal_hold);
    anneal_steps = std::max(0, c->anneal_cycles);
  }
  std::vector<double> h_eelec(nat, 0.0), h_scal(2);
  int iscf = 0;
  bool converged = false;
  double eelec_sum = 0.0;
  if (ctx->verbosity > 0) {
    ctx->message(std::string(60, '-'));
    ctx->message("  cycle        total energy    energy error   density error");
    ctx->message(std::string(60, '-'));
  }
  std::vector<double> h_erep;
  w.erep.download(h_erep, nat, s);
  if (c->has_d4) {  // non-self-consistent energies: repulsion + three-body dispersion
    std::vector<double> h_e3;
    w.d4_e3.download(h_e3, nat, s);
    stream_wait(s);
    for (int i = 0; i < nat; ++i) h_erep[i] += h_e3[i];
  }
  std::vector<int> h_cnt(2);
  // eigenvalues per iteration: the occupied levels and a margin (the rest once converged)
  int nev = scf_eigenvalue_count(n, std::max(nalp, nbet));
  double kt = target_kt;
  while (!converged && iscf < c->max_iter) {
    const double elast = eelec_sum;
    if (elevated_kt > target_kt) {  // singlepoint.f90:286-296
      if (iscf < anneal_hold) kt = elevated_kt;
      else if (anneal_steps > 0 && iscf < anneal_hold + anneal_steps)
        kt = elevated_kt + (double)(iscf - anneal_hold + 1) / anneal_steps * (target_kt - elevated_kt);
      else kt = target_kt;
    }
    if (iscf > 0) {
      g_prof.begin(PH_MIXER, s);
      launch_broyden_next(b, s);
      int st = 0;
      cuda_check(cudaMemcpyAsync(&st, w.b_status.p, sizeof(int), cudaMemcpyDeviceToHost, s), "st");
      stream_wait(s);
      if (st != 0) throw std::runtime_error("Broyden mixing failed to obtain next iteration");
      launch_unpack(m, w.b_q.p, w.qsh.p, w.qat.p, w.dpat.p, w.qpat.p, s, with_mp);
      g_prof.end(s);
    }
    ++iscf;
    g_prof.begin(PH_POTENTIAL, s);
    launch_coulomb_potential(m, p, w.mrad.p, w.qsh.p, w.qat.p, w.dpat.p, w.qpat.p, w.vsh.p, w.vat.p,
                             w.vdp.p, w.vqp.p, s);
    if (c->has_d4) d4_potential(m, d4, d4w, w.qat.p, w.vat.p, s);
    if (c->solv) solv_potential(dsolv, w.xyz.p, w.qat.p, w.vat.p, s);
    if (c->has_field) launch_field_potential(nat, w.xyz.p, c->efield, w.vat.p, w.vdp.p, s);
    launch_vao(m, w.vsh.p, w.vat.p, w.vao.p, s);
    g_prof.end(s);
    g_prof.begin(PH_FOCK, s);
    launch_fock(n, w.ao_at.p, w.H.p, w.S.p, with_mp ? w.D.p : nullptr, w.Q.p, w.vao.p, w.vdp.p,
                w.vqp.p, w.F.p, s);
    launch_pack(m, w.qsh.p, w.dpat.p, w.qpat.p, w.b_q.p, s, with_mp);  // mixer%set
    g_prof.end(s);
    if (purify) {  // P from the Fock matrix by products alone; 0/1 occupations carry no entropy
      g_prof.begin(PH_DENSITY, s);
      if (purify_density(w.pur, w.F.p, nocc, w.P.p) < 0) {
        pipeline_check(w);
        throw std::runtime_error("spectral projection (SP2) did not converge");
      }
      cuda_check(cudaMemsetAsync(w.scal.p, 0, sizeof(double), s), "ts");
      g_prof.end(s);
    } else {
      g_prof.begin(PH_EIGEN, s);
      const int info = eigen_values(w.eig, w.F.p, w.emo.p, nev);
      if (info != 0)
        throw std::runtime_error("(sygvd) failed to solve eigenvalue problem. info=" +
                                 std::to_string(info));
      launch_fermi(n, w.emo.p, nalp, nbet, kt, w.focc.p, w.scal.p, w.icount.p, s, nev);
      w.icount.download(h_cnt, 2, s);
      stream_wait(s);
      if (h_cnt[1] != 0) {  // the Fermi level needs more levels: all of them from now on
        eigen_values_rest(w.eig, nev, w.emo.p);
        nev = n;
        launch_fermi(n, w.emo.p, nalp, nbet, kt, w.focc.p, w.scal.p, w.icount.p, s, nev);
        w.icount.download(h_cnt, 2, s);
        stream_wait(s);
      }
      eigen_vectors(w.eig, h_cnt[0], w.C.p);
      g_prof.end(s);
      g_prof.begin(PH_DENSITY, s);
      density_matrix(n, h_cnt[0], w.C.p, w.focc.p, w.P.p, w.scratch.p, s,
                     eigen_gemm_status(w.eig));
      g_prof.end(s);
    }
    g_prof.begin(PH_MULLIKEN, s);
    launch_mulliken(m, w.P.p, w.S.p, w.H.p, w.D.p, w.Q.p, w.mull.p, mulliken_chunks(n), w.qsh_o.p,
                    w.qat_o.p, w.dpat_o.p, w.qpat_o.p, w.eband.p, s);
    launch_pack(m, w.qsh_o.p, w.dpat_o.p, w.qpat_o.p, w.vec_out.p, s, with_mp);
    launch_diff((int)nd, w.vec_out.p, w.b_q.p, w.b_dq.p, w.scal.p + 1, s);  // mixer%diff
    launch_eelec_init(nat, w.scal.p, w.eband.p, w.eelec.p, s);
    launch_coulomb_energy(m, p, w.mrad.p, w.qsh_o.p, w.qat_o.p, w.dpat_o.p, w.qpat_o.p, w.eelec.p,
                          s);
    if (c->has_d4) d4_energy(m, d4, d4w, w.qat_o.p, w.eelec.p, s);
    if (c->solv) solv_energy(dsolv, w.xyz.p, w.qat_o.p, w.eelec.p, s);
    if (c->has_field)
      launch_field_energy(nat, w.xyz.p, c->efield, w.qat_o.p, w.dpat_o.p, w.eelec.p, s);
    g_prof.end(s);
    w.eelec.download(h_eelec, nat, s);
    w.scal.download(h_scal, 2, s);
    stream_wait(s);
    eelec_sum = 0.0;
    for (int i = 0; i < nat; ++i) eelec_sum += h_eelec[i];
    const bool econv_ok = fabs(eelec_sum - elast) < econv;
    const bool pconv_ok = h_scal[1] < pconv;
    converged = econv_ok && pconv_ok && kt <= target_kt;
    if (ctx->verbosity > 0) {
      double etot = eelec_sum;
      for (int i = 0; i < nat; ++i) etot += h_erep[i];
      char buf[128];
      snprintf(buf, sizeof(buf), "%7d%24.13g%16.7e%16.7e", iscf, etot, eelec_sum - elast, h_scal[1]);
      ctx->message(buf);
    }
  }
  // results (singlepoint.f90:315-322)
  res->nat = nat;
  res->nsh = nsh;
  res->nao = n;
  res->energies.resize(nat);
  res->energy = 0.0;
  for (int i = 0; i < nat; ++i) {
    res->energies[i] = h_erep[i] + h_eelec[i];
    res->energy += res->energies[i];
  }
  res->has_energy = true;
  res->gap.clear();
  if (purify) {  // the 0/1 occupations hold only with a gap of many kT
    std::vector<double> gap(3);
    g_prof.begin(PH_DENSITY, s);
    purify_gap(w.pur, gap.data());
    g_prof.end(s);
    const double lower = gap[1] - gap[0] - gap[2];
    if (!(lower >= purify_gap_kt() * kt)) {
      char buf[200];
      snprintf(buf, sizeof(buf),
               "HOMO-LUMO gap %.3e Eh is below %.0f kT: the spectral-projection density solver "
               "needs a gapped system (use diagonalisation)", gap[1] - gap[0], purify_gap_kt());
      throw std::runtime_error(buf);
    }
    res->gap = gap;
  }

  // gradient (singlepoint.f90:343-381): Coulomb at output moments, H0 with last potential
  g_prof.begin(PH_GRADIENT, s);
  launch_coulomb_gradient(m, p, w.mrad.p, w.dmrdcn.p, w.qsh_o.p, w.qat_o.p, w.dpat_o.p, w.qpat_o.p,
                          w.grad.p, w.sig_at.p, w.dEdcn.p, s);
  if (c->has_d4) d4_gradient(m, d4, d4w, w.qat_o.p, w.grad.p, w.sig_at.p, s);
  if (c->solv) solv_gradient(dsolv, w.xyz.p, w.qat_o.p, w.grad.p, s);
  // W = C diag(f e) C^T  (scf/diag.f90:110-143); after projection W = P F P / 2
  if (purify) {
    purify_weighted(w.pur, w.F.p, w.P.p, w.W.p);
  } else {
    launch_fe(n, w.focc.p, w.emo.p, w.vec_out.p, s);
    density_matrix(n, h_cnt[0], w.C.p, w.vec_out.p, w.W.p, w.scratch.p, s,
                   eigen_gemm_status(w.eig));
  }
  launch_h0_gradient(m, p, w.se.p, w.P.p, w.W.p, w.vao.p, w.vdp.p, w.vqp.p, w.grad.p, w.sigma.p,
                     w.dEdcn.p, s);
  launch_cn_grad(m, p, w.dEdcn.p, w.grad.p, w.sig_at.p, s);
  std::vector<double> h_zgrad;
  if (c->param_grad) {  // dE/d(Slater exponent): needs W, so before W is reused below
    w.zgrad.alloc(nsh);
    launch_zeta_grad(m, p, w.se.p, w.P.p, w.W.p, w.vao.p, w.vdp.p, w.vqp.p, w.zgrad.p, s);
    w.zgrad.download(h_zgrad, nsh, s);
  }
  g_prof.end(s);
  // the result carries every orbital (wavefunction/type.f90 coeff(nao, nao)): the SCF only
  // needed the occupied ones, the empty ones come from the last tridiagonal form
  if (!purify) {  // the projection has no orbitals
    g_prof.begin(PH_EIGEN, s);
    eigen_values_rest(w.eig, nev, w.emo.p);
    eigen_vectors_range(w.eig, h_cnt[0], (int)n, w.C.p);
    g_prof.end(s);
  }
  // Wiberg/Mayer bond orders (post_processing/wbo.f90:60-115): closed shell from P; restricted
  // open shell from the spin densities with the factor 2, then (up, down) -> (total, up-down)
  g_prof.begin(PH_GRADIENT, s);
  const bool open_shell = nalp != nbet;
  const bool want_wbo = c->wants("bond-orders");
  const int nch = want_wbo ? (open_shell ? 2 : 1) : 0;
  w.wbo.alloc((size_t)std::max(nch, 1) * nat * nat);
  cuda_check(cudaMemsetAsync(w.wbo.p, 0, sizeof(double) * std::max(nch, 1) * nat * nat, s),
             "zero");
  if (!want_wbo) {
    // bond orders not requested (post-processing list without "bond-orders")
  } else if (!open_shell) {
    if (purify) purify_product(w.pur, w.P.p, w.S.p, w.scratch.p);
    else gemm64(false, false, n, n, n, 1.0, w.P.p, n, w.S.p, n, 0.0, w.scratch.p, n, KM_NONE, s);
    launch_wbo(m, w.scratch.p, w.wbo.p, 1.0, s);
  } else {
    for (int sp = 0; sp < 2; ++sp) {  // W is free after the gradient: it holds the spin density
      density_matrix(n, h_cnt[0], w.C.p, w.focc.p + (size_t)(1 + sp) * n, w.W.p, w.scratch.p, s,
                     eigen_gemm_status(w.eig));
      gemm64(false, false, n, n, n, 1.0, w.W.p, n, w.S.p, n, 0.0, w.scratch.p, n, KM_NONE, s);
      launch_wbo(m, w.scratch.p, w.wbo.p + (size_t)sp * nat * nat, 2.0, s);
    }
  }
  // parameter gradient (on request): H0 rebuilt with unit self energies into the scratch
  // matrix (S, D and Q are rebuilt with identical values), then one thread per shell
  std::vector<double> h_pgrad, h_cn;
  if (c->param_grad) {
    w.ones.upload(std::vector<double>(nsh, 1.0), s);
    launch_build_h0(m, p, w.ones.p, w.S.p, w.scratch.p, w.D.p, w.Q.p, s);
    w.pgrad.alloc((size_t)3 * nsh);
    launch_param_grad(m, p, w.P.p, w.scratch.p, w.qsh_o.p, w.pgrad.p, s);
    w.pgrad.download(h_pgrad, (size_t)3 * nsh, s);
    w.cn.download(h_cn, nat, s);
  }
  g_prof.end(s);
  g_prof.begin(PH_TRANSFER, s);
  if (!purify) w.C.download(res->C, (size_t)n * n, s);
  w.wbo.download(res->wbo, (size_t)nch * nat * nat, s);
  w.grad.download(res->gradient, 3 * nat, s);
  std::vector<double> h_sig_at, h_sigma;
  w.sig_at.download(h_sig_at, 9 * nat, s);
  w.sigma.download(h_sigma, 9, s);
  w.qsh_o.download(res->qsh, nsh, s);
  w.qat_o.download(res->qat, nat, s);
  w.dpat_o.download(res->dpat, 3 * nat, s);
  w.qpat_o.download(res->qpat, 6 * nat, s);
  if (purify) {
    res->C.clear();
    res->emo.clear();
    res->focc.clear();
  } else {
    w.emo.download(res->emo, n, s);
    w.focc.download(res->focc, n, s);
  }
  w.P.download(res->P, (size_t)n * n, s);
  if (c->save_integrals) {
    w.S.download(res->S, (size_t)n * n, s);
    w.H.download(res->H, (size_t)n * n, s);
  }
  std::vector<int> h_sv_status;
  if (c->solv) w.sv_status.download(h_sv_status, 1, s);
  g_prof.end(s);
  stream_wait(s);
  cuda_check(cudaGetLastError(), "results");
  int pur_status = 0;
  if (purify)
    cuda_check(cudaMemcpy(&pur_status, purify_status(w.pur), sizeof(int), cudaMemcpyDeviceToHost),
               "purify status");
  if (eigen_gemm_failed(w.eig) || pur_status != 0)
    throw std::runtime_error("tensor-core matrix product did not complete (wait limit reached)");
  g_prof.collect();
  g_prof.iterations = iscf;
  if (c->solv) {
    if (h_sv_status[0] != 0)
      throw std::runtime_error("solvent accessible surface: more neighbours than the GPU kernel holds");
    alpb_shape_gradient(*c->solv, mol->xyz.data(), res->qat.data(), res->gradient.data());
  }
  res->sigma.assign(9, 0.0);
  for (int k = 0; k < 9; ++k) {
    double acc = h_sigma[k];
    for (int i = 0; i < nat; ++i) acc += h_sig_at[9 * i + k];
    res->sigma[k] = acc;
  }
  if (c->has_field) {  // external/field.f90 get_gradient: gradient -= E, sigma -= sym(E R^T)
    double st[3][3] = {};
    for (int i = 0; i < nat; ++i)
      for (int a = 0; a < 3; ++a) {
        res->gradient[3 * i + a] -= c->efield[a];
        for (int b = 0; b < 3; ++b) st[a][b] += c->efield[a] * mol->xyz[3 * i + b];
      }
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) res->sigma[3 * a + b] -= 0.5 * (st[a][b] + st[b][a]);
  }
  res->has_wfn = true;
  res->n0sh.assign(c->sh_refocc.begin(), c->sh_refocc.begin() + nsh);
  res->n0at.assign(nat, 0.0);
  for (int i = 0; i < nsh; ++i) res->n0at[c->sh_atom[i]] += c->sh_refocc[i];
  res->nel[0] = nalp;
  res->nel[1] = nbet;
  res->kt = c->etemp;
  if (nch == 2) {  // updown_to_magnet (wavefunction/spin.f90:130-140)
    const size_t na2 = (size_t)nat * nat;
    for (size_t t = 0; t < na2; ++t) {
      const double up = res->wbo[t], dn = res->wbo[na2 + t];
      res->wbo[t] = up + dn;
      res->wbo[na2 + t] = up - dn;
    }
  }
  res->wbo_channels = nch;
  molecular_moments(mol, res);
  res->set_post_processing(c->post_proc);
  if (c->param_grad) {  // self energy e_s = se0_s - kcn_s CN_A  =>  dE/dkcn_s = -CN_A dE/de_s
    res->dse.assign(h_pgrad.begin(), h_pgrad.begin() + nsh);
    res->dhub.assign(h_pgrad.begin() + nsh, h_pgrad.begin() + 2 * nsh);
    res->dgam3.assign(h_pgrad.begin() + 2 * nsh, h_pgrad.end());
    res->dkcn.resize(nsh);
    for (int i = 0; i < nsh; ++i) res->dkcn[i] = -h_cn[c->sh_atom[i]] * res->dse[i];
    res->dzeta = h_zgrad;
  } else {
    res->dzeta.clear();
    res->dse.clear();
    res->dhub.clear();
    res->dgam3.clear();
    res->dkcn.clear();
  }
  if (!converged)
    throw std::runtime_error("SCF not converged in " + std::to_string(iscf) + " cycles");
}

// --------------------------------------------------------------------------------------
// C ABI
// --------------------------------------------------------------------------------------
// --------------------------------------------------------------------------------------
// ALPB(water) + CDS + shift model: parameters per atom (solvation/data/alpb.f90:227-249,
// data/cds.f90:225-249, data/shift.f90:221-233; alpb.f90:173-206; cds.f90:166-184;
// surface.f90:80-140; shift.f90:150-241) and the 230-point Lebedev grid from its orbits
// --------------------------------------------------------------------------------------
static std::vector<double> lebedev230() {
  std::vector<double> g;
  for (int o = 0; o < LEB230_NORB; ++o) {
    const int t = LEB230_TYPE[o];
    const double a = LEB230_A[o], b = LEB230_B[o], v = LEB230_V[o] * 4.0 * M_PI;
    double base[3];
    if (t == 1) {
      base[0] = 1.0; base[1] = 0.0; base[2] = 0.0;
    } else if (t == 3) {
      const double s = sqrt(1.0 / 3.0);
      base[0] = s; base[1] = s; base[2] = s;
    } else if (t == 4) {
      base[0] = a; base[1] = a; base[2] = sqrt(1.0 - 2.0 * a * a);
    } else if (t == 5) {
      base[0] = a; base[1] = sqrt(1.0 - a * a); base[2] = 0.0;
    } else if (t == 6) {
      base[0] = a; base[1] = b; base[2] = sqrt(1.0 - a * a - b * b);
    } else {
      throw std::runtime_error("unknown Lebedev orbit type");
    }
    // every distinct signed permutation of the generator
    std::vector<std::array<double, 3>> pts;
    const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    for (auto& pm : perm)
      for (int sg = 0; sg < 8; ++sg) {
        std::array<double, 3> p;
        for (int k = 0; k < 3; ++k) {
          const double c = base[pm[k]];
          p[k] = c == 0.0 ? 0.0 : ((sg >> k) & 1 ? -c : c);
        }
        if (std::find(pts.begin(), pts.end(), p) == pts.end()) pts.push_back(p);
      }
    std::sort(pts.begin(), pts.end());
    for (auto& p : pts) {
      g.push_back(p[0]);
      g.push_back(p[1]);
      g.push_back(p[2]);
      g.push_back(v);
    }
  }
  if (g.size() != 4 * 230) throw std::runtime_error("Lebedev grid has the wrong size");
  return g;
}

// gbsa: the GBSA(water) tables and the Still kernel without the ALPB shape term
// (api/solvation.f90:272-283, data/alpb.f90:92-249), else ALPB(water) with the P16 kernel
std::unique_ptr<SolvModel> build_solvation(const _tblite_structure* mol, int state, bool gbsa) {
  auto m = std::make_unique<SolvModel>();
  const int nat = mol->nat;
  m->nat = nat;
  m->state = state;
  m->kernel = gbsa ? 1 : 2;
  const double eps = gbsa ? GBSA_WATER_EPSV : ALPB_WATER_EPSV;
  m->alpbet = gbsa ? 0.0 : 0.571412 / eps;
  m->keps = (1.0 / eps - 1.0) / (1.0 + m->alpbet);
  m->born_scale = gbsa ? GBSA_WATER_C1 : ALPB_WATER_C1;
  m->lrcut = 35.0 * SOLV_AATOAU;
  const double* sx = gbsa ? GBSA_WATER_SX : ALPB_WATER_SX;
  const double soset = gbsa ? GBSA_WATER_SOSET : ALPB_WATER_SOSET;
  const double* gamscale = gbsa ? CDS_GBSA_WATER_GAMSCALE : CDS_WATER_GAMSCALE;
  const double* sqrtghb = gbsa ? CDS_GBSA_WATER_SQRTGHB : CDS_WATER_SQRTGHB;
  const double probe = (gbsa ? CDS_GBSA_WATER_RPROBE : CDS_WATER_RPROBE) * SOLV_AATOAU;
  const double w = 0.3 * SOLV_AATOAU;
  m->ah0 = 0.5;
  m->ah1 = 3.0 / (4.0 * w);
  m->ah3 = -1.0 / (4.0 * w * w * w);
  double maxsa = 0.0;
  for (int i = 0; i < nat; ++i) {
    const int z = mol->num[i];
    if (z < 1 || z > 94) throw std::runtime_error("No solvation parameters for Z > 94");
    const double rv = SOLV_RVDW_D3[z - 1];
    m->vdwr.push_back(rv);
    m->rho.push_back(rv * sx[z - 1]);
    m->svdw.push_back(rv - soset * 0.1 * SOLV_AATOAU);
    const double vs = rv + probe;
    maxsa = std::max(maxsa, vs);
    m->vdwsa.push_back(vs);
    m->trj2_lo.push_back((vs - w) * (vs - w));
    m->trj2_hi.push_back((vs + w) * (vs + w));
    auto part = [&](double r) {
      return (0.25 / w + 3.0 * m->ah3 * (0.2 * r * r - 0.5 * r * vs + vs * vs / 3.0)) * r * r * r;
    };
    m->wrp.push_back(part(vs + w) - part(vs - w));
    m->tension.push_back(gamscale[z - 1] * 1.0e-5);
    const double hb = -SOLV_KCALTOAU * sqrtghb[z - 1] * sqrtghb[z - 1];
    m->hbond.push_back(hb / (4.0 * M_PI * vs * vs));
  }
  m->srcut = 2.0 * (w + maxsa) + 2.0 * SOLV_AATOAU;
  // free-energy shift and reference state (shift.f90:191-241; CODATA 2018 constants)
  const double kb_au = 1.380649e-23 / 4.3597447222071e-18, temp = 298.15, amb = 298.15;
  const double vm = 8.314462618 * amb / 1.0e2;
  double stateshift = 0.0;
  if (state == 2) stateshift = temp * kb_au * log(vm * temp / amb);
  const double rhos = gbsa ? SHIFT_GBSA_WATER_RHOS : SHIFT_WATER_RHOS;
  const double smass = gbsa ? SHIFT_GBSA_WATER_SMASS : SHIFT_WATER_SMASS;
  if (state == 3)
    stateshift = temp * kb_au * (log(vm * temp / amb) + log(rhos / 1.0e-3 * 1.0 / smass));
  m->shift = (gbsa ? SHIFT_GBSA_WATER_GSHIFT : SHIFT_WATER_GSHIFT) * SOLV_KCALTOAU + stateshift;
  m->grid = lebedev230();
  return m;
}

// generalized Born model with a dielectric constant (api/solvation.f90:185-229, alpb.f90:146-204,
// born.f90:60-107): COSMO radii, descreening 0.8, Born scale 1, no offset; alpb adds the ALPB
// shape term (version 10), kernel 1 Still or 2 P16; no surface term and no free-energy shift
std::unique_ptr<SolvModel> build_gb_epsilon(const _tblite_structure* mol, double eps, bool alpb,
                                            int kernel) {
  auto m = std::make_unique<SolvModel>();
  const int nat = mol->nat;
  m->nat = nat;
  m->kernel = kernel;
  m->cds = false;
  m->alpbet = alpb ? 0.571412 / eps : 0.0;
  m->keps = (1.0 / eps - 1.0) / (1.0 + m->alpbet);
  m->born_scale = 1.0;
  m->lrcut = 35.0 * SOLV_AATOAU;
  for (int i = 0; i < nat; ++i) {
    const int z = mol->num[i];
    if (z < 1 || z > 94) throw std::runtime_error("No solvation parameters for Z > 94");
    const double rv = SOLV_RVDW_COSMO[z - 1];
    m->vdwr.push_back(rv);
    m->rho.push_back(rv * 0.8);
    m->svdw.push_back(rv);
    // no surface: the surface arrays only keep the device layout
    m->vdwsa.push_back(rv);
    m->wrp.push_back(0.0);
    m->trj2_lo.push_back(0.0);
    m->trj2_hi.push_back(0.0);
    m->tension.push_back(0.0);
    m->hbond.push_back(0.0);
  }
  m->grid = lebedev230();
  return m;
}

// shape descriptor of the ALPB term (alpb.f90:656-691) and its gradient (693-787)
static void alpb_shape(const SolvModel& sm, const double* xyz, double* adet, double cen[3],
                       double I[3][3], double* vol_out) {
  double vol = 0.0;
  cen[0] = cen[1] = cen[2] = 0.0;
  for (int i = 0; i < sm.nat; ++i) {
    const double r3 = sm.vdwr[i] * sm.vdwr[i] * sm.vdwr[i];
    vol += r3;
    for (int k = 0; k < 3; ++k) cen[k] += xyz[3 * i + k] * r3;
  }
  for (int k = 0; k < 3; ++k) cen[k] /= vol;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) I[a][b] = 0.0;
  for (int i = 0; i < sm.nat; ++i) {
    const double r2 = sm.vdwr[i] * sm.vdwr[i], r3 = r2 * sm.vdwr[i];
    double v[3], vv = 0.0;
    for (int k = 0; k < 3; ++k) {
      v[k] = xyz[3 * i + k] - cen[k];
      vv += v[k] * v[k];
    }
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) I[a][b] += r3 * ((a == b ? vv + 0.4 * r2 : 0.0) - v[a] * v[b]);
  }
  const double det = I[0][0] * (I[1][1] * I[2][2] - I[1][2] * I[2][1]) -
                     I[0][1] * (I[1][0] * I[2][2] - I[1][2] * I[2][0]) +
                     I[0][2] * (I[1][0] * I[2][1] - I[1][1] * I[2][0]);
  *adet = sqrt(pow(det, 1.0 / 3.0) / (0.4 * vol));
  *vol_out = vol;
}

static void alpb_shape_gradient(const SolvModel& sm, const double* xyz, const double* qat,
                                double* grad) {
  double adet, cen[3], I[3][3], vol;
  alpb_shape(sm, xyz, &adet, cen, I, &vol);
  double qt = 0.0;
  for (int i = 0; i < sm.nat; ++i) qt += qat[i];
  double d[3][3];
  d[0][0] = I[0][0] * (I[1][1] + I[2][2]) - I[0][1] * I[0][1] - I[0][2] * I[0][2];
  d[1][1] = I[1][1] * (I[0][0] + I[2][2]) - I[0][1] * I[0][1] - I[1][2] * I[1][2];
  d[2][2] = I[2][2] * (I[0][0] + I[1][1]) - I[0][2] * I[0][2] - I[1][2] * I[1][2];
  d[0][1] = d[1][0] = I[0][1] * I[2][2] - I[0][2] * I[1][2];
  d[0][2] = d[2][0] = I[0][2] * I[1][1] - I[0][1] * I[2][1];
  d[1][2] = d[2][1] = I[0][0] * I[1][2] - I[0][1] * I[0][2];
  const double f = 250.0 / (48.0 * vol * vol * vol * pow(adet, 5)) *
                   (-0.5 * sm.keps * sm.alpbet * qt * qt / (adet * adet));
  for (int i = 0; i < sm.nat; ++i) {
    const double r3 = sm.vdwr[i] * sm.vdwr[i] * sm.vdwr[i];
    double v[3];
    for (int k = 0; k < 3; ++k) v[k] = xyz[3 * i + k] - cen[k];
    for (int a = 0; a < 3; ++a)
      grad[3 * i + a] += r3 * f * (d[a][0] * v[0] + d[a][1] * v[1] + d[a][2] * v[2]);
  }
}

void molecular_moments(const _tblite_structure* mol, _tblite_result* res) {
  const int nat = res->nat;
  for (int k = 0; k < 3; ++k) res->dipole[k] = 0.0;
  for (int k = 0; k < 6; ++k) res->quadrupole[k] = 0.0;
  for (int i = 0; i < nat; ++i) {
    const double* x = &mol->xyz[3 * i];
    const double q = res->qat[i];
    const double* d = &res->dpat[3 * i];
    for (int k = 0; k < 3; ++k) res->dipole[k] += x[k] * q + d[k];
    // cartesian second moment of the point charge and dipole, made traceless (xx xy yy xz yz zz)
    const double v[3] = {x[0] * q, x[1] * q, x[2] * q};
    double c[6];
    c[0] = x[0] * (v[0] + 2 * d[0]);
    c[2] = x[1] * (v[1] + 2 * d[1]);
    c[5] = x[2] * (v[2] + 2 * d[2]);
    c[1] = x[0] * (v[1] + d[1]) + d[0] * x[1];
    c[3] = x[0] * (v[2] + d[2]) + d[0] * x[2];
    c[4] = x[1] * (v[2] + d[2]) + d[1] * x[2];
    const double tr = 0.5 * (c[0] + c[2] + c[5]);
    c[0] = 1.5 * c[0] - tr;
    c[1] = 3.0 * c[1];
    c[2] = 1.5 * c[2] - tr;
    c[3] = 3.0 * c[3];
    c[4] = 3.0 * c[4];
    c[5] = 1.5 * c[5] - tr;
    for (int k = 0; k < 6; ++k) res->quadrupole[k] += res->qpat[6 * i + k] + c[k];
  }
}

void run_singlepoint(_tblite_context* ctx, const _tblite_structure* mol, _tblite_calculator* c,
                     _tblite_result* res) {
  singlepoint(ctx, mol, c, res);
}

static void copy_msg(const std::string& msg, char* buffer, const int* buffersize) {
  if (!buffer) return;
  size_t cap = buffersize ? (size_t)std::max(*buffersize, 0) : msg.size() + 1;
  if (cap == 0) return;
  const size_t len = std::min(cap - 1, msg.size());
  memcpy(buffer, msg.data(), len);
  buffer[len] = '\0';
}

static void set_err(tblite_error e, const std::string& m) {
  if (e) {
    e->msg = m;
    e->set = true;
  }
}

extern "C" {

void tblite_gb300_set_profiling(int enable) { g_prof.enabled = enable != 0; }

int tblite_gb300_get_profile(double* phase_ms, int* phase_count, int nphase, double* total_ms,
                             int* iterations) {
  const int m = std::min(nphase, (int)PH_COUNT);
  for (int k = 0; k < m; ++k) {
    if (phase_ms) phase_ms[k] = g_prof.phase_ms[k];
    if (phase_count) phase_count[k] = g_prof.phase_n[k];
  }
  if (total_ms) *total_ms = g_prof.total_ms;
  if (iterations) *iterations = g_prof.iterations;
  return PH_COUNT;
}

int tblite_gb300_get_kernel_profile(double* kernel_ms, int* kernel_count, int nslot) {
  const int m = std::min(nslot, (int)KS_COUNT);
  for (int k = 0; k < m; ++k) {
    if (kernel_ms) kernel_ms[k] = g_prof.kernel_ms[k];
    if (kernel_count) kernel_count[k] = g_prof.kernel_n[k];
  }
  return KS_COUNT;
}

unsigned long long tblite_gb300_get_launch_count(void) { return g_kernel_launches; }
unsigned long long tblite_gb300_get_split_gemm_flops(void) { return g_split_flops; }

int tblite_gb300_get_result_bond_order_channels(tblite_result res) {
  return res ? res->wbo_channels : 0;
}

void tblite_gb300_set_calculator_parameter_gradient(tblite_context ctx, tblite_calculator calc,
                                                    int enable) {
  if (!ctx) return;
  if (!calc) {
    ctx->push("Calculator object is missing");
    return;
  }
  if (enable && calc->method != 2) {
    ctx->push("parameter gradients are available for GFN2-xTB calculators only");
    return;
  }
  calc->param_grad = enable != 0;
}

void tblite_gb300_set_calculator_density_solver(tblite_context ctx, tblite_calculator calc,
                                                int solver) {
  if (!ctx) return;
  if (!calc) {
    ctx->push("Calculator object is missing");
    return;
  }
  if (solver != 0 && solver != 1) {
    ctx->push("density solver must be 0 (diagonalisation) or 1 (spectral projection)");
    return;
  }
  calc->density_solver = solver;
}

void tblite_gb300_get_result_gap(tblite_error error, tblite_result res, double* gap) {
  if (!res) {
    set_err(error, "Result container is missing");
    return;
  }
  if (res->gap.size() != 3) {
    set_err(error, "Result does not contain a certified gap (spectral projection only)");
    return;
  }
  if (gap) std::copy(res->gap.begin(), res->gap.end(), gap);
}

void tblite_gb300_get_calculator_shell_parameters(tblite_context ctx, tblite_calculator calc,
                                                  double* selfenergy, double* kcn,
                                                  double* hubbard, double* hubbard_deriv) {
  if (!ctx) return;
  if (!calc) {
    ctx->push("Calculator object is missing");
    return;
  }
  const size_t nsh = calc->nsh;
  if (selfenergy) std::copy(calc->sh_se0.begin(), calc->sh_se0.begin() + nsh, selfenergy);
  if (kcn) std::copy(calc->sh_kcn.begin(), calc->sh_kcn.begin() + nsh, kcn);
  if (hubbard) std::copy(calc->sh_hub.begin(), calc->sh_hub.begin() + nsh, hubbard);
  if (hubbard_deriv) std::copy(calc->sh_gam3.begin(), calc->sh_gam3.begin() + nsh, hubbard_deriv);
}

void tblite_gb300_set_calculator_shell_parameters(tblite_context ctx, tblite_calculator calc,
                                                  const double* selfenergy, const double* kcn,
                                                  const double* hubbard,
                                                  const double* hubbard_deriv) {
  if (!ctx) return;
  if (!calc) {
    ctx->push("Calculator object is missing");
    return;
  }
  const size_t nsh = calc->nsh;
  if (hubbard)
    for (size_t i = 0; i < nsh; ++i)
      if (!(hubbard[i] > 0.0)) {
        ctx->push("Shell hardness must be positive");
        return;
      }
  if (selfenergy) std::copy(selfenergy, selfenergy + nsh, calc->sh_se0.begin());
  if (kcn) std::copy(kcn, kcn + nsh, calc->sh_kcn.begin());
  if (hubbard) std::copy(hubbard, hubbard + nsh, calc->sh_hub.begin());
  if (hubbard_deriv) std::copy(hubbard_deriv, hubbard_deriv + nsh, calc->sh_gam3.begin());
  calc->params_dirty = true;
}

void tblite_gb300_get_result_parameter_gradient(tblite_error error, tblite_result res,
                                                double* dselfenergy, double* dkcn,
                                                double* dhubbard, double* dhubbard_deriv) {
  if (!res) {
    set_err(error, "Result container is missing");
    return;
  }
  if (res->dse.empty()) {
    set_err(error, "Result does not contain a parameter gradient");
    return;
  }
  if (dselfenergy) std::copy(res->dse.begin(), res->dse.end(), dselfenergy);
  if (dkcn) std::copy(res->dkcn.begin(), res->dkcn.end(), dkcn);
  if (dhubbard) std::copy(res->dhub.begin(), res->dhub.end(), dhubbard);
  if (dhubbard_deriv) std::copy(res->dgam3.begin(), res->dgam3.end(), dhubbard_deriv);
}

void tblite_gb300_get_calculator_slater_exponents(tblite_context ctx, tblite_calculator calc,
                                                   double* zeta) {
  if (!ctx) return;
  if (!calc || !zeta) {
    ctx->push("Calculator object or output array is missing");
    return;
  }
  std::copy(calc->sh_zeta.begin(), calc->sh_zeta.begin() + calc->nsh, zeta);
}

// new Slater exponents: the STO-nG expansion of every shell is redone (slater.f90:409-511)
void tblite_gb300_set_calculator_slater_exponents(tblite_context ctx, tblite_calculator calc,
                                                   const double* zeta) {
  if (!ctx) return;
  if (!calc || !zeta) {
    ctx->push("Calculator object or input array is missing");
    return;
  }
  if (calc->method != 2 || (int)calc->sh_pqn.size() != calc->nsh) {
    ctx->push("Slater exponents can be changed for GFN2-xTB calculators only");
    return;
  }
  for (int i = 0; i < calc->nsh; ++i)
    if (!(zeta[i] > 0.0)) {
      ctx->push("Slater exponents must be positive");
      return;
    }
  double min_alpha = 1e300;
  for (int i = 0; i < calc->nsh; ++i) {
    double a[MAXG] = {0}, cc[MAXG] = {0};
    const int ng = calc->sh_nprim[i];
    slater_to_gauss(ng, calc->sh_pqn[i], calc->sh_l[i], zeta[i], a, cc);
    for (int k = 0; k < MAXG; ++k) {
      calc->sh_alpha[(size_t)i * MAXG + k] = a[k];
      calc->sh_coeff[(size_t)i * MAXG + k] = cc[k];
      if (k < ng) min_alpha = std::min(min_alpha, a[k]);
    }
    calc->sh_zeta[i] = zeta[i];
  }
  calc->min_alpha = min_alpha;
  calc->params_dirty = true;
}

void tblite_gb300_get_result_slater_gradient(tblite_error error, tblite_result res, double* dzeta) {
  if (!res) {
    set_err(error, "Result container is missing");
    return;
  }
  if (res->dzeta.empty()) {
    set_err(error, "Result does not contain a parameter gradient");
    return;
  }
  if (dzeta) std::copy(res->dzeta.begin(), res->dzeta.end(), dzeta);
}

int tblite_get_version(void) { return 7 * 100 + 0; }  // 0.7.0 -> 700 (reference version.h)

int tblite_get_feature(const char* flag) {
  if (!flag) return 0;
  return 0;
}

tblite_error tblite_new_error(void) { return new _tblite_error(); }
void tblite_delete_error(tblite_error* e) {
  if (e && *e) {
    delete *e;
    *e = nullptr;
  }
}
int tblite_check_error(tblite_error e) { return e && e->set ? 1 : 0; }
void tblite_clear_error(tblite_error e) {
  if (e) {
    e->set = false;
    e->msg.clear();
  }
}
void tblite_get_error(tblite_error e, char* buffer, const int* buffersize) {
  if (e && e->set) copy_msg(e->msg, buffer, buffersize);
}
void tblite_set_error(tblite_error e, char* buffer, const int* buffersize) {
  if (!e || !buffer) return;
  std::string m = buffersize ? std::string(buffer, strnlen(buffer, *buffersize)) : std::string(buffer);
  set_err(e, m);
}

tblite_context tblite_new_context(void) { return new _tblite_context(); }
void tblite_delete_context(tblite_context* c) {
  if (c && *c) {
    delete *c;
    *c = nullptr;
  }
}
int tblite_check_context(tblite_context c) { return c && !c->errors.empty() ? 1 : 0; }
void tblite_get_context_error(tblite_context c, char* buffer, const int* buffersize) {
  if (!c || c->errors.empty()) return;
  std::string m = c->errors.front();
  c->errors.erase(c->errors.begin());
  copy_msg(m, buffer, buffersize);
}
void tblite_set_context_logger(tblite_context c, tblite_logger_callback cb, void* ud) {
  if (!c) return;
  c->logger = cb;
  c->userdata = ud;
}
void tblite_set_context_color(tblite_context c, int color) {
  if (c) c->color = color;
}
void tblite_set_context_verbosity(tblite_context c, int v) {
  if (c) c->verbosity = v;
}

tblite_structure tblite_new_structure(tblite_error error, const int natoms, const int* numbers,
                                      const double* positions, const double* charge, const int* uhf,
                                      const double* lattice, const bool* periodic) {
  if (natoms <= 0 || !numbers || !positions) {
    set_err(error, "Invalid molecular structure data");
    return nullptr;
  }
  if (periodic) {
    for (int k = 0; k < 3; ++k)
      if (periodic[k]) {
        set_err(error, "Periodic systems are not supported by the GPU engine");
        return nullptr;
      }
  }
  (void)lattice;
  auto* m = new _tblite_structure();
  m->nat = natoms;
  m->num.assign(numbers, numbers + natoms);
  m->xyz.assign(positions, positions + 3 * natoms);
  for (double x : m->xyz)
    if (!std::isfinite(x)) {
      delete m;
      set_err(error, "Non-finite atomic coordinates");
      return nullptr;
    }
  m->charge = charge ? *charge : 0.0;
  m->uhf = uhf ? *uhf : 0;
  return m;
}
void tblite_delete_structure(tblite_structure* m) {
  if (m && *m) {
    delete *m;
    *m = nullptr;
  }
}
void tblite_update_structure_geometry(tblite_error error, tblite_structure m,
                                      const double* positions, const double* lattice) {
  (void)lattice;
  if (!m) {
    set_err(error, "Molecular structure data is missing");
    return;
  }
  if (!positions) {
    set_err(error, "Position array is missing");
    return;
  }
  m->xyz.assign(positions, positions + 3 * m->nat);
}
void tblite_update_structure_charge(tblite_error error, tblite_structure m, const double* charge) {
  if (!m) {
    set_err(error, "Molecular structure data is missing");
    return;
  }
  m->charge = charge ? *charge : 0.0;
}
void tblite_update_structure_uhf(tblite_error error, tblite_structure m, const int* uhf) {
  if (!m) {
    set_err(error, "Molecular structure data is missing");
    return;
  }
  m->uhf = uhf ? *uhf : 0;
}

tblite_result tblite_new_result(void) { return new _tblite_result(); }
tblite_result tblite_copy_result(tblite_result r) { return r ? new _tblite_result(*r) : nullptr; }

// wavefunction restart files (api/result.f90:597-642, wavefunction/restart.f90): a NumPy .npz
// archive with the members tblite0_{kt, nel, n0at, n0sh, density, coeff, emo, focc, qat, qsh,
// dpat, qpat}, Fortran order, one spin channel (the closed-shell / total representation)
void tblite_save_result_wavefunction(tblite_error error, tblite_result res, const char* filename) {
  if (!res) {
    set_err(error, "Result container is missing");
    return;
  }
  const size_t nat = res->nat, nsh = res->nsh, nao = res->nao;
  if (!res->has_wfn || res->P.size() != nao * nao || res->C.size() != nao * nao ||
      res->emo.size() < nao || res->focc.size() < nao || res->n0at.size() != nat) {
    set_err(error, "Result does not contain wavefunction");
    return;
  }
  auto arr = [](std::vector<size_t> shape, const double* p) {
    tb::NpyArray a;
    size_t count = 1;
    for (size_t d : shape) count *= d;
    a.shape = std::move(shape);
    a.data.assign(p, p + count);
    return a;
  };
  const std::string pre = "tblite0_";
  std::vector<std::pair<std::string, tb::NpyArray>> out = {
      {pre + "kt", arr({1}, &res->kt)},
      {pre + "nel", arr({2}, res->nel)},
      {pre + "n0at", arr({nat}, res->n0at.data())},
      {pre + "n0sh", arr({nsh}, res->n0sh.data())},
      {pre + "density", arr({nao, nao, 1}, res->P.data())},
      {pre + "coeff", arr({nao, nao, 1}, res->C.data())},
      {pre + "emo", arr({nao, 1}, res->emo.data())},
      {pre + "focc", arr({nao, 1}, res->focc.data())},
      {pre + "qat", arr({nat, 1}, res->qat.data())},
      {pre + "qsh", arr({nsh, 1}, res->qsh.data())},
      {pre + "dpat", arr({3, nat, 1}, res->dpat.data())},
      {pre + "qpat", arr({6, nat, 1}, res->qpat.data())}};
  try {
    tb::npz_write(filename ? filename : "", out);
  } catch (const std::exception& e) {
    set_err(error, e.what());
  }
}

void tblite_load_result_wavefunction(tblite_error error, tblite_result res, const char* filename) {
  if (!res) {
    set_err(error, "Result container is missing");
    return;
  }
  const std::string file = filename ? filename : "";
  try {
    const auto m = tb::npz_read(file);
    auto get = [&](const char* key) -> const tb::NpyArray& {
      const auto it = m.find(std::string("tblite0_") + key);
      if (it == m.end()) throw std::runtime_error(std::string("'") + file + "' has no " + key);
      return it->second;
    };
    const auto &n0at = get("n0at"), &n0sh = get("n0sh"), &emo = get("emo"), &qat = get("qat"),
               &qsh = get("qsh"), &dpat = get("dpat"), &qpat = get("qpat"), &den = get("density"),
               &coeff = get("coeff"), &focc = get("focc"), &nel = get("nel"), &kt = get("kt");
    auto dim = [](const tb::NpyArray& a, size_t k) { return k < a.shape.size() ? a.shape[k] : 1; };
    const size_t nat = n0at.data.size(), nsh = n0sh.data.size(), nao = dim(emo, 0);
    if (dim(qat, 0) != nat || dim(dpat, 1) != nat || dim(qpat, 1) != nat || dim(dpat, 0) != 3 ||
        dim(qpat, 0) != 6)
      throw std::runtime_error("Dimension mismatch in '" + file + "' for number of atoms");
    if (dim(qsh, 0) != nsh)
      throw std::runtime_error("Dimension mismatch in '" + file + "' for number of shells");
    if (dim(den, 0) != nao || dim(den, 1) != nao || dim(coeff, 0) != nao ||
        dim(coeff, 1) != nao || dim(focc, 0) != nao)
      throw std::runtime_error("Dimension mismatch in '" + file + "' for number of orbitals");
    if (nel.data.size() < 2 || kt.data.empty())
      throw std::runtime_error("Dimension mismatch in '" + file + "' for number of spins");
    // first spin channel: the total (closed shell) or charge part of the restart data
    auto first = [&file](const tb::NpyArray& a, size_t count) {
      if (a.data.size() < count)  // e.g. a trailing dimension of 0
        throw std::runtime_error("Dimension mismatch in '" + file + "'");
      return std::vector<double>(a.data.begin(), a.data.begin() + count);
    };
    res->nat = (int)nat;
    res->nsh = (int)nsh;
    res->nao = (int)nao;
    res->n0at = n0at.data;
    res->n0sh = n0sh.data;
    res->nel[0] = nel.data[0];
    res->nel[1] = nel.data[1];
    res->kt = kt.data[0];
    res->qat = first(qat, nat);
    res->qsh = first(qsh, nsh);
    res->dpat = first(dpat, 3 * nat);
    res->qpat = first(qpat, 6 * nat);
    res->P = first(den, nao * nao);
    res->C = first(coeff, nao * nao);
    res->emo = first(emo, nao);
    res->focc = first(focc, nao);
    res->has_wfn = true;
    res->has_energy = false;
    res->gap.clear();
  } catch (const std::exception& e) {
    set_err(error, e.what());
  }
}
void tblite_delete_result(tblite_result* r) {
  if (r && *r) {
    delete *r;
    *r = nullptr;
  }
}

#define RESULT_GUARD(cond, msg)  \
  if (!res) {                    \
    set_err(error, "Result container is missing"); \
    return;                      \
  }                              \
  if (!(cond)) {                 \
    set_err(error, msg);         \
    return;                      \
  }

void tblite_get_result_number_of_atoms(tblite_error error, tblite_result res, int* nat) {
  RESULT_GUARD(res->has_energy, "Result does not contain number of atoms");
  *nat = res->nat;
}
void tblite_get_result_number_of_shells(tblite_error error, tblite_result res, int* nsh) {
  RESULT_GUARD(res->has_wfn, "Result does not contain number of shells");
  *nsh = res->nsh;
}
void tblite_get_result_number_of_orbitals(tblite_error error, tblite_result res, int* nao) {
  RESULT_GUARD(res->has_wfn, "Result does not contain number of orbitals");
  *nao = res->nao;
}
void tblite_get_result_number_of_spins(tblite_error error, tblite_result res, int* nspin) {
  RESULT_GUARD(res->has_wfn, "Result does not contain number of spins");
  *nspin = 1;
}
void tblite_get_result_energy(tblite_error error, tblite_result res, double* energy) {
  RESULT_GUARD(res->has_energy, "Result does not contain energy");
  *energy = res->energy;
}
void tblite_get_result_energies(tblite_error error, tblite_result res, double* energies) {
  RESULT_GUARD(res->has_energy, "Result does not contain atom-resolved energies");
  std::copy(res->energies.begin(), res->energies.end(), energies);
}
void tblite_get_result_gradient(tblite_error error, tblite_result res, double* gradient) {
  RESULT_GUARD(!res->gradient.empty(), "Result does not contain gradient");
  std::copy(res->gradient.begin(), res->gradient.end(), gradient);
}
void tblite_get_result_virial(tblite_error error, tblite_result res, double* sigma) {
  RESULT_GUARD(!res->sigma.empty(), "Result does not contain virial");
  std::copy(res->sigma.begin(), res->sigma.end(), sigma);
}
void tblite_get_result_charges(tblite_error error, tblite_result res, double* charges) {
  RESULT_GUARD(res->has_wfn, "Result does not contain atomic charges");
  std::copy(res->qat.begin(), res->qat.end(), charges);
}
void tblite_gb300_get_result_shell_charges(tblite_error error, tblite_result res, double* qsh) {
  RESULT_GUARD(res->has_wfn && (int)res->qsh.size() == res->nsh,
               "Result does not contain shell charges");
  std::copy(res->qsh.begin(), res->qsh.end(), qsh);
}
void tblite_get_result_bond_orders(tblite_error error, tblite_result res, double* mbo) {
  RESULT_GUARD(res->has_energy || res->has_wfn, "Result does not contain bond orders");
  RESULT_GUARD(res->has_pp("bond-orders") && !res->wbo.empty(),
               "Could not find bond orders in results dictionary");
  std::copy(res->wbo.begin(), res->wbo.end(), mbo);
}
void tblite_get_result_dipole(tblite_error error, tblite_result res, double dipole[3]) {
  RESULT_GUARD(res->has_pp("molecular-dipole"), "Result does not contain dipole moment");
  for (int k = 0; k < 3; ++k) dipole[k] = res->dipole[k];
}
void tblite_get_result_quadrupole(tblite_error error, tblite_result res, double quadrupole[6]) {
  RESULT_GUARD(res->has_pp("molecular-quadrupole"), "Result does not contain quadrupole moment");
  for (int k = 0; k < 6; ++k) quadrupole[k] = res->quadrupole[k];
}
void tblite_get_result_orbital_energies(tblite_error error, tblite_result res, double* emo) {
  RESULT_GUARD(res->has_wfn && !res->emo.empty(), "Result does not contain orbital energies");
  std::copy(res->emo.begin(), res->emo.end(), emo);
}
void tblite_get_result_orbital_occupations(tblite_error error, tblite_result res, double* occ) {
  RESULT_GUARD(res->has_wfn && !res->focc.empty(), "Result does not contain orbital occupations");
  std::copy(res->focc.begin(), res->focc.end(), occ);
}
void tblite_get_result_orbital_coefficients(tblite_error error, tblite_result res, double* cmat) {
  RESULT_GUARD(!res->C.empty(), "Result does not contain orbital coefficients");
  std::copy(res->C.begin(), res->C.end(), cmat);
}
void tblite_get_result_density_matrix(tblite_error error, tblite_result res, double* pmat) {
  RESULT_GUARD(!res->P.empty(), "Result does not contain density matrix");
  std::copy(res->P.begin(), res->P.end(), pmat);
}
void tblite_get_result_overlap_matrix(tblite_error error, tblite_result res, double* smat) {
  RESULT_GUARD(!res->S.empty(), "Result does not contain overlap matrix");
  std::copy(res->S.begin(), res->S.end(), smat);
}
void tblite_get_result_hamiltonian_matrix(tblite_error error, tblite_result res, double* hmat) {
  RESULT_GUARD(!res->H.empty(), "Result does not contain Hamiltonian matrix");
  std::copy(res->H.begin(), res->H.end(), hmat);
}

void tblite_calculator_push_back(tblite_context ctx, tblite_calculator calc,
                                 tblite_container* cont) {
  if (!ctx) return;
  if (!calc) {
    ctx->push("Calculator object is missing");
    return;
  }
  if (!cont || !*cont) {
    ctx->push("Container object is missing");
    return;
  }
  if ((*cont)->solv) {
    if (calc->solv) {
      ctx->push("Calculator already holds an implicit solvation model");
      return;
    }
    if ((*cont)->solv->nat != calc->nat) {
      ctx->push("Solvation model was built for a different structure");
      return;
    }
    calc->solv = std::move((*cont)->solv);
  }
  if ((*cont)->field) {
    if (calc->method != 2) {
      ctx->push("An electric field needs the atomic dipole moments of the GFN2-xTB form in the "
                "GPU engine");
      return;
    }
    if (calc->has_field) {
      ctx->push("Calculator already holds an electric field");
      return;
    }
    calc->has_field = true;
    for (int k = 0; k < 3; ++k) calc->efield[k] = (*cont)->efield[k];
  }
  delete *cont;  // the container moves into the calculator (api/container.f90:53-94)
  *cont = nullptr;
}

void tblite_delete_container(tblite_container* cont) {
  if (cont && *cont) {
    delete *cont;
    *cont = nullptr;
  }
}

// interactions of the reference that the GPU engine does not provide: each reports an error and
// returns NULL (include/tblite/container.h:31-45, solvation.h:54-95)
// homogeneous electric field (external/field.f90): vat -= E.R_A, vdp -= E; the container
// moves into a calculator of the GFN2 form (its dipole moments enter the SCF)
tblite_container tblite_new_electric_field(double* efield) {
  if (!efield) return nullptr;  // the reference's signature has no error handle
  auto* cont = new _tblite_container();
  cont->field = true;
  for (int k = 0; k < 3; ++k) cont->efield[k] = efield[k];
  return cont;
}
tblite_container tblite_new_spin_polarization(tblite_context ctx, tblite_structure mol,
                                              tblite_calculator calc, double wscale) {
  (void)mol;
  (void)calc;
  (void)wscale;
  if (ctx) ctx->push("Spin polarization is not available in the GPU engine");
  return nullptr;
}
tblite_container tblite_new_gb_solvation_epsilon(tblite_error error, tblite_structure mol,
                                                 double eps, enum tblite_solvation_param version,
                                                 enum tblite_born_kernel born) {
  if (!error) return nullptr;
  if (!mol) {
    set_err(error, "Molecular structure data is missing");
    return nullptr;
  }
  if (version != tblite_solvation_gbe && version != tblite_solvation_gb) {
    set_err(error, "Unknown solvation model requested");
    return nullptr;
  }
  if (born != tblite_born_still && born != tblite_born_p16) {
    set_err(error, "Unknown Born interaction kernel requested");
    return nullptr;
  }
  if (!(eps > 0.0)) {
    set_err(error, "Dielectric constant must be positive");
    return nullptr;
  }
  try {
    auto* cont = new _tblite_container();
    cont->solv = build_gb_epsilon(mol, eps, version == tblite_solvation_gbe, (int)born);
    return cont;
  } catch (const std::exception& e) {
    set_err(error, e.what());
    return nullptr;
  }
}
tblite_container tblite_new_ddx_solvation_epsilon(tblite_error error, tblite_structure mol,
                                                  double eps, enum tblite_solvation_param model) {
  (void)mol;
  (void)eps;
  (void)model;
  set_err(error, "ddX solvation is not available in the GPU engine");
  return nullptr;
}
tblite_container tblite_new_ddx_solvation_solvent(tblite_error error, tblite_structure mol,
                                                  char* solvent, enum tblite_solvation_param model) {
  (void)mol;
  (void)solvent;
  (void)model;
  set_err(error, "ddX solvation is not available in the GPU engine");
  return nullptr;
}
tblite_container tblite_new_alpb_solvation_solvent(tblite_error error, tblite_structure mol,
                                                   char* solvent,
                                                   enum tblite_solvation_param version,
                                                   enum tblite_ref_solvation_state refstate) {
  if (!error) return nullptr;
  if (!mol) {
    set_err(error, "Molecular structure data is missing");
    return nullptr;
  }
  std::string name = solvent ? solvent : "";
  for (auto& ch : name) ch = (char)tolower((unsigned char)ch);
  if (name != "water" && name != "h2o") {
    set_err(error, "Solvent '" + name + "' is not available: the GPU engine provides water only");
    return nullptr;
  }
  if (version != tblite_solvation_alpb_gfn2 && version != tblite_solvation_gbsa_gfn2) {
    set_err(error, "Only the ALPB and GBSA models with GFN2 parameters are available in the GPU "
                   "engine");
    return nullptr;
  }
  if (refstate < 1 || refstate > 3) {
    set_err(error, "Unknown reference state for the solvation free energy");
    return nullptr;
  }
  try {
    auto* cont = new _tblite_container();
    cont->solv = build_solvation(mol, (int)refstate, version == tblite_solvation_gbsa_gfn2);
    return cont;
  } catch (const std::exception& e) {
    set_err(error, e.what());
    return nullptr;
  }
}

tblite_calculator tblite_new_gfn2_calculator(tblite_context ctx, tblite_structure mol,
                                            tblite_xtb_config* config) {
  (void)config;
  if (!ctx) return nullptr;
  if (!mol) {
    ctx->push("Molecular structure data is missing");
    return nullptr;
  }
  auto* c = new _tblite_calculator();
  try {
    ParamRecord rec;
    export_gfn2(rec);
    build_calculator(c, mol, rec);
  } catch (const std::exception& e) {
    ctx->push(e.what());
    delete c;
    return nullptr;
  }
  return c;
}
tblite_calculator tblite_new_gfn1_calculator(tblite_context ctx, tblite_structure mol,
                                            tblite_xtb_config* config) {
  (void)config;
  if (!ctx) return nullptr;
  if (!mol) {
    ctx->push("Molecular structure data is missing");
    return nullptr;
  }
  auto* c = new _tblite_calculator();
  try {
    ParamRecord rec;
    export_gfn1(rec);
    build_calculator(c, mol, rec);
  } catch (const std::exception& e) {
    ctx->push(e.what());
    delete c;
    return nullptr;
  }
  return c;
}
tblite_calculator tblite_new_xtb_calculator(tblite_context ctx, tblite_structure mol,
                                           tblite_param param, tblite_xtb_config* config) {
  (void)config;
  if (!ctx) return nullptr;
  if (!mol) {
    ctx->push("Molecular structure data is missing");
    return nullptr;
  }
  if (!param) {
    ctx->push("Parametrization record is missing");
    return nullptr;
  }
  if (!param->set) {
    ctx->push("Parametrization record is empty");
    return nullptr;
  }
  auto* c = new _tblite_calculator();
  try {
    build_calculator(c, mol, param->rec);
  } catch (const std::exception& e) {
    ctx->push(e.what());
    delete c;
    return nullptr;
  }
  return c;
}
void tblite_gb300_set_calculator_fault(tblite_context ctx, tblite_calculator calc, int kind) {
  if (!ctx) return;
  if (!calc) {
    ctx->push("Calculator object is missing");
    return;
  }
  if (kind < 0 || kind > 1) {
    ctx->push("fault kind must be 0 (none) or 1 (overlap not positive definite)");
    return;
  }
  calc->fault = kind;
}
tblite_calculator tblite_new_ipea1_calculator(tblite_context ctx, tblite_structure mol,
                                             tblite_xtb_config* config) {
  (void)config;
  if (!ctx) return nullptr;
  if (!mol) {
    ctx->push("Molecular structure data is missing");
    return nullptr;
  }
  auto* c = new _tblite_calculator();
  try {
    ParamRecord rec;
    export_ipea1(rec);  // the GFN1 form with IPEA1-xTB's tables (xtb/ipea1.f90:529-564)
    build_calculator(c, mol, rec);
  } catch (const std::exception& e) {
    ctx->push(e.what());
    delete c;
    return nullptr;
  }
  return c;
}
void tblite_delete_calculator(tblite_calculator* c) {
  if (c && *c) {
    delete *c;
    *c = nullptr;
  }
}

#define CALC_GUARD                                   \
  if (!ctx) return;                                  \
  if (!calc) {                                       \
    ctx->push("Calculator object is missing");       \
    return;                                          \
  }

void tblite_set_calculator_accuracy(tblite_context ctx, tblite_calculator calc, double acc) {
  CALC_GUARD;
  calc->accuracy = acc;
}
void tblite_set_calculator_max_iter(tblite_context ctx, tblite_calculator calc, int max_iter) {
  CALC_GUARD;
  calc->max_iter = max_iter;
}
void tblite_set_calculator_mixer_damping(tblite_context ctx, tblite_calculator calc, double d) {
  CALC_GUARD;
  calc->damping = d;
}
void tblite_set_calculator_mixer_memory(tblite_context ctx, tblite_calculator calc, int memory) {
  CALC_GUARD;
  calc->memory = memory;
}
void tblite_set_calculator_mixer(tblite_context ctx, tblite_calculator calc, tblite_mixer mixer) {
  CALC_GUARD;
  if (mixer != TBLITE_MIXER_BROYDEN) ctx->push("Unknown mixer selected");
}
void tblite_set_calculator_temperature_annealing(tblite_context ctx, tblite_calculator calc,
                                                 double initial_etemp, int hold, int cycles) {
  CALC_GUARD;
  calc->anneal = true;
  calc->anneal_kt = initial_etemp;
  calc->anneal_hold = hold;
  calc->anneal_cycles = cycles;
}
void tblite_set_calculator_guess(tblite_context ctx, tblite_calculator calc, tblite_guess guess) {
  CALC_GUARD;
  if (guess != TBLITE_GUESS_SAD) {
    ctx->push("Only the SAD guess is available in the GPU engine");
    return;
  }
  calc->guess = guess;
}
void tblite_set_calculator_temperature(tblite_context ctx, tblite_calculator calc, double etemp) {
  CALC_GUARD;
  calc->etemp = etemp;
}
void tblite_set_calculator_save_integrals(tblite_context ctx, tblite_calculator calc, int v) {
  CALC_GUARD;
  calc->save_integrals = v;
}
void tblite_get_calculator_shell_count(tblite_context ctx, tblite_calculator calc, int* nsh) {
  CALC_GUARD;
  *nsh = calc->nsh;
}
void tblite_get_calculator_shell_map(tblite_context ctx, tblite_calculator calc, int* sh2at) {
  CALC_GUARD;
  std::copy(calc->sh_atom.begin(), calc->sh_atom.end(), sh2at);
}
void tblite_get_calculator_angular_momenta(tblite_context ctx, tblite_calculator calc, int* am) {
  CALC_GUARD;
  std::copy(calc->sh_l.begin(), calc->sh_l.end(), am);
}
void tblite_get_calculator_orbital_count(tblite_context ctx, tblite_calculator calc, int* nao) {
  CALC_GUARD;
  *nao = calc->nao;
}
void tblite_get_calculator_orbital_map(tblite_context ctx, tblite_calculator calc, int* ao2sh) {
  CALC_GUARD;
  std::copy(calc->ao_sh.begin(), calc->ao_sh.end(), ao2sh);
}

void tblite_get_singlepoint(tblite_context ctx, tblite_structure mol, tblite_calculator calc,
                            tblite_result res) {
  if (!ctx) return;
  if (!mol) {
    ctx->push("Molecular structure data is missing");
    return;
  }
  if (!calc) {
    ctx->push("Calculator object is missing");
    return;
  }
  if (!res) {
    ctx->push("Result container is missing");
    return;
  }
  calc->default_post_processing();  // bond orders and molecular moments unless asked otherwise
  try {
    singlepoint(ctx, mol, calc, res);
  } catch (const std::exception& e) {
    ctx->push(e.what());
  }
}

}  // extern "C"
