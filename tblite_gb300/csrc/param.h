// Parametrisation records of the xTB methods (reference include/tblite/param.h,
// src/tblite/param.f90 and param/*.f90): the global model constants and the element records of
// a method, in atomic units (levels and CN shifts in Hartree).  They are filled from the
// built-in GFN2-xTB / GFN1-xTB tables (tblite_export_gfn2_param, tblite_export_gfn1_param), read
// from or written to data tables in the reference's TOML layout (tblite_load_param,
// tblite_dump_param), and turned into a calculator (tblite_new_xtb_calculator).  The built-in
// calculators are made from the exported records by the same code, so a record that is exported
// and used unchanged gives the same calculator bit for bit.
#pragma once
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "table.h"

namespace tb {

struct ElementRecord {
  std::string sym;
  int num = 0;
  int nsh = 0;
  std::vector<int> lsh, pqn, ngauss;
  std::vector<double> levels, slater, refocc, kcn, shpoly, lgam;
  double gam = 0.0, gam3 = 0.0, zeff = 0.0, arep = 0.0, xbond = 0.0, en = 0.0;
  double dkernel = 0.0, qkernel = 0.0, mprad = 0.0, mpvcn = 0.0;
};

struct ParamRecord {
  int version = 0;
  std::string name, reference;
  // hamiltonian.xtb
  std::string cn;
  double wexp = 0.0, kpol = 2.0, enscale = 0.0;
  int lmax = 0;
  double ksh[5][5] = {};  // ksh[l][k]
  std::map<std::pair<int, int>, double> kpair;  // (Z_i >= Z_j) -> factor, entries != 1
  // dispersion.d3 / dispersion.d4
  bool has_dispersion = false, d3 = false, sc = true, smooth = false;
  double s6 = 1.0, s8 = 0.0, a1 = 0.0, a2 = 0.0, s9 = 0.0;
  // repulsion.effective
  bool has_repulsion = false;
  double kexp = 0.0, klight = 0.0;
  // charge.effective
  bool has_charge = false;
  double gexp = 0.0;
  std::string average;
  // thirdorder (shell-resolved Hubbard derivatives, or atom-resolved)
  bool has_thirdorder = false, third_shell = false;
  int third_lmax = 0;
  double third_ksh[5] = {};
  // multipole.damped
  bool has_multipole = false;
  double dmp3 = 0.0, dmp5 = 0.0, mp_kexp = 0.0, mp_shift = 0.0, mp_rmax = 0.0;
  // halogen.classical
  bool has_halogen = false;
  double hal_damping = 0.0, hal_rscale = 0.0;
  std::vector<ElementRecord> element;

  const ElementRecord* get(int z) const {
    for (const auto& e : element)
      if (e.num == z) return &e;
    return nullptr;
  }
  double pair(int zi, int zj) const {
    const auto it = kpair.find(zi >= zj ? std::make_pair(zi, zj) : std::make_pair(zj, zi));
    return it == kpair.end() ? 1.0 : it->second;
  }
};

void export_gfn2(ParamRecord& r);
void export_gfn1(ParamRecord& r);
void export_ipea1(ParamRecord& r);
// reference layout: meta, hamiltonian, dispersion, repulsion, charge, thirdorder, multipole,
// halogen, element.<symbol>; throws std::runtime_error with the reference's messages
void param_load(ParamRecord& r, const TTable& t);
void param_dump(const ParamRecord& r, TTable& t);
// element-pair factor of the GFN1-xTB valence Hamiltonian (the GPU kernel applies the same)
double gfn1_pair_factor(int zi, int zj);
// element-pair factor of IPEA1-xTB (the d-block rule of the GFN1 form only)
double dblock_pair_factor(int zi, int zj);
// element symbol of Z (1..118) and the inverse (0 for an unknown symbol)
std::string element_symbol(int z);
int element_number(const std::string& sym);

}  // namespace tb

struct _tblite_param {
  tb::ParamRecord rec;
  bool set = false;  // filled by an export or a load
};
