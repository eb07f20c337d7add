// Parametrisation records (reference include/tblite/param.h; src/tblite/param.f90,
// param/{element,hamiltonian,dispersion,repulsion,charge,thirdorder,multipole,halogen}.f90;
// the exports of xtb/gfn2.f90:914-1022 and xtb/gfn1.f90:931-1054).  Layout of the tables:
//
//   [meta] name, reference, version, format
//   [hamiltonian.xtb] wexp, kpol, enscale, cn, [hamiltonian.xtb.shell] ss, pp, ... (and the
//        off-diagonal pairs that differ from the mean of the diagonal), [hamiltonian.xtb.kpair]
//        "A-B" factors that differ from 1
//   [dispersion.d4] sc, smooth, s6, s8, a1, a2, s9   or   [dispersion.d3] s6, s8, a1, a2, s9
//   [repulsion.effective] kexp, klight
//   [charge.effective] gexp, average
//   [thirdorder] shell = false  or  [thirdorder.shell] s, p, d, ...
//   [multipole.damped] dmp3, dmp5, kexp, shift, rmax
//   [halogen.classical] damping, rscale
//   [element.<symbol>] shells ("1s", "2p", ...), levels (eV), slater, ngauss, refocc, shpoly,
//        kcn (eV), gam, lgam, gam3, zeff, arep, xbond, en, dkernel, qkernel, mprad, mpvcn
//
// The TOML tables hold levels and CN shifts in eV (divided by 1/27.21138505 Hartree per eV, the
// conversion of param/element.f90); the records hold Hartree.
#include "param.h"

#include <cmath>
#include <cstring>
#include <stdexcept>

#include "api_internal.h"
#include "element_data.inc"
#include "params_gfn1.inc"
#include "params_ipea1.inc"
#include "params_gfn2.inc"

namespace tb {

namespace {

constexpr double EV_TO_AU = 1.0 / 27.21138505;  // param/element.f90
constexpr int MAX_ELEM = 86;
const char* const ANG = "spdfg";

const char* const SYMBOLS[] = {
    "H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg", "Al", "Si", "P",
    "S",  "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn",
    "Ga", "Ge", "As", "Se", "Br", "Kr", "Rb", "Sr", "Y",  "Zr", "Nb", "Mo", "Tc", "Ru", "Rh",
    "Pd", "Ag", "Cd", "In", "Sn", "Sb", "Te", "I",  "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd",
    "Pm", "Sm", "Eu", "Gd", "Tb", "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W",  "Re",
    "Os", "Ir", "Pt", "Au", "Hg", "Tl", "Pb", "Bi", "Po", "At", "Rn", "Fr", "Ra", "Ac", "Th",
    "Pa", "U",  "Np", "Pu", "Am", "Cm", "Bk", "Cf", "Es", "Fm", "Md", "No", "Lr", "Rf", "Db",
    "Sg", "Bh", "Hs", "Mt", "Ds", "Rg", "Cn", "Nh", "Fl", "Mc", "Lv", "Ts", "Og"};

int dblock_row(int z) {
  if (z >= 21 && z <= 29) return 1;
  if (z >= 39 && z <= 47) return 2;
  if (z >= 57 && z <= 79) return 3;
  return 0;
}
}  // namespace

// GFN1-xTB pair factors of the valence Hamiltonian (xtb/gfn1.f90 get_pair_param): H-H, H-B,
// H-N, H-Ni, H-Re, H-Pt, B-P, N-Si, and the mean of the d-block row factors for two transition
// metals
double gfn1_pair_factor(int zi, int zj) {
  const int a = zi < zj ? zi : zj, b = zi < zj ? zj : zi;
  if (a == 1 && b == 1) return 0.96;
  if (a == 1 && b == 5) return 0.95;
  if (a == 1 && b == 7) return 1.04;
  if (a == 1 && b == 28) return 0.90;
  if (a == 1 && (b == 75 || b == 78)) return 0.80;
  if (a == 5 && b == 15) return 0.97;
  if (a == 7 && b == 14) return 1.01;
  const int ti = dblock_row(zi), tj = dblock_row(zj);
  if (ti > 0 && tj > 0) {
    const double kp[3] = {1.1, 1.2, 1.2};
    return 0.5 * (kp[ti - 1] + kp[tj - 1]);
  }
  return 1.0;
}

// IPEA1-xTB pair factors (xtb/ipea1.f90:752-765): the mean of the d-block row factors for two
// transition metals, 1 otherwise
double dblock_pair_factor(int zi, int zj) {
  const int ti = dblock_row(zi), tj = dblock_row(zj);
  if (ti > 0 && tj > 0) {
    const double kp[3] = {1.1, 1.2, 1.2};
    return 0.5 * (kp[ti - 1] + kp[tj - 1]);
  }
  return 1.0;
}

namespace {

// ---- table helpers ------------------------------------------------------------------------
[[noreturn]] void fail(const std::string& m) { throw std::runtime_error(m); }

const TValue* child(const TTable& t, const char* key, int type) {
  const TValue* v = t.find(key);
  return (v && v->type == type) ? v : nullptr;
}
bool get_double(const TTable& t, const char* key, double& out) {
  const TValue* v = t.find(key);
  if (!v) return false;
  if (v->type == T_DOUBLE) out = v->d;
  else if (v->type == T_INT) out = (double)v->i;
  else return false;
  return true;
}
void need_double(const TTable& t, const char* key, double& out, const std::string& msg) {
  if (!get_double(t, key, out)) fail(msg);
}
std::vector<double> doubles(const TValue& v, const std::string& msg) {
  std::vector<double> out;
  for (const TValue& e : v.a->v) {
    if (e.type == T_DOUBLE) out.push_back(e.d);
    else if (e.type == T_INT) out.push_back((double)e.i);
    else fail(msg);
  }
  return out;
}
std::shared_ptr<TArray> darray(TTable& t, const char* key, const std::vector<double>& v,
                               double scale = 1.0) {
  auto a = t.add_array(key);
  for (double x : v) a->v.push_back(TValue::of(x / scale));
  return a;
}

void load_element(ElementRecord& e, const std::string& sym, const TTable& t) {
  e.sym = sym;
  e.num = element_number(sym);
  const TValue* v = child(t, "shells", T_ARRAY);
  if (!v) fail("No shells specified for " + sym);
  e.nsh = (int)v->a->v.size();
  for (const TValue& s : v->a->v) {
    if (s.type != T_CHAR || s.s.size() != 2 || s.s[0] < '1' || s.s[0] > '6' ||
        !std::strchr(ANG, s.s[1]) || !s.s[1])
      fail("Cannot read shell specification for " + sym);
    e.pqn.push_back(s.s[0] - '0');
    e.lsh.push_back((int)(std::strchr(ANG, s.s[1]) - ANG));
  }
  auto per_shell = [&](const char* key, const std::string& what, bool required, double def,
                       double scale) {
    std::vector<double> out;
    const TValue* a = child(t, key, T_ARRAY);
    if (!a) {
      if (required) fail("No " + what + " specified for " + sym);
      out.assign(e.nsh, def);
      return out;
    }
    out = doubles(*a, "Cannot read " + what + " for " + sym);
    if ((int)out.size() != e.nsh) fail("Number of " + what + " does not match shells for " + sym);
    for (double& x : out) x *= scale;
    return out;
  };
  e.levels = per_shell("levels", "atomic levels", true, 0.0, EV_TO_AU);
  e.slater = per_shell("slater", "slater exponents", true, 0.0, 1.0);
  e.refocc = per_shell("refocc", "reference occupation", true, 0.0, 1.0);
  {
    const std::vector<double> ng = per_shell("ngauss", "number of primitives", false, 6.0, 1.0);
    for (double x : ng) e.ngauss.push_back((int)x);
  }
  e.shpoly = per_shell("shpoly", "shell-polynomials", true, 0.0, 1.0);
  e.kcn = per_shell("kcn", "CN shifts", false, 0.0, EV_TO_AU);
  need_double(t, "gam", e.gam, "Invalid atomic Hubbard parameter for " + sym);
  e.lgam = per_shell("lgam", "shell hardness scaling", false, 1.0, 1.0);
  need_double(t, "gam3", e.gam3, "Invalid atomic Hubbard derivative for " + sym);
  need_double(t, "zeff", e.zeff, "Invalid effective nuclear charge for " + sym);
  need_double(t, "arep", e.arep, "Invalid repulsion exponent for " + sym);
  e.dkernel = e.qkernel = e.mprad = e.mpvcn = 0.0;
  get_double(t, "dkernel", e.dkernel);
  get_double(t, "qkernel", e.qkernel);
  get_double(t, "mprad", e.mprad);
  get_double(t, "mpvcn", e.mpvcn);
  e.xbond = 0.0;
  get_double(t, "xbond", e.xbond);
  // the reference defaults the electronegativity to its Pauling table (mctc-lib); here the
  // element-data pack of the engine stands in for that table
  e.en = (e.num >= 1 && e.num <= MAX_ELEM) ? EXT_EN[e.num - 1] : NAN;
  get_double(t, "en", e.en);
}

void dump_element(const ElementRecord& e, TTable& t) {
  auto sh = t.add_array("shells");
  for (int i = 0; i < e.nsh; ++i)
    sh->v.push_back(TValue::of(std::string(1, (char)('0' + e.pqn[i])) + ANG[e.lsh[i]]));
  darray(t, "levels", e.levels, EV_TO_AU);
  darray(t, "slater", e.slater);
  auto ng = t.add_array("ngauss");
  for (int g : e.ngauss) ng->v.push_back(TValue::of((int64_t)g));
  darray(t, "refocc", e.refocc);
  darray(t, "shpoly", e.shpoly);
  darray(t, "kcn", e.kcn, EV_TO_AU);
  t.set("gam", TValue::of(e.gam));
  darray(t, "lgam", e.lgam);
  t.set("gam3", TValue::of(e.gam3));
  t.set("zeff", TValue::of(e.zeff));
  t.set("arep", TValue::of(e.arep));
  t.set("xbond", TValue::of(e.xbond));
  t.set("en", TValue::of(e.en));
  t.set("dkernel", TValue::of(e.dkernel));
  t.set("qkernel", TValue::of(e.qkernel));
  t.set("mprad", TValue::of(e.mprad));
  t.set("mpvcn", TValue::of(e.mpvcn));
}

}  // namespace

std::string element_symbol(int z) {
  return (z >= 1 && z <= 118) ? SYMBOLS[z - 1] : std::string();
}
int element_number(const std::string& sym) {
  for (int z = 1; z <= 118; ++z)
    if (sym == SYMBOLS[z - 1]) return z;
  return 0;
}

// ---- exports of the built-in methods -----------------------------------------------------
void export_gfn2(ParamRecord& r) {
  r = ParamRecord();
  r.version = 1;
  r.name = "GFN2-xTB";
  r.reference =
      "C. Bannwarth, S. Ehlert and S. Grimme., J. Chem. Theory Comput., 2019, 15, 1652-1671. "
      "DOI: 10.1021/acs.jctc.8b01176";
  r.cn = "dexp";
  r.enscale = GFN2_ENSCALE;
  r.wexp = GFN2_WEXP;
  r.lmax = 2;
  for (int l = 0; l < 5; ++l)
    for (int k = 0; k < 5; ++k) r.ksh[l][k] = GFN2_KSHELL[l * 5 + k];
  r.kpol = 2.0;
  r.has_dispersion = true;
  r.d3 = false;
  r.sc = true;
  r.smooth = false;
  r.s6 = GFN2_S6;
  r.s8 = GFN2_S8;
  r.a1 = GFN2_A1;
  r.a2 = GFN2_A2;
  r.s9 = GFN2_S9;
  r.has_repulsion = true;
  r.kexp = GFN2_REP_KEXP;
  r.klight = GFN2_REP_KEXP_LIGHT;
  r.has_charge = true;
  r.gexp = GFN2_GEXP;
  r.average = "arithmetic";
  r.has_thirdorder = true;
  r.third_shell = true;
  r.third_lmax = 2;
  for (int l = 0; l < 5; ++l) r.third_ksh[l] = GFN2_SHELL_HUBBARD_DERIVS[l];
  r.has_multipole = true;
  r.dmp3 = GFN2_MP_DMP3;
  r.dmp5 = GFN2_MP_DMP5;
  r.mp_kexp = GFN2_MP_KEXP;
  r.mp_shift = GFN2_MP_SHIFT;
  r.mp_rmax = GFN2_MP_RMAX;
  for (int z = 1; z <= MAX_ELEM; ++z) {
    ElementRecord e;
    e.sym = element_symbol(z);
    e.num = z;
    e.zeff = GFN2_REP_ZEFF[z - 1];
    e.arep = GFN2_REP_ALPHA[z - 1];
    e.nsh = GFN2_NSHELL[z - 1];
    for (int s = 0; s < e.nsh; ++s) {
      const int l = GFN2_ANG_SHELL[(z - 1) * 3 + s];
      e.lsh.push_back(l);
      e.pqn.push_back(GFN2_PRINCIPAL_QUANTUM_NUMBER[(z - 1) * 3 + s]);
      e.ngauss.push_back(GFN2_NUMBER_OF_PRIMITIVES[(z - 1) * 3 + s]);
      e.levels.push_back(GFN2_P_SELFENERGY[(z - 1) * 3 + s]);
      e.slater.push_back(GFN2_SLATER_EXPONENT[(z - 1) * 3 + s]);
      e.refocc.push_back(GFN2_REFERENCE_OCC[(z - 1) * 3 + l]);
      e.kcn.push_back(GFN2_P_KCN[(z - 1) * 3 + l]);
      e.shpoly.push_back(GFN2_P_SHPOLY[(z - 1) * 3 + l]);
      e.lgam.push_back(GFN2_SHELL_HUBBARD[(z - 1) * 3 + l]);
    }
    e.gam = GFN2_HUBBARD_PARAMETER[z - 1];
    e.gam3 = GFN2_P_HUBBARD_DERIVS[z - 1];
    e.mpvcn = GFN2_P_VCN[z - 1];
    e.mprad = GFN2_P_RAD[z - 1];
    e.dkernel = GFN2_P_DKERNEL[z - 1];
    e.qkernel = GFN2_P_QKERNEL[z - 1];
    e.en = EXT_EN[z - 1];
    r.element.push_back(std::move(e));
  }
}

// element tables of the two GFN1-form parametrisations, as types for export_xtb1
#define XTB1_TABLES(P)                                                                      \
  static constexpr const double& ENSCALE = P##_ENSCALE;                                    \
  static constexpr const double& KDIFF = P##_KDIFF;                                        \
  static constexpr const double& S6 = P##_S6;                                              \
  static constexpr const double& S8 = P##_S8;                                              \
  static constexpr const double& A1 = P##_A1;                                              \
  static constexpr const double& A2 = P##_A2;                                              \
  static constexpr const double& S9 = P##_S9;                                              \
  static constexpr const double& REP_KEXP = P##_REP_KEXP;                                  \
  static constexpr const double& GEXP = P##_GEXP;                                          \
  static constexpr const double& HALOGEN_DAMPING = P##_HALOGEN_DAMPING;                    \
  static constexpr const double& HALOGEN_RADSCALE = P##_HALOGEN_RADSCALE;                  \
  static constexpr const double* KSHELL = P##_KSHELL;                                      \
  static constexpr const double* REP_ZEFF = P##_REP_ZEFF;                                  \
  static constexpr const double* REP_ALPHA = P##_REP_ALPHA;                                \
  static constexpr const int* NSHELL = P##_NSHELL;                                         \
  static constexpr const int* ANG_SHELL = P##_ANG_SHELL;                                   \
  static constexpr const int* PRINCIPAL_QUANTUM_NUMBER = P##_PRINCIPAL_QUANTUM_NUMBER;     \
  static constexpr const int* NUMBER_OF_PRIMITIVES = P##_NUMBER_OF_PRIMITIVES;             \
  static constexpr const double* P_SELFENERGY = P##_P_SELFENERGY;                          \
  static constexpr const double* SLATER_EXPONENT = P##_SLATER_EXPONENT;                    \
  static constexpr const double* REFERENCE_OCC = P##_REFERENCE_OCC;                        \
  static constexpr const double* P_KCN = P##_P_KCN;                                        \
  static constexpr const double* P_SHPOLY = P##_P_SHPOLY;                                  \
  static constexpr const double* SHELL_HUBBARD = P##_SHELL_HUBBARD;                        \
  static constexpr const double* HUBBARD_PARAMETER = P##_HUBBARD_PARAMETER;                \
  static constexpr const double* P_HUBBARD_DERIVS = P##_P_HUBBARD_DERIVS;                  \
  static constexpr const double* HALOGEN_BOND = P##_HALOGEN_BOND;
struct Gfn1Tables {
  XTB1_TABLES(GFN1)
};
struct Ipea1Tables {
  XTB1_TABLES(IPEA1)
};
#undef XTB1_TABLES

template <class T>
static void export_xtb1(ParamRecord& r, bool ipea1) {
  r = ParamRecord();
  r.version = 1;
  r.name = ipea1 ? "IPEA1-xTB" : "GFN1-xTB";
  r.reference =
      ipea1 ? "V. Asgeirsson, C. Bauer and S. Grimme, Chem. Sci., 2017, 8, 4879. DOI: "
              "10.1039/c7sc00601b"
            : "S. Grimme, C. Bannwarth, P. Shushkov, J. Chem. Theory Comput., 2017, 13, "
              "1989-2009. DOI: 10.1021/acs.jctc.7b00118";
  r.cn = "exp";
  r.enscale = T::ENSCALE;
  r.wexp = 0.0;
  r.lmax = 2;
  for (int l = 0; l < 5; ++l)
    for (int k = 0; k < 5; ++k) r.ksh[l][k] = (l < 3 && k < 3) ? T::KSHELL[l * 3 + k] : 0.0;
  r.kpol = T::KDIFF;
  for (int zi = 1; zi <= MAX_ELEM; ++zi)
    for (int zj = 1; zj <= zi; ++zj) {
      const double k = ipea1 ? dblock_pair_factor(zi, zj) : gfn1_pair_factor(zi, zj);
      if (k != 1.0) r.kpair[{zi, zj}] = k;
    }
  r.has_dispersion = true;
  r.d3 = true;
  r.sc = false;
  r.smooth = false;
  r.s6 = T::S6;
  r.s8 = T::S8;
  r.a1 = T::A1;
  r.a2 = T::A2;
  r.s9 = T::S9;
  r.has_repulsion = true;
  r.kexp = T::REP_KEXP;
  r.klight = T::REP_KEXP;
  r.has_charge = true;
  r.gexp = T::GEXP;
  r.average = "harmonic";
  r.has_thirdorder = true;
  r.third_shell = false;
  r.third_lmax = 0;
  r.has_halogen = true;
  r.hal_damping = T::HALOGEN_DAMPING;
  r.hal_rscale = T::HALOGEN_RADSCALE;
  for (int z = 1; z <= MAX_ELEM; ++z) {
    ElementRecord e;
    e.sym = element_symbol(z);
    e.num = z;
    e.zeff = T::REP_ZEFF[z - 1];
    e.arep = T::REP_ALPHA[z - 1];
    e.nsh = T::NSHELL[z - 1];
    bool seen[5] = {false, false, false, false, false};
    for (int s = 0; s < e.nsh; ++s) {
      const int l = T::ANG_SHELL[(z - 1) * 3 + s];
      const bool valence = !seen[l];
      seen[l] = true;
      e.lsh.push_back(l);
      e.pqn.push_back(T::PRINCIPAL_QUANTUM_NUMBER[(z - 1) * 3 + s]);
      e.ngauss.push_back(T::NUMBER_OF_PRIMITIVES[(z - 1) * 3 + s]);
      e.levels.push_back(T::P_SELFENERGY[(z - 1) * 3 + s]);
      e.slater.push_back(T::SLATER_EXPONENT[(z - 1) * 3 + s]);
      // the reference's IPEA1 export keeps the occupation of polarisation shells too
      // (xtb/ipea1.f90:1015); calculators take occupations of valence shells only
      e.refocc.push_back(valence || ipea1 ? T::REFERENCE_OCC[(z - 1) * 3 + l] : 0.0);
      e.kcn.push_back(T::P_KCN[(z - 1) * 3 + s]);
      e.shpoly.push_back(T::P_SHPOLY[(z - 1) * 3 + l]);
      e.lgam.push_back(T::SHELL_HUBBARD[(z - 1) * 3 + l]);
    }
    e.gam = T::HUBBARD_PARAMETER[z - 1];
    e.gam3 = T::P_HUBBARD_DERIVS[z - 1];
    e.xbond = T::HALOGEN_BOND[z - 1];
    e.en = EXT_EN[z - 1];
    r.element.push_back(std::move(e));
  }
}

void export_gfn1(ParamRecord& r) { export_xtb1<Gfn1Tables>(r, false); }
void export_ipea1(ParamRecord& r) { export_xtb1<Ipea1Tables>(r, true); }

// ---- table <-> record ---------------------------------------------------------------------
void param_load(ParamRecord& r, const TTable& t) {
  r = ParamRecord();
  if (const TValue* m = child(t, "meta", T_TABLE)) {
    double fmt = 1.0;
    get_double(*m->t, "format", fmt);
    if (fmt < 1) fail("Parametrer file format must be a positive version");
    if (fmt > 1) fail("Requested future parameter file format which is not yet supported");
    double v = 0.0;
    if (get_double(*m->t, "version", v)) r.version = (int)v;
    if (const TValue* s = child(*m->t, "name", T_CHAR)) r.name = s->s;
    if (const TValue* s = child(*m->t, "reference", T_CHAR)) r.reference = s->s;
  }
  // hamiltonian
  const TValue* h = child(t, "hamiltonian", T_TABLE);
  const TValue* x = h ? child(*h->t, "xtb", T_TABLE) : nullptr;
  if (!x) fail("No entry for xTB Hamiltonian found");
  const TTable& xt = *x->t;
  if (const TValue* s = xt.find("cn")) {
    if (s->type != T_CHAR) fail("Invalid entry for CN type in Hamiltonian");
    r.cn = s->s;
  }
  need_double(xt, "wexp", r.wexp, "Invalid entry for Slater exponent weighting of Hamiltonian");
  r.kpol = 2.0;
  get_double(xt, "kpol", r.kpol);
  if (const TValue* sh = child(xt, "shell", T_TABLE)) {
    bool have = false;
    double last = 0.0;
    for (int l = 0; l < 5; ++l) {
      const std::string key(2, ANG[l]);
      double v;
      if (!sh->t->find(key)) {
        if (!have) fail("No entry for " + key + "-shell pair scaling parameter");
        r.ksh[l][l] = last;
        continue;
      }
      if (!get_double(*sh->t, key.c_str(), v))
        fail("Cannot read " + key + "-shell pair scaling parameter");
      r.ksh[l][l] = last = v;
      r.lmax = l;
      have = true;
    }
    for (int l = 0; l < 5; ++l)
      for (int k = 0; k < l; ++k) {
        const std::string key = std::string(1, ANG[k]) + ANG[l];
        double v = 0.5 * (r.ksh[k][k] + r.ksh[l][l]);
        if (sh->t->find(key) && !get_double(*sh->t, key.c_str(), v))
          fail("Cannot read " + key + "-shell pair scaling parameter");
        r.ksh[k][l] = r.ksh[l][k] = v;
      }
  }
  need_double(xt, "enscale", r.enscale, "Invalid entry for EN scaling parameter in Hamiltonian");
  if (const TValue* kp = child(xt, "kpair", T_TABLE))
    for (const auto& [key, v] : kp->t->kv) {
      const size_t dash = key.find('-');
      const int zi = dash == std::string::npos ? 0 : element_number(key.substr(0, dash));
      const int zj = dash == std::string::npos ? 0 : element_number(key.substr(dash + 1));
      double f;
      if (!zi || !zj || !get_double(*kp->t, key.c_str(), f))
        fail("Invalid entry '" + key + "' for element pair scaling in Hamiltonian");
      r.kpair[{std::max(zi, zj), std::min(zi, zj)}] = f;
    }
  // dispersion
  if (const TValue* d = child(t, "dispersion", T_TABLE)) {
    r.has_dispersion = true;
    const TValue* d3 = child(*d->t, "d3", T_TABLE);
    const TValue* d4 = child(*d->t, "d4", T_TABLE);
    if (!d3 && !d4) fail("Dispersion model not provided in dispersion table");
    r.d3 = d3 != nullptr;
    const TTable& dt = r.d3 ? *d3->t : *d4->t;
    if (!r.d3) {
      r.sc = true;
      if (const TValue* v = dt.find("sc")) {
        if (v->type != T_BOOL) fail("Cannot read self-consistency for D4 dispersion");
        r.sc = v->b;
      }
      if (const TValue* v = dt.find("smooth")) {
        if (v->type != T_BOOL) fail("Cannot read smoothing for dispersion (D4S)");
        r.smooth = v->b;
      }
    } else {
      r.sc = false;
    }
    r.s6 = 1.0;
    get_double(dt, "s6", r.s6);
    need_double(dt, "s8", r.s8, "Cannot read s8 parameter for dispersion");
    need_double(dt, "a1", r.a1, "Cannot read a1 parameter for dispersion");
    need_double(dt, "a2", r.a2, "Cannot read a2 parameter for dispersion");
    r.s9 = 0.0;
    get_double(dt, "s9", r.s9);
  }
  if (const TValue* rp = child(t, "repulsion", T_TABLE)) {
    const TValue* e = child(*rp->t, "effective", T_TABLE);
    if (!e) fail("No entry for effective repulsion found");
    r.has_repulsion = true;
    need_double(*e->t, "kexp", r.kexp, "Invalid entry for repulsion exponent");
    r.klight = r.kexp;
    get_double(*e->t, "klight", r.klight);
  }
  if (const TValue* c = child(t, "charge", T_TABLE)) {
    const TValue* e = child(*c->t, "effective", T_TABLE);
    if (!e) fail("No entry for Coulomb electrostatic found");
    r.has_charge = true;
    need_double(*e->t, "gexp", r.gexp, "Invalid entry for effective Coulomb exponent");
    const TValue* a = child(*e->t, "average", T_CHAR);
    if (!a) fail("Invalid entry for hardness averaging");
    r.average = a->s;
    if (r.average != "harmonic" && r.average != "geometric" && r.average != "arithmetic")
      fail("Invalid '" + r.average + "' averaging for hardness");
  }
  if (const TValue* th = child(t, "thirdorder", T_TABLE)) {
    r.has_thirdorder = true;
    const TValue* sh = child(*th->t, "shell", T_TABLE);
    r.third_shell = sh != nullptr;
    if (sh) {
      bool have = false;
      double last = 0.0;
      for (int l = 0; l < 5; ++l) {
        const std::string key(1, ANG[l]);
        double v;
        if (!sh->t->find(key)) {
          if (!have) fail("No entry for " + key + "-shell Hubbard derivative");
          r.third_ksh[l] = last;
          continue;
        }
        if (!get_double(*sh->t, key.c_str(), v))
          fail("Cannot read " + key + "-shell Hubbard derivative");
        r.third_ksh[l] = last = v;
        r.third_lmax = l;
        have = true;
      }
    }
  }
  if (const TValue* mp = child(t, "multipole", T_TABLE)) {
    const TValue* d = child(*mp->t, "damped", T_TABLE);
    if (!d) fail("No entry for damped multipole electrostatic found");
    r.has_multipole = true;
    const std::string bad = "Invalid entry for ";
    need_double(*d->t, "dmp3", r.dmp3, bad + "multipole range separation parameter");
    need_double(*d->t, "dmp5", r.dmp5, bad + "multipole range separation parameter");
    need_double(*d->t, "kexp", r.mp_kexp, bad + "multipole damping function exponent");
    need_double(*d->t, "shift", r.mp_shift, bad + "CN multipole shift");
    need_double(*d->t, "rmax", r.mp_rmax, bad + "maximum multipole radius");
  }
  if (const TValue* hl = child(t, "halogen", T_TABLE)) {
    const TValue* c = child(*hl->t, "classical", T_TABLE);
    if (!c) fail("No entry for classical halogen bonding correction found");
    r.has_halogen = true;
    need_double(*c->t, "damping", r.hal_damping,
                "Invalid entry for halogen bonding damping parameter");
    need_double(*c->t, "rscale", r.hal_rscale, "Invalid entry for halogen bonding radii scaling");
  }
  const TValue* el = child(t, "element", T_TABLE);
  if (!el) fail("No element records in parameter table");
  for (const auto& [sym, v] : el->t->kv) {
    if (v.type != T_TABLE) fail("Invalid element record for " + sym);
    ElementRecord e;
    load_element(e, sym, *v.t);
    if (e.num == 0) fail("Unknown element symbol '" + sym + "'");
    r.element.push_back(std::move(e));
  }
}

void param_dump(const ParamRecord& r, TTable& t) {
  t.kv.clear();
  auto meta = t.add_table("meta");
  if (!r.name.empty()) meta->set("name", TValue::of(r.name));
  if (!r.reference.empty()) meta->set("reference", TValue::of(r.reference));
  meta->set("version", TValue::of((int64_t)r.version));
  meta->set("format", TValue::of((int64_t)1));
  auto x = t.add_table("hamiltonian")->add_table("xtb");
  x->set("wexp", TValue::of(r.wexp));
  x->set("kpol", TValue::of(r.kpol));
  x->set("enscale", TValue::of(r.enscale));
  if (!r.cn.empty()) x->set("cn", TValue::of(r.cn));
  auto sh = x->add_table("shell");
  for (int l = 0; l <= r.lmax; ++l) sh->set(std::string(2, ANG[l]), TValue::of(r.ksh[l][l]));
  for (int l = 0; l <= r.lmax; ++l)
    for (int k = 0; k < l; ++k)
      if (std::fabs(r.ksh[k][l] - 0.5 * (r.ksh[l][l] + r.ksh[k][k])) > 2.220446049250313e-16)
        sh->set(std::string(1, ANG[k]) + ANG[l], TValue::of(r.ksh[k][l]));
  if (!r.kpair.empty()) {
    auto kp = x->add_table("kpair");
    for (const auto& [zz, f] : r.kpair)
      kp->set(element_symbol(zz.first) + "-" + element_symbol(zz.second), TValue::of(f));
  }
  if (r.has_dispersion) {
    auto d = t.add_table("dispersion")->add_table(r.d3 ? "d3" : "d4");
    if (!r.d3) {
      d->set("sc", TValue::of(r.sc));
      if (r.smooth) d->set("smooth", TValue::of(true));
    }
    d->set("s6", TValue::of(r.s6));
    d->set("s8", TValue::of(r.s8));
    d->set("a1", TValue::of(r.a1));
    d->set("a2", TValue::of(r.a2));
    d->set("s9", TValue::of(r.s9));
  }
  if (r.has_repulsion) {
    auto e = t.add_table("repulsion")->add_table("effective");
    e->set("kexp", TValue::of(r.kexp));
    if (r.klight != r.kexp) e->set("klight", TValue::of(r.klight));
  }
  if (r.has_charge) {
    auto e = t.add_table("charge")->add_table("effective");
    e->set("gexp", TValue::of(r.gexp));
    e->set("average", TValue::of(r.average));
  }
  if (r.has_thirdorder) {
    auto th = t.add_table("thirdorder");
    if (r.third_shell) {
      auto s = th->add_table("shell");
      for (int l = 0; l <= r.third_lmax; ++l) s->set(std::string(1, ANG[l]), TValue::of(r.third_ksh[l]));
    } else {
      th->set("shell", TValue::of(false));
    }
  }
  if (r.has_multipole) {
    auto d = t.add_table("multipole")->add_table("damped");
    d->set("dmp3", TValue::of(r.dmp3));
    d->set("dmp5", TValue::of(r.dmp5));
    d->set("kexp", TValue::of(r.mp_kexp));
    d->set("shift", TValue::of(r.mp_shift));
    d->set("rmax", TValue::of(r.mp_rmax));
  }
  if (r.has_halogen) {
    auto c = t.add_table("halogen")->add_table("classical");
    c->set("damping", TValue::of(r.hal_damping));
    c->set("rscale", TValue::of(r.hal_rscale));
  }
  auto el = t.add_table("element");
  for (const auto& e : r.element) dump_element(e, *el->add_table(e.sym));
}

}  // namespace tb

// ---- C API: include/tblite/param.h -----------------------------------------------------------
namespace {
void set_error(tblite_error error, const std::string& m) {
  if (error) {
    error->msg = m;
    error->set = true;
  }
}
}  // namespace

extern "C" {

tblite_param tblite_new_param(void) { return new _tblite_param(); }

void tblite_delete_param(tblite_param* param) {
  if (param && *param) {
    delete *param;
    *param = nullptr;
  }
}

void tblite_load_param(tblite_error error, tblite_param param, tblite_table table) {
  if (!error) return;
  if (!param) return set_error(error, "Parametrization record is missing");
  if (!table) return set_error(error, "Data table object is missing");
  try {
    tb::ParamRecord r;
    tb::param_load(r, *table->p);
    param->rec = std::move(r);
    param->set = true;
  } catch (const std::exception& e) {
    set_error(error, e.what());
  }
}

void tblite_dump_param(tblite_error error, tblite_param param, tblite_table table) {
  if (!error) return;
  if (!param) return set_error(error, "Parametrization record is missing");
  if (!table) return set_error(error, "Data table object is missing");
  tb::param_dump(param->rec, *table->p);
}

void tblite_export_gfn2_param(tblite_error error, tblite_param param) {
  if (!error) return;
  if (!param) return set_error(error, "Parametrization record is missing");
  tb::export_gfn2(param->rec);
  param->set = true;
}

void tblite_export_gfn1_param(tblite_error error, tblite_param param) {
  if (!error) return;
  if (!param) return set_error(error, "Parametrization record is missing");
  tb::export_gfn1(param->rec);
  param->set = true;
}

void tblite_export_ipea1_param(tblite_error error, tblite_param param) {
  if (!error) return;
  if (!param) return set_error(error, "Parametrization record is missing");
  tb::export_ipea1(param->rec);
  param->set = true;
}

// post-processing named in a parametrisation record: none is kept by the records here (the
// reference's records carry xtbml / molmom settings from TOML files), so the call only checks
// its handles
void tblite_push_back_post_processing_param(tblite_context ctx, tblite_calculator calc,
                                            tblite_structure mol, tblite_param param) {
  if (!ctx) return;
  if (!param) return ctx->push("Param object is missing");
  if (!calc) return ctx->push("Calculator object is missing");
  if (!mol) return ctx->push("Molecular structure data is missing");
  ctx->push("Post processing from a parametrization record is not available in this library");
}

}  // extern "C"
