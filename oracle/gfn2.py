"""CPU oracle: GFN2-xTB single point (energy + analytic gradient).

TEST INFRASTRUCTURE ONLY -- a CPU restatement of the reference algorithm
(tblite 0.7.0) used to check the CUDA engine.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` may import it;
the product (``tblite_gb300``) never does.

Pair loops live in ``xtb_oracle.c`` (built by ``oracle/build.py``); the SCF
driver below follows ``src/tblite/xtb/singlepoint.f90:73-433`` and
``src/tblite/scf/iterator.f90:46-353``.  The generalised eigenproblem is
solved with LAPACK ``dsygvd`` (itype 1, jobz V, uplo U) through
``scipy.linalg.eigh(..., type=1, driver="gvd", lower=False)``, the same
routine and arguments as ``src/tblite/lapack/sygvd.f90:146``.

Parity status: the data-free part (basis, integrals, H0 on-site terms,
Coulomb/third-order/AES on-site terms, Fermi smearing, Broyden mixing) is
pinned against the reference's single-atom GFN2 energies
(``test/unit/test_gfn2_xtb.f90:61-272``).  Terms that need the
coordination-number, electronegativity, atomic-radius and D4 tables of
mctc-lib / dftd4 (not part of the reference tree) run on an injected
element-data pack; with the synthetic pack their parity against the
reference is unpinned.
"""
from __future__ import annotations

import ctypes
import json
import math
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np
import scipy.linalg

HERE = Path(__file__).resolve().parent
DATA = HERE.parent / "tblite_gb300" / "data"
MAXG = 12
KT_300K = 300.0 * 3.166808578545117e-06  # reference api/calculator.f90:81

_lib = None


def lib():
    """Load (building if needed) the C part of the oracle."""
    global _lib
    if _lib is None:
        from oracle.build import build_oracle

        path = build_oracle()
        _lib = ctypes.CDLL(str(path))
    return _lib


class _Basis(ctypes.Structure):
    _fields_ = [("nat", ctypes.c_int), ("nsh", ctypes.c_int), ("nao", ctypes.c_int),
                ("xyz", ctypes.c_void_p), ("sh_atom", ctypes.c_void_p),
                ("sh_l", ctypes.c_void_p), ("sh_nprim", ctypes.c_void_p),
                ("sh_alpha", ctypes.c_void_p), ("sh_coeff", ctypes.c_void_p),
                ("sh_ao", ctypes.c_void_p), ("at_sh", ctypes.c_void_p)]


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def load_params():
    return json.loads((DATA / "gfn2.json").read_text())


def load_sto():
    return json.loads((DATA / "sto_ng.json").read_text())


def load_element_data(path=None):
    path = path or os.environ.get("TBLITE_GB300_ELEMENT_DATA") or DATA / "element_data_synthetic.json"
    return json.loads(Path(path).read_text())


# --------------------------------------------------------------------------
# STO-nG expansion, reference src/tblite/basis/slater.f90:409-511
# --------------------------------------------------------------------------
def slater_to_gauss(ng, n, l, zeta, sto):
    if l == 0:
        ityp = n
    elif l == 1:
        ityp = 4 + n
    elif l == 2:
        ityp = 7 + n
    else:
        raise ValueError("angular momentum > d not supported")
    if ng == 1:
        alpha = np.array([sto["pAlpha1"][ityp - 1]]) * zeta**2
        coeff = np.array([1.0])
    elif ng == 6 and n == 6:
        key = "6s" if l == 0 else "6p"
        alpha = np.array(sto["pAlpha" + key]) * zeta**2
        coeff = np.array(sto["pCoeff" + key])
    else:
        alpha = np.array(sto[f"pAlpha{ng}"][ityp - 1]) * zeta**2
        coeff = np.array(sto[f"pCoeff{ng}"][ityp - 1])
    dfac = [1.0, 1.0, 3.0, 15.0, 105.0, 945.0, 10395.0, 135135.0]
    top = 2.0 / math.pi
    # dfactorial(l+1) of the reference is 1-based: (2l-1)!!
    coeff = coeff * (top * alpha) ** 0.75 * np.sqrt(4 * alpha) ** l / math.sqrt(dfac[l])
    return alpha, coeff


@dataclass
class Molecule:
    numbers: np.ndarray
    positions: np.ndarray  # Bohr, [nat][3]
    charge: float = 0.0
    uhf: int = 0


@dataclass
class Calc:
    """GFN2-xTB calculator data for one molecule (reference xtb/gfn2.f90:570-716)."""

    mol: Molecule
    params: dict
    edata: dict | None
    sh_atom: np.ndarray = field(default=None)
    sh_l: np.ndarray = field(default=None)
    sh_nprim: np.ndarray = field(default=None)
    sh_alpha: np.ndarray = field(default=None)
    sh_coeff: np.ndarray = field(default=None)
    sh_ao: np.ndarray = field(default=None)
    at_sh: np.ndarray = field(default=None)
    sh_zeta: np.ndarray = field(default=None)
    nao: int = 0
    accuracy: float = 1.0
    kt: float = KT_300K
    max_iter: int = 250
    damping: float = 0.4
    include_dispersion: bool = True


def new_calc(mol: Molecule, edata=None, **kw):
    p = load_params()
    sto = load_sto()
    nat = len(mol.numbers)
    if edata is None and nat > 1:
        edata = load_element_data()
    sh_atom, sh_l, sh_nprim, sh_alpha, sh_coeff, sh_ao, sh_zeta, at_sh = [], [], [], [], [], [], [], [0]
    nao = 0
    for iat, z in enumerate(mol.numbers):
        nsh = int(p["nshell"][z - 1])
        for ish in range(nsh):
            l = int(p["ang_shell"][z - 1][ish])
            n = int(p["principal_quantum_number"][z - 1][ish])
            ng = int(p["number_of_primitives"][z - 1][ish])
            zeta = p["slater_exponent"][z - 1][ish]
            a, c = slater_to_gauss(ng, n, l, zeta, sto)
            aa = np.zeros(MAXG)
            cc = np.zeros(MAXG)
            aa[:ng] = a
            cc[:ng] = c
            sh_atom.append(iat)
            sh_l.append(l)
            sh_nprim.append(ng)
            sh_alpha.append(aa)
            sh_coeff.append(cc)
            sh_ao.append(nao)
            sh_zeta.append(zeta)
            nao += 2 * l + 1
        at_sh.append(at_sh[-1] + nsh)
    calc = Calc(mol=mol, params=p, edata=edata)
    calc.sh_atom = np.array(sh_atom, dtype=np.int32)
    calc.sh_l = np.array(sh_l, dtype=np.int32)
    calc.sh_nprim = np.array(sh_nprim, dtype=np.int32)
    calc.sh_alpha = np.ascontiguousarray(sh_alpha, dtype=np.float64)
    calc.sh_coeff = np.ascontiguousarray(sh_coeff, dtype=np.float64)
    calc.sh_ao = np.array(sh_ao, dtype=np.int32)
    calc.at_sh = np.array(at_sh, dtype=np.int32)
    calc.sh_zeta = np.array(sh_zeta, dtype=np.float64)
    calc.nao = nao
    for k, v in kw.items():
        setattr(calc, k, v)
    return calc


def _basis_struct(calc, xyz):
    b = _Basis()
    b.nat = len(calc.mol.numbers)
    b.nsh = len(calc.sh_l)
    b.nao = calc.nao
    keep = [xyz, calc.sh_atom, calc.sh_l, calc.sh_nprim, calc.sh_alpha, calc.sh_coeff,
            calc.sh_ao, calc.at_sh]
    b.xyz, b.sh_atom, b.sh_l, b.sh_nprim, b.sh_alpha, b.sh_coeff, b.sh_ao, b.at_sh = [
        _p(a) for a in keep]
    return b, keep


def _elem(edata, key, z):
    try:
        return edata[key][str(int(z))]
    except KeyError as exc:  # loud failure: no silent defaults for external data
        raise KeyError(f"element data pack '{edata.get('name')}' has no '{key}' for Z={z}") from exc


# --------------------------------------------------------------------------
# Broyden mixer, reference src/tblite/scf/mixer/broyden.f90:72-278
# --------------------------------------------------------------------------
class Broyden:
    def __init__(self, ndim, memory, damp):
        self.ndim, self.memory, self.damp = ndim, memory, damp
        self.iter = 0
        self.df = np.zeros((memory, ndim))
        self.u = np.zeros((memory, ndim))
        self.a = np.zeros((memory, memory))
        self.omega = np.zeros(memory)
        self.dq = np.zeros(ndim)
        self.dqlast = np.zeros(ndim)
        self.qlast = np.zeros(ndim)
        self.q = np.zeros(ndim)

    def set(self, q):
        self.q = np.array(q, dtype=float)

    def diff(self, qout):
        self.dq = np.asarray(qout, dtype=float) - self.q

    def error(self):
        return math.sqrt(float(np.sum(self.dq**2 / self.ndim)))

    def next(self):
        self.iter += 1
        it = self.iter
        alpha = self.damp
        if it == 1:
            self.dqlast = self.dq.copy()
            self.qlast = self.q.copy()
            self.q = self.q + alpha * self.dq
            return
        itn = it - 1
        it1 = (itn - 1) % self.memory
        nhist = min(self.memory, itn)
        first = max(1, itn - self.memory + 1)
        hist = [(first + ih - 2) % self.memory for ih in range(1, nhist + 1)]
        omega0, minw, maxw, wfac = 0.01, 1.0, 100000.0, 0.01
        w = math.sqrt(float(self.dq @ self.dq))
        w = wfac / w if w > wfac / maxw else maxw
        self.omega[it1] = max(w, minw)
        self.df[it1] = self.dq - self.dqlast
        inv = max(math.sqrt(float(self.df[it1] @ self.df[it1])), np.finfo(float).eps)
        inv = 1.0 / inv
        self.df[it1] *= inv
        c = np.array([self.omega[i] * (self.df[i] @ self.dq) for i in hist])
        for i in hist:
            for j in hist:
                self.a[i, j] = self.df[i] @ self.df[j]
        beta = np.array([[self.omega[i] * self.omega[j] * self.a[i, j] for j in hist] for i in hist])
        beta += omega0 * omega0 * np.eye(nhist)
        lu, piv = scipy.linalg.lu_factor(beta)
        c = scipy.linalg.lu_solve((lu, piv), c, trans=1)
        self.u[it1] = alpha * self.df[it1] + inv * (self.q - self.qlast)
        self.dqlast = self.dq.copy()
        self.qlast = self.q.copy()
        q = self.q + alpha * self.dq
        for ih, i in enumerate(hist):
            q = q - self.omega[i] * c[ih] * self.u[i]
        self.q = q


# --------------------------------------------------------------------------
# Fermi smearing, reference src/tblite/wavefunction/fermi.f90:31-106
# --------------------------------------------------------------------------
def fermi_filling(nel, kt, emo):
    n = len(emo)
    occ = np.zeros(n)
    homo = int(math.floor(nel))
    occ[: min(homo, n)] = 1.0
    if homo < n:
        occ[homo] = math.fmod(nel, 1.0)
    homo = homo + 1 if math.fmod(nel, 1.0) > 0.5 else homo
    if homo <= 0:
        return occ
    ef = 0.5 * (emo[max(homo, 1) - 1] + emo[min(homo + 1, n) - 1])
    occt = float(homo)
    thr = math.sqrt(np.finfo(float).eps)
    sqrttiny = math.sqrt(np.finfo(float).tiny)
    for _ in range(200):
        x = (emo - ef) / kt
        mask = x < 50
        ex = np.exp(np.where(mask, x, 0.0))
        f = np.where(mask, 1.0 / (ex + 1.0), 0.0)
        df = np.where(mask, ex / (kt * (ex + 1.0) ** 2), 0.0)
        total = float(np.sum(f))
        dtot = float(np.sum(df))
        occ = f
        change = (occt - total) / dtot if dtot > sqrttiny else 0.0
        ef += change
        if abs(occt - total) <= thr:
            break
    return occ


def entropy(occ, kt):
    with np.errstate(divide="ignore", invalid="ignore"):
        t = occ**occ * (1 - occ) ** (1 - occ)
    return float(np.sum(np.log(t))) * kt


# --------------------------------------------------------------------------
# Single point
# --------------------------------------------------------------------------
@dataclass
class Result:
    energy: float
    energies: np.ndarray
    gradient: np.ndarray | None
    sigma: np.ndarray | None
    qsh: np.ndarray
    qat: np.ndarray
    dpat: np.ndarray
    qpat: np.ndarray
    density: np.ndarray
    emo: np.ndarray
    focc: np.ndarray
    iterations: int
    converged: bool
    parts: dict


def setup(calc: Calc):
    """Geometry-dependent data: CN, self energies, integrals, Coulomb matrices."""
    mol = calc.mol
    p = calc.params
    nat = len(mol.numbers)
    xyz = np.ascontiguousarray(mol.positions, dtype=np.float64)
    z = mol.numbers
    L = lib()
    nsh = len(calc.sh_l)
    ed = calc.edata
    # coordination number (dexp), reference xtb/singlepoint.f90:218-225
    cn = np.zeros(nat)
    if nat > 1:
        cnp = ed["cn"]
        rcov = np.array([_elem(cnp, "rcov", zz) for zz in z])
        L.orc_cn_dexp(ctypes.c_int(nat), _p(xyz), _p(rcov), ctypes.c_double(cnp["ka"]),
                      ctypes.c_double(cnp["kb"]), ctypes.c_double(cnp["rshift"]),
                      ctypes.c_double(cnp["cutoff"]), _p(cn))
    # self energies, reference xtb/h0.f90:113-217
    se0 = np.array([p["p_selfenergy"][z[calc.sh_atom[i]] - 1][i - calc.at_sh[calc.sh_atom[i]]]
                    for i in range(nsh)])
    kcn = np.array([p["p_kcn"][z[calc.sh_atom[i]] - 1][calc.sh_l[i]] for i in range(nsh)])
    selfenergy = se0 - kcn * cn[calc.sh_atom]
    dsedcn = -kcn
    shpoly = np.array([p["p_shpoly"][z[calc.sh_atom[i]] - 1][calc.sh_l[i]] for i in range(nsh)])
    if nat > 1:
        at_en = np.array([_elem(ed, "pauling_en", zz) for zz in z])
        at_rad = np.array([_elem(ed, "atomic_rad", zz) for zz in z])
    else:
        at_en = np.zeros(nat)
        at_rad = np.ones(nat)
    min_alpha = min(float(np.min(calc.sh_alpha[i, : calc.sh_nprim[i]])) for i in range(nsh))
    intcut = 25.0  # integral_cutoff(acc) always yields 25, basis/type.f90:250-267
    cutoff = min(math.sqrt(2.0 * intcut / min_alpha), 40.0)
    n = calc.nao
    S = np.zeros((n, n))
    H = np.zeros((n, n))
    D = np.zeros((3, n, n))
    Q = np.zeros((6, n, n))
    b, keep = _basis_struct(calc, xyz)
    ksh = np.ascontiguousarray(p["kshell"], dtype=np.float64)
    sc = p["scalars"]
    L.orc_build_h0(ctypes.byref(b), _p(selfenergy), _p(shpoly), _p(calc.sh_zeta), _p(at_en),
                   _p(at_rad), _p(ksh), ctypes.c_double(sc["wexp"]), ctypes.c_double(sc["enscale"]),
                   ctypes.c_double(intcut), ctypes.c_double(cutoff), _p(S), _p(D), _p(Q), _p(H),
                   None)
    # shell hardness and Hubbard derivatives, xtb/gfn2.f90:717-763
    hub = np.array([p["hubbard_parameter"][z[calc.sh_atom[i]] - 1]
                    * p["shell_hubbard"][z[calc.sh_atom[i]] - 1][calc.sh_l[i]] for i in range(nsh)])
    gam3 = np.array([p["p_hubbard_derivs"][z[calc.sh_atom[i]] - 1]
                     * p["shell_hubbard_derivs"][calc.sh_l[i]] for i in range(nsh)])
    gamma = np.zeros((nsh, nsh))
    L.orc_gamma(ctypes.c_int(nat), _p(xyz), _p(calc.at_sh), _p(hub), ctypes.c_double(sc["gexp"]),
                ctypes.c_int(0), _p(gamma))
    # AES radii and matrices, coulomb/multipole.f90:141-190,389-420,488-535
    vcn = np.array([p["p_vcn"][zz - 1] for zz in z])
    rad = np.array([p["p_rad"][zz - 1] for zz in z])
    arg = cn - vcn - sc["mp_shift"]
    t1 = np.exp(-sc["mp_kexp"] * arg)
    t2 = (sc["mp_rmax"] - rad) / (1.0 + t1)
    mrad = rad + t2
    dmrdcn = -t2 * sc["mp_kexp"] * t1 / (1.0 + t1)
    asd = np.zeros((nat, nat, 3))
    add = np.zeros((nat, nat, 3, 3))
    asq = np.zeros((nat, nat, 6))
    L.orc_aes_matrices(ctypes.c_int(nat), _p(xyz), _p(mrad), ctypes.c_double(sc["mp_dmp3"]),
                       ctypes.c_double(sc["mp_dmp5"]), _p(asd), _p(add), _p(asq))
    dkernel = np.array([p["p_dkernel"][zz - 1] for zz in z])
    qkernel = np.array([p["p_qkernel"][zz - 1] for zz in z])
    # reference occupations, xtb/h0.f90:669-700
    refocc = np.array([p["reference_occ"][z[calc.sh_atom[i]] - 1][calc.sh_l[i]] for i in range(nsh)])
    n0at = np.zeros(nat)
    np.add.at(n0at, calc.sh_atom, refocc)
    return dict(xyz=xyz, cn=cn, selfenergy=selfenergy, dsedcn=dsedcn, shpoly=shpoly, at_en=at_en,
                at_rad=at_rad, intcut=intcut, cutoff=cutoff, S=S, H=H, D=D, Q=Q, hub=hub,
                gam3=gam3, gamma=gamma, mrad=mrad, dmrdcn=dmrdcn, asd=asd, add=add, asq=asq,
                dkernel=dkernel, qkernel=qkernel, n0sh=refocc, n0at=n0at, ksh=ksh)


MPSCALE = np.array([1.0, 2.0, 1.0, 2.0, 2.0, 1.0])


def potentials(calc, st, qsh, qat, dpat, qpat, disp=None, solv=None, efield=None):
    """vsh, vat, vdp, vqp; reference coulomb get_potential routines (and the homogeneous
    electric field of external/field.f90:77-86: vat -= E.R, vdp -= E)."""
    vsh = st["gamma"] @ qsh + qsh**2 * st["gam3"]
    vat = np.einsum("ijk,jk->i", st["asd"], dpat) + np.einsum("ijq,jq->i", st["asq"], qpat)
    vdp = np.einsum("ijk,i->jk", st["asd"], qat) + np.einsum("ijac,ic->ja", st["add"], dpat)
    vdp += 2 * st["dkernel"][:, None] * dpat
    vqp = np.einsum("ijq,i->jq", st["asq"], qat) + 2 * st["qkernel"][:, None] * qpat * MPSCALE
    if disp is not None:
        vat = vat + disp.potential(qat)
    if solv is not None:
        vat = vat + solv.potential(qat)
    if efield is not None:
        vat = vat - st["xyz"] @ efield
        vdp = vdp - efield[None, :]
    return vsh, vat, vdp, vqp


def electrostatic_energies(calc, st, qsh, qat, dpat, qpat):
    nat = len(qat)
    e = np.zeros(nat)
    e2sh = 0.5 * (st["gamma"] @ qsh) * qsh + qsh**3 * st["gam3"] / 3.0
    np.add.at(e, calc.sh_atom, e2sh)
    vd = np.einsum("ijk,i->jk", st["asd"], qat) + 0.5 * np.einsum("ijac,ic->ja", st["add"], dpat)
    vq = np.einsum("ijq,i->jq", st["asq"], qat)
    e += np.sum(dpat * vd, 1) + np.sum(qpat * vq, 1)
    e += st["dkernel"] * np.sum(dpat * dpat, 1) + st["qkernel"] * np.sum(qpat * qpat * MPSCALE, 1)
    return e


def fock(calc, st, vsh, vat, vdp, vqp):
    """add_pot_to_h1, reference scf/potential.f90:122-255."""
    vsh = vsh + vat[calc.sh_atom]
    nao = calc.nao
    ao2sh = np.repeat(np.arange(len(calc.sh_l)), 2 * calc.sh_l + 1)
    ao2at = calc.sh_atom[ao2sh]
    vao = vsh[ao2sh]
    F = st["H"] - 0.5 * st["S"] * (vao[:, None] + vao[None, :])
    # D[k][row][col] with operator on atom of col
    mp = np.einsum("krc,ck->rc", st["D"], vdp[ao2at]) + np.einsum("qrc,cq->rc", st["Q"], vqp[ao2at])
    F -= 0.5 * (mp + mp.T)
    return F, vao, ao2at, ao2sh


def singlepoint(calc: Calc, grad=True, verbose=False, dispersion=None, solvation=None,
                efield=None):
    mol = calc.mol
    nat = len(mol.numbers)
    st = setup(calc)
    p = calc.params
    sc = p["scalars"]
    L = lib()
    nsh = len(calc.sh_l)
    n = calc.nao
    xyz = st["xyz"]
    # occupation, xtb/singlepoint.f90:140-156
    nocc = float(np.sum(st["n0sh"])) - mol.charge
    nel = float(np.sum(st["n0at"])) - mol.charge
    if mol.uhf % 2 == round(nel) % 2:
        nuhf = mol.uhf
    else:
        if mol.uhf != 0:
            raise ValueError("number of electrons and unpaired electrons incompatible")
        nuhf = round(nel) % 2
    diff = min(nuhf, nocc)
    nalp = (nocc - diff) / 2 + diff
    nbet = (nocc - diff) / 2
    energies = np.zeros(nat)
    gradient = np.zeros((nat, 3)) if grad else None
    sigma = np.zeros((3, 3)) if grad else None
    # repulsion, repulsion/effective.f90
    erep = np.zeros(nat)
    if nat > 1:
        alpha = np.array([p["rep_alpha"][zz - 1] for zz in mol.numbers])
        zeff = np.array([p["rep_zeff"][zz - 1] for zz in mol.numbers])
        num = np.ascontiguousarray(mol.numbers, dtype=np.int32)
        g = gradient if grad else None
        L.orc_repulsion(ctypes.c_int(nat), _p(xyz), _p(num), _p(alpha), _p(zeff),
                        ctypes.c_double(sc["rep_kexp"]), ctypes.c_double(sc["rep_kexp_light"]),
                        ctypes.c_double(sc["rep_rexp"]), ctypes.c_double(25.0), _p(erep),
                        _p(g) if grad else None, _p(sigma) if grad else None)
    energies += erep
    # dispersion (non self-consistent three-body part)
    disp = None
    edisp = np.zeros(nat)
    if calc.include_dispersion and nat > 1:
        from oracle.d4 import D4

        disp = D4(calc, st)
        edisp = disp.energy_nonsc(gradient, sigma)
    energies += edisp
    field = None if efield is None else np.asarray(efield, dtype=float).reshape(3)
    # implicit solvation (interactions container: ALPB + CDS + shift), geometry part
    solv = solvation
    esolv = np.zeros(nat)
    if solv is not None:
        solv.update(xyz)
        esolv = solv.nonsc_energies()
    energies += esolv
    # SAD guess, wavefunction/guess.f90:51-120
    qat = np.full(nat, mol.charge / nat)
    qsh = st["n0sh"] / st["n0at"][calc.sh_atom] * qat[calc.sh_atom]
    dpat = np.zeros((nat, 3))
    qpat = np.zeros((nat, 6))
    econv = 1.0e-6 * calc.accuracy
    pconv = 2.0e-5 * calc.accuracy
    mixer = Broyden(nsh + 9 * nat, calc.max_iter, calc.damping)
    eelec = np.zeros(nat)
    converged = False
    iscf = 0
    while not converged and iscf < calc.max_iter:
        elast = float(np.sum(eelec))
        if iscf > 0:
            mixer.next()
            qv = mixer.q
            qsh = qv[:nsh].copy()
            dpat = qv[nsh:nsh + 3 * nat].reshape(nat, 3).copy()
            qpat = qv[nsh + 3 * nat:].reshape(nat, 6).copy()
            qat = np.zeros(nat)
            np.add.at(qat, calc.sh_atom, qsh)
        iscf += 1
        vsh, vat, vdp, vqp = potentials(calc, st, qsh, qat, dpat, qpat, disp, solv, field)
        F, vao, ao2at, ao2sh = fock(calc, st, vsh, vat, vdp, vqp)
        mixer.set(np.concatenate([qsh, dpat.ravel(), qpat.ravel()]))
        emo, C = scipy.linalg.eigh(F, st["S"], type=1, driver="gvd", lower=False)
        fa = fermi_filling(nalp, calc.kt, emo)
        fb = fermi_filling(nbet, calc.kt, emo)
        focc = fa + fb
        ts = entropy(fa, calc.kt) + entropy(fb, calc.kt)
        P = (C * focc) @ C.T
        PS = P * st["S"]
        qsh_ao = -np.sum(PS, 0)
        qsh = np.zeros(nsh)
        np.add.at(qsh, ao2sh, qsh_ao)
        qsh += st["n0sh"]
        qat = np.zeros(nat)
        np.add.at(qat, calc.sh_atom, qsh)
        dpat = np.zeros((nat, 3))
        qpat = np.zeros((nat, 6))
        dcol = -np.einsum("krc,rc->ck", st["D"], P)
        qcol = -np.einsum("qrc,rc->cq", st["Q"], P)
        np.add.at(dpat, ao2at, dcol)
        np.add.at(qpat, ao2at, qcol)
        mixer.diff(np.concatenate([qsh, dpat.ravel(), qpat.ravel()]))
        eao = np.sum(st["H"] * P, 0)
        eelec = np.full(nat, ts / nat)
        np.add.at(eelec, ao2at, eao)
        eelec += electrostatic_energies(calc, st, qsh, qat, dpat, qpat)
        if disp is not None:
            eelec += disp.energy_sc(qat)
        if solv is not None:
            eelec += solv.energies(qat)
        if field is not None:  # external/field.f90:64-75, with the output moments
            eelec -= (xyz @ field) * qat + dpat @ field
        econverged = abs(float(np.sum(eelec)) - elast) < econv
        pconverged = mixer.error() < pconv
        converged = econverged and pconverged
        if verbose:
            print(iscf, float(np.sum(eelec + energies)), float(np.sum(eelec)) - elast, mixer.error())
    energies = energies + eelec
    energy = float(np.sum(energies))
    parts = dict(erep=float(np.sum(erep)), edisp_nonsc=float(np.sum(edisp)),
                 eelec=float(np.sum(eelec)), cn=st["cn"], vao=vao, vdp=vdp, vqp=vqp)
    parts.update(post_processing(st["S"], C, fa, fb, P, nalp, nbet, xyz, qat, dpat, qpat, ao2at))
    if grad:
        gradient, sigma = _gradient(calc, st, gradient, sigma, C, emo, focc, P, qsh, qat, dpat,
                                    qpat, vao, vdp, vqp, disp)
        if solv is not None:
            gradient += solv.gradient(qat)
        if field is not None:  # external/field.f90:100-113
            gradient -= field[None, :]
            stmp = np.outer(field, xyz.sum(0))
            sigma -= 0.5 * (stmp + stmp.T)
    return Result(energy=energy, energies=energies, gradient=gradient, sigma=sigma, qsh=qsh,
                  qat=qat, dpat=dpat, qpat=qpat, density=P, emo=emo, focc=focc, iterations=iscf,
                  converged=converged, parts=parts)



def post_processing(S, C, fa, fb, P, nalp, nbet, xyz, qat, dpat, qpat, ao2at):
    """Wiberg/Mayer bond orders (post_processing/wbo.f90:60-115 ->
    wavefunction/mulliken.f90:176-235) and molecular moments (mulliken.f90:133-172)."""
    nat = len(qat)
    parts = {}
    if nalp != nbet:
        spin_p = [(C * fa) @ C.T, (C * fb) @ C.T]
        scale = 2.0
    else:
        spin_p = [P]
        scale = 1.0
    # atom blocks of P S (P S)^T summed with np.add.reduceat over the atom-sorted AOs
    starts = np.flatnonzero(np.r_[True, ao2at[1:] != ao2at[:-1]])
    wbo = np.zeros((len(spin_p), nat, nat))
    for s_, Ps in enumerate(spin_p):
        PS_ = Ps @ S
        prod = PS_ * PS_.T
        blk = np.add.reduceat(np.add.reduceat(prod, starts, axis=0), starts, axis=1)
        wbo[s_] = scale * blk
        np.fill_diagonal(wbo[s_], 0.0)
    if len(spin_p) == 2:
        wbo = np.stack([wbo[0] + wbo[1], wbo[0] - wbo[1]])
    parts["wbo"] = wbo
    parts["dipole"] = np.sum(xyz * qat[:, None] + dpat, axis=0)
    v = xyz * qat[:, None]
    c = np.zeros((nat, 6))
    c[:, [0, 2, 5]] = xyz * (v + 2 * dpat)
    c[:, 1] = xyz[:, 0] * (v[:, 1] + dpat[:, 1]) + dpat[:, 0] * xyz[:, 1]
    c[:, 3] = xyz[:, 0] * (v[:, 2] + dpat[:, 2]) + dpat[:, 0] * xyz[:, 2]
    c[:, 4] = xyz[:, 1] * (v[:, 2] + dpat[:, 2]) + dpat[:, 1] * xyz[:, 2]
    tr = 0.5 * (c[:, 0] + c[:, 2] + c[:, 5])
    cq = np.stack([1.5 * c[:, 0] - tr, 3 * c[:, 1], 1.5 * c[:, 2] - tr, 3 * c[:, 3], 3 * c[:, 4],
                   1.5 * c[:, 5] - tr], axis=1)
    quad = np.sum(qpat + cq, axis=0)
    parts["quadrupole"] = quad
    return parts


def _gradient(calc, st, gradient, sigma, C, emo, focc, P, qsh, qat, dpat, qpat, vao, vdp, vqp, disp):
    """Nuclear gradient, reference xtb/singlepoint.f90:343-381."""
    mol = calc.mol
    nat = len(mol.numbers)
    p = calc.params
    sc = p["scalars"]
    L = lib()
    xyz = st["xyz"]
    if nat == 1:
        return gradient, sigma
    # Coulomb: es2 (coulomb/charge/type.f90:266-294) and AES (multipole.f90:746-852)
    L.orc_gamma_grad(ctypes.c_int(nat), _p(xyz), _p(calc.at_sh), _p(st["hub"]),
                     ctypes.c_double(sc["gexp"]), ctypes.c_int(0), _p(qsh), _p(gradient), _p(sigma))
    dEdr = np.zeros(nat)
    dp = np.ascontiguousarray(dpat)
    qp = np.ascontiguousarray(qpat)
    L.orc_aes_grad(ctypes.c_int(nat), _p(xyz), _p(st["mrad"]), ctypes.c_double(sc["mp_dmp3"]),
                   ctypes.c_double(sc["mp_dmp5"]), _p(qat), _p(dp), _p(qp), _p(dEdr), _p(gradient),
                   _p(sigma))
    dEdcn = dEdr * st["dmrdcn"]
    if disp is not None:
        disp.gradient(qat, gradient, sigma)
    # H0: W = C diag(f e) C^T (scf/diag.f90:110-143), h0.f90:432-666
    W = (C * (focc * emo)) @ C.T
    b, keep = _basis_struct(calc, xyz)
    sc_ = p["scalars"]
    vdp_c = np.ascontiguousarray(vdp)
    vqp_c = np.ascontiguousarray(vqp)
    P_c = np.ascontiguousarray(P)
    L.orc_h0_gradient(ctypes.byref(b), _p(st["selfenergy"]), _p(np.ascontiguousarray(st["dsedcn"])),
                      _p(st["shpoly"]), _p(calc.sh_zeta), _p(st["at_en"]), _p(st["at_rad"]),
                      _p(st["ksh"]), ctypes.c_double(sc_["wexp"]), ctypes.c_double(sc_["enscale"]),
                      ctypes.c_double(st["intcut"]), ctypes.c_double(st["cutoff"]), _p(P_c), _p(W),
                      _p(np.ascontiguousarray(vao)), _p(vdp_c), _p(vqp_c), _p(gradient), _p(sigma),
                      _p(dEdcn), None)
    cnp = calc.edata["cn"]
    rcov = np.array([_elem(cnp, "rcov", zz) for zz in mol.numbers])
    L.orc_cn_dexp_grad(ctypes.c_int(nat), _p(xyz), _p(rcov), ctypes.c_double(cnp["ka"]),
                       ctypes.c_double(cnp["kb"]), ctypes.c_double(cnp["rshift"]),
                       ctypes.c_double(cnp["cutoff"]), _p(dEdcn), _p(gradient), _p(sigma))
    return gradient, sigma
