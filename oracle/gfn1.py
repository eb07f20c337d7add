"""CPU oracle: GFN1-xTB single point (energy + analytic gradient).

TEST INFRASTRUCTURE ONLY -- a CPU restatement of the reference algorithm (tblite 0.7.0) used to
check the CUDA engine.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` may import it; the product (``tblite_gb300``) never does.

Follows:
  basis (H 2s orthogonalised to 1s)   src/tblite/xtb/gfn1.f90:556-596, basis/ortho.f90:33-72
  H0 scaling (valence / polarisation shells, element-pair factors)
                                      src/tblite/xtb/gfn1.f90:704-828, 1056-1060
  self energies, CN shift, shell polynomial, reference occupation
                                      src/tblite/xtb/gfn1.f90:831-905, xtb/h0.f90
  isotropic Coulomb (harmonic mean of the shell hardnesses), atom-resolved third order
                                      src/tblite/xtb/gfn1.f90:625-668, coulomb/thirdorder.f90
  repulsion                           src/tblite/xtb/gfn1.f90:612-622
  SCF driver                          src/tblite/xtb/singlepoint.f90 (as the GFN2 oracle)
The pair integrals, the H0 build and its gradient and the Coulomb matrix come from the C part
shared with the GFN2 oracle.  Parity status: the data-free part is pinned against the
reference's single-atom GFN1 energies (test/unit/test_gfn1_xtb.f90:135-349).  The coordination
number and the D3 dispersion need data from mctc-lib / s-dftd3, which is not in the reference
tree; they run on the injected element-data pack, so multi-atom totals are unpinned.
"""
from __future__ import annotations

import ctypes
import json
import math
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg

from oracle.gfn2 import (DATA, KT_300K, MAXG, Broyden, Molecule, Result, _basis_struct, _elem,
                         _p, entropy, fermi_filling, lib, load_element_data, load_sto,
                         post_processing, slater_to_gauss)


def load_params1(method="gfn1"):
    """GFN1-xTB tables, or with method="ipea1" the IPEA1-xTB tables of the same form
    (xtb/ipea1.f90:47-490, extracted into ipea1.json)."""
    return json.loads((DATA / f"{method}.json").read_text())


def orthogonalize(ai, ci, aj, cj):
    """Orthogonalise s function (aj, cj) to (ai, ci): basis/ortho.f90:33-72."""
    ov = 0.0
    for a, c in zip(ai, ci):
        for b, d in zip(aj, cj):
            ov += c * d * math.sqrt(math.pi / (a + b)) ** 3
    a_new = list(aj) + list(ai)
    c_new = list(cj) + [-ov * c for c in ci]
    norm = 0.0
    for a, c in zip(a_new, c_new):
        for b, d in zip(a_new, c_new):
            norm += c * d * math.sqrt(math.pi / (a + b)) ** 3
    return np.array(a_new), np.array(c_new) / math.sqrt(norm)


@dataclass
class Calc1:
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
    sh_valence: np.ndarray = field(default=None)
    sh_index: np.ndarray = field(default=None)  # shell index within its atom
    nao: int = 0
    accuracy: float = 1.0
    kt: float = KT_300K
    max_iter: int = 250
    damping: float = 0.4
    include_dispersion: bool = True


def new_calc(mol: Molecule, edata=None, method="gfn1", **kw):
    """Calculator of the GFN1 form: GFN1-xTB, or IPEA1-xTB with method="ipea1" (its own tables,
    the s-p H0 scale 2.25 and element-pair factors from the d-block rule only,
    xtb/ipea1.f90:752-765, 1037-1041)."""
    p = load_params1(method)
    p["ipea1"] = method == "ipea1"
    sto = load_sto()
    nat = len(mol.numbers)
    if edata is None and nat > 1:
        edata = load_element_data()
    cols = {k: [] for k in ("atom", "l", "nprim", "alpha", "coeff", "ao", "zeta", "val", "idx")}
    at_sh = [0]
    nao = 0
    for iat, z in enumerate(mol.numbers):
        if p["halogen_bond"][z - 1] > 0.0:
            raise ValueError(f"Z={z}: the halogen-bond correction is not part of this path")
        nsh = int(p["nshell"][z - 1])
        prims, first_of_l = [], {}
        for ish in range(nsh):
            l = int(p["ang_shell"][z - 1][ish])
            if l > 1:
                raise ValueError(f"Z={z} has d shells")
            n = int(p["principal_quantum_number"][z - 1][ish])
            ng = int(p["number_of_primitives"][z - 1][ish])
            zeta = p["slater_exponent"][z - 1][ish]
            a, c = slater_to_gauss(ng, n, l, zeta, sto)
            valence = l not in first_of_l
            if valence:
                first_of_l[l] = ish
            prims.append([l, a, c, zeta, valence, first_of_l[l]])
        for ish in range(nsh):  # orthogonalise after all shells of the atom exist
            l, a, c, zeta, valence, ref = prims[ish]
            if not valence:
                a, c = orthogonalize(prims[ref][1], prims[ref][2], a, c)
                prims[ish][1], prims[ish][2] = a, c
        for ish in range(nsh):
            l, a, c, zeta, valence, _ = prims[ish]
            aa, cc = np.zeros(MAXG), np.zeros(MAXG)
            aa[:len(a)] = a
            cc[:len(c)] = c
            for key, v in (("atom", iat), ("l", l), ("nprim", len(a)), ("alpha", aa),
                           ("coeff", cc), ("ao", nao), ("zeta", zeta), ("val", valence),
                           ("idx", ish)):
                cols[key].append(v)
            nao += 2 * l + 1
        at_sh.append(at_sh[-1] + nsh)
    calc = Calc1(mol=mol, params=p, edata=edata)
    calc.sh_atom = np.array(cols["atom"], dtype=np.int32)
    calc.sh_l = np.array(cols["l"], dtype=np.int32)
    calc.sh_nprim = np.array(cols["nprim"], dtype=np.int32)
    calc.sh_alpha = np.ascontiguousarray(cols["alpha"], dtype=np.float64)
    calc.sh_coeff = np.ascontiguousarray(cols["coeff"], dtype=np.float64)
    calc.sh_ao = np.array(cols["ao"], dtype=np.int32)
    calc.at_sh = np.array(at_sh, dtype=np.int32)
    calc.sh_zeta = np.array(cols["zeta"], dtype=np.float64)
    calc.sh_valence = np.array(cols["val"], dtype=bool)
    calc.sh_index = np.array(cols["idx"], dtype=np.int32)
    calc.nao = nao
    for k, v in kw.items():
        setattr(calc, k, v)
    return calc


def pair_param(zi, zj, ipea1=False):
    """get_pair_param, xtb/gfn1.f90:734-772 (IPEA1-xTB: xtb/ipea1.f90:752-765, the d-block
    rule only)."""
    pairs = {(1, 1): 0.96, (1, 5): 0.95, (1, 7): 1.04, (1, 28): 0.90, (1, 75): 0.80,
             (1, 78): 0.80, (5, 15): 0.97, (7, 14): 1.01}
    key = (min(zi, zj), max(zi, zj))
    if key in pairs and not ipea1:
        return pairs[key]

    def row(z):
        if 20 < z < 30:
            return 1
        if 38 < z < 48:
            return 2
        if 56 < z < 80:
            return 3
        return 0

    kp = [1.1, 1.2, 1.2]
    ti, tj = row(zi), row(zj)
    if ti > 0 and tj > 0:
        return 0.5 * (kp[ti - 1] + kp[tj - 1])
    return 1.0


def hscale_pairs(calc, at_en):
    """get_hscale, xtb/gfn1.f90:797-828, for every shell pair [jsh][ish]."""
    p = calc.params
    ksh = np.array(p["kshell"])
    kdiff = p["scalars"]["kdiff"]
    enscale = p["scalars"]["enscale"]
    z = calc.mol.numbers
    nsh = len(calc.sh_l)
    hs = np.zeros((nsh, nsh))
    for i in range(nsh):
        for j in range(nsh):
            ai, aj = calc.sh_atom[i], calc.sh_atom[j]
            li, lj = calc.sh_l[i], calc.sh_l[j]
            vi, vj = calc.sh_valence[i], calc.sh_valence[j]
            if vi and vj:
                den = (at_en[ai] - at_en[aj]) ** 2
                km = pair_param(z[aj], z[ai], p.get("ipea1", False)) * ksh[lj][li] * (1.0 + enscale * den)
            elif vi:
                km = 0.5 * (ksh[li][li] + kdiff)
            elif vj:
                km = 0.5 * (ksh[lj][lj] + kdiff)
            else:
                km = kdiff
            hs[j, i] = km
    return np.ascontiguousarray(hs)


def _cn_exp(xyz, rcov, k, cutoff):
    """Exponential counting function and its derivative, per atom pair."""
    nat = len(rcov)
    cn = np.zeros(nat)
    dcn = np.zeros((nat, nat, 3))  # dcn[i, k] = d cn_i / d x_k
    for i in range(nat):
        for j in range(i):
            v = xyz[i] - xyz[j]
            r = np.linalg.norm(v)
            if r > cutoff:
                continue
            r0 = rcov[i] + rcov[j]
            e = math.exp(-k * (r0 / r - 1.0))
            c = 1.0 / (1.0 + e)
            dc = -c * c * e * k * r0 / (r * r)  # d c / d r
            cn[i] += c
            cn[j] += c
            g = dc * v / r
            dcn[i, i] += g
            dcn[i, j] -= g
            dcn[j, j] -= g
            dcn[j, i] += g
    return cn, dcn


class D3:
    """Two-body D3(BJ) dispersion on the pack's reference data (s9 = 0 for GFN1)."""

    def __init__(self, calc, xyz):
        ed = calc.edata
        d3, d4 = ed["d3"], ed["d4"]
        sc = calc.params["scalars"]
        z = calc.mol.numbers
        self.s6, self.s8, self.a1, self.a2 = sc["s6"], sc["s8"], sc["a1"], sc["a2"]
        rcov = np.array([_elem(d4, "rcov", zz) for zz in z])
        self.r4r2 = np.array([_elem(d4, "r4r2", zz) for zz in z])
        self.cn, self.dcn = _cn_exp(xyz, rcov, d3["k1"], d3["cn_cutoff"])
        self.cut = d3["disp2_cutoff"]
        self.xyz = xyz
        nat = len(z)
        self.z = [int(v) for v in z]
        self.d4 = d4
        # normalised Gaussian weights of the reference CNs and their CN derivatives
        self.w, self.dw = [], []
        for i in range(nat):
            refcn = np.array(d4["refcn"][str(z[i])])
            w = np.exp(-d3["k3"] * (self.cn[i] - refcn) ** 2)
            dw = -2.0 * d3["k3"] * (self.cn[i] - refcn) * w
            norm = w.sum()
            self.w.append(w / norm)
            self.dw.append((dw * norm - w * dw.sum()) / norm ** 2)

    def _c6(self, i, j):
        """C6 of the pair (i, j) = sum_rs w_ir w_js C6ref(r, s) and its CN_i, CN_j derivatives"""
        from oracle.d4 import pair_c6

        t = pair_c6(self.d4, self.z[i], self.z[j])
        return (self.w[i] @ t @ self.w[j], self.dw[i] @ t @ self.w[j],
                self.w[i] @ t @ self.dw[j])

    def energy_gradient(self, gradient=None, sigma=None):
        nat = len(self.w)
        e = np.zeros(nat)
        dedcn = np.zeros(nat)
        xyz = self.xyz
        for i in range(nat):
            for j in range(i):
                v = xyz[i] - xyz[j]
                r = np.linalg.norm(v)
                if r > self.cut:
                    continue
                c6, dc6i, dc6j = self._c6(i, j)
                q = 3.0 * self.r4r2[i] * self.r4r2[j]
                r0 = self.a1 * math.sqrt(q) + self.a2
                t6 = 1.0 / (r ** 6 + r0 ** 6)
                t8 = 1.0 / (r ** 8 + r0 ** 8)
                eij = -(self.s6 * t6 + self.s8 * q * t8) * c6
                e[i] += 0.5 * eij
                e[j] += 0.5 * eij
                if gradient is not None:
                    de = c6 * (self.s6 * 6 * r ** 5 * t6 * t6 + self.s8 * q * 8 * r ** 7 * t8 * t8)
                    g = de * v / r
                    gradient[i] += g
                    gradient[j] -= g
                    if sigma is not None:
                        sigma += np.outer(g, v)
                    dedc6 = -(self.s6 * t6 + self.s8 * q * t8)
                    dedcn[i] += dedc6 * dc6i
                    dedcn[j] += dedc6 * dc6j
        if gradient is not None:
            gradient += np.einsum("i,ikx->kx", dedcn, self.dcn)
            if sigma is not None:
                for i in range(nat):
                    for k in range(nat):
                        sigma += dedcn[i] * np.outer(self.dcn[i, k], xyz[k])
        return e


def setup(calc):
    mol = calc.mol
    p = calc.params
    sc = p["scalars"]
    nat = len(mol.numbers)
    z = mol.numbers
    xyz = np.ascontiguousarray(mol.positions, dtype=np.float64)
    L = lib()
    nsh = len(calc.sh_l)
    ed = calc.edata
    if nat > 1:
        rcov = np.array([_elem(ed["cn"], "rcov", zz) for zz in z])
        cn, dcn = _cn_exp(xyz, rcov, ed["cn_exp"]["k"], ed["cn_exp"]["cutoff"])
        at_en = np.array([_elem(ed, "pauling_en", zz) for zz in z])
        at_rad = np.array([_elem(ed, "atomic_rad", zz) for zz in z])
    else:
        cn, dcn = np.zeros(nat), np.zeros((nat, nat, 3))
        at_en, at_rad = np.zeros(nat), np.ones(nat)
    zs = z[calc.sh_atom]
    se0 = np.array([p["p_selfenergy"][zs[i] - 1][calc.sh_index[i]] for i in range(nsh)])
    kcn = np.array([p["p_kcn"][zs[i] - 1][calc.sh_index[i]] for i in range(nsh)])
    selfenergy = se0 - kcn * cn[calc.sh_atom]
    shpoly = np.array([p["p_shpoly"][zs[i] - 1][calc.sh_l[i]] for i in range(nsh)])
    min_alpha = min(float(np.min(calc.sh_alpha[i, : calc.sh_nprim[i]])) for i in range(nsh))
    intcut = 25.0
    cutoff = min(math.sqrt(2.0 * intcut / min_alpha), 40.0)
    n = calc.nao
    S, H = np.zeros((n, n)), np.zeros((n, n))
    D, Q = np.zeros((3, n, n)), np.zeros((6, n, n))
    b, keep = _basis_struct(calc, xyz)
    hs = hscale_pairs(calc, at_en)
    ksh = np.zeros((5, 5))
    L.orc_build_h0(ctypes.byref(b), _p(selfenergy), _p(shpoly), _p(calc.sh_zeta), _p(at_en),
                   _p(at_rad), _p(ksh), ctypes.c_double(0.0), ctypes.c_double(0.0),
                   ctypes.c_double(intcut), ctypes.c_double(cutoff), _p(S), _p(D), _p(Q), _p(H),
                   _p(hs))
    hub = np.array([p["hubbard_parameter"][zs[i] - 1] * p["shell_hubbard"][zs[i] - 1][calc.sh_l[i]]
                    for i in range(nsh)])
    gamma = np.zeros((nsh, nsh))
    L.orc_gamma(ctypes.c_int(nat), _p(xyz), _p(calc.at_sh), _p(hub), ctypes.c_double(sc["gexp"]),
                ctypes.c_int(1), _p(gamma))
    gam3 = np.array([p["p_hubbard_derivs"][zz - 1] for zz in z])
    refocc = np.array([p["reference_occ"][zs[i] - 1][calc.sh_l[i]] if calc.sh_valence[i] else 0.0
                       for i in range(nsh)])
    n0at = np.zeros(nat)
    np.add.at(n0at, calc.sh_atom, refocc)
    return dict(xyz=xyz, cn=cn, dcn=dcn, selfenergy=selfenergy, dsedcn=-kcn, shpoly=shpoly,
                at_en=at_en, at_rad=at_rad, intcut=intcut, cutoff=cutoff, S=S, H=H, D=D, Q=Q,
                hs=hs, ksh=ksh, hub=hub, gamma=gamma, gam3=gam3, n0sh=refocc, n0at=n0at)


def singlepoint(calc: Calc1, grad=True, verbose=False, solvation=None):
    mol = calc.mol
    nat = len(mol.numbers)
    st = setup(calc)
    p = calc.params
    sc = p["scalars"]
    L = lib()
    nsh = len(calc.sh_l)
    xyz = st["xyz"]
    nocc = float(np.sum(st["n0sh"])) - mol.charge
    nel = nocc
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
    erep = np.zeros(nat)
    if nat > 1:
        alpha = np.array([p["rep_alpha"][zz - 1] for zz in mol.numbers])
        zeff = np.array([p["rep_zeff"][zz - 1] for zz in mol.numbers])
        num = np.ascontiguousarray(mol.numbers, dtype=np.int32)
        L.orc_repulsion(ctypes.c_int(nat), _p(xyz), _p(num), _p(alpha), _p(zeff),
                        ctypes.c_double(sc["rep_kexp"]), ctypes.c_double(sc["rep_kexp"]),
                        ctypes.c_double(sc["rep_rexp"]), ctypes.c_double(25.0), _p(erep),
                        _p(gradient) if grad else None, _p(sigma) if grad else None)
    energies += erep
    edisp = np.zeros(nat)
    if calc.include_dispersion and nat > 1:
        disp = D3(calc, xyz)
        edisp = disp.energy_gradient(gradient, sigma)
    energies += edisp
    # implicit solvation (the dielectric-constant GB models take atomic Mulliken charges for
    # every method), geometry part
    solv = solvation
    if solv is not None:
        solv.update(xyz)
        energies += solv.nonsc_energies()
    ao2sh = np.repeat(np.arange(nsh), 2 * calc.sh_l + 1)
    ao2at = calc.sh_atom[ao2sh]
    qat = np.full(nat, mol.charge / nat)
    qsh = st["n0sh"] / np.where(st["n0at"] > 0, st["n0at"], 1.0)[calc.sh_atom] * qat[calc.sh_atom]
    econv, pconv = 1.0e-6 * calc.accuracy, 2.0e-5 * calc.accuracy
    mixer = Broyden(nsh, calc.max_iter, calc.damping)
    eelec = np.zeros(nat)
    converged = False
    iscf = 0
    while not converged and iscf < calc.max_iter:
        elast = float(np.sum(eelec))
        if iscf > 0:
            mixer.next()
            qsh = mixer.q.copy()
            qat = np.zeros(nat)
            np.add.at(qat, calc.sh_atom, qsh)
        iscf += 1
        vsh = st["gamma"] @ qsh
        vat = st["gam3"] * qat ** 2
        if solv is not None:
            vat = vat + solv.potential(qat)
        vao = (vsh + vat[calc.sh_atom])[ao2sh]
        F = st["H"] - 0.5 * st["S"] * (vao[:, None] + vao[None, :])
        mixer.set(qsh.copy())
        emo, C = scipy.linalg.eigh(F, st["S"], type=1, driver="gvd", lower=False)
        fa = fermi_filling(nalp, calc.kt, emo)
        fb = fermi_filling(nbet, calc.kt, emo)
        focc = fa + fb
        ts = entropy(fa, calc.kt) + entropy(fb, calc.kt)
        P = (C * focc) @ C.T
        qsh_ao = -np.sum(P * st["S"], 0)
        qsh = np.zeros(nsh)
        np.add.at(qsh, ao2sh, qsh_ao)
        qsh += st["n0sh"]
        qat = np.zeros(nat)
        np.add.at(qat, calc.sh_atom, qsh)
        mixer.diff(qsh.copy())
        eao = np.sum(st["H"] * P, 0)
        eelec = np.full(nat, ts / nat)
        np.add.at(eelec, ao2at, eao)
        e2sh = 0.5 * (st["gamma"] @ qsh) * qsh
        np.add.at(eelec, calc.sh_atom, e2sh)
        eelec += st["gam3"] * qat ** 3 / 3.0
        if solv is not None:
            eelec += solv.energies(qat)
        converged = abs(float(np.sum(eelec)) - elast) < econv and mixer.error() < pconv
        if verbose:
            print(iscf, float(np.sum(eelec + energies)), float(np.sum(eelec)) - elast, mixer.error())
    energies = energies + eelec
    energy = float(np.sum(energies))
    # atomic multipoles of the final density (scf/iterator.f90:120-123 runs for every method)
    dpat = np.zeros((nat, 3))
    qpat = np.zeros((nat, 6))
    np.add.at(dpat, ao2at, -np.einsum("krc,rc->ck", st["D"], P))
    np.add.at(qpat, ao2at, -np.einsum("qrc,rc->cq", st["Q"], P))
    parts = dict(erep=float(np.sum(erep)), edisp=float(np.sum(edisp)), eelec=float(np.sum(eelec)),
                 cn=st["cn"], vao=vao)
    parts.update(post_processing(st["S"], C, fa, fb, P, nalp, nbet, xyz, qat, dpat, qpat, ao2at))
    if grad:
        n = calc.nao
        dEdcn = np.zeros(nat)
        W = (C * (focc * emo)) @ C.T
        b, keep = _basis_struct(calc, xyz)
        zero3 = np.zeros(3 * nat)
        zero6 = np.zeros(6 * nat)
        L.orc_h0_gradient(ctypes.byref(b), _p(st["selfenergy"]),
                          _p(np.ascontiguousarray(st["dsedcn"])), _p(st["shpoly"]),
                          _p(calc.sh_zeta), _p(st["at_en"]), _p(st["at_rad"]), _p(st["ksh"]),
                          ctypes.c_double(0.0), ctypes.c_double(0.0), ctypes.c_double(st["intcut"]),
                          ctypes.c_double(st["cutoff"]), _p(np.ascontiguousarray(P)),
                          _p(np.ascontiguousarray(W)), _p(np.ascontiguousarray(vao)), _p(zero3),
                          _p(zero6), _p(gradient), _p(sigma), _p(dEdcn), _p(st["hs"]))
        L.orc_gamma_grad(ctypes.c_int(nat), _p(xyz), _p(calc.at_sh), _p(st["hub"]),
                         ctypes.c_double(sc["gexp"]), ctypes.c_int(1), _p(qsh), _p(gradient),
                         _p(sigma))
        gradient += np.einsum("i,ikx->kx", dEdcn, st["dcn"])
        if solv is not None:
            gradient += solv.gradient(qat)
        for i in range(nat):
            for k in range(nat):
                sigma += dEdcn[i] * np.outer(st["dcn"][i, k], xyz[k])
    return Result(energy=energy, energies=energies, gradient=gradient, sigma=sigma, qsh=qsh,
                  qat=qat, dpat=dpat, qpat=qpat, density=P, emo=emo, focc=focc, iterations=iscf,
                  converged=converged, parts=parts)
