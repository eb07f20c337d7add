"""CPU oracle: self-consistent D4 dispersion for GFN2-xTB (test infrastructure only).

The reference wraps dftd4 v4.2.0 (src/tblite/disp/d4.f90:79-474); dftd4 is not
part of the reference tree, so the D4 model is restated here from its published
form and its element data come from the injected element-data pack:

* coordination number: EN-weighted error-function counting (orc_d4_cn);
* reference weights: Gaussian weights in (CN - CN_ref) with charge scaling
  zeta(q) = exp(ga (1 - exp(gc * gam * (1 - (Z+q_ref)/(Z+q)))));
* two-body energy with rational damping, self-consistent through the charges
  (energy, potential and gradient as in d4.f90:217-352);
* three-body ATM term with charge-free weights (d4.f90:193-213, 422-474).

With the synthetic pack the numbers are not the reference's; the engine is
checked against this oracle with the same injected data.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from oracle.gfn2 import _elem, _p, lib

MREF = 7


def pair_c6(d4, za, zb):
    """nref(za) x nref(zb) reference C6 matrix of an element pair from the pack (stored once
    per unordered pair as "Za-Zb", Za <= Zb)."""
    if za <= zb:
        return np.array(d4["c6"][f"{za}-{zb}"], dtype=float)
    return np.array(d4["c6"][f"{zb}-{za}"], dtype=float).T


def species_c6(d4, species, nref):
    """[nsp, MREF, nsp, MREF] reference C6 of the species pairs, zero beyond nref."""
    nsp = len(species)
    out = np.zeros((nsp, MREF, nsp, MREF))
    for a, za in enumerate(species):
        for b, zb in enumerate(species):
            out[a, :nref[a], b, :nref[b]] = pair_c6(d4, za, zb)
    return out


class D4:
    def __init__(self, calc, st):
        self.calc = calc
        mol = calc.mol
        self.nat = nat = len(mol.numbers)
        d4 = calc.edata["d4"]
        self.par = d4
        sc = calc.params["scalars"]
        self.s6, self.s8, self.a1, self.a2, self.s9 = sc["s6"], sc["s8"], sc["a1"], sc["a2"], sc["s9"]
        z = mol.numbers
        species = sorted(set(int(v) for v in z))
        self.sp = np.array([species.index(int(v)) for v in z], dtype=np.int32)
        nsp = len(species)
        self.nsp = nsp
        self.nref = np.array([len(_elem(d4, "refcn", s)) for s in species])
        self.refcn = np.zeros((nsp, MREF))
        self.refq = np.zeros((nsp, MREF))
        self.ngw = np.zeros((nsp, MREF), dtype=int)
        for k, s in enumerate(species):
            nr = self.nref[k]
            self.refcn[k, :nr] = _elem(d4, "refcn", s)
            self.refq[k, :nr] = _elem(d4, "refq", s)
            self.ngw[k, :nr] = _elem(d4, "ngw", s)
        if d4.get("width2", 0.0) != 0.0 or d4.get("width3", 0.0) != 0.0:
            raise ValueError("smooth dispersion cutoffs are not restated (widths must be 0)")
        # reference C6 per species pair from the pack's per-element-pair table, the layout of
        # dftd4's c6(iref, jref, izp, jzp) read by disp/d4.f90:410-413
        self.c6ref = species_c6(d4, species, self.nref)
        self.zeff = np.array([_elem(d4, "zeff", s) for s in species])[self.sp]
        self.gam = np.array([_elem(d4, "gam", s) for s in species])[self.sp]
        self.r4r2 = np.array([_elem(d4, "r4r2", s) for s in species])[self.sp]
        self.rcov = np.array([_elem(d4, "rcov", s) for s in species])[self.sp]
        self.en = np.array([_elem(d4, "en", s) for s in species])[self.sp]
        self.xyz = st["xyz"]
        self.cn = np.zeros(nat)
        lib().orc_d4_cn(nat, _p(self.xyz), _p(self.rcov), _p(self.en), ctypes.c_double(d4["cn_kn"]),
                        ctypes.c_double(d4["cn_k4"]), ctypes.c_double(d4["cn_k5"]),
                        ctypes.c_double(d4["cn_k6"]), ctypes.c_double(d4["cn_cutoff"]), None,
                        _p(self.cn), None, None)
        self.gw, self.dgwdcn = self._cn_weights()

    # Gaussian weights in the coordination number (charge independent part)
    def _cn_weights(self):
        wf = self.par["wf"]
        gw = np.zeros((self.nat, MREF))
        dgw = np.zeros((self.nat, MREF))
        for i in range(self.nat):
            a = self.sp[i]
            nr = self.nref[a]
            num = np.zeros(MREF)
            dnum = np.zeros(MREF)
            for r in range(nr):
                for k in range(1, self.ngw[a, r] + 1):
                    w = math.exp(-wf * k * (self.cn[i] - self.refcn[a, r]) ** 2)
                    num[r] += w
                    dnum[r] += 2.0 * wf * k * (self.refcn[a, r] - self.cn[i]) * w
            norm = num.sum()
            dnorm = dnum.sum()
            if norm < 1e-300:
                raise ValueError("D4 reference weights underflow")
            gw[i] = num / norm
            dgw[i] = dnum / norm - num * dnorm / norm**2
        return gw, dgw

    def _zeta(self, q):
        ga, gc = self.par["ga"], self.par["gc"]
        zeta = np.zeros((self.nat, MREF))
        dzeta = np.zeros((self.nat, MREF))
        for i in range(self.nat):
            a = self.sp[i]
            z = self.zeff[i] + q[i]
            for r in range(self.nref[a]):
                zr = self.zeff[i] + self.refq[a, r]
                if z > 0:
                    t = math.exp(gc * self.gam[i] * (1.0 - zr / z))
                    zeta[i, r] = math.exp(ga * (1.0 - t))
                    dzeta[i, r] = zeta[i, r] * (-ga * t) * gc * self.gam[i] * zr / (z * z)
                else:
                    zeta[i, r] = math.exp(ga)
        return zeta, dzeta

    def _u(self, gwvec):
        u = np.zeros((self.nat, MREF))
        lib().orc_d4_twobody(self.nat, _p(self.xyz), _p(self.sp), self.nsp, _p(self.c6ref),
                             _p(self.r4r2), ctypes.c_double(self.a1), ctypes.c_double(self.a2),
                             ctypes.c_double(self.s6), ctypes.c_double(self.s8),
                             ctypes.c_double(self.par["disp2_cutoff"]), _p(gwvec), None, 0, _p(u),
                             None, None, None)
        return u

    def potential(self, qat):
        zeta, dzeta = self._zeta(qat)
        u = self._u(self.gw * zeta)
        return np.sum(u * self.gw * dzeta, 1)

    def energy_sc(self, qat):
        zeta, _ = self._zeta(qat)
        gwv = self.gw * zeta
        u = self._u(gwv)
        return 0.5 * np.sum(u * gwv, 1)

    def energy_nonsc(self, gradient, sigma):
        """Three-body ATM term with charge-free weights (and its gradient)."""
        zeta, _ = self._zeta(np.zeros(self.nat))
        gwv = self.gw * zeta
        dgwv = self.dgwdcn * zeta
        c6, dc6 = self._atomic_c6(gwv, dgwv)
        e = np.zeros(self.nat)
        dEdc6 = np.zeros((self.nat, self.nat))
        g = gradient if gradient is not None else np.zeros((self.nat, 3))
        s = sigma if sigma is not None else np.zeros((3, 3))
        lib().orc_d4_atm(self.nat, _p(self.xyz), _p(c6), _p(self.r4r2), ctypes.c_double(self.a1),
                         ctypes.c_double(self.a2), ctypes.c_double(self.s9),
                         ctypes.c_double(self.par["atm_alpha"]),
                         ctypes.c_double(self.par["disp3_cutoff"]), _p(e), _p(dEdc6), _p(g), _p(s))
        if gradient is not None:
            dEdc6 = dEdc6 + dEdc6.T
            dEdcn = np.einsum("ij,ij->i", dEdc6, dc6)
            self._cn_chain(dEdcn, gradient, sigma)
        return e

    def _atomic_c6(self, gwv, dgwv):
        t = self.c6ref[self.sp][:, :, self.sp, :]  # [i, r, j, s]
        c6 = np.einsum("ir,irjs,js->ij", gwv, t, gwv)
        dc6 = np.einsum("ir,irjs,js->ij", dgwv, t, gwv)  # d c6_ij / d cn_i
        return np.ascontiguousarray(c6), dc6

    def _cn_chain(self, dEdcn, gradient, sigma):
        d4 = self.par
        lib().orc_d4_cn(self.nat, _p(self.xyz), _p(self.rcov), _p(self.en), ctypes.c_double(d4["cn_kn"]),
                        ctypes.c_double(d4["cn_k4"]), ctypes.c_double(d4["cn_k5"]),
                        ctypes.c_double(d4["cn_k6"]), ctypes.c_double(d4["cn_cutoff"]),
                        _p(np.ascontiguousarray(dEdcn)), None, _p(gradient), _p(sigma))

    def gradient(self, qat, gradient, sigma):
        """Two-body gradient at the final charges (d4.f90:315-352)."""
        zeta, _ = self._zeta(qat)
        gwv = np.ascontiguousarray(self.gw * zeta)
        dgwv = np.ascontiguousarray(self.dgwdcn * zeta)
        dEdcn = np.zeros(self.nat)
        lib().orc_d4_twobody(self.nat, _p(self.xyz), _p(self.sp), self.nsp, _p(self.c6ref),
                             _p(self.r4r2), ctypes.c_double(self.a1), ctypes.c_double(self.a2),
                             ctypes.c_double(self.s6), ctypes.c_double(self.s8),
                             ctypes.c_double(self.par["disp2_cutoff"]), _p(gwv), _p(dgwv), 1, None,
                             _p(gradient), _p(sigma), _p(dEdcn))
        self._cn_chain(dEdcn, gradient, sigma)
