"""CPU oracle: generalized Born implicit solvation -- ALPB(water) and GBSA(water) with CDS and
free-energy shift (GFN2 parameters), and the dielectric-constant GB models (GB-epsilon with or
without the ALPB shape term, Still or P16 kernel).

TEST INFRASTRUCTURE ONLY -- a CPU restatement of the reference's solvation containers used to
check the CUDA engine.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` may import it; the product (``tblite_gb300``) never does.

Follows (reference tblite 0.7.0):
  Born radii        src/tblite/solvation/born.f90:135-454 (compute_bornr, compute_psi; GBOBC
                    integrator, 35 Angstrom pair cutoff)
  ALPB kernel       src/tblite/solvation/alpb.f90:173-206 (new_alpb), 218-256 (update),
                    426-535 (add_born_mat_p16, add_born_deriv_p16), 562-684 (add_born_mat_still,
                    add_born_deriv_still), 656-787 (get_adet, get_adet_deriv); energy/potential/
                    gradient 260-365; dielectric-constant models api/solvation.f90:185-229 with
                    the COSMO radii of data.f90:103-130 and born.f90:52-107 defaults
  CDS               src/tblite/solvation/cds.f90:166-365; surface.f90:80-387 (SASA with the
                    230-point Lebedev grid, smoothed step function)
  shift             src/tblite/solvation/shift.f90:150-241
  parameters        data/alpb.f90:227-249, data/cds.f90:225-249, data/shift.f90:221-233 and
                    the gfn2 water tables (extracted into tblite_gb300/data/solvation_water.json)
Parity of this restatement against the reference itself is unpinned: the reference tests of
these containers use molecules from mstore, which is not in the reference tree.
"""
from __future__ import annotations

import itertools
import json
import math
from pathlib import Path

import numpy as np

DATA = Path(__file__).resolve().parent.parent / "tblite_gb300" / "data" / "solvation_water.json"
ZETA_P16 = 1.028
ALPHA_ALPB = 0.571412
OBC = (1.0, 0.8, 4.85)
KB_AU = 1.380649e-23 / 4.3597447222071e-18      # Boltzmann constant in Hartree/K (CODATA 2018)
R_GAS = 8.314462618                              # J/(mol K)


def lebedev230(orbits):
    """Points and weights (x 4 pi) of the 230-point grid from its orbit generators."""
    pts, wts = [], []
    for o in orbits:
        t, a, b, v = o["type"], o["a"], o["b"], o["v"]
        if t == 1:
            base = [(1.0, 0.0, 0.0)]
        elif t == 3:
            s = math.sqrt(1.0 / 3.0)
            base = [(s, s, s)]
        elif t == 4:
            base = [(a, a, math.sqrt(1.0 - 2.0 * a * a))]
        elif t == 5:
            base = [(a, math.sqrt(1.0 - a * a), 0.0)]
        elif t == 6:
            base = [(a, b, math.sqrt(1.0 - a * a - b * b))]
        else:
            raise ValueError(t)
        orbit = set()
        for p in base:
            for perm in itertools.permutations(p):
                for sg in itertools.product((1.0, -1.0), repeat=3):
                    orbit.add(tuple(0.0 if c == 0.0 else c * s_ for c, s_ in zip(perm, sg)))
        for p in sorted(orbit):
            pts.append(p)
            wts.append(v)
    pts = np.array(pts)
    assert pts.shape == (230, 3)
    return pts, np.array(wts) * 4.0 * math.pi


class ALPBWater:
    """ALPB(water) + CDS + shift for GFN2 (tblite_new_alpb_solvation_solvent(..., 12, state));
    with model="gbsa" the GBSA(water) tables and the Still kernel (version 22)."""

    def __init__(self, numbers, state=1, model="alpb"):
        d = json.loads(DATA.read_text())
        aatoau, kcaltoau = d["constants"]["aatoau"], d["constants"]["kcaltoau"]
        z = np.asarray(numbers) - 1
        self.nat = len(z)
        gbsa = model == "gbsa"
        self.kernel = "still" if gbsa else "p16"
        self.cds = True
        # ALPB / GBSA (load_alpb_param, new_alpb, new_born_integrator)
        a = d["gbsa" if gbsa else "alpb"]
        eps = a["epsv"]
        self.alpbet = 0.0 if gbsa else ALPHA_ALPB / eps
        self.keps = (1.0 / eps - 1.0) / (1.0 + self.alpbet)
        self.vdwr = np.array(d["rvdw_d3"])[z]
        self.rho = self.vdwr * np.array(a["sx"])[z]
        self.svdw = self.vdwr - a["soset"] * 0.1 * aatoau
        self.born_scale = a["c1"]
        self.lrcut = 35.0 * aatoau
        # CDS (load_cds_param, new_cds, new_surface_integrator)
        c = d["gbsa_cds" if gbsa else "cds"]
        probe = c["rprobe"] * aatoau
        rad = np.array(d["rvdw_d3"])[z]
        self.tension = np.array(c["gamscale"])[z] * 1.0e-5
        hb = -kcaltoau * np.array(c["sqrtghbond"])[z] ** 2
        self.hbond = hb / (4.0 * math.pi * (rad + probe) ** 2)
        w = 0.3 * aatoau
        self.ah0, self.ah1, self.ah3 = 0.5, 3.0 / (4.0 * w), -1.0 / (4.0 * w ** 3)
        self.vdwsa = rad + probe
        self.trj2 = np.stack([(self.vdwsa - w) ** 2, (self.vdwsa + w) ** 2])

        def wpart(r, vs):
            return (0.25 / w + 3.0 * self.ah3 * (0.2 * r * r - 0.5 * r * vs + vs * vs / 3.0)) * r ** 3

        self.wrp = wpart(self.vdwsa + w, self.vdwsa) - wpart(self.vdwsa - w, self.vdwsa)
        self.srcut = 2.0 * (w + self.vdwsa.max()) + 2.0 * aatoau
        self.grid, self.gw = lebedev230(d["lebedev230"])
        # shift (load_shift_param, new_shift, get_stateshift)
        s = d["gbsa_shift" if gbsa else "shift"]
        gshift = s["gshift"] * kcaltoau
        temp, amb = 298.15, 298.15
        vm = R_GAS * amb / 1.0e2  # ideal-gas molar volume, reference units (L/mol)
        if state == 2:
            stateshift = temp * KB_AU * math.log(vm * temp / amb)
        elif state == 3:
            stateshift = temp * KB_AU * (math.log(vm * temp / amb) +
                                         math.log(s["rhos"] / 1.0e-3 * 1.0 / s["smass"]))
        else:
            stateshift = 0.0
        self.total_shift = gshift + stateshift

    # ---------------------------------------------------------------- geometry
    def update(self, xyz):
        xyz = np.asarray(xyz, dtype=float)
        self.xyz = xyz
        self.brad, self.dbrad = self._born(xyz)
        self.adet = self._adet(xyz)
        if self.cds:
            self.surface, self.dsdr = self._sasa(xyz)
        else:
            self.surface, self.dsdr = np.zeros(self.nat), np.zeros((self.nat, self.nat, 3))

    def _born(self, xyz):
        nat = self.nat
        psi = np.zeros(nat)
        dpsi = np.zeros((nat, nat, 3))   # dpsi[i, k] = d psi_i / d x_k
        for i in range(nat):
            for j in range(nat):
                if i == j:
                    continue
                vec = xyz[i] - xyz[j]
                r = np.linalg.norm(vec)
                if r > self.lrcut:
                    continue
                g, dg = self._psi_term(r, self.rho[j], self.vdwr[i])
                psi[i] += g
                dpsi[i, i] += dg * vec
                dpsi[i, j] -= dg * vec
        brad = np.zeros(nat)
        dbrad = np.zeros((nat, nat, 3))
        c1 = self.born_scale
        for i in range(nat):
            s1, v1, s2 = 1.0 / self.svdw[i], 1.0 / self.vdwr[i], 0.5 * self.svdw[i]
            br = psi[i] * s2
            arg2 = br * (OBC[2] * br - OBC[1])
            arg = br * (OBC[0] + arg2)
            arg2 = 2.0 * arg2 + OBC[0] + OBC[2] * br * br
            th, ch = math.tanh(arg), math.cosh(arg)
            brad[i] = c1 / (s1 - v1 * th)
            dp = ch * (s1 - v1 * th)
            dp = c1 * s2 * v1 * arg2 / (dp * dp)
            dbrad[i] = dpsi[i] * dp
        return brad, dbrad

    @staticmethod
    def _psi_term(r, rhoj, rvdwi):
        """Contribution of partner j to psi_i and its radial derivative factor (d/dr = dg r)."""
        if r >= rvdwi + rhoj:  # no overlap of i's sphere with j's descreening sphere
            r1 = 1.0 / r
            ap, am = r + rhoj, r - rhoj
            ab = ap * am
            rhab = rhoj / ab
            lnab = 0.5 * math.log(am / ap) * r1
            g = rhab + lnab
            dg = -2.0 * rhab / ab + (rhab - lnab) * r1 * r1
            return g, dg
        if r + rhoj > rvdwi:
            r1 = 1.0 / r
            r12 = 0.5 * r1
            r24 = r12 * r12
            ap, am = r + rhoj, r - rhoj
            rh1 = 1.0 / rvdwi
            rhr1 = 1.0 / ap
            aprh1 = ap * rh1
            lnab = math.log(aprh1)
            g = rh1 - rhr1 + r12 * (0.5 * am * (rhr1 - rh1 * aprh1) - lnab)
            dg = (rhr1 * rhr1 * (1.0 - 0.25 * am * r1 * (1.0 + aprh1 * aprh1))
                  + rhoj * r24 * (rhr1 - rh1 * aprh1) + r12 * (r1 * lnab - rhr1)) * r1
            return g, dg
        return 0.0, 0.0

    def _adet(self, xyz):
        rad3 = self.vdwr ** 3
        vol = rad3.sum()
        center = (xyz * rad3[:, None]).sum(0) / vol
        inertia = np.zeros((3, 3))
        for i in range(self.nat):
            v = xyz[i] - center
            inertia += rad3[i] * ((v @ v + 0.4 * self.vdwr[i] ** 2) * np.eye(3) - np.outer(v, v))
        return math.sqrt(np.linalg.det(inertia) ** (1.0 / 3.0) / (0.4 * vol))

    def _sasa(self, xyz):
        nat = self.nat
        surface = np.zeros(nat)
        dsdr = np.zeros((nat, nat, 3))  # dsdr[i, k] = d surface_i / d x_k
        for i in range(nat):
            nb = [j for j in range(nat) if j != i and np.linalg.norm(xyz[i] - xyz[j]) <= self.srcut]
            for p in range(230):
                xp = xyz[i] + self.vdwsa[i] * self.grid[p]
                sasap = 1.0
                grads = []
                for j in nb:
                    tj = xp - xyz[j]
                    tj2 = tj @ tj
                    if tj2 < self.trj2[1, j]:
                        if tj2 <= self.trj2[0, j]:
                            sasap = 0.0
                            break
                        sq = math.sqrt(tj2)
                        uj = sq - self.vdwsa[j]
                        a3 = self.ah3 * uj * uj
                        s_ij = self.ah0 + (self.ah1 + a3) * uj
                        ds = (self.ah1 + 3.0 * a3) / (s_ij * sq)
                        sasap *= s_ij
                        grads.append((j, ds * tj))
                if sasap > 1.0e-6:
                    wsa = self.gw[p] * self.wrp[i] * sasap
                    surface[i] += wsa
                    for j, g in grads:
                        dsdr[i, i] += wsa * g
                        dsdr[i, j] -= wsa * g
        return surface, dsdr

    # ---------------------------------------------------------------- SCF terms
    def jmat(self):
        nat, xyz = self.nat, self.xyz
        J = np.zeros((nat, nat))
        for i in range(nat):
            for j in range(i):
                r = np.linalg.norm(xyz[i] - xyz[j])
                if self.kernel == "still":
                    aa = self.brad[i] * self.brad[j]
                    J[i, j] = J[j, i] = self.keps / math.sqrt(r * r + aa * math.exp(-0.25 * r * r / aa))
                    continue
                ab = math.sqrt(self.brad[i] * self.brad[j])
                arg = ab / (ab + ZETA_P16 / 16.0 * r)
                arg = arg ** 16
                J[i, j] = J[j, i] = self.keps / (r + ab * arg)
            J[i, i] = self.keps / self.brad[i]
        J += self.keps * self.alpbet / self.adet
        return J

    def nonsc_energies(self):
        """Geometry-only energy per atom: surface tension term and the free-energy shift."""
        return self.surface * self.tension + self.total_shift / self.nat

    def potential(self, qat):
        return self.jmat() @ qat + 2.0 * self.hbond * self.surface * qat

    def energies(self, qat):
        return 0.5 * qat * (self.jmat() @ qat) + self.hbond * self.surface * qat ** 2

    def gradient(self, qat):
        """Gradient of surface tension + hbond + ALPB energy at charges qat ([nat, 3])."""
        nat, xyz, keps = self.nat, self.xyz, self.keps
        g = np.zeros((nat, 3))
        # CDS: sum_i (tension_i + hbond_i q_i^2) d surface_i
        c = self.tension + self.hbond * qat ** 2
        g += np.einsum("i,ikx->kx", c, self.dsdr)
        # ALPB pair terms and Born radius chain rule
        dedbr = np.zeros(nat)
        for i in range(nat):
            for j in range(i):
                vec = xyz[i] - xyz[j]
                r = np.linalg.norm(vec)
                qq = qat[i] * qat[j]
                if self.kernel == "still":  # add_born_deriv_still
                    aa = self.brad[i] * self.brad[j]
                    dd = 0.25 * r * r / aa
                    expd = math.exp(-dd)
                    dfgb2 = 1.0 / (r * r + aa * expd)
                    dfgb3 = dfgb2 * math.sqrt(dfgb2) * keps
                    dG = (1.0 - 0.25 * expd) * dfgb3 * vec * qq
                    g[i] -= dG
                    g[j] += dG
                    bp = -0.5 * expd * (1.0 + dd) * dfgb3
                    dedbr[i] += self.brad[j] * bp * qq
                    dedbr[j] += self.brad[i] * bp * qq
                    continue
                ab = math.sqrt(self.brad[i] * self.brad[j])
                arg1 = ab / (ab + ZETA_P16 / 16.0 * r)
                arg16 = arg1 ** 16
                fgb = r + ab * arg16
                dfgb2 = 1.0 / (fgb * fgb)
                ap = (1.0 - ZETA_P16 * arg1 * arg16) * dfgb2
                dG = ap * vec * keps / r * qq
                g[i] -= dG
                g[j] += dG
                bp = -0.5 * (r * ZETA_P16 / ab * arg1 + 1.0) / ab * arg16 * dfgb2
                dedbr[i] += self.brad[j] * bp * keps * qq
                dedbr[j] += self.brad[i] * bp * keps * qq
            bp = 1.0 / self.brad[i]
            dedbr[i] += -0.5 * keps * qat[i] * bp * bp * qat[i]
        g += np.einsum("i,ikx->kx", dedbr, self.dbrad)
        # shape term of ALPB (get_adet_deriv)
        rad3 = self.vdwr ** 3
        vol = rad3.sum()
        center = (xyz * rad3[:, None]).sum(0) / vol
        inertia = np.zeros((3, 3))
        for i in range(nat):
            v = xyz[i] - center
            inertia += rad3[i] * ((v @ v + 0.4 * self.vdwr[i] ** 2) * np.eye(3) - np.outer(v, v))
        adet = math.sqrt(np.linalg.det(inertia) ** (1.0 / 3.0) / (0.4 * vol))
        I = inertia
        ad = np.array([
            [I[0, 0] * (I[1, 1] + I[2, 2]) - I[0, 1] ** 2 - I[0, 2] ** 2,
             I[0, 1] * I[2, 2] - I[0, 2] * I[1, 2],
             I[0, 2] * I[1, 1] - I[0, 1] * I[2, 1]],
            [I[0, 1] * I[2, 2] - I[0, 2] * I[1, 2],
             I[1, 1] * (I[0, 0] + I[2, 2]) - I[0, 1] ** 2 - I[1, 2] ** 2,
             I[0, 0] * I[1, 2] - I[0, 1] * I[0, 2]],
            [I[0, 2] * I[1, 1] - I[0, 1] * I[2, 1],
             I[0, 0] * I[1, 2] - I[0, 1] * I[0, 2],
             I[2, 2] * (I[0, 0] + I[1, 1]) - I[0, 2] ** 2 - I[1, 2] ** 2]])
        qt = qat.sum()
        ad *= 250.0 / (48.0 * vol ** 3 * adet ** 5) * (-0.5 * keps * self.alpbet * qt ** 2 / adet ** 2)
        for i in range(nat):
            g[i] += rad3[i] * (ad @ (xyz[i] - center))
        return g


class GBEpsilon(ALPBWater):
    """Generalized Born model with a dielectric constant (tblite_new_gb_solvation_epsilon):
    alpb=True is version 10 (GB-epsilon with the ALPB shape term), False version 20; kernel
    "still" or "p16".  COSMO radii, descreening 0.8, Born scale 1, no offset, no surface term
    and no free-energy shift."""

    def __init__(self, numbers, eps, alpb=True, kernel="p16"):
        d = json.loads(DATA.read_text())
        aatoau = d["constants"]["aatoau"]
        z = np.asarray(numbers) - 1
        self.nat = len(z)
        self.kernel = kernel
        self.cds = False
        self.alpbet = ALPHA_ALPB / eps if alpb else 0.0
        self.keps = (1.0 / eps - 1.0) / (1.0 + self.alpbet)
        self.vdwr = np.array(d["rvdw_cosmo"])[z]
        self.rho = self.vdwr * 0.8
        self.svdw = self.vdwr.copy()
        self.born_scale = 1.0
        self.lrcut = 35.0 * aatoau
        self.tension = np.zeros(self.nat)
        self.hbond = np.zeros(self.nat)
        self.total_shift = 0.0
