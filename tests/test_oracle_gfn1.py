"""GFN1-xTB CPU oracle checks against the reference's own known-answer tests.

Pins the GFN1 restatement (basis with the orthogonalised hydrogen 2s shell, valence /
polarisation H0 scaling, harmonic-mean Coulomb, atom-resolved third order) before it checks
the CUDA engine: single-atom energies of test/unit/test_gfn1_xtb.f90:135-349 (thr = sqrt(eps))
for every element without d shells or a halogen-bond correction, and the analytic molecular
gradient against central finite differences.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import gfn1, gfn2

GOLDEN = Path(__file__).resolve().parent / "golden"


def _cases():
    d = json.loads((GOLDEN / "atoms_gfn1.json").read_text())
    p = gfn1.load_params1()
    out = []
    for key, c in d["cases"].items():
        for z in range(1, 87):
            if z in c["skip"]:
                continue
            lmax = max(p["ang_shell"][z - 1][: int(p["nshell"][z - 1])])
            if lmax > 1 or p["halogen_bond"][z - 1] > 0.0:
                continue  # d shells and halogen-bond elements are not on this path
            out.append((key, z, c["charge"], c["uhf"][z - 1], c["energy"][z - 1]))
    return d, out


_D, _CASES = _cases()


def test_case_count():
    assert len(_CASES) >= 50


@pytest.mark.parametrize("key,z,charge,uhf,ref", _CASES, ids=[f"{c[0]}-{c[1]}" for c in _CASES])
def test_atom_energy(key, z, charge, uhf, ref):
    mol = gfn2.Molecule(np.array([z]), np.zeros((1, 3)), charge=charge, uhf=uhf)
    calc = gfn1.new_calc(mol, accuracy=_D["accuracy"], kt=_D["kt"])
    res = gfn1.singlepoint(calc, grad=False)
    assert abs(res.energy - ref) < _D["thr"]


def test_hydrogen_2s_is_orthogonal_to_1s():
    from oracle.gfn2 import load_sto, slater_to_gauss

    p = gfn1.load_params1()
    sto = load_sto()
    shells = []
    for ish in range(2):
        a, c = slater_to_gauss(int(p["number_of_primitives"][0][ish]),
                               int(p["principal_quantum_number"][0][ish]), 0,
                               p["slater_exponent"][0][ish], sto)
        shells.append((a, c))
    a2, c2 = gfn1.orthogonalize(shells[0][0], shells[0][1], shells[1][0], shells[1][1])

    def ov(a, c, b, d):
        return sum(ci * dj * (np.pi / (ai + bj)) ** 1.5 for ai, ci in zip(a, c) for bj, dj in zip(b, d))

    # the projection assumes a normalised 1s; the STO-nG fit is normalised to ~1e-9, which
    # leaves an overlap of that size (the reference does the same)
    assert abs(ov(*shells[0], a2, c2)) < 1e-8
    assert abs(ov(a2, c2, a2, c2) - 1.0) < 1e-13


@pytest.mark.parametrize("mol", ["water", "alkane"])
def test_molecular_gradient_fd(mol):
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster_k(2, seed=3) if mol == "water" else workloads.alkane(3, seed=5)

    def run(xx, grad):
        calc = gfn1.new_calc(gfn2.Molecule(np.asarray(z), xx), accuracy=1e-5)
        return gfn1.singlepoint(calc, grad=grad)

    ref = run(x, True)
    h = 1e-4
    for a, k in [(0, 0), (1, 2), (len(z) - 1, 1)]:
        xp, xm = x.copy(), x.copy()
        xp[a, k] += h
        xm[a, k] -= h
        fd = (run(xp, False).energy - run(xm, False).energy) / (2 * h)
        assert abs(fd - ref.gradient[a, k]) < 2e-8
