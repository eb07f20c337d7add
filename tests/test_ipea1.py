"""IPEA1-xTB: the GFN1 form with IPEA1-xTB's tables (reference src/tblite/xtb/ipea1.f90).

CPU part: the oracle (oracle/gfn1.py with method="ipea1") against the reference's own
single-atom energies (test/unit/test_ipea1_xtb.f90:133-347, thr = sqrt(eps)) for every element
without d shells or a halogen-bond correction, its molecular gradient against central finite
differences, and the exported parameter record (tblite_export_ipea1_param): name, s-p H0 scale,
pair factors, the occupation of polarisation shells the reference's export keeps.
GPU part (marked): the engine against the same golden energies and against the oracle for
molecules at |dE| <= 1e-7 Eh, charges <= 1e-6 e, gradient <= 1e-6 Eh/Bohr; the calculator made
from the exported record gives the built-in calculator's energy.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import gfn1, gfn2

GOLDEN = Path(__file__).resolve().parent / "golden"
E_TOL, Q_TOL, G_TOL = 1e-7, 1e-6, 1e-6


def _cases():
    d = json.loads((GOLDEN / "atoms_ipea1.json").read_text())
    p = gfn1.load_params1("ipea1")
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
    assert len(_CASES) >= 40


@pytest.mark.parametrize("key,z,charge,uhf,ref", _CASES, ids=[f"{c[0]}-{c[1]}" for c in _CASES])
def test_oracle_atom_energy(key, z, charge, uhf, ref):
    mol = gfn2.Molecule(np.array([z]), np.zeros((1, 3)), charge=charge, uhf=uhf)
    calc = gfn1.new_calc(mol, method="ipea1", accuracy=_D["accuracy"], kt=_D["kt"])
    res = gfn1.singlepoint(calc, grad=False)
    assert abs(res.energy - ref) < _D["thr"]


def test_oracle_gradient_fd():
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster_k(2, seed=3)

    def run(xx, grad):
        calc = gfn1.new_calc(gfn2.Molecule(np.asarray(z), xx), method="ipea1", accuracy=1e-5)
        return gfn1.singlepoint(calc, grad=grad)

    ref = run(x, True)
    h = 1e-4
    for a, k in [(0, 0), (1, 1), (3, 2)]:
        xp, xm = x.copy(), x.copy()
        xp[a, k] += h
        xm[a, k] -= h
        fd = (run(xp, False).energy - run(xm, False).energy) / (2 * h)
        assert abs(fd - ref.gradient[a, k]) < 1e-7


def test_exported_record():
    from tblite_gb300 import _build, library

    _build.build()
    d = library.export_param("IPEA1-xTB")
    assert d["meta"]["name"] == "IPEA1-xTB"
    assert d["hamiltonian"]["xtb"]["shell"]["sp"] == 2.25
    assert d["hamiltonian"]["xtb"]["cn"] == "exp"
    # element-pair factors only between transition metals (no H-H 0.96 as in GFN1-xTB)
    pairs = d["hamiltonian"]["xtb"].get("kpair", {})
    assert pairs and all("H" not in k.split("-") for k in pairs)
    assert library.export_param("GFN1-xTB")["hamiltonian"]["xtb"]["kpair"]["H-H"] == 0.96
    # the reference's export keeps the occupation of the diffuse 3s shell of carbon
    assert d["element"]["C"]["refocc"] == [2.0, 2.0, 2.0]
    g1 = library.export_param("GFN1-xTB")
    assert g1["element"]["H"]["refocc"][1] == 0.0


def _gpu(z, x, charge=None, uhf=None, acc=1.0, **settings):
    from tblite_gb300.interface import Calculator

    calc = Calculator("IPEA1-xTB", z, x, charge=charge, uhf=uhf)
    calc.set("accuracy", acc)
    for k, v in settings.items():
        calc.set(k, v)
    return calc.singlepoint()


@pytest.mark.gpu
@pytest.mark.parametrize("key,z,charge,uhf,ref", _CASES, ids=[f"{c[0]}-{c[1]}" for c in _CASES])
def test_gpu_atom_golden(key, z, charge, uhf, ref):
    res = _gpu([z], np.zeros((1, 3)), charge=charge, uhf=uhf, acc=_D["accuracy"],
               temperature=_D["kt"])
    assert abs(res.get("energy") - ref) < _D["thr"]


@pytest.mark.gpu
@pytest.mark.parametrize("mol", ["water4", "alkane6", "cation"])
def test_gpu_molecules_vs_oracle(mol):
    from tblite_gb300 import workloads

    charge = 0.0
    if mol == "water4":
        z, x = workloads.water_cluster_k(4, seed=41)
    elif mol == "alkane6":
        z, x = workloads.alkane(6, seed=42)
    else:
        z, x = workloads.water_cluster_k(2, seed=43)
        charge = 1.0
    uhf = 1 if charge else 0
    res = _gpu(z, x, charge=charge, uhf=uhf, acc=1e-3)
    ref = gfn1.singlepoint(gfn1.new_calc(gfn2.Molecule(np.asarray(z), np.asarray(x),
                                                        charge=charge, uhf=uhf),
                                         method="ipea1", accuracy=1e-3))
    assert abs(res.get("energy") - ref.energy) < E_TOL
    assert np.max(np.abs(res.get("charges") - ref.qat)) < Q_TOL
    assert np.max(np.abs(res.get("gradient") - ref.gradient)) < G_TOL


@pytest.mark.gpu
def test_gpu_record_calculator_matches_builtin():
    from tblite_gb300 import library, workloads
    from tblite_gb300.interface import Calculator

    z, x = workloads.alkane(4, seed=44)
    ref = Calculator("IPEA1-xTB", z, x).singlepoint()
    res = Calculator(library.export_param("IPEA1-xTB"), z, x).singlepoint()
    assert abs(res.get("energy") - ref.get("energy")) < 1e-10


@pytest.mark.gpu
def test_gpu_batch_mixes_methods():
    """GFN2-xTB, GFN1-xTB and IPEA1-xTB calculators in one batch call: every memory chunk runs
    one set of model constants, and each molecule agrees with its one-molecule single point."""
    from tblite_gb300 import workloads
    from tblite_gb300.interface import Calculator, batch_fallbacks, batch_singlepoint

    mols = [workloads.water_cluster_k(k, seed=50 + k) for k in (1, 3, 6)] + \
           [workloads.alkane(n, seed=60 + n) for n in (2, 5)]
    calcs, ref = [], []
    for i, (z, x) in enumerate(mols):
        for method in ("IPEA1-xTB", "GFN1-xTB", "GFN2-xTB"):
            calcs.append(Calculator(method, z, x))
            ref.append(Calculator(method, z, x).singlepoint())
    res = batch_singlepoint(calcs)
    assert batch_fallbacks() == 0
    for r, p in zip(res, ref):
        assert abs(r.get("energy") - p.get("energy")) < E_TOL
        assert np.max(np.abs(r.get("gradient") - p.get("gradient"))) < G_TOL
        assert np.max(np.abs(r.get("charges") - p.get("charges"))) < Q_TOL
