"""GFN1-xTB on the CUDA engine vs the GFN1 CPU oracle and the reference's single-atom energies
(needs a GPU).

Single atoms: test/unit/test_gfn1_xtb.f90:135-349 (neutral, cation, anion; thr = sqrt(eps)) for
every element without d shells or a halogen-bond correction.  Molecules: energy, atomic
energies, charges, gradient, virial, dipole, quadrupole and bond orders against the oracle at
|dE| <= 1e-7 Eh, charges <= 1e-6 e, gradient <= 1e-6 Eh/Bohr.
"""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
E_TOL, Q_TOL, G_TOL = 1e-7, 1e-6, 1e-6


@pytest.fixture(scope="module", autouse=True)
def built():
    from tblite_gb300 import _build

    _build.build()


def _gpu(z, x, charge=None, uhf=None, acc=1.0, **settings):
    from tblite_gb300.interface import Calculator

    calc = Calculator("GFN1-xTB", z, x, charge=charge, uhf=uhf)
    calc.set("accuracy", acc)
    for k, v in settings.items():
        calc.set(k, v)
    return calc.singlepoint()


def _oracle(z, x, charge=0.0, uhf=0, acc=1.0):
    from oracle import gfn1, gfn2

    mol = gfn2.Molecule(np.asarray(z), np.asarray(x, dtype=float), charge=charge, uhf=uhf)
    return gfn1.singlepoint(gfn1.new_calc(mol, accuracy=acc))


def _atom_cases():
    d = json.loads((GOLDEN / "atoms_gfn1.json").read_text())
    p = json.loads((Path(__file__).resolve().parents[1] / "tblite_gb300" / "data"
                    / "gfn1.json").read_text())
    out = []
    for key, c in d["cases"].items():
        for z in range(1, 87):
            if z in c["skip"]:
                continue
            lmax = max(p["ang_shell"][z - 1][: int(p["nshell"][z - 1])])
            if lmax > 1 or p["halogen_bond"][z - 1] > 0.0:
                continue
            out.append((key, z, c["charge"], c["uhf"][z - 1], c["energy"][z - 1]))
    return d, out


_D, _ATOMS = _atom_cases()


@pytest.mark.parametrize("key,z,charge,uhf,ref", _ATOMS, ids=[f"{c[0]}-{c[1]}" for c in _ATOMS])
def test_atom_golden(key, z, charge, uhf, ref):
    res = _gpu([z], np.zeros((1, 3)), charge=charge, uhf=uhf, acc=_D["accuracy"],
               temperature=_D["kt"])
    assert abs(res.get("energy") - ref) < _D["thr"]


def _compare(z, x, acc, charge=0.0, uhf=None):
    res = _gpu(z, x, charge=charge, uhf=uhf, acc=acc)
    ref = _oracle(z, x, charge=charge, uhf=uhf or 0, acc=acc)
    assert abs(res.get("energy") - ref.energy) < E_TOL
    assert np.max(np.abs(res.get("energies") - ref.energies)) < E_TOL
    assert np.max(np.abs(res.get("charges") - ref.qat)) < Q_TOL
    assert np.max(np.abs(res.get("gradient") - ref.gradient)) < G_TOL
    assert np.max(np.abs(res.get("virial") - ref.sigma)) < 1e-5
    assert np.max(np.abs(res.get("dipole") - ref.parts["dipole"])) < 1e-6
    assert np.max(np.abs(res.get("quadrupole") - ref.parts["quadrupole"])) < 1e-5
    wbo = res.get("bond-orders")
    ref_wbo = ref.parts["wbo"]
    if ref_wbo.shape[0] == 1:
        assert np.max(np.abs(wbo - ref_wbo[0])) < 1e-6
    else:
        for ch in range(2):
            assert np.max(np.abs(wbo[:, :, ch] - ref_wbo[ch])) < 1e-6
    return res, ref


def test_water_dimer():
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster((2, 1, 1), seed=11)
    _compare(z, x, acc=1e-3)


@pytest.mark.parametrize("charge", [1.0, -1.0])
def test_water_dimer_ions(charge):
    """Restricted open shell (doublets): total and magnetisation bond-order channels."""
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster((2, 1, 1), seed=15)
    _compare(z, x, acc=1e-3, charge=charge)


def test_alkane():
    from tblite_gb300 import workloads

    z, x = workloads.alkane(10, seed=5)
    _compare(z, x, acc=1e-3)


def test_water_cluster_8():
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster((2, 2, 2), seed=7)
    _compare(z, x, acc=1e-3)


def test_triplet_oxygen():
    x = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 2.28]])
    _compare([8, 8], x, acc=1e-3, uhf=2)


def test_formamide_ammonia():
    """N-containing molecules: formamide next to ammonia (H, C, N, O)."""
    rng = np.random.default_rng(3)
    z = np.array([6, 8, 1, 7, 1, 1, 7, 1, 1, 1])
    x = np.array([[0.0, 0.0, 0.0], [2.28, 0.0, 0.0], [-1.0, 1.75, 0.0], [-1.28, -2.23, 0.0],
                  [-3.2, -2.1, 0.0], [-0.4, -3.9, 0.0], [1.5, -6.8, 0.5], [2.9, -6.0, 1.5],
                  [0.3, -7.6, 1.7], [2.1, -8.2, -0.6]]) + 0.05 * rng.standard_normal((10, 3))
    _compare(z, x, acc=1e-3)


def test_parameter_gradient_is_refused():
    from tblite_gb300 import library
    from tblite_gb300.interface import Calculator

    z, x = [1, 1], np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 1.4]])
    calc = Calculator("GFN1-xTB", z, x)
    with pytest.raises(Exception):
        library.set_parameter_gradient(calc._ctx, calc._calc)
