"""CUDA engine vs the CPU oracle and the reference's golden vectors (needs a GPU).

Tolerances: |dE| <= 1e-7 Eh, shell charges <= 1e-6 e, gradient <= 1e-6 Eh/Bohr
(the engine and the oracle converge the same SCF with the same thresholds).
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

    calc = Calculator("GFN2-xTB", z, x, charge=charge, uhf=uhf)
    calc.set("accuracy", acc)
    for k, v in settings.items():
        calc.set(k, v)
    return calc, calc.singlepoint()


def _oracle(z, x, charge=0.0, uhf=0, acc=1.0, grad=True):
    from oracle import gfn2

    calc = gfn2.new_calc(gfn2.Molecule(np.asarray(z), np.asarray(x), charge=charge, uhf=uhf),
                         accuracy=acc)
    return gfn2.singlepoint(calc, grad=grad)


ATOMS = [(z, key) for z in (1, 2, 3, 6, 7, 8, 9) for key in ("neutral", "cation", "anion")]


@pytest.mark.parametrize("z,key", ATOMS)
def test_atom_golden(z, key):
    d = json.loads((GOLDEN / "atoms_gfn2.json").read_text())
    c = d["cases"][key]
    if z in c["skip"]:
        pytest.skip("skipped by the reference test")
    _, res = _gpu([z], np.zeros((1, 3)), charge=c["charge"], uhf=c["uhf"][z - 1], acc=d["accuracy"])
    assert abs(res.get("energy") - c["energy"][z - 1]) < d["thr"]


def _compare(z, x, acc, charge=0.0):
    _, res = _gpu(z, x, charge=charge, acc=acc)
    ref = _oracle(z, x, charge=charge, acc=acc)
    assert abs(res.get("energy") - ref.energy) < E_TOL
    assert np.max(np.abs(res.get("charges") - ref.qat)) < Q_TOL
    assert np.max(np.abs(res.get("shell-charges") - ref.qsh)) < Q_TOL
    assert np.max(np.abs(res.get("gradient") - ref.gradient)) < G_TOL
    assert np.max(np.abs(res.get("energies") - ref.energies)) < E_TOL
    assert np.max(np.abs(res.get("virial") - ref.sigma)) < 1e-5
    return res, ref


def test_water_dimer():
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster((2, 1, 1), seed=11)
    _compare(z, x, acc=1e-3)


def test_water_cation():
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster((2, 1, 1), seed=12)
    _compare(z, x, acc=1e-3, charge=1.0)


def test_alkane_c8():
    from tblite_gb300 import workloads

    z, x = workloads.alkane(8, seed=7)
    _compare(z, x, acc=1e-2)


def test_h2o32_config0():
    """(H2O)32, 192 AOs, accuracy 0.01 (the configuration's SCF threshold)."""
    from tblite_gb300 import workloads

    z, x = workloads.config("h2o32")
    _compare(z, x, acc=0.01)


def test_restart_reuses_wavefunction():
    from tblite_gb300 import workloads
    from tblite_gb300.interface import Calculator

    z, x = workloads.alkane(6, seed=3)
    calc = Calculator("GFN2-xTB", z, x)
    res = calc.singlepoint()
    e1 = res.get("energy")
    calc.singlepoint(res)
    assert abs(res.get("energy") - e1) < 1e-6


def test_nonconvergence_is_an_error_with_results():
    from tblite_gb300 import workloads
    from tblite_gb300.exceptions import TBLiteRuntimeError
    from tblite_gb300.interface import Calculator, Result

    z, x = workloads.alkane(5, seed=3)
    calc = Calculator("GFN2-xTB", z, x)
    calc.set("max-iter", 3)
    res = Result()
    with pytest.raises(TBLiteRuntimeError, match="SCF not converged in 3 cycles"):
        calc.singlepoint(res)
    assert np.isfinite(res.get("energy"))


def test_energy_is_deterministic():
    from tblite_gb300 import workloads

    z, x = workloads.alkane(12, seed=4)
    _, r1 = _gpu(z, x)
    _, r2 = _gpu(z, x)
    assert r1.get("energy") == r2.get("energy")
    assert np.array_equal(r1.get("charges"), r2.get("charges"))


@pytest.mark.parametrize("charge", [0.0, 1.0])
def test_bond_orders_and_moments(charge):
    """Wiberg/Mayer bond orders and molecular dipole/quadrupole vs the oracle's post-processing;
    the cation is a restricted open shell (total and magnetisation channels)."""
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster((2, 1, 1), seed=12)
    res, ref = _compare(z, x, acc=1e-3, charge=charge)
    wbo = res.get("bond-orders")
    ref_wbo = ref.parts["wbo"]
    if ref_wbo.shape[0] == 1:
        assert wbo.shape == (len(z), len(z))
        assert np.max(np.abs(wbo - ref_wbo[0])) < 1e-6
    else:
        assert wbo.shape == (len(z), len(z), 2)
        for ch in range(2):
            assert np.max(np.abs(wbo[:, :, ch] - ref_wbo[ch])) < 1e-6
    assert np.max(np.abs(res.get("dipole") - ref.parts["dipole"])) < 1e-6
    assert np.max(np.abs(res.get("quadrupole") - ref.parts["quadrupole"])) < 1e-5


def test_split_gemm_plain_path():
    """One-molecule path: the tensor-core split GEMM (FP64-accurate operand splitting, used
    from 128 orbitals on) against the FP64 tile GEMM on (H2O)32 (192 orbitals)."""
    from tblite_gb300 import library, workloads

    z, x = workloads.water_cluster((4, 4, 2), seed=0)
    try:
        library.set_split_gemm(False)
        _, ref = _gpu(z, x, acc=0.01)
    finally:
        library.set_split_gemm(True)
    _, res = _gpu(z, x, acc=0.01)
    assert abs(res.get("energy") - ref.get("energy")) < E_TOL
    assert np.max(np.abs(res.get("gradient") - ref.get("gradient"))) < G_TOL
    assert np.max(np.abs(res.get("charges") - ref.get("charges"))) < Q_TOL
    assert np.max(np.abs(res.get("bond-orders") - ref.get("bond-orders"))) < 1e-6
