"""Homogeneous external electric field (reference src/tblite/external/field.f90).

The field adds -E.R_A to the atomic potential and -E to the atomic dipole potential; the energy
takes the output charges and dipole moments, E_field = -sum_A (q_A E.R_A + E.mu_A).  The
reference's gradient of the container is -E for every atom and its virial -sym(E (sum_A R_A)^T)
(field.f90:100-113); this library returns the same, so the gradient of a molecule in a field is
checked against the oracle, not against finite differences of the energy.  The energy is
checked through its field derivative: dE/dE_k = -mu_k, the molecular dipole (the reference's
test_d_mb03/04 in test/unit/test_xtb_external.f90).
"""
import numpy as np
import pytest

from oracle import gfn2

E_FIELD = np.array([0.002, -0.001, 0.003])


def _oracle(z, x, efield, acc=1e-5):
    calc = gfn2.new_calc(gfn2.Molecule(np.asarray(z), np.asarray(x, dtype=float)), accuracy=acc)
    return gfn2.singlepoint(calc, grad=True, efield=efield)


def test_oracle_energy_derivative_is_the_dipole():
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster_k(2, seed=3)
    ref = _oracle(z, x, E_FIELD)
    h = 1e-4
    for k in range(3):
        ep, em = E_FIELD.copy(), E_FIELD.copy()
        ep[k] += h
        em[k] -= h
        num = -(_oracle(z, x, ep).energy - _oracle(z, x, em).energy) / (2 * h)
        assert abs(num - ref.parts["dipole"][k]) < 1e-6


def test_capi_field_container():
    from tblite_gb300 import _build, library, workloads
    from tblite_gb300.exceptions import TBLiteRuntimeError
    from tblite_gb300.interface import Calculator

    _build.build()
    lib = library.load()
    assert not lib.tblite_new_electric_field(None)
    z, x = workloads.water_cluster_k(1, seed=4)
    calc = Calculator("GFN2-xTB", z, x)
    calc.add("electric-field", E_FIELD)
    with pytest.raises(TBLiteRuntimeError, match="already holds an electric field"):
        calc.add("electric-field", E_FIELD)
    with pytest.raises(TBLiteRuntimeError, match="GFN2-xTB form"):
        Calculator("GFN1-xTB", z, x).add("electric-field", E_FIELD)


def _gpu(z, x, efield, acc=1e-5):
    from tblite_gb300.interface import Calculator

    calc = Calculator("GFN2-xTB", z, x)
    calc.set("accuracy", acc)
    calc.add("electric-field", efield)
    return calc.singlepoint()


@pytest.mark.gpu
@pytest.mark.parametrize("mol", ["water3", "alkane4"])
def test_gpu_field_vs_oracle(mol):
    from tblite_gb300 import workloads

    z, x = (workloads.water_cluster_k(3, seed=5) if mol == "water3"
            else workloads.alkane(4, seed=6))
    res = _gpu(z, x, E_FIELD, acc=1e-3)
    ref = _oracle(z, x, E_FIELD, acc=1e-3)
    assert abs(res.get("energy") - ref.energy) < 1e-7
    assert np.max(np.abs(res.get("charges") - ref.qat)) < 1e-6
    assert np.max(np.abs(res.get("gradient") - ref.gradient)) < 1e-6
    assert np.max(np.abs(res.get("virial") - ref.sigma)) < 1e-5
    assert np.max(np.abs(res.get("dipole") - ref.parts["dipole"])) < 1e-6


@pytest.mark.gpu
def test_gpu_energy_derivative_is_the_dipole():
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster_k(2, seed=7)
    dip = _gpu(z, x, E_FIELD).get("dipole")
    h = 1e-4
    for k in range(3):
        ep, em = E_FIELD.copy(), E_FIELD.copy()
        ep[k] += h
        em[k] -= h
        num = -(_gpu(z, x, ep).get("energy") - _gpu(z, x, em).get("energy")) / (2 * h)
        assert abs(num - dip[k]) < 1e-6
