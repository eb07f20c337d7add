"""Implicit solvation: ALPB(water) and GBSA(water) with CDS and shift, and the generalized Born
models with a dielectric constant (GB-epsilon with or without the ALPB shape term, Still or P16
kernel).

CPU part: the oracle's solvation gradient against finite differences of its own energy (every
model and kernel), the Lebedev grid integrating low-order spherical polynomials exactly, and the
C ABI constructors' error handling.  GPU part (marked): the engine against the oracle at
|dE| <= 1e-7 Eh, charges <= 1e-6 e, gradient <= 1e-6 Eh/Bohr, for GFN2 and GFN1.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_lebedev230_integrates_polynomials():
    from oracle.solvation import lebedev230

    d = json.loads((ROOT / "tblite_gb300" / "data" / "solvation_water.json").read_text())
    x, w = lebedev230(d["lebedev230"])
    assert np.allclose(np.sum(x * x, axis=1), 1.0)
    assert abs(w.sum() - 4 * math.pi) < 1e-12
    assert abs(np.sum(w * x[:, 0] ** 2) - 4 * math.pi / 3) < 1e-12
    assert abs(np.sum(w * x[:, 0] ** 2 * x[:, 1] ** 2) - 4 * math.pi / 15) < 1e-12
    assert abs(np.sum(w * x[:, 2] ** 4) - 4 * math.pi / 5) < 1e-12


def _model(name, z):
    from oracle.solvation import ALPBWater, GBEpsilon

    return {"alpb": lambda: ALPBWater(z),
            "gbsa": lambda: ALPBWater(z, model="gbsa"),
            "gbe-still": lambda: GBEpsilon(z, 7.0, alpb=True, kernel="still"),
            "gbe-p16": lambda: GBEpsilon(z, 7.0, alpb=True, kernel="p16"),
            "gb-p16": lambda: GBEpsilon(z, 7.0, alpb=False, kernel="p16")}[name]()


@pytest.mark.parametrize("model", ["alpb", "gbsa", "gbe-still", "gb-p16"])
def test_oracle_solvation_gradient_matches_fd(model):
    from oracle import gfn2
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster_k(2, seed=3)

    def run(xx, grad):
        calc = gfn2.new_calc(gfn2.Molecule(np.asarray(z), xx), accuracy=1e-5)
        return gfn2.singlepoint(calc, grad=grad, solvation=_model(model, z))

    ref = run(x, True)
    h = 1e-4
    for a, k in [(0, 0), (2, 1), (4, 2)]:
        xp, xm = x.copy(), x.copy()
        xp[a, k] += h
        xm[a, k] -= h
        fd = (run(xp, False).energy - run(xm, False).energy) / (2 * h)
        assert abs(fd - ref.gradient[a, k]) < 1e-7


def test_capi_rejects_unknown_solvent():
    from tblite_gb300 import _build, library
    from tblite_gb300.exceptions import TBLiteRuntimeError

    _build.build()
    mol = library.new_structure(np.array([8, 1, 1]), np.array([[0, 0, 0], [0, 0, 1.8], [1.8, 0, 0.0]]))
    with pytest.raises(TBLiteRuntimeError, match="water only"):
        library.new_alpb_solvation(mol, "benzene")
    with pytest.raises(TBLiteRuntimeError, match="GFN2"):
        library.new_alpb_solvation(mol, "water", version=1)
    cont = library.new_alpb_solvation(mol, "water", state="bar1mol")
    assert cont.value
    library.load().tblite_delete_container(library.byref(cont))
    assert not cont.value
    cont = library.new_gbsa_solvation(mol, "water")
    assert cont.value
    library.load().tblite_delete_container(library.byref(cont))
    with pytest.raises(TBLiteRuntimeError, match="GFN2"):
        library.new_gbsa_solvation(mol, "water", version=1)


def test_capi_gb_epsilon_constructor():
    from tblite_gb300 import _build, library
    from tblite_gb300.exceptions import TBLiteRuntimeError, TBLiteValueError

    _build.build()
    lib = library.load()
    mol = library.new_structure(np.array([8, 1, 1]), np.array([[0, 0, 0], [0, 0, 1.8], [1.8, 0, 0.0]]))
    for alpb in (True, False):
        for born in ("still", "p16"):
            cont = library.new_gb_solvation_epsilon(mol, 7.0, born, alpb=alpb)
            assert cont.value
            lib.tblite_delete_container(library.byref(cont))
    err = library._Error()
    assert not lib.tblite_new_gb_solvation_epsilon(err.h, mol, 7.0, 12, 1)
    with pytest.raises(TBLiteRuntimeError, match="Unknown solvation model"):
        err.check()
    err = library._Error()
    assert not lib.tblite_new_gb_solvation_epsilon(err.h, mol, 7.0, 20, 3)
    with pytest.raises(TBLiteRuntimeError, match="Born interaction kernel"):
        err.check()
    err = library._Error()
    assert not lib.tblite_new_gb_solvation_epsilon(err.h, mol, -1.0, 20, 1)
    with pytest.raises(TBLiteRuntimeError, match="Dielectric constant"):
        err.check()
    with pytest.raises(TBLiteValueError):
        library.new_gb_solvation_epsilon(mol, 7.0, "born", alpb=False)


def _compare(z, x, state="gsolv", acc=1e-3):
    from oracle import gfn2
    from oracle.solvation import ALPBWater
    from tblite_gb300.interface import Calculator

    calc = Calculator("GFN2-xTB", z, x)
    calc.set("accuracy", acc)
    calc.add("alpb-solvation", "water", state)
    res = calc.singlepoint()
    ocalc = gfn2.new_calc(gfn2.Molecule(np.asarray(z), np.asarray(x)), accuracy=acc)
    ref = gfn2.singlepoint(ocalc, grad=True,
                           solvation=ALPBWater(z, state={"gsolv": 1, "bar1mol": 2, "reference": 3}[state]))
    assert abs(res.get("energy") - ref.energy) < 1e-7
    assert np.max(np.abs(res.get("charges") - ref.qat)) < 1e-6
    assert np.max(np.abs(res.get("gradient") - ref.gradient)) < 1e-6
    return res, ref


@pytest.mark.gpu
@pytest.mark.parametrize("state", ["gsolv", "bar1mol", "reference"])
def test_gpu_alpb_water_dimer(state):
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster_k(2, seed=3)
    _compare(z, x, state)


@pytest.mark.gpu
def test_gpu_alpb_water_cluster_and_alkane():
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster((2, 2, 2), seed=21)
    _compare(z, x)
    z, x = workloads.alkane(5, seed=22)
    _compare(z, x)


def _compare_model(method, z, x, interaction, args, model, acc=1e-3):
    from oracle import gfn1, gfn2
    from tblite_gb300.interface import Calculator

    calc = Calculator(method, z, x)
    calc.set("accuracy", acc)
    calc.add(interaction, *args)
    res = calc.singlepoint()
    orc = gfn2 if method == "GFN2-xTB" else gfn1
    ocalc = orc.new_calc(orc.Molecule(np.asarray(z), np.asarray(x)), accuracy=acc)
    ref = orc.singlepoint(ocalc, grad=True, solvation=_model(model, z))
    assert abs(res.get("energy") - ref.energy) < 1e-7
    assert np.max(np.abs(res.get("charges") - ref.qat)) < 1e-6
    assert np.max(np.abs(res.get("gradient") - ref.gradient)) < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("interaction,args,model", [
    ("gbsa-solvation", ("water",), "gbsa"),
    ("gbe-solvation", (7.0, "still"), "gbe-still"),
    ("gb-solvation", (7.0, "p16"), "gb-p16"),
])
def test_gpu_gb_models_gfn2(interaction, args, model):
    """GBSA(water) and the dielectric-constant GB models against the oracle (GFN2)."""
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster((2, 2, 2), seed=21)
    _compare_model("GFN2-xTB", z, x, interaction, args, model)
    z, x = workloads.alkane(5, seed=22)
    _compare_model("GFN2-xTB", z, x, interaction, args, model)


@pytest.mark.gpu
def test_gpu_gb_epsilon_gfn1():
    """GFN1-xTB with GB-epsilon (the reference's python test_solvation_gfn1_gbe uses this model
    with epsilon 7 and the P16 kernel) against the GFN1 oracle."""
    from tblite_gb300 import workloads

    z, x = workloads.water_cluster_k(3, seed=23)
    _compare_model("GFN1-xTB", z, x, "gbe-solvation", (7.0, "p16"), "gbe-p16")
