"""The benchmark configurations against the CPU oracle (needs a GPU).

* C200H402 (602 atoms, 1202 AOs), the one-molecule configuration: the plain path with
  diagonalisation (the shared-memory tridiagonalisation over a cooperative grid) and with the
  spectral-projection density, against the oracle's result in ``golden/c200h402.npz``.
* 40 molecules of the 4096-molecule ensemble (``golden/ensemble_sample.npz``: 16 drawn
  uniformly, 24 with at least 157 orbitals, which the batched path tridiagonalises in a
  thread-block cluster), through the batched entry point (GFN2, and GFN1 for every fourth
  molecule) and, for a subset, the plain path.

Fixtures: ``tests/golden/make_parity_fixtures.py``.  Bars: |dE| <= 1e-7 Eh, shell and atomic
charges <= 1e-6 e, gradient <= 1e-6 Eh/Bohr, virial <= 1e-5 Eh, dipole <= 1e-6 e Bohr.
"""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
E_TOL, Q_TOL, G_TOL, V_TOL = 1e-7, 1e-6, 1e-6, 1e-5


@pytest.fixture(scope="module", autouse=True)
def built():
    from tblite_gb300 import _build

    _build.build()


def _check(res, ref, energies=True):
    """res: a Result; ref: mapping with the oracle's arrays."""
    assert abs(res.get("energy") - float(ref["energy"])) <= E_TOL
    assert np.max(np.abs(res.get("shell-charges") - ref["qsh"])) <= Q_TOL
    assert np.max(np.abs(res.get("charges") - ref["qat"])) <= Q_TOL
    assert np.max(np.abs(res.get("gradient") - ref["gradient"])) <= G_TOL
    if "virial" in ref:
        assert np.max(np.abs(res.get("virial") - ref["virial"])) <= V_TOL
    if "dipole" in ref:
        assert np.max(np.abs(res.get("dipole") - ref["dipole"])) <= 1e-6
    if energies and "energies" in ref:
        assert np.max(np.abs(res.get("energies") - ref["energies"])) <= E_TOL


@pytest.mark.parametrize("solver", ["diagonalization", "purification"])
def test_c200h402_plain_path(solver):
    from tblite_gb300.interface import Calculator

    ref = dict(np.load(GOLDEN / "c200h402.npz"))
    calc = Calculator("GFN2-xTB", ref["numbers"], ref["positions"])
    calc.set("density-solver", solver)
    res = calc.singlepoint()
    assert res.get("norbitals") == 1202
    _check(res, ref)


def _sample():
    d = dict(np.load(GOLDEN / "ensemble_sample.npz"))
    nat, nsh = d["natoms"], d["nshells"]
    ao = np.concatenate([[0], np.cumsum(nat)])
    so = np.concatenate([[0], np.cumsum(nsh)])
    mols, refs = [], []
    for j in range(len(nat)):
        a = slice(ao[j], ao[j + 1])
        mols.append((d["numbers"][a], d["positions"][a]))
        refs.append({"energy": d["energy"][j], "gradient": d["gradient"][a], "qat": d["qat"][a],
                     "qsh": d["qsh"][so[j]:so[j + 1]], "virial": d["virial"][j],
                     "dipole": d["dipole"][j]})
    g1 = {}
    so1 = np.concatenate([[0], np.cumsum(d["gfn1_nshells"])])
    ao1 = np.concatenate([[0], np.cumsum(nat[d["gfn1_index"]])])
    for t, j in enumerate(d["gfn1_index"]):
        a = slice(ao1[t], ao1[t + 1])
        g1[int(j)] = {"energy": d["gfn1_energy"][t], "gradient": d["gfn1_gradient"][a],
                      "qat": d["gfn1_qat"][a], "qsh": d["gfn1_qsh"][so1[t]:so1[t + 1]]}
    return mols, refs, g1


def test_sample_covers_cluster_tridiagonalisation():
    from tblite_gb300.interface import Calculator

    mols, _, _ = _sample()
    nao = [Calculator("GFN2-xTB", z, x).get("orbital-map").size for z, x in mols]
    assert sum(n >= 288 for n in nao) >= 10 and sum(157 <= n < 288 for n in nao) >= 10
    waters = sum(int(np.all(np.isin(z, (1, 8)))) for z, _ in mols)
    assert 0 < waters < len(mols)


def test_ensemble_sample_batched_gfn2():
    from tblite_gb300.interface import Calculator, batch_fallbacks, batch_singlepoint

    mols, refs, _ = _sample()
    res = batch_singlepoint([Calculator("GFN2-xTB", z, x) for z, x in mols])
    assert batch_fallbacks() == 0  # every molecule stayed on the batched kernels
    for r, ref in zip(res, refs):
        _check(r, ref, energies=False)


def test_ensemble_sample_batched_gfn1():
    from tblite_gb300.interface import Calculator, batch_fallbacks, batch_singlepoint

    mols, _, g1 = _sample()
    pick = sorted(g1)
    res = batch_singlepoint([Calculator("GFN1-xTB", *mols[j]) for j in pick])
    assert batch_fallbacks() == 0
    for r, j in zip(res, pick):
        _check(r, g1[j], energies=False)


def test_ensemble_sample_plain_path():
    from tblite_gb300.interface import Calculator

    mols, refs, _ = _sample()
    for j in (0, 5, 17, 29, 39):
        _check(Calculator("GFN2-xTB", *mols[j]).singlepoint(), refs[j], energies=False)
