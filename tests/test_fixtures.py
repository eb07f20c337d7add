"""The committed oracle fixtures of the configuration parity tests (CPU).

``golden/ensemble_sample.npz`` and ``golden/c200h402.npz`` are written by
``golden/make_parity_fixtures.py``; here the stored geometries are checked against the workload
generators, and the oracle is re-run on the smallest sampled molecules to confirm the stored
results.
"""
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_sample_geometries_come_from_the_ensemble():
    import importlib.util

    from tblite_gb300 import workloads

    spec = importlib.util.spec_from_file_location("mk", GOLDEN / "make_parity_fixtures.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    d = np.load(GOLDEN / "ensemble_sample.npz")
    mols = workloads.mixed_ensemble(4096, seed=mk.ENSEMBLE_SEED)
    assert np.array_equal(mk.ensemble_sample_indices(mols), d["index"])
    off = np.concatenate([[0], np.cumsum(d["natoms"])])
    for j, i in enumerate(d["index"]):
        z, x = mols[i]
        assert np.array_equal(d["numbers"][off[j]:off[j + 1]], z)
        assert np.array_equal(d["positions"][off[j]:off[j + 1]], x)
    z, x = workloads.config("c200h402")
    c = np.load(GOLDEN / "c200h402.npz")
    assert np.array_equal(c["numbers"], z) and np.array_equal(c["positions"], x)


def test_stored_results_reproduce():
    from oracle import gfn1, gfn2

    d = np.load(GOLDEN / "ensemble_sample.npz")
    off = np.concatenate([[0], np.cumsum(d["natoms"])])
    soff = np.concatenate([[0], np.cumsum(d["nshells"])])
    small = np.argsort(d["natoms"])[:3]
    for j in small:
        z, x = d["numbers"][off[j]:off[j + 1]], d["positions"][off[j]:off[j + 1]]
        r = gfn2.singlepoint(gfn2.new_calc(gfn2.Molecule(z, x)), grad=True)
        assert abs(r.energy - d["energy"][j]) < 1e-9
        assert np.max(np.abs(r.gradient - d["gradient"][off[j]:off[j + 1]])) < 1e-9
        assert np.max(np.abs(r.qsh - d["qsh"][soff[j]:soff[j + 1]])) < 1e-9
    t = int(np.argmin(d["natoms"][d["gfn1_index"]]))
    j = int(d["gfn1_index"][t])
    z, x = d["numbers"][off[j]:off[j + 1]], d["positions"][off[j]:off[j + 1]]
    r1 = gfn1.singlepoint(gfn1.new_calc(gfn2.Molecule(z, x)))
    assert abs(r1.energy - d["gfn1_energy"][t]) < 1e-9
