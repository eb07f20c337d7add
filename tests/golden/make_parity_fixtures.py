"""Oracle results for the parity tests of the one-molecule C200H402 configuration and of a
sample of the 4096-molecule benchmark ensemble.

Writes next to this file:

* ``c200h402.npz``: the CPU oracle (``oracle.gfn2``, default settings: accuracy 1, 300 K) on
  ``workloads.config("c200h402")`` (602 atoms, 1202 AOs): total and atomic energies, gradient,
  virial, shell and atomic charges, dipole, SCF iterations, positions.
* ``ensemble_sample.npz``: 40 molecules of ``workloads.mixed_ensemble(4096, seed=4)``, drawn
  with ``numpy.random.default_rng(2024)``: 16 uniformly from the whole ensemble and 24 from its
  molecules with at least 157 orbitals (those the batched path tridiagonalises in a thread-block
  cluster; 12 of them with at least 288), so both molecule kinds and every size class appear.
  For each, the geometry and the GFN2 oracle results (energy, gradient, virial, shell and
  atomic charges, dipole); for every fourth molecule also the GFN1 oracle results.  Ragged
  per-molecule arrays are concatenated with offsets.

The geometries are stored, so the tests do not depend on the random generator of the numpy
version that runs them.

Usage: ``python tests/golden/make_parity_fixtures.py`` (about a minute on 8 cores).
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ENSEMBLE_SEED, SAMPLE_SEED = 4, 2024
N_UNIFORM, N_LARGE, N_XLARGE = 16, 12, 12


def ensemble_sample_indices(mols):
    """Indices of the stratified sample (see the module docstring)."""
    nao = np.array([sum({1: 1, 6: 4, 8: 4}[int(q)] for q in z) for z, _ in mols])
    rng = np.random.default_rng(SAMPLE_SEED)
    uni = rng.choice(len(mols), N_UNIFORM, replace=False)
    large = np.flatnonzero((nao >= 157) & (nao < 288))
    xlarge = np.flatnonzero(nao >= 288)
    pick = np.concatenate([uni, rng.choice(large, N_LARGE, replace=False),
                           rng.choice(xlarge, N_XLARGE, replace=False)])
    _, first = np.unique(pick, return_index=True)
    return pick[np.sort(first)]


def _result_arrays(res):
    return dict(energy=res.energy, energies=res.energies, gradient=res.gradient, virial=res.sigma,
                qsh=res.qsh, qat=res.qat, dipole=res.parts["dipole"], iterations=res.iterations)


def main():
    root = HERE.parents[1]
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))
    from oracle import gfn1, gfn2
    from oracle.build import build_oracle
    from tblite_gb300 import workloads

    build_oracle()
    t0 = time.perf_counter()
    z, x = workloads.config("c200h402")
    res = gfn2.singlepoint(gfn2.new_calc(gfn2.Molecule(np.asarray(z), np.asarray(x))), grad=True)
    np.savez_compressed(HERE / "c200h402.npz", numbers=np.asarray(z), positions=np.asarray(x),
                        **_result_arrays(res))
    print(f"c200h402 energy {res.energy:.12f} iterations {res.iterations} "
          f"({time.perf_counter() - t0:.1f} s)")

    mols = workloads.mixed_ensemble(4096, seed=ENSEMBLE_SEED)
    idx = ensemble_sample_indices(mols)
    out = {"index": idx, "natoms": np.array([len(mols[i][0]) for i in idx])}
    cols = {k: [] for k in ("numbers", "positions", "energy", "gradient", "virial", "qsh",
                            "qat", "dipole", "nshells")}
    g1 = {k: [] for k in ("index", "energy", "gradient", "qsh", "qat", "nshells")}
    for j, i in enumerate(idx):
        z, x = np.asarray(mols[i][0]), np.asarray(mols[i][1])
        r = gfn2.singlepoint(gfn2.new_calc(gfn2.Molecule(z, x)), grad=True)
        cols["numbers"].append(z)
        cols["positions"].append(x)
        cols["energy"].append(r.energy)
        cols["gradient"].append(r.gradient)
        cols["virial"].append(r.sigma)
        cols["qsh"].append(r.qsh)
        cols["qat"].append(r.qat)
        cols["dipole"].append(r.parts["dipole"])
        cols["nshells"].append(len(r.qsh))
        if j % 4 == 0:
            r1 = gfn1.singlepoint(gfn1.new_calc(gfn2.Molecule(z, x)))
            g1["index"].append(j)
            g1["energy"].append(r1.energy)
            g1["gradient"].append(r1.gradient)
            g1["qsh"].append(r1.qsh)
            g1["qat"].append(r1.qat)
            g1["nshells"].append(len(r1.qsh))
    for k in ("numbers", "positions", "gradient", "qsh", "qat"):
        out[k] = np.concatenate(cols[k])
    for k in ("energy", "virial", "dipole", "nshells"):
        out[k] = np.array(cols[k])
    for k, v in g1.items():
        out["gfn1_" + k] = (np.array(v) if k in ("index", "energy", "nshells")
                            else np.concatenate(v))
    np.savez_compressed(HERE / "ensemble_sample.npz", **out)
    print(f"ensemble sample: {len(idx)} molecules, {int(out['natoms'].sum())} atoms, "
          f"{len(g1['index'])} with GFN1 ({time.perf_counter() - t0:.1f} s)")


if __name__ == "__main__":
    main()
