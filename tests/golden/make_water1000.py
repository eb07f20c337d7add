"""Oracle result for the 1000-water cluster with ALPB(water) solvation (3000 atoms, 6000 AOs).

Runs the CPU oracle (``oracle.gfn2`` with ``oracle.solvation.ALPBWater``, default settings:
accuracy 1, 300 K) on ``workloads.config("h2o1000")`` and writes ``water1000_alpb.npz`` next
to this file: total energy, atomic charges, gradient, SCF iterations and the HOMO/LUMO of the
final Fock matrix.  The oracle diagonalises a 6000 x 6000 generalised eigenproblem per SCF
iteration, so the run takes tens of minutes; the GPU tests read the fixture instead.

Usage: ``python tests/golden/make_water1000.py``
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def main():
    root = HERE.parents[1]
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))
    from oracle import gfn2
    from oracle.solvation import ALPBWater
    from tblite_gb300 import workloads

    z, x = workloads.config("h2o1000")
    t0 = time.perf_counter()
    calc = gfn2.new_calc(gfn2.Molecule(np.asarray(z), np.asarray(x, dtype=float)))
    res = gfn2.singlepoint(calc, grad=True, solvation=ALPBWater(z), verbose=True)
    nocc = int(round(float(np.sum(res.focc)) / 2))
    np.savez_compressed(HERE / "water1000_alpb.npz", energy=res.energy, charges=res.qat,
                        gradient=res.gradient, iterations=res.iterations,
                        homo=res.emo[nocc - 1], lumo=res.emo[nocc])
    print(f"energy {res.energy:.12f} iterations {res.iterations} "
          f"gap {res.emo[nocc] - res.emo[nocc - 1]:.6f} time {time.perf_counter() - t0:.0f} s")


if __name__ == "__main__":
    main()
