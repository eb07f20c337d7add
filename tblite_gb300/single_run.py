"""Plain-path single points (energy + gradient) of a named workload.

    python -m tblite_gb300.single_run [--geometry h2o1000] [--solvent] [--solver purification]
                                      [--calls 1]

The geometry is ``workloads.config(name)``; ``--solvent`` adds ALPB(water), ``--solver`` picks
the density solver.  Each call goes through ``tblite_get_singlepoint`` and prints the energy and
the SCF iterations.  It is the fixed command behind the kernel profiles of the plain path.
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--geometry", default="h2o1000")
    ap.add_argument("--solvent", action="store_true")
    ap.add_argument("--solver", default="diagonalization",
                    choices=["diagonalization", "purification"])
    ap.add_argument("--method", default="GFN2-xTB", choices=["GFN2-xTB", "GFN1-xTB"])
    ap.add_argument("--calls", type=int, default=1)
    args = ap.parse_args(argv)
    root = Path(__file__).resolve().parents[1]
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))
    from tblite_gb300 import _build, library, workloads
    from tblite_gb300.interface import Calculator

    _build.build()
    z, x = workloads.config(args.geometry)
    calc = Calculator(args.method, z, x)
    if args.solvent:
        calc.add("alpb-solvation", "water")
    calc.set("density-solver", args.solver)
    library.set_profiling(True)
    for _ in range(args.calls):
        res = calc.singlepoint()
        prof = library.get_profile()
        print(f"atoms {len(z)} energy {res.get('energy'):.10f} "
              f"iterations {prof['iterations']}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
