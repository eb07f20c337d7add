"""One batched energy + gradient call over the seeded mixed ensemble.

    python -m tblite_gb300.ensemble_run [--molecules 512] [--method GFN2-xTB] [--calls 1]
                                        [--tridiag-ctas 1]

The molecules are ``workloads.mixed_ensemble(count, seed=4)`` (50 % water clusters, 50 %
alkanes, 3-192 atoms).  Each call goes through ``tblite_gb300_batch_singlepoint``; the script
prints the number of molecules, the fallbacks to the one-molecule path and the energy sum.  It is
the fixed command behind the kernel profiles of the batched path.
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--molecules", type=int, default=512)
    ap.add_argument("--method", default="GFN2-xTB", choices=["GFN2-xTB", "GFN1-xTB"])
    ap.add_argument("--calls", type=int, default=1)
    ap.add_argument("--tridiag-ctas", type=int, default=0,
                    help="CTAs per SM of the batched tridiagonalisation (0: library default)")
    args = ap.parse_args(argv)
    root = Path(__file__).resolve().parents[1]
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))
    from tblite_gb300 import _build, library, workloads
    from tblite_gb300.interface import Calculator, batch_fallbacks, batch_singlepoint

    _build.build()
    if args.tridiag_ctas:
        library.set_tridiag_ctas_per_sm(args.tridiag_ctas)
    mols = workloads.mixed_ensemble(args.molecules, seed=4)
    calcs = [Calculator(args.method, z, x) for z, x in mols]
    for _ in range(args.calls):
        res = batch_singlepoint(calcs)
        print(f"molecules {len(res)} fallbacks {batch_fallbacks()} "
              f"energy_sum {sum(r.get('energy') for r in res):.10f} "
              f"device_ms {library.load().tblite_gb300_batch_last_device_ms():.1f}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
