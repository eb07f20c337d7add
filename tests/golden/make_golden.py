"""Extract golden vectors from the reference's own unit tests.

Reads ``test/unit/test_gfn2_xtb.f90``, ``test/unit/test_gfn1_xtb.f90`` and
``test/unit/test_ipea1_xtb.f90`` of the reference repository (as text; nothing is compiled or
run) and writes ``atoms_gfn2.json`` / ``atoms_gfn1.json`` / ``atoms_ipea1.json`` next to this
file: total energies of isolated atoms Z = 1..86 for the neutral, cation and anion cases, with
the unpaired-electron counts the reference uses, the accuracy (0.01) and the tolerance of that
test (reference ``test/unit/test_gfn2_xtb.f90:34-36,61-272``,
``test/unit/test_gfn1_xtb.f90:135-349``, ``test/unit/test_ipea1_xtb.f90:33-36,133-347``).

Isolated atoms need no coordination-number or dispersion data, so these
energies pin the basis, the on-site integrals, the self energies, the
shell-resolved Coulomb / third-order terms, Fermi smearing, the entropy term
and the Broyden-mixed SCF of the oracle and of the CUDA engine.

Usage: ``python tests/golden/make_golden.py REFERENCE_ROOT``
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path


def _array(block: str, name: str):
    m = re.search(name + r"\(86\) = \[(.*?)\]", block, re.S)
    body = re.sub(r"[&\s]", "", m.group(1))
    return [v.replace("_wp", "") for v in body.split(",")]


def main():
    if len(sys.argv) < 2:
        raise SystemExit(f"usage: python {Path(__file__).name} <tblite source tree>")
    root = Path(sys.argv[1])
    for method, src in (("gfn2", "test/unit/test_gfn2_xtb.f90:61-272"),
                        ("gfn1", "test/unit/test_gfn1_xtb.f90:135-349"),
                        ("ipea1", "test/unit/test_ipea1_xtb.f90:133-347")):
        extract(root, method, src)


def extract(root: Path, method: str, src: str):
    text = (root / f"test/unit/test_{method}_xtb.f90").read_text()
    out = {"source": "reference " + src, "accuracy": 0.01,
           "kt": 300.0 * 3.166808578545117e-06,
           # thresholds of the reference tests: 10 sqrt(eps) (gfn2), sqrt(eps) (gfn1, ipea1)
           "thr": (10.0 if method == "gfn2" else 1.0) * (2.220446049250313e-16) ** 0.5,
           "cases": {}}
    for key, sub, charge in (("neutral", "test_e_pse(", 0), ("cation", "test_e_pse_cation(", 1),
                             ("anion", "test_e_pse_anion(", -1)):
        i = text.index("subroutine " + sub)
        j = text.index("end subroutine", i)
        block = text[i:j]
        uhf = [int(v) for v in _array(block, "uhf")]
        ref = [float(v) for v in _array(block, "ref")]
        skip = []
        m = re.search(r"if \(any\(izp == \[([\d, ]+)\]\)\) cycle", block)
        if m:
            skip = [int(v) for v in m.group(1).split(",")]
        m = re.search(r"if \(izp == (\d+)\) cycle", block)
        if m:
            skip.append(int(m.group(1)))
        out["cases"][key] = {"charge": charge, "uhf": uhf, "energy": ref, "skip": skip}
    dst = Path(__file__).resolve().parent / f"atoms_{method}.json"
    dst.write_text(json.dumps(out, indent=1))
    print("wrote", dst)


if __name__ == "__main__":
    main()
