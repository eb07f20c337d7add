"""Generate the implicit-solvation tables (ALPB + CDS + shift, GFN2, water) used by this package.

ALPB(water) is defined by its parameter tables, so a drop-in engine must use the very same
numbers.  This script reads them from the reference sources and writes

* ``solvation_water.json`` next to this file (read by the CPU oracle), and
* ``../csrc/params_solv.inc`` (compiled into the CUDA/C++ library).

Sources read (reference repository, read only):

* ``src/tblite/solvation/data.f90:75-100``   D3 van-der-Waals radii (Angstrom)
* ``src/tblite/solvation/data/alpb/param_alpb_water.fh``  gfn2: epsilon, Born scale, offset,
  descreening per element
* ``src/tblite/solvation/data/cds/param_alpb_water.fh``   gfn2: probe radius, surface
  tension scale and sqrt(H-bond strength) per element
* ``src/tblite/solvation/data/shift/param_alpb_water.fh`` gfn2: solvent molar mass, density,
  free-energy shift
* ``src/tblite/mesh/lebedev.f90:544-579``    generator parameters of the 230-point Lebedev
  grid (orbit types and their a, b, weight values)
* ``src/tblite/solvation/data.f90:103-130``  COSMO van-der-Waals radii (Angstrom; the
  ``cosmostub`` entries 2.223) of the generalized Born model with a dielectric constant
* ``src/tblite/solvation/data/{alpb,cds,shift}/param_gbsa_water.fh`` gfn2: the GBSA(water)
  counterparts of the three ALPB tables above

Unit conversions use the CODATA 2018 constants (Bohr radius 0.529177210903 Angstrom,
Hartree 2625.4996394799 kJ/mol, 1 kcal = 4.184 kJ), the values of the reference's mctc-lib.

Usage::

    python tblite_gb300/data/extract_solvation.py REFERENCE_ROOT
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
AATOAU = 1.0 / 0.529177210903
KCALTOAU = 4.184 / 2625.4996394799


def _numbers(text: str) -> list[float]:
    return [float(x.replace("_wp", "").replace("d", "e").replace("D", "e"))
            for x in re.findall(r"[-+]?\d+\.\d*(?:[eEdD][-+]?\d+)?_wp", text)]


def _block(text: str, name: str) -> str:
    start = text.index(name)
    end = text.find("type(", start + len(name))
    return text[start:end if end > 0 else len(text)]


def extract(root: Path) -> dict:
    sol = root / "src" / "tblite" / "solvation"
    data = (sol / "data.f90").read_text()
    i0 = data.index("vdw_rad_d3(1:94)")
    i1 = data.index("]", i0)
    rvdw = [v * AATOAU for v in _numbers(data[i0:i1])]
    assert len(rvdw) == 94
    alpb = _numbers(_block((sol / "data" / "alpb" / "param_alpb_water.fh").read_text(),
                           "gfn2_alpb_water"))
    assert len(alpb) == 3 + 94
    cds = _numbers(_block((sol / "data" / "cds" / "param_alpb_water.fh").read_text(),
                          "gfn2_alpb_water"))
    assert len(cds) == 1 + 2 * 94
    shift = _numbers(_block((sol / "data" / "shift" / "param_alpb_water.fh").read_text(),
                            "gfn2_alpb_water"))
    assert len(shift) == 3
    gbsa = _numbers(_block((sol / "data" / "alpb" / "param_gbsa_water.fh").read_text(),
                           "gfn2_water"))
    assert len(gbsa) == 3 + 94
    gcds = _numbers(_block((sol / "data" / "cds" / "param_gbsa_water.fh").read_text(),
                           "gfn2_water"))
    assert len(gcds) == 1 + 2 * 94
    gshift = _numbers(_block((sol / "data" / "shift" / "param_gbsa_water.fh").read_text(),
                             "gfn2_water"))
    assert len(gshift) == 3
    k0 = data.index("cosmostub =")
    stub = _numbers(data[k0:data.index("\n", k0)])[0]
    c0 = data.index("vdw_rad_cosmo(1:94)")
    c1 = data.index("]", c0)
    cosmo = []
    for tok in re.findall(r"cosmostub|[-+]?\d+\.\d*_wp", data[c0 + len("vdw_rad_cosmo(1:94)"):c1]):
        cosmo.append((stub if tok == "cosmostub" else float(tok.replace("_wp", ""))) * AATOAU)
    assert len(cosmo) == 94
    leb = (root / "src" / "tblite" / "mesh" / "lebedev.f90").read_text()
    j0 = leb.index("pure subroutine ld0230")
    j1 = leb.index("end subroutine ld0230")
    orbits = []
    cur = {}
    for line in leb[j0:j1].splitlines():
        m = re.match(r"\s*([abv])\s*=\s*(\S+)_wp", line)
        if m:
            cur[m.group(1)] = float(m.group(2))
            continue
        m = re.match(r"\s*call gen_oh(\d)", line)
        if m:
            orbits.append({"type": int(m.group(1)), "a": cur.get("a", 0.0), "b": cur.get("b", 0.0),
                           "v": cur["v"]})
    return {
        "source": "tblite solvation data, gfn2 / ALPB and GBSA / water, COSMO radii",
        "rvdw_d3": rvdw,
        "alpb": {"epsv": alpb[0], "c1": alpb[1], "soset": alpb[2], "sx": alpb[3:]},
        "cds": {"rprobe": cds[0], "gamscale": cds[1:95], "sqrtghbond": cds[95:]},
        "shift": {"smass": shift[0], "rhos": shift[1], "gshift": shift[2]},
        "gbsa": {"epsv": gbsa[0], "c1": gbsa[1], "soset": gbsa[2], "sx": gbsa[3:]},
        "gbsa_cds": {"rprobe": gcds[0], "gamscale": gcds[1:95], "sqrtghbond": gcds[95:]},
        "gbsa_shift": {"smass": gshift[0], "rhos": gshift[1], "gshift": gshift[2]},
        "rvdw_cosmo": cosmo,
        "lebedev230": orbits,
        "constants": {"aatoau": AATOAU, "kcaltoau": KCALTOAU},
    }


def write_inc(d: dict, path: Path) -> None:
    def arr(name, vals):
        body = ",\n  ".join(", ".join(repr(float(v)) for v in vals[i:i + 4])
                            for i in range(0, len(vals), 4))
        return f"static const double {name}[{len(vals)}] = {{\n  {body}}};\n"

    out = ["// Generated by tblite_gb300/data/extract_solvation.py from the reference's solvation",
           "// tables (gfn2, ALPB and GBSA, water; COSMO radii) and its 230-point Lebedev",
           "// generator.  Do not edit.",
           "#pragma once",
           f"static const double SOLV_AATOAU = {AATOAU!r};",
           f"static const double SOLV_KCALTOAU = {KCALTOAU!r};",
           f"static const double ALPB_WATER_EPSV = {d['alpb']['epsv']!r};",
           f"static const double ALPB_WATER_C1 = {d['alpb']['c1']!r};",
           f"static const double ALPB_WATER_SOSET = {d['alpb']['soset']!r};",
           f"static const double CDS_WATER_RPROBE = {d['cds']['rprobe']!r};",
           f"static const double SHIFT_WATER_SMASS = {d['shift']['smass']!r};",
           f"static const double SHIFT_WATER_RHOS = {d['shift']['rhos']!r};",
           f"static const double SHIFT_WATER_GSHIFT = {d['shift']['gshift']!r};",
           arr("SOLV_RVDW_D3", d["rvdw_d3"]),
           arr("ALPB_WATER_SX", d["alpb"]["sx"]),
           arr("CDS_WATER_GAMSCALE", d["cds"]["gamscale"]),
           arr("CDS_WATER_SQRTGHB", d["cds"]["sqrtghbond"]),
           f"static const double GBSA_WATER_EPSV = {d['gbsa']['epsv']!r};",
           f"static const double GBSA_WATER_C1 = {d['gbsa']['c1']!r};",
           f"static const double GBSA_WATER_SOSET = {d['gbsa']['soset']!r};",
           f"static const double CDS_GBSA_WATER_RPROBE = {d['gbsa_cds']['rprobe']!r};",
           f"static const double SHIFT_GBSA_WATER_SMASS = {d['gbsa_shift']['smass']!r};",
           f"static const double SHIFT_GBSA_WATER_RHOS = {d['gbsa_shift']['rhos']!r};",
           f"static const double SHIFT_GBSA_WATER_GSHIFT = {d['gbsa_shift']['gshift']!r};",
           arr("GBSA_WATER_SX", d["gbsa"]["sx"]),
           arr("CDS_GBSA_WATER_GAMSCALE", d["gbsa_cds"]["gamscale"]),
           arr("CDS_GBSA_WATER_SQRTGHB", d["gbsa_cds"]["sqrtghbond"]),
           arr("SOLV_RVDW_COSMO", d["rvdw_cosmo"])]
    orb = d["lebedev230"]
    out.append(f"static const int LEB230_NORB = {len(orb)};")
    out.append("static const int LEB230_TYPE[] = {" + ", ".join(str(o["type"]) for o in orb) + "};")
    out.append(arr("LEB230_A", [o["a"] for o in orb]))
    out.append(arr("LEB230_B", [o["b"] for o in orb]))
    out.append(arr("LEB230_V", [o["v"] for o in orb]))
    path.write_text("\n".join(out) + "\n")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        raise SystemExit(f"usage: python {Path(__file__).name} <tblite source tree>")
    root = Path(sys.argv[1])
    d = extract(root)
    (HERE / "solvation_water.json").write_text(json.dumps(d, indent=1))
    write_inc(d, HERE.parent / "csrc" / "params_solv.inc")
    print("lebedev orbits", [o["type"] for o in d["lebedev230"]])
