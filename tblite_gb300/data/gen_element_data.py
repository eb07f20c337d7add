"""Compile an element-data pack (JSON) into ``../csrc/element_data.inc``.

The element-data pack carries the per-element numbers that GFN2-xTB and GFN1-xTB take
from libraries outside the reference tree: mctc-lib covalent radii, Pauling
electronegativities, atomic radii and coordination-number constants (double-exponential
and exponential counting functions), the D3 model constants, and the
dftd4 model data (reference coordination numbers and charges, Gaussian weight
counts, reference C6 values, effective charges, hardnesses, <r4>/<r2> ratios).
Elements absent from the pack are stored as NaN (nref = 0); the library rejects
molecules that need them with an error naming the element.

Reference C6 values come per element pair (the pack's d4.c6["Za-Zb"], Za <= Zb, an
nref(Za) x nref(Zb) matrix): EXT_D4_C6OFF[(Za-1)*86 + Zb-1] is the offset of that matrix
(row-major) in EXT_D4_C6PAIR, -1 when the pack has no entry for the pair.

Usage: ``python tblite_gb300/data/gen_element_data.py [PACK.json]``
(default: ``element_data_synthetic.json``).
"""
import json
import math
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
MREF = 7


def table(d, default=math.nan):
    out = [default] * 86
    for k, v in d.items():
        out[int(k) - 1] = float(v)
    return out


def fmt(name, vals, ctype="double"):
    if ctype == "int":
        body = ", ".join(str(int(v)) for v in vals)
    else:
        body = ", ".join("NAN" if math.isnan(v) else repr(float(v)) for v in vals)
    return f"static const {ctype} {name}[{len(vals)}] = {{{body}}};\n"


def main():
    src = Path(sys.argv[1]) if len(sys.argv) > 1 else HERE / "element_data_synthetic.json"
    pack = json.loads(src.read_text())
    cn = pack["cn"]
    d4 = pack["d4"]
    lines = ["// Generated by tblite_gb300/data/gen_element_data.py -- do not edit.\n",
             f"// pack: {pack['name']}\n", "#pragma once\n#include <cmath>\n",
             f'static const char* const EXT_PACK_NAME = "{pack["name"]}";\n',
             f"static const double EXT_CN_KA = {cn['ka']!r};\n",
             f"static const double EXT_CN_KB = {cn['kb']!r};\n",
             f"static const double EXT_CN_RSHIFT = {cn['rshift']!r};\n",
             f"static const double EXT_CN_CUTOFF = {cn['cutoff']!r};\n",
             fmt("EXT_RCOV", table(cn["rcov"])), fmt("EXT_EN", table(pack["pauling_en"])),
             fmt("EXT_RAD", table(pack["atomic_rad"])),
             f"static const int EXT_D4_MREF = {MREF};\n"]
    for key in ("ga", "gc", "wf", "cn_kn", "cn_k4", "cn_k5", "cn_k6", "cn_cutoff", "disp2_cutoff",
                "disp3_cutoff", "atm_alpha", "width2", "width3"):
        lines.append(f"static const double EXT_D4_{key.upper()} = {float(d4.get(key, 0.0))!r};\n")
    nref = [0] * 86
    refcn = [0.0] * (86 * MREF)
    refq = [0.0] * (86 * MREF)
    ngw = [0] * (86 * MREF)
    for k, v in d4["refcn"].items():
        z = int(k) - 1
        nref[z] = len(v)
        for r in range(len(v)):
            refcn[z * MREF + r] = v[r]
            refq[z * MREF + r] = d4["refq"][k][r]
            ngw[z * MREF + r] = d4["ngw"][k][r]
    c6off = [-1] * (86 * 86)
    c6pair = []
    for key, mat in sorted(d4["c6"].items(), key=lambda kv: tuple(map(int, kv[0].split("-")))):
        za, zb = map(int, key.split("-"))
        if za > zb or len(mat) != nref[za - 1] or any(len(row) != nref[zb - 1] for row in mat):
            raise SystemExit(f"pack: C6 pair {key} does not match the reference counts")
        c6off[(za - 1) * 86 + zb - 1] = len(c6pair)
        c6pair += [float(x) for row in mat for x in row]
    lines += [fmt("EXT_D4_NREF", nref, "int"), fmt("EXT_D4_REFCN", refcn), fmt("EXT_D4_REFQ", refq),
              fmt("EXT_D4_NGW", ngw, "int"), fmt("EXT_D4_C6OFF", c6off, "int"),
              fmt("EXT_D4_C6PAIR", c6pair or [0.0]),
              fmt("EXT_D4_ZEFF", table(d4["zeff"])), fmt("EXT_D4_GAM", table(d4["gam"])),
              fmt("EXT_D4_R4R2", table(d4["r4r2"])), fmt("EXT_D4_RCOV", table(d4["rcov"])),
              fmt("EXT_D4_EN", table(d4["en"]))]
    cx = pack["cn_exp"]
    lines += [f"static const double EXT_CNEXP_K = {float(cx['k'])!r};\n",
              f"static const double EXT_CNEXP_CUTOFF = {float(cx['cutoff'])!r};\n"]
    d3 = pack["d3"]
    for key in ("k1", "k3", "cn_cutoff", "disp2_cutoff"):
        lines.append(f"static const double EXT_D3_{key.upper()} = {float(d3[key])!r};\n")
    (HERE.parent / "csrc" / "element_data.inc").write_text("".join(lines))
    print("wrote element_data.inc from", src.name)


if __name__ == "__main__":
    main()
