"""Compile an element-data pack (JSON) into ``../csrc/element_data.inc``.

The element-data pack carries the per-element numbers that GFN2-xTB takes from
libraries outside the reference tree (mctc-lib covalent radii, Pauling
electronegativities, atomic radii and the coordination-number constants).
Elements absent from the pack are stored as NaN; the library rejects molecules
that need them with an error naming the element.

Usage: ``python tblite_gb300/data/gen_element_data.py [PACK.json]``
(default: ``element_data_synthetic.json``).
"""
import json
import math
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def table(d):
    out = [math.nan] * 86
    for k, v in d.items():
        out[int(k) - 1] = float(v)
    return out


def fmt(name, vals):
    body = ", ".join("NAN" if math.isnan(v) else repr(v) for v in vals)
    return f"static const double {name}[86] = {{{body}}};\n"


def main():
    src = Path(sys.argv[1]) if len(sys.argv) > 1 else HERE / "element_data_synthetic.json"
    pack = json.loads(src.read_text())
    cn = pack["cn"]
    lines = ["// Generated by tblite_gb300/data/gen_element_data.py -- do not edit.\n",
             f"// pack: {pack['name']}\n", "#pragma once\n#include <cmath>\n",
             f'static const char* const EXT_PACK_NAME = "{pack["name"]}";\n',
             f"static const double EXT_CN_KA = {cn['ka']!r};\n",
             f"static const double EXT_CN_KB = {cn['kb']!r};\n",
             f"static const double EXT_CN_RSHIFT = {cn['rshift']!r};\n",
             f"static const double EXT_CN_CUTOFF = {cn['cutoff']!r};\n",
             fmt("EXT_RCOV", table(cn["rcov"])), fmt("EXT_EN", table(pack["pauling_en"])),
             fmt("EXT_RAD", table(pack["atomic_rad"]))]
    (HERE.parent / "csrc" / "element_data.inc").write_text("".join(lines))
    print("wrote element_data.inc from", src.name)


if __name__ == "__main__":
    main()
