"""Generate the GFN2-xTB / STO-nG parameter tables used by this package.

The GFN2-xTB method is defined by its parameter tables; a drop-in engine
must use the very same numbers.  This script reads the Fortran parameter
declarations of the reference sources and writes them out as

* ``gfn2.json`` / ``sto_ng.json`` next to this file (read by the CPU oracle
  and the Python layer), and
* ``../csrc/params_gfn2.inc`` (compiled into the CUDA/C++ library).

Sources read (reference repository, read only):

* ``src/tblite/xtb/gfn2.f90:47-543``  (element tables, global constants)
* ``src/tblite/basis/slater.f90:44-376`` (STO-nG exponents/coefficients,
  R. F. Stewart, J. Chem. Phys. 52, 431 (1970))

The arithmetic in the declarations (``0.1_wp * [...]``, ``reshape(...) *
evtoau`` ...) is evaluated element by element in IEEE double precision,
which reproduces the compile-time folding of the reference bit for bit.

Usage::

    python tblite_gb300/data/extract_params.py REFERENCE_ROOT

It is only needed when regenerating the committed outputs.
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _declarations(text: str) -> dict[str, tuple[str, str]]:
    """Return {name: (dims, expression)} for every ``parameter`` declaration."""
    # strip comments and join continuation lines
    lines = []
    for raw in text.splitlines():
        line = raw.split("!")[0].rstrip()
        lines.append(line)
    joined = []
    buf = ""
    for line in lines:
        s = line.strip()
        if not s:
            continue
        if s.startswith("&"):
            s = s[1:]
        if buf.endswith("&"):
            buf = buf[:-1] + " " + s
        else:
            if buf:
                joined.append(buf)
            buf = s
    if buf:
        joined.append(buf)
    out = {}
    pat = re.compile(r"^(real\(wp\)|integer)\s*,\s*parameter\s*::\s*(.*)$", re.I)
    for stmt in joined:
        m = pat.match(stmt)
        if not m:
            continue
        body = m.group(2)
        # a statement may declare several scalars: a = 1.0_wp, b = 2.0_wp
        parts = _split_top(body)
        for part in parts:
            if "=" not in part:
                continue
            lhs, rhs = part.split("=", 1)
            lhs = lhs.strip()
            mm = re.match(r"(\w+)\s*(\((.*)\))?", lhs)
            out[mm.group(1)] = (mm.group(3) or "", rhs.strip())
    return out


def _split_top(s: str) -> list[str]:
    depth = 0
    parts, cur = [], ""
    for ch in s:
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return parts


def _to_python(expr: str) -> str:
    e = expr.replace("_wp", "")
    e = re.sub(r"reshape\s*\(", "_reshape(", e)
    e = re.sub(r"shape\s*\(\s*(\w+)\s*\)", r"'\1'", e)
    e = re.sub(r"spread\s*\(\s*([^,]+),\s*1\s*,\s*(\d+)\s*\)", r"*np.full(\2, \1)", e)
    e = e.replace("[", "np.array([").replace("]", "], dtype=float)")
    return e


def _reshape(arr, _name):
    return np.asarray(arr, dtype=float)


def evaluate(decls, names, env=None):
    env = dict(env or {})
    env.update(np=np, _reshape=_reshape, sqrt=np.sqrt)
    vals = {}
    for name in names:
        dims, expr = decls[name]
        val = eval(_to_python(expr), env)  # noqa: S307 - trusted local transform
        env[name] = val
        vals[name] = val
    return vals


def extract(root: Path):
    gfn2 = (root / "src/tblite/xtb/gfn2.f90").read_text()
    slater = (root / "src/tblite/basis/slater.f90").read_text()

    d = _declarations(gfn2)
    scalars = ["evtoau", "s6", "s8", "a1", "a2", "s9", "rep_kexp", "rep_kexp_light",
               "rep_rexp", "wexp", "enscale", "gexp", "mp_dmp3", "mp_dmp5", "mp_shift",
               "mp_kexp", "mp_rmax"]
    env = {}
    sc = evaluate(d, scalars, env)
    env.update(sc)
    tables = ["kdiag", "rep_alpha", "rep_zeff", "hubbard_parameter", "shell_hubbard",
              "shell_hubbard_derivs", "p_hubbard_derivs", "nshell", "ang_shell",
              "principal_quantum_number", "number_of_primitives", "p_shpoly", "p_kcn",
              "reference_occ", "slater_exponent", "p_selfenergy", "p_dkernel",
              "p_qkernel", "p_vcn", "p_rad"]
    tv = evaluate(d, tables, env)
    max_elem = 86
    shapes = {
        "shell_hubbard": (3, max_elem), "ang_shell": (3, max_elem),
        "principal_quantum_number": (3, max_elem), "number_of_primitives": (3, max_elem),
        "p_shpoly": (3, max_elem), "p_kcn": (3, max_elem), "reference_occ": (3, max_elem),
        "slater_exponent": (3, max_elem), "p_selfenergy": (3, max_elem),
    }
    out = {"scalars": {k: float(v) for k, v in sc.items()}}
    for name, val in tv.items():
        arr = np.asarray(val, dtype=float)
        if name in shapes:
            rows, cols = shapes[name]
            if arr.size != rows * cols:
                raise ValueError(f"{name}: {arr.size} values for shape {shapes[name]}")
            # Fortran column-major (first index fastest) -> [element][slot]
            arr = arr.reshape((cols, rows))
        if name in ("p_vcn", "p_rad"):
            arr = arr[:max_elem]
        out[name] = arr.tolist()
    # ``kshell`` elemental function (gfn2.f90:1024-1028)
    kdiag = np.asarray(tv["kdiag"])
    ksh = np.zeros((5, 5))
    for k in range(5):
        for ll in range(5):
            if (k == 2 and ll in (0, 1)) or (ll == 2 and k in (0, 1)):
                ksh[k, ll] = 2.0
            else:
                ksh[k, ll] = (kdiag[ll] + kdiag[k]) / 2
    out["kshell"] = ksh.tolist()

    s = _declarations(slater)
    names = ["pAlpha1"] + [f"p{kind}{ng}" for ng in range(2, 7) for kind in ("Alpha", "Coeff")] \
        + ["pAlpha6s", "pCoeff6s", "pAlpha6p", "pCoeff6p"]
    sv = evaluate(s, names)
    sto = {}
    for name, val in sv.items():
        arr = np.asarray(val, dtype=float)
        m = re.match(r"p(Alpha|Coeff)(\d)$", name)
        if m and m.group(2) != "1":
            ng = int(m.group(2))
            arr = arr.reshape((15, ng))  # [ityp][primitive]
        sto[name] = arr.tolist()
    return out, sto


def write_inc(params, sto, path: Path):
    def arr1(name, ctype, vals):
        body = ", ".join(repr(float(v)) if ctype == "double" else str(int(v)) for v in vals)
        return f"static const {ctype} {name}[{len(vals)}] = {{{body}}};\n"

    lines = ["// Generated by tblite_gb300/data/extract_params.py -- do not edit.\n",
             "// GFN2-xTB element tables (reference src/tblite/xtb/gfn2.f90:47-543)\n",
             "// and STO-nG expansions (reference src/tblite/basis/slater.f90:44-376).\n",
             "#pragma once\n"]
    for k, v in params["scalars"].items():
        lines.append(f"static const double GFN2_{k.upper()} = {v!r};\n")
    flat = lambda x: np.asarray(x).ravel().tolist()  # noqa: E731
    for name in ["rep_alpha", "rep_zeff", "hubbard_parameter", "p_hubbard_derivs", "p_dkernel",
                 "p_qkernel", "p_vcn", "p_rad"]:
        lines.append(arr1("GFN2_" + name.upper(), "double", flat(params[name])))
    for name in ["shell_hubbard", "p_shpoly", "p_kcn", "reference_occ", "slater_exponent",
                 "p_selfenergy"]:
        lines.append(f"// [Z-1][slot], slot = shell index or angular momentum\n")
        lines.append(arr1("GFN2_" + name.upper(), "double", flat(params[name])))
    for name in ["ang_shell", "principal_quantum_number", "number_of_primitives"]:
        lines.append(arr1("GFN2_" + name.upper(), "int", flat(params[name])))
    lines.append(arr1("GFN2_NSHELL", "int", flat(params["nshell"])))
    lines.append(arr1("GFN2_SHELL_HUBBARD_DERIVS", "double", flat(params["shell_hubbard_derivs"])))
    lines.append(arr1("GFN2_KSHELL", "double", flat(params["kshell"])))
    lines.append(arr1("STO_ALPHA1", "double", flat(sto["pAlpha1"])))
    for ng in range(2, 7):
        lines.append(arr1(f"STO_ALPHA{ng}", "double", flat(sto[f"pAlpha{ng}"])))
        lines.append(arr1(f"STO_COEFF{ng}", "double", flat(sto[f"pCoeff{ng}"])))
    for nm in ["pAlpha6s", "pCoeff6s", "pAlpha6p", "pCoeff6p"]:
        lines.append(arr1("STO_" + nm[1:].upper(), "double", flat(sto[nm])))
    path.write_text("".join(lines))


def extract_gfn1(root: Path, method: str = "gfn1"):
    """GFN1-xTB tables (reference src/tblite/xtb/gfn1.f90:47-496, kshell at :1056-1060); with
    method="ipea1" the IPEA1-xTB tables of the same form (src/tblite/xtb/ipea1.f90:47-490,
    kshell at :1037-1041; its hardnesses are named chemical_hardness / shell_hardness)."""
    d = _declarations((root / f"src/tblite/xtb/{method}.f90").read_text())
    if method == "ipea1":
        d["hubbard_parameter"] = d["chemical_hardness"]
        d["shell_hubbard"] = d["shell_hardness"]
    scalars = ["evtoau", "s6", "s8", "a1", "a2", "s9", "rep_kexp", "rep_rexp", "gexp",
               "enscale", "kdiff", "halogen_radscale", "halogen_damping"]
    env = {}
    sc = evaluate(d, scalars, env)
    env.update(sc)
    tables = ["kdiag", "rep_alpha", "rep_zeff", "hubbard_parameter", "shell_hubbard",
              "p_hubbard_derivs", "nshell", "ang_shell", "principal_quantum_number",
              "number_of_primitives", "p_shpoly", "reference_occ", "slater_exponent",
              "p_selfenergy", "p_kcn", "halogen_bond"]
    tv = evaluate(d, tables, env)
    max_elem = 86
    shaped = {"shell_hubbard", "ang_shell", "principal_quantum_number", "number_of_primitives",
              "p_shpoly", "reference_occ", "slater_exponent", "p_selfenergy", "p_kcn"}
    out = {"scalars": {k: float(v) for k, v in sc.items()}}
    for name, val in tv.items():
        arr = np.asarray(val, dtype=float)
        if name in shaped:
            if arr.size != 3 * max_elem:
                raise ValueError(f"{name}: {arr.size} values")
            arr = arr.reshape((max_elem, 3))  # [element][slot]
        out[name] = arr.tolist()
    kdiag = np.asarray(tv["kdiag"])
    ksh = np.zeros((3, 3))
    for k in range(3):
        for ll in range(3):
            sp = 2.25 if method == "ipea1" else 2.08
            ksh[k, ll] = sp if (k, ll) in ((0, 1), (1, 0)) else (kdiag[ll] + kdiag[k]) / 2
    out["kshell"] = ksh.tolist()
    return out


def write_inc_gfn1(params, path: Path, prefix: str = "GFN1"):
    def arr1(name, ctype, vals):
        body = ", ".join(repr(float(v)) if ctype == "double" else str(int(v)) for v in vals)
        return f"static const {ctype} {name}[{len(vals)}] = {{{body}}};\n"

    flat = lambda x: np.asarray(x).ravel().tolist()  # noqa: E731
    src = "gfn1.f90:47-496" if prefix == "GFN1" else "ipea1.f90:47-490"
    lines = ["// Generated by tblite_gb300/data/extract_params.py -- do not edit.\n",
             f"// {prefix} element tables (reference src/tblite/xtb/{src}).\n",
             "#pragma once\n"]
    for k, v in params["scalars"].items():
        lines.append(f"static const double {prefix}_{k.upper()} = {v!r};\n")
    for name in ["rep_alpha", "rep_zeff", "hubbard_parameter", "p_hubbard_derivs",
                 "halogen_bond"]:
        lines.append(arr1(prefix + "_" + name.upper(), "double", flat(params[name])))
    lines.append("// [Z-1][slot]: slot = shell index (selfenergy, kcn, slater, ang, pqn, ngauss)\n")
    lines.append("// or angular momentum (shell_hubbard, shpoly, reference_occ)\n")
    for name in ["shell_hubbard", "p_shpoly", "reference_occ", "slater_exponent",
                 "p_selfenergy", "p_kcn"]:
        lines.append(arr1(prefix + "_" + name.upper(), "double", flat(params[name])))
    for name in ["ang_shell", "principal_quantum_number", "number_of_primitives"]:
        lines.append(arr1(prefix + "_" + name.upper(), "int", flat(params[name])))
    lines.append(arr1(prefix + "_NSHELL", "int", flat(params["nshell"])))
    lines.append(arr1(prefix + "_KSHELL", "double", flat(params["kshell"])))
    path.write_text("".join(lines))


def main():
    if len(sys.argv) < 2:
        raise SystemExit(f"usage: python {Path(__file__).name} <tblite source tree>")
    root = Path(sys.argv[1])
    params, sto = extract(root)
    (HERE / "gfn2.json").write_text(json.dumps(params, indent=0))
    (HERE / "sto_ng.json").write_text(json.dumps(sto, indent=0))
    write_inc(params, sto, HERE.parent / "csrc" / "params_gfn2.inc")
    g1 = extract_gfn1(root)
    (HERE / "gfn1.json").write_text(json.dumps(g1, indent=0))
    write_inc_gfn1(g1, HERE.parent / "csrc" / "params_gfn1.inc")
    i1 = extract_gfn1(root, "ipea1")
    (HERE / "ipea1.json").write_text(json.dumps(i1, indent=0))
    write_inc_gfn1(i1, HERE.parent / "csrc" / "params_ipea1.inc", "IPEA1")
    print("wrote gfn2.json, sto_ng.json, params_gfn2.inc, gfn1.json, params_gfn1.inc, "
          "ipea1.json, params_ipea1.inc")


if __name__ == "__main__":
    main()
