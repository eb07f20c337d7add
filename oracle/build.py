"""Build recipe for the C part of the CPU oracle (test infrastructure only).

Compiles ``oracle/xtb_oracle.c`` with gcc into ``oracle/_build/liboracle.so``.
The output is rebuilt when the source is newer than the library.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"


def build_oracle(force: bool = False) -> Path:
    src = HERE / "xtb_oracle.c"
    lib = OUT / "liboracle.so"
    if not force and lib.exists() and lib.stat().st_mtime >= src.stat().st_mtime:
        return lib
    OUT.mkdir(exist_ok=True)
    tmp = OUT / f"liboracle.{os.getpid()}.so"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-o", str(tmp), str(src), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build_oracle(force=True))
