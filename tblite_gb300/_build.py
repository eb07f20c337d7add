"""Build the CUDA engine (``libtblite_gb300.so``) in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into one shared
library next to this file (``tblite_gb300/lib/``).  A unit is rebuilt when its
source, ``engine.h`` or a generated include is newer than its object file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OUT = PKG / "lib"
OBJ = PKG / "_build"
LIBNAME = "libtblite_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = ["integrals.cu", "scf.cu", "disp.cu", "linalg.cu", "eigen.cu", "noalloc.cu", "solv.cu",
         "ozaki.cu", "ozaki_pipe.cu", "purify.cu", "capi.cpp", "batch.cpp", "npz.cpp",
         "dictionary.cpp", "sp2.cu", "table.cpp", "param.cpp"]
HEADERS = ["engine.h", "api_internal.h", "npz.h", "table.h", "param.h", "params_solv.inc", "params_gfn1.inc", "params_gfn2.inc",
           "element_data.inc"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")
    return cand


def _compile(src: Path, obj: Path) -> None:
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-fvisibility=default", "-Xcompiler", "-pthread", "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cu":
        cmd[1:1] = ["-Xptxas", "-O3"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")


def library_path() -> Path:
    return OUT / LIBNAME


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    hdr_time = max((SRC / h).stat().st_mtime for h in HEADERS)
    jobs = []
    for unit in UNITS:
        src = SRC / unit
        obj = OBJ / (unit + ".o")
        stale = force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_time)
        jobs.append((src, obj, stale))
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        futs = [ex.submit(_compile, s, o) for s, o, stale in jobs if stale]
        for f in futs:
            f.result()
    lib = library_path()
    newest = max(o.stat().st_mtime for _, o, _ in jobs)
    if force or not lib.exists() or lib.stat().st_mtime < newest:
        tmp = OUT / f".{LIBNAME}.{os.getpid()}"
        cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-pthread", "-o", str(tmp),
               *[str(o) for _, o, _ in jobs], "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, lib)
        if verbose:
            print("built", lib)
    return lib


if __name__ == "__main__":
    print(build(force=True, verbose=True))
