"""The reference's own Python package over this library (CPU; runs where the reference's
source tree is present, and is skipped elsewhere).

A maintainer switching the reference's ``tblite`` Python package to this library rebuilds its
cffi extension (python/ffi-builder.py: API mode, the header preprocessed with TBLITE_CFFI)
against ``include/tblite.h`` and ``libtblite_gb300.so``.  This test does exactly that in a
temporary directory and then imports the UNMODIFIED ``tblite.library`` and ``tblite.interface``
modules from the reference tree (not copied): every entry point they bind when they are
imported must exist.  It then drives them: structures, calculators by method name and by a
parameter dictionary (the table and parameter-record API), settings, maps, the post-processing
names, and the errors of calls that need a GPU (no CPU fallback) or a single point first.
"""
import importlib
import shutil
import subprocess
import sys
import sysconfig
import types
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
REF_PY = Path("/root/reference/python/tblite")


@pytest.fixture(scope="module")
def tblite(tmp_path_factory):
    if not (REF_PY / "interface.py").exists():
        pytest.skip("the reference's source tree is not present")
    cffi = pytest.importorskip("cffi")
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None or not (Path(sysconfig.get_paths()["include"]) / "Python.h").exists():
        pytest.skip("no C compiler or Python headers")
    from tblite_gb300 import _build, library

    _build.build()
    libdir = str(library.library_path().parent)
    inc = str(ROOT / "include")
    cdefs = subprocess.run([cc, "-DTBLITE_CFFI", "-E", "-P", f"{inc}/tblite.h"],
                           capture_output=True, text=True, check=True).stdout
    work = tmp_path_factory.mktemp("binding")
    ffi = cffi.FFI()
    ffi.set_source("tblite._libtblite", '#include "tblite.h"', include_dirs=[inc],
                   libraries=["tblite_gb300"], library_dirs=[libdir],
                   runtime_library_dirs=[libdir])
    ffi.cdef(cdefs)
    built = Path(ffi.compile(tmpdir=str(work), verbose=False))
    pkgdir = work / "tblite"
    pkgdir.mkdir(exist_ok=True)
    if built.parent != pkgdir:
        shutil.move(str(built), pkgdir / built.name)
    saved = {k: v for k, v in sys.modules.items() if k == "tblite" or k.startswith("tblite.")}
    for k in saved:
        del sys.modules[k]
    pkg = types.ModuleType("tblite")
    pkg.__path__ = [str(pkgdir), str(REF_PY)]  # the extension here, the Python from the reference
    sys.modules["tblite"] = pkg
    try:
        yield types.SimpleNamespace(interface=importlib.import_module("tblite.interface"),
                                    library=importlib.import_module("tblite.library"),
                                    exceptions=importlib.import_module("tblite.exceptions"))
    finally:
        for k in [k for k in sys.modules if k == "tblite" or k.startswith("tblite.")]:
            del sys.modules[k]
        sys.modules.update(saved)


def _water_dimer():
    from tblite_gb300 import workloads

    return workloads.water_cluster((2, 1, 1), seed=11)


def test_calculators_settings_and_maps(tblite):
    numbers, positions = _water_dimer()
    calc = tblite.interface.Calculator("GFN2-xTB", numbers, positions)
    for key, value in (("accuracy", 0.1), ("max-iter", 100), ("mixer-damping", 0.3),
                       ("temperature", 1e-3), ("save-integrals", 1)):
        calc.set(key, value)
    assert list(calc.get("shell-map")) == [0, 0, 1, 2, 3, 3, 4, 5]
    assert list(calc.get("angular-momenta")) == [0, 1, 0, 0, 0, 1, 0, 0]
    assert len(calc.get("orbital-map")) == 12
    calc.add("bond-orders")
    calc.add("molecular-multipoles")
    gfn1 = tblite.interface.Calculator("GFN1-xTB", numbers, positions)
    assert len(gfn1.get("shell-map")) == 12  # H carries a second s shell in GFN1-xTB
    with pytest.raises(tblite.exceptions.TBLiteValueError):
        tblite.interface.Calculator("GFN0-xTB", numbers, positions)


def test_parameter_dictionary_through_the_table_api(tblite):
    from tblite_gb300 import library as ours

    numbers, positions = _water_dimer()
    params = ours.export_param("GFN2-xTB")
    calc = tblite.interface.Calculator(params, numbers, positions)
    assert list(calc.get("shell-map")) == [0, 0, 1, 2, 3, 3, 4, 5]
    # the reference's own round trip of the exported GFN2 parameters
    lib = tblite.library
    p = lib.new_param()
    lib.export_gfn2_param(p)
    table = lib.new_table()
    lib.dump_param(p, table)
    data = lib.table_to_dict(table)
    assert data["hamiltonian"]["xtb"]["cn"] == "dexp"
    assert np.allclose(data["element"]["O"]["levels"], params["element"]["O"]["levels"])


def test_gpu_calls_fail_loudly_and_results_need_a_single_point(tblite):
    import torch

    numbers, positions = _water_dimer()
    calc = tblite.interface.Calculator("GFN2-xTB", numbers, positions)
    res = tblite.interface.Result()
    with pytest.raises(tblite.exceptions.TBLiteRuntimeError, match="Result does not contain"):
        res.get("energy")
    with pytest.raises(tblite.exceptions.TBLiteRuntimeError, match="post processing"):
        res.get("bond-orders")
    if not torch.cuda.is_available():
        with pytest.raises(tblite.exceptions.TBLiteRuntimeError, match="CUDA"):
            calc.singlepoint()


def test_interactions_through_the_reference_package(tblite):
    numbers, positions = _water_dimer()
    calc = tblite.interface.Calculator("GFN2-xTB", numbers, positions)
    with pytest.raises(tblite.exceptions.TBLiteRuntimeError, match="not available"):
        calc.add("spin-polarization", 1.0)
    with pytest.raises(tblite.exceptions.TBLiteRuntimeError, match="water only"):
        calc.add("alpb-solvation", "benzene")
    calc.add("alpb-solvation", "water")  # ALPB(water) is available
    for interaction, args in (("gbsa-solvation", ("water",)), ("gbe-solvation", (7.0, "p16")),
                              ("gb-solvation", (78.4, "still"))):
        other = tblite.interface.Calculator("GFN2-xTB", numbers, positions)
        other.add(interaction, *args)
