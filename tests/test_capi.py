"""Host-side checks of the C ABI (no GPU needed): exports, handles, errors, basis maps."""
import re
from ctypes import byref, c_int, c_void_p
from pathlib import Path

import numpy as np
import pytest

from tblite_gb300 import _build, library
from tblite_gb300.exceptions import TBLiteRuntimeError

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return library.load()


def test_header_symbols_exported(lib):
    header = "".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    macros = set(re.findall(r"#define\s+(tblite_[a-z0-9_]+)\(", header))
    names = sorted(set(re.findall(r"\b(tblite_[a-z0-9_]+)\s*\(", header)) - macros)
    assert len(names) > 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_header_parses_with_cffi(lib):
    """The reference's Python package binds the preprocessed header with cffi."""
    import shutil
    import subprocess

    cffi = pytest.importorskip("cffi")
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C preprocessor")
    src = subprocess.run([cc, "-E", "-P", "-DTBLITE_CFFI", str(ROOT / "include" / "tblite.h")],
                         capture_output=True, text=True, check=True).stdout
    ffi = cffi.FFI()
    ffi.cdef(src)
    clib = ffi.dlopen(str(library.library_path()))
    assert clib.tblite_get_version() == lib.tblite_get_version()
    err = clib.tblite_new_error()
    assert clib.tblite_check_error(err) == 0
    perr = ffi.new("tblite_error *", err)
    clib.tblite_delete_error(perr)
    assert perr[0] == ffi.NULL


def test_error_roundtrip(lib):
    err = c_void_p(lib.tblite_new_error())
    assert lib.tblite_check_error(err) == 0
    msg = b"some failure"
    size = c_int(len(msg))
    lib.tblite_set_error(err, msg, byref(size))
    assert lib.tblite_check_error(err) == 1
    import ctypes
    buf = ctypes.create_string_buffer(64)
    cap = c_int(64)
    lib.tblite_get_error(err, buf, byref(cap))
    assert buf.value == msg
    lib.tblite_clear_error(err)
    assert lib.tblite_check_error(err) == 0
    lib.tblite_delete_error(byref(err))
    assert err.value is None


def test_null_handles_report_errors(lib):
    ctx = c_void_p(lib.tblite_new_context())
    res = c_void_p(lib.tblite_new_result())
    lib.tblite_get_singlepoint(ctx, None, None, res)
    assert lib.tblite_check_context(ctx) == 1
    with pytest.raises(TBLiteRuntimeError, match="structure data is missing"):
        library.context_check(ctx)
    lib.tblite_delete_result(byref(res))
    lib.tblite_delete_context(byref(ctx))


def test_structure_validation():
    with pytest.raises(TBLiteRuntimeError, match="Non-finite"):
        library.new_structure([8, 1], [[0, 0, 0], [np.nan, 0, 0]])
    with pytest.raises(TBLiteRuntimeError, match="Invalid"):
        library.new_structure([], np.zeros((0, 3)))


def test_result_without_data(lib):
    res = c_void_p(lib.tblite_new_result())
    with pytest.raises(TBLiteRuntimeError, match="does not contain energy"):
        library.result_array(res, "energy", (1,))
    lib.tblite_delete_result(byref(res))


def test_basis_maps_match_oracle():
    from oracle import gfn2
    from tblite_gb300 import interface, workloads

    z, x = workloads.water_cluster((2, 1, 1), seed=5)
    calc = interface.Calculator("GFN2-xTB", z, x)
    ref = gfn2.new_calc(gfn2.Molecule(z, x))
    assert np.array_equal(calc.get("shell-map"), ref.sh_atom)
    assert np.array_equal(calc.get("angular-momenta"), ref.sh_l)
    ao2sh = np.repeat(np.arange(len(ref.sh_l)), 2 * ref.sh_l + 1)
    assert np.array_equal(calc.get("orbital-map"), ao2sh)


def test_unsupported_element_message():
    from tblite_gb300 import interface

    with pytest.raises(TBLiteRuntimeError, match="d shells"):
        interface.Calculator("GFN2-xTB", [26, 1], [[0, 0, 0], [0, 0, 3.0]])
    # fluorine has no d shell, but the element-data pack covers H, C, N, O only: the error names
    # the library whose tables are missing
    with pytest.raises(TBLiteRuntimeError, match=r"Z=9 \(mctc-lib v0\.5\.2 data"):
        interface.Calculator("GFN2-xTB", [9, 1], [[0, 0, 0], [0, 0, 1.7]])
    with pytest.raises(TBLiteRuntimeError, match=r"Z=9 \(mctc-lib v0\.5\.2 data"):
        interface.Calculator("GFN1-xTB", [9, 1], [[0, 0, 0], [0, 0, 1.7]])


def test_density_solver_setting():
    """The density-solver key takes the two solver names; other codes are refused, and a result
    without a spectral projection has no gap certificate."""
    from tblite_gb300 import interface, workloads

    z, x = workloads.water_cluster((2, 1, 1), seed=5)
    calc = interface.Calculator("GFN2-xTB", z, x)
    calc.set("density-solver", "purification")
    calc.set("density-solver", "diagonalization")
    with pytest.raises(TBLiteRuntimeError, match="density solver"):
        calc.set("density-solver", 2)
    with pytest.raises(ValueError):
        calc.set("density-solver", "lanczos")
    with pytest.raises(TBLiteRuntimeError, match="gap"):
        interface.Result().get("gap")


def test_batch_host_settings_without_a_gpu(lib):
    """Host-side batch settings need no device: the projection threshold setter returns the
    previous value (0 only queries), and the host phases of the last batch call are reported
    by name (zeros before any call in this process)."""
    old = library.set_projection_threshold(0)
    assert old > 0
    try:
        assert library.set_projection_threshold(120) == old
        assert library.set_projection_threshold(0) == 120
    finally:
        library.set_projection_threshold(old)
    assert library.set_projection_threshold(0) == old
    host = library.batch_host_ms()
    assert tuple(host) == library.BATCH_HOST_PHASES
    assert all(v >= 0.0 for v in host.values())
