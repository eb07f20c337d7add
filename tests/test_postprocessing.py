"""Post-processing list and dictionary (reference include/tblite/double_dictionary.h,
result.h:243-246, calculator.h:270-279; api/double_dictionary.f90, post_processing/list.f90).

CPU: error behaviour of the dictionary entry points and of the post-processing list, the
generic tblite_delete / tblite_check macros in C.  GPU (marked): the dictionary of a single
point holds the reference's default entries (bond orders [nat, nat, 1], molecular dipole and
quadrupole) with the values of the result getters; a calculator asked only for bond orders
computes no moments; the batched path returns the same bond orders as the plain path (closed and
open shells).
"""
import ctypes
import shutil
import subprocess
from ctypes import byref, c_int, c_void_p
from pathlib import Path

import numpy as np
import pytest

from tblite_gb300 import library
from tblite_gb300.exceptions import TBLiteRuntimeError

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    from tblite_gb300 import _build

    _build.build()
    return library.load()


def test_dictionary_errors(lib):
    err = library._Error()
    res = c_void_p(lib.tblite_new_result())
    try:
        assert lib.tblite_get_post_processing_dict(err.h, res) is None
        with pytest.raises(TBLiteRuntimeError, match="post processing dictionary"):
            err.check()
        assert lib.tblite_get_n_entries_dict(err.h, None) == 0
        with pytest.raises(TBLiteRuntimeError, match="Dictionary is missing"):
            err.check()
        idx = c_int(1)
        dims = [c_int(7), c_int(7), c_int(7)]
        lib.tblite_get_array_size_index(err.h, None, byref(idx), *[byref(d) for d in dims])
        assert [d.value for d in dims] == [0, 0, 0]
        with pytest.raises(TBLiteRuntimeError, match="Dictionary is missing"):
            err.check()
        null = c_void_p()
        lib.tblite_delete_double_dictionary(byref(null))  # a null handle is ignored
    finally:
        lib.tblite_delete_result(byref(res))


def test_post_processing_names(lib):
    from tblite_gb300 import workloads
    from tblite_gb300.interface import Calculator

    z, x = workloads.water_cluster((2, 1, 1), seed=11)
    calc = Calculator("GFN2-xTB", z, x)
    calc.add("bond-orders")
    calc.add("molecular-multipoles")
    for name in ("xtbml", "missing-file.toml"):
        with pytest.raises(TBLiteRuntimeError, match="not available"):
            library.post_processing_push_back(calc._ctx, calc._calc, calc._mol, name)


def test_generic_macros_compile_and_run(lib, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "macros.c"
    src.write_text(
        '#include "tblite.h"\n'
        "int main(void) {\n"
        "  tblite_error e = tblite_new_error();\n"
        "  tblite_context c = tblite_new_context();\n"
        "  tblite_result r = tblite_new_result();\n"
        "  tblite_double_dictionary d = tblite_get_post_processing_dict(e, r);\n"
        "  int rc = tblite_check(e) == 1 ? 0 : 1;\n"
        "  rc += tblite_check(c);\n"
        "  tblite_delete(d); tblite_delete(r); tblite_delete(c); tblite_delete(e);\n"
        "  return rc + (e != 0) + (c != 0) + (r != 0) + (d != 0);\n"
        "}\n")
    exe = tmp_path / "macros"
    libdir = library.library_path().parent
    subprocess.run([cc, "-std=c11", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src),
                    f"-L{libdir}", "-ltblite_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                   check=True)
    assert subprocess.run([str(exe)]).returncode == 0


@pytest.mark.gpu
def test_default_dictionary_matches_getters(lib):
    from tblite_gb300 import workloads
    from tblite_gb300.interface import Calculator

    z, x = workloads.water_cluster((2, 1, 1), seed=11)
    res = Calculator("GFN2-xTB", z, x).singlepoint()
    d = res.get("post-processing-dict")
    assert list(d) == ["bond-orders", "molecular-dipole", "molecular-quadrupole"]
    assert d["bond-orders"].shape == (len(z), len(z), 1)
    # the dictionary keeps Fortran order (wbo(a, b)); Result.get reads the same buffer in C order
    assert np.array_equal(d["bond-orders"][:, :, 0].T, res.get("bond-orders"))
    assert np.array_equal(d["molecular-dipole"], res.get("dipole"))
    assert np.array_equal(d["molecular-quadrupole"], res.get("quadrupole"))
    # by label, through the C ABI
    err = library._Error()
    h = c_void_p(lib.tblite_get_post_processing_dict(err.h, res._res))
    try:
        dims = [c_int(0), c_int(0), c_int(0)]
        lib.tblite_get_array_size_label(err.h, h, b"molecular-dipole", *[byref(v) for v in dims])
        assert [v.value for v in dims] == [3, 0, 0]
        out = np.zeros(3)
        lib.tblite_get_array_entry_label(err.h, h, b"molecular-dipole", library._dp(out))
        err.check()
        assert np.array_equal(out, res.get("dipole"))
        lib.tblite_get_array_entry_label(err.h, h, b"no-such-entry", library._dp(out))
        with pytest.raises(TBLiteRuntimeError, match="Label is not a key"):
            err.check()
        idx = c_int(4)
        label = ctypes.create_string_buffer(8)
        lib.tblite_get_label_entry_index(err.h, h, byref(idx), label, None)
        with pytest.raises(TBLiteRuntimeError, match="Index is not a key"):
            err.check()
    finally:
        lib.tblite_delete_double_dictionary(byref(h))


@pytest.mark.gpu
def test_bond_orders_only(lib):
    from tblite_gb300 import workloads
    from tblite_gb300.interface import Calculator

    z, x = workloads.water_cluster((2, 1, 1), seed=11)
    calc = Calculator("GFN2-xTB", z, x)
    calc.add("bond-orders")
    res = calc.singlepoint()
    assert list(res.get("post-processing-dict")) == ["bond-orders"]
    with pytest.raises(TBLiteRuntimeError, match="dipole"):
        res.get("dipole")
    ref = Calculator("GFN2-xTB", z, x).singlepoint()
    assert np.array_equal(res.get("bond-orders"), ref.get("bond-orders"))


@pytest.mark.gpu
def test_batched_bond_orders_match_plain_path(lib):
    """Closed shells and a restricted open shell (two channels) in one batch call; the plain
    path is the reference for the values, which the plain-path parity tests pin to the
    oracle."""
    from tblite_gb300 import workloads
    from tblite_gb300.interface import Calculator, batch_fallbacks, batch_singlepoint

    mols = [(workloads.water_cluster_k(k, seed=50 + k), None) for k in (2, 7, 40)]
    mols += [(workloads.alkane(n, seed=60 + n), None) for n in (3, 30)]
    mols += [(workloads.water_cluster((2, 1, 1), seed=12), 1.0)]  # cation: open shell
    calcs = [Calculator("GFN2-xTB", z, x, charge=q) for (z, x), q in mols]
    res_b = batch_singlepoint(calcs)
    assert batch_fallbacks() == 0
    for ((z, x), q), rb in zip(mols, res_b):
        rp = Calculator("GFN2-xTB", z, x, charge=q).singlepoint()
        wb, wp = rb.get("bond-orders"), rp.get("bond-orders")
        assert wb.shape == wp.shape
        assert np.max(np.abs(wb - wp)) <= 1e-6
        assert list(rb.get("post-processing-dict")) == list(rp.get("post-processing-dict"))
