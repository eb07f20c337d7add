"""Data tables of the C API (reference include/tblite/table.h, src/tblite/api/table.f90), CPU.

Nested tables of scalars, arrays and sub-tables are built through the C ABI, read back (types,
values, 1-based key and array indices, errors for missing keys and handles), and written as TOML
text that Python's own TOML reader parses to the same data.
"""
import ctypes
import tomllib
from ctypes import byref, c_bool, c_char_p, c_double, c_int, c_int64, c_void_p

import pytest

from tblite_gb300 import library
from tblite_gb300.exceptions import TBLiteRuntimeError


@pytest.fixture(scope="module")
def lib():
    from tblite_gb300 import _build

    _build.build()
    return library.load()


def test_build_read_and_dump(lib, tmp_path):
    err = library._Error()
    t = c_void_p(lib.tblite_new_table(None))
    x = (c_double * 3)(1.5, -2.0, 1e-300)
    lib.tblite_table_set_double(err.h, t, b"levels", x, 3)
    one = c_double(0.25)
    lib.tblite_table_set_double(err.h, t, b"wexp", byref(one), 0)
    n = c_int64(7)
    lib.tblite_table_set_int64_t(err.h, t, b"version", byref(n), 0)
    b = c_bool(True)
    lib.tblite_table_set_bool(err.h, t, b"sc", byref(b), 0)
    s = ctypes.create_string_buffer(b"GFN2-xTB")
    lib.tblite_table_set_char(err.h, t, b"name", s, 0)
    sub = c_void_p(lib.tblite_table_add_table(err.h, t, b"element"))
    h = c_void_p(lib.tblite_table_add_table(err.h, sub, b"H"))
    arr = c_void_p(lib.tblite_new_array())
    lib.tblite_array_push_back_char(err.h, arr, b"1s")
    lib.tblite_array_push_back_char(err.h, arr, b"2s")
    lib.tblite_table_set_array(err.h, h, b"shells", arr)
    err.check()
    lib.tblite_delete_array(byref(arr))
    lib.tblite_delete_table(byref(sub))  # the child handle lives on by itself
    assert lib.tblite_table_get_n_keys(err.h, t) == 6
    key = ctypes.create_string_buffer(16)
    lib.tblite_table_get_key(err.h, t, 1, key, 16)
    assert key.value == b"levels"
    types = {k: lib.tblite_table_get_type(err.h, t, k)
             for k in (b"levels", b"wexp", b"version", b"sc", b"name", b"element", b"nope")}
    assert types == {b"levels": 5, b"wexp": 3, b"version": 2, b"sc": 1, b"name": 4,
                     b"element": 6, b"nope": 0}
    v = c_double()
    lib.tblite_table_get_double(err.h, t, b"version", byref(v))  # integers read as doubles
    assert v.value == 7.0
    a = c_void_p(lib.tblite_table_get_array(err.h, t, b"levels"))
    assert lib.tblite_array_size(err.h, a) == 3
    lib.tblite_array_get_double(err.h, a, 3, byref(v))
    assert v.value == 1e-300
    lib.tblite_array_get_double(err.h, a, 4, byref(v))
    with pytest.raises(TBLiteRuntimeError, match="double value from data array"):
        err.check()
    lib.tblite_delete_array(byref(a))
    shells = c_void_p(lib.tblite_table_get_array(err.h, h, b"shells"))
    lib.tblite_array_get_char(err.h, shells, 2, key, 16)
    assert key.value == b"2s"
    lib.tblite_delete_array(byref(shells))
    lib.tblite_table_get_double(err.h, t, b"name", byref(v))
    with pytest.raises(TBLiteRuntimeError, match="double value from data table"):
        err.check()
    assert lib.tblite_table_get_table(err.h, t, b"missing") is None
    with pytest.raises(TBLiteRuntimeError, match="subtable"):
        err.check()
    lib.tblite_table_get_key(err.h, t, 7, key, 16)
    with pytest.raises(TBLiteRuntimeError, match="out of range"):
        err.check()
    path = tmp_path / "table.toml"
    lib.tblite_dump_table(err.h, t, str(path).encode())
    err.check()
    data = tomllib.loads(path.read_text())
    assert data == {"levels": [1.5, -2.0, 1e-300], "wexp": 0.25, "version": 7, "sc": True,
                    "name": "GFN2-xTB", "element": {"H": {"shells": ["1s", "2s"]}}}
    lib.tblite_delete_table(byref(h))
    lib.tblite_delete_table(byref(t))
    assert t.value is None


def test_missing_handles(lib):
    err = library._Error()
    v = c_double()
    lib.tblite_table_get_double(err.h, None, b"x", byref(v))
    with pytest.raises(TBLiteRuntimeError, match="Data table object is missing"):
        err.check()
    assert lib.tblite_array_size(err.h, None) == 0
    with pytest.raises(TBLiteRuntimeError, match="Data array object is missing"):
        err.check()
    lib.tblite_table_set_double(None, None, b"x", byref(v), 0)  # no error handle: no action
