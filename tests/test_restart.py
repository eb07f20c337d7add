"""Wavefunction restart files (tblite_save_result_wavefunction / tblite_load_result_wavefunction,
reference include/tblite/result.h:253-265, wavefunction/restart.f90): a NumPy .npz archive with
the members tblite0_{kt, nel, n0at, n0sh, density, coeff, emo, focc, qat, qsh, dpat, qpat}.

CPU: an archive written by numpy (C-order members, as numpy writes by default) is loaded and
saved again; numpy reads the saved archive back bit for bit, damaged or incomplete files are
refused.  GPU (marked): a single point saved, loaded into a fresh result and used as the restart
of the next single point gives the same energy in fewer iterations.
"""
from ctypes import c_void_p

import numpy as np
import pytest

from tblite_gb300 import library
from tblite_gb300.exceptions import TBLiteRuntimeError


def _arrays(nat=3, nsh=5, nao=7, seed=1):
    rng = np.random.default_rng(seed)
    return {
        "tblite0_kt": np.array([9.5e-4]), "tblite0_nel": np.array([4.0, 4.0]),
        "tblite0_n0at": rng.random(nat), "tblite0_n0sh": rng.random(nsh),
        "tblite0_density": rng.random((nao, nao, 1)), "tblite0_coeff": rng.random((nao, nao, 1)),
        "tblite0_emo": rng.random((nao, 1)), "tblite0_focc": rng.random((nao, 1)),
        "tblite0_qat": rng.random((nat, 1)), "tblite0_qsh": rng.random((nsh, 1)),
        "tblite0_dpat": rng.random((3, nat, 1)), "tblite0_qpat": rng.random((6, nat, 1)),
    }


def _call(fn, res, path):
    err = library._Error()
    getattr(library.load(), fn)(err.h, res, str(path).encode())
    err.check()


def test_numpy_archive_round_trip(tmp_path):
    lib = library.load()
    ref = _arrays()
    np.savez(tmp_path / "in.npz", **ref)
    res = c_void_p(lib.tblite_new_result())
    try:
        _call("tblite_load_result_wavefunction", res, tmp_path / "in.npz")
        _call("tblite_save_result_wavefunction", res, tmp_path / "out.npz")
    finally:
        lib.tblite_delete_result(res)
    out = np.load(tmp_path / "out.npz")
    assert sorted(out.files) == sorted(ref)
    for k, v in ref.items():
        assert out[k].shape == v.shape and np.array_equal(out[k], v), k


def test_refuses_bad_files(tmp_path):
    lib = library.load()
    res = c_void_p(lib.tblite_new_result())
    try:
        with pytest.raises(TBLiteRuntimeError, match="Could not find"):
            _call("tblite_load_result_wavefunction", res, tmp_path / "missing.npz")
        ref = _arrays()
        del ref["tblite0_qsh"]
        np.savez(tmp_path / "incomplete.npz", **ref)
        with pytest.raises(TBLiteRuntimeError, match="qsh"):
            _call("tblite_load_result_wavefunction", res, tmp_path / "incomplete.npz")
        ref = _arrays()
        ref["tblite0_qat"] = np.zeros((4, 1))
        np.savez(tmp_path / "mismatch.npz", **ref)
        with pytest.raises(TBLiteRuntimeError, match="Dimension mismatch"):
            _call("tblite_load_result_wavefunction", res, tmp_path / "mismatch.npz")
        np.savez(tmp_path / "good.npz", **_arrays())
        raw = bytearray((tmp_path / "good.npz").read_bytes())
        raw[200] ^= 0xFF  # inside the first member's data
        (tmp_path / "damaged.npz").write_bytes(bytes(raw))
        with pytest.raises(TBLiteRuntimeError):
            _call("tblite_load_result_wavefunction", res, tmp_path / "damaged.npz")
        with pytest.raises(TBLiteRuntimeError, match="wavefunction"):
            _call("tblite_save_result_wavefunction", res, tmp_path / "empty.npz")
    finally:
        lib.tblite_delete_result(res)


def _npy_bytes(header_shape, payload):
    """A .npy 1.0 member with the given shape text in its header (not checked by numpy)."""
    hdr = "{'descr': '<f8', 'fortran_order': True, 'shape': %s, }" % header_shape
    hdr = hdr + " " * (63 - (10 + len(hdr)) % 64) + "\n"
    return b"\x93NUMPY\x01\x00" + len(hdr).to_bytes(2, "little") + hdr.encode() + payload


def _archive_with(tmp_path, name, member, data):
    import zipfile

    ref = _arrays()
    path = tmp_path / name
    with zipfile.ZipFile(path, "w", compression=zipfile.ZIP_STORED) as zf:
        for k, v in ref.items():
            if k == member:
                zf.writestr(k + ".npy", data)
            else:
                import io

                buf = io.BytesIO()
                np.save(buf, v)
                zf.writestr(k + ".npy", buf.getvalue())
    return path


def test_refuses_malformed_headers_and_offsets(tmp_path):
    """Malformed shapes, empty trailing dimensions and wrapped offsets give an error, never a
    hang or a read outside the file."""
    lib = library.load()
    res = c_void_p(lib.tblite_new_result())
    payload = np.zeros(3).tobytes()
    try:
        for i, (shape, match) in enumerate([("(3L,)", "bad shape"), ("(3,x)", "bad shape"),
                                            ("(99999999999999999999,)", "truncated"),
                                            ("(4611686018427387904, 4)", "truncated"),
                                            ("(3, 0)", "Dimension mismatch")]):
            path = _archive_with(tmp_path, f"shape{i}.npz", "tblite0_qat",
                                 _npy_bytes(shape, payload))
            with pytest.raises(TBLiteRuntimeError, match=match):
                _call("tblite_load_result_wavefunction", res, path)
        np.savez(tmp_path / "good.npz", **_arrays())
        raw = bytearray((tmp_path / "good.npz").read_bytes())
        cd = raw.index(b"PK\x01\x02")
        raw[cd + 42:cd + 46] = (0xFFFFFFF0).to_bytes(4, "little")  # local header offset
        (tmp_path / "offset.npz").write_bytes(bytes(raw))
        with pytest.raises(TBLiteRuntimeError, match="damaged member"):
            _call("tblite_load_result_wavefunction", res, tmp_path / "offset.npz")
    finally:
        lib.tblite_delete_result(res)


@pytest.mark.gpu
def test_restart_from_file(tmp_path):
    from tblite_gb300 import _build, workloads
    from tblite_gb300.interface import Calculator, Result

    _build.build()
    z, x = workloads.water_cluster((2, 2, 1), seed=3)
    calc = Calculator("GFN2-xTB", z, x)
    # tight convergence, so that two differently started SCF runs agree beyond the parity bar
    calc.set("accuracy", 1e-4)
    library.set_profiling(True)
    first = calc.singlepoint()
    it_first = library.get_profile()["iterations"]
    _call("tblite_save_result_wavefunction", first._res, tmp_path / "wfn.npz")
    res = Result()
    _call("tblite_load_result_wavefunction", res._res, tmp_path / "wfn.npz")
    again = calc.singlepoint(res)
    assert library.get_profile()["iterations"] < it_first
    assert abs(again.get("energy") - first.get("energy")) < 1e-7
    assert np.max(np.abs(again.get("charges") - first.get("charges"))) < 1e-6
