"""Parametrisation records (reference include/tblite/param.h, src/tblite/param.f90 and
param/*.f90; exports xtb/gfn2.f90:914-1022, xtb/gfn1.f90:931-1054) and
tblite_new_xtb_calculator (calculator.h:92-107).

CPU: the exported GFN2-xTB and GFN1-xTB records written as tables have the reference's TOML
layout (levels and CN shifts in eV), survive a dump -> load -> dump round trip, and give the same
basis as the built-in calculators; malformed tables are refused with the reference's messages.
GPU (marked): a calculator from the exported record gives the built-in calculator's results bit
for bit; a record that went through the table (eV conversion) agrees to 1e-10 Eh; a changed
element level moves the energy by the amount the analytic parameter gradient predicts.
"""
import tomllib

import numpy as np
import pytest

from tblite_gb300 import library
from tblite_gb300.exceptions import TBLiteRuntimeError

EV = 27.21138505


@pytest.fixture(scope="module", autouse=True)
def built():
    from tblite_gb300 import _build

    _build.build()


def test_gfn2_layout():
    d = library.export_param("GFN2-xTB")
    assert d["meta"]["name"] == "GFN2-xTB" and d["meta"]["format"] == 1
    xtb = d["hamiltonian"]["xtb"]
    assert xtb["cn"] == "dexp" and set(xtb["shell"]) >= {"ss", "pp", "dd"}
    assert "kpair" not in xtb
    assert d["dispersion"]["d4"]["sc"] is True
    assert d["charge"]["effective"]["average"] == "arithmetic"
    assert set(d["thirdorder"]["shell"]) == {"s", "p", "d"}
    assert set(d["multipole"]["damped"]) == {"dmp3", "dmp5", "kexp", "shift", "rmax"}
    o = d["element"]["O"]
    assert o["shells"] == ["2s", "2p"]
    from oracle import gfn2

    p = gfn2.load_params()
    # levels in eV in the table, Hartree in the method's own tables
    assert np.allclose(np.array(o["levels"]) / EV, p["p_selfenergy"][7][:2], rtol=1e-14)


def test_gfn1_layout():
    d = library.export_param("GFN1-xTB")
    xtb = d["hamiltonian"]["xtb"]
    assert xtb["cn"] == "exp" and xtb["wexp"] == 0.0
    assert xtb["kpair"]["H-H"] == 0.96 and xtb["kpair"]["N-H"] == 1.04
    assert "d3" in d["dispersion"] and d["thirdorder"]["shell"] is False
    assert "multipole" not in d and "classical" in d["halogen"]
    h = d["element"]["H"]
    assert h["shells"] == ["1s", "2s"] and h["refocc"][1] == 0.0


@pytest.mark.parametrize("method", ["GFN2-xTB", "GFN1-xTB"])
def test_round_trip_and_toml(method, tmp_path):
    d1 = library.export_param(method)
    d2 = library.table_to_dict(_dump(library.param_from_dict(d1)))
    assert d2 == _with_float_tolerance(d1, d2)
    # written as TOML, the text parses back to the same data
    t = library.dict_to_table(d1)
    err = library._Error()
    library.load().tblite_dump_table(err.h, t.h, str(tmp_path / "p.toml").encode())
    err.check()
    d3 = tomllib.loads((tmp_path / "p.toml").read_text())
    assert d3["meta"] == d1["meta"]
    assert d3["element"]["C"]["levels"] == d1["element"]["C"]["levels"]
    assert d3["element"]["O"]["en"] == d1["element"]["O"]["en"]
    assert d3["hamiltonian"] == d1["hamiltonian"]


def _dump(param):
    t = library.Table()
    err = library._Error()
    library.load().tblite_dump_param(err.h, param.h, t.h)
    err.check()
    return t


def _with_float_tolerance(a, b):
    """a with each float replaced by b's value where both agree to 1e-12 relative (the eV
    conversion of levels and CN shifts rounds on the way in and out)"""
    if isinstance(a, dict):
        return {k: _with_float_tolerance(v, b.get(k) if isinstance(b, dict) else None)
                for k, v in a.items()}
    if isinstance(a, list):
        return [_with_float_tolerance(x, y) for x, y in zip(a, b or [None] * len(a))]
    if isinstance(a, float) and isinstance(b, float):
        if (a != a and b != b) or abs(a - b) <= 1e-12 * max(1.0, abs(a)):
            return b  # equal within the conversion, or both missing (NaN) in the data pack
    return a


def test_refusals():
    d = library.export_param("GFN2-xTB")
    bad = dict(d)
    del bad["hamiltonian"]
    with pytest.raises(TBLiteRuntimeError, match="No entry for xTB Hamiltonian found"):
        library.param_from_dict(bad)
    bad = {k: v for k, v in d.items()}
    bad["charge"] = {"effective": {"gexp": 2.0, "average": "median"}}
    with pytest.raises(TBLiteRuntimeError, match="Invalid 'median' averaging"):
        library.param_from_dict(bad)
    bad = {k: v for k, v in d.items()}
    bad["element"] = {"O": {k: v for k, v in d["element"]["O"].items() if k != "levels"}}
    with pytest.raises(TBLiteRuntimeError, match="No atomic levels specified for O"):
        library.param_from_dict(bad)
    # a GFN1-form record whose element-pair factors follow neither GFN1-xTB nor IPEA1-xTB
    from tblite_gb300 import workloads
    from tblite_gb300.interface import Calculator

    g1 = library.export_param("GFN1-xTB")
    g1["hamiltonian"]["xtb"]["kpair"]["H-H"] = 0.5
    z, x = workloads.water_cluster((2, 1, 1), seed=11)
    with pytest.raises(TBLiteRuntimeError, match="element-pair scaling factors"):
        Calculator(g1, z, x)


def test_xtb_calculator_basis_matches_builtin():
    from tblite_gb300 import workloads
    from tblite_gb300.interface import Calculator

    z, x = workloads.water_cluster((2, 1, 1), seed=11)
    for method in ("GFN2-xTB", "GFN1-xTB", "IPEA1-xTB"):
        a = Calculator(method, z, x)
        b = Calculator(library.export_param(method), z, x)
        for key in ("shell-map", "angular-momenta", "orbital-map"):
            assert np.array_equal(a.get(key), b.get(key))
    # a form the GPU engine does not have is refused
    d = library.export_param("GFN2-xTB")
    d["hamiltonian"]["xtb"]["cn"] = "erf"
    with pytest.raises(TBLiteRuntimeError, match="coordination number"):
        Calculator(d, z, x)


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["GFN2-xTB", "GFN1-xTB"])
def test_exported_record_is_bitwise_the_builtin(method):
    from tblite_gb300 import workloads
    from tblite_gb300.interface import Calculator

    z, x = workloads.alkane(6, seed=5)
    ref = Calculator(method, z, x).singlepoint()
    # the record as exported, without the table (no unit conversion)
    lib = library.load()
    err = library._Error()
    p = library.Param()
    getattr(lib, "tblite_export_gfn2_param" if method == "GFN2-xTB"
            else "tblite_export_gfn1_param")(err.h, p.h)
    err.check()
    calc = Calculator(method, z, x)  # structure and context; the calculator is replaced
    lib.tblite_delete_calculator(__import__("ctypes").byref(calc._calc))
    calc._calc = library.new_xtb_calculator(calc._ctx, calc._mol, p.h)
    res = calc.singlepoint()
    assert res.get("energy") == ref.get("energy")
    # the gradient kernels sum some pair terms with atomics: equal to the last bits
    assert np.max(np.abs(res.get("gradient") - ref.get("gradient"))) < 1e-14
    # through the table in the TOML layout (levels in eV and back)
    res2 = Calculator(library.export_param(method), z, x).singlepoint()
    assert abs(res2.get("energy") - ref.get("energy")) < 1e-10
    assert np.max(np.abs(res2.get("gradient") - ref.get("gradient"))) < 1e-9


@pytest.mark.gpu
def test_changed_level_matches_parameter_gradient():
    """A custom parameter set: the oxygen 2p level moved by h (in eV, through the table) changes
    the energy by h x dE/d(level) summed over the O 2p shells, the analytic parameter gradient of
    the built-in calculator."""
    from tblite_gb300 import workloads
    from tblite_gb300.interface import Calculator

    z, x = workloads.water_cluster((2, 1, 1), seed=11)
    base = Calculator("GFN2-xTB", z, x)
    base.set("accuracy", 1e-5)
    library.set_parameter_gradient(base._ctx, base._calc, True)
    res = base.singlepoint()
    dse = np.zeros(len(base.get("shell-map")))
    dk, dh, dg = np.zeros_like(dse), np.zeros_like(dse), np.zeros_like(dse)
    lib = library.load()
    err = library._Error()
    lib.tblite_gb300_get_result_parameter_gradient(err.h, res._res, library._dp(dse),
                                                   library._dp(dk), library._dp(dh),
                                                   library._dp(dg))
    err.check()
    sh_at, ang = base.get("shell-map"), base.get("angular-momenta")
    o2p = [i for i in range(len(dse)) if z[sh_at[i]] == 8 and ang[i] == 1]
    h = 1e-4  # eV
    energies = []
    for sign in (1.0, -1.0):
        d = library.export_param("GFN2-xTB")
        d["element"]["O"]["levels"][1] += sign * h
        c = Calculator(d, z, x)
        c.set("accuracy", 1e-5)
        energies.append(c.singlepoint().get("energy"))
    fd = (energies[0] - energies[1]) / (2 * h / EV)
    assert abs(fd - float(np.sum(dse[o2p]))) < 1e-6
