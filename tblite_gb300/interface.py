"""Python surface of the engine: ``Structure``, ``Calculator`` and ``Result``.

Same class names, constructor arguments, ``set``/``get`` keys and
``singlepoint(res=None, copy=False)`` semantics as the reference's
``tblite.interface`` (python/tblite/interface.py:31-685), implemented on the
C ABI of ``libtblite_gb300.so`` (CUDA, FP64).  Inputs and outputs are in
atomic units (Bohr, Hartree).
"""
from __future__ import annotations

from ctypes import byref, c_int, c_void_p
from typing import Optional

import numpy as np

from . import library
from .exceptions import TBLiteRuntimeError, TBLiteTypeError, TBLiteValueError


class Structure:
    """Molecular structure (reference interface.py:31-172)."""

    def __init__(self, numbers, positions, charge: Optional[float] = None,
                 uhf: Optional[int] = None, lattice=None, periodic=None):
        numbers = np.asarray(numbers)
        positions = np.asarray(positions, dtype=np.float64)
        if numbers.ndim != 1:
            raise TBLiteValueError("Expected one dimensional numbers array")
        if positions.shape != (len(numbers), 3):
            raise TBLiteValueError("Expected tripels of cartesian coordinates")
        if lattice is not None or (periodic is not None and np.any(periodic)):
            raise TBLiteValueError("Periodic systems are not supported by the GPU engine")
        self._natoms = len(numbers)
        self._mol = library.new_structure(numbers, positions, charge, uhf)

    def __len__(self):
        return self._natoms

    def update(self, positions, lattice=None):
        positions = np.asarray(positions, dtype=np.float64)
        if positions.shape != (self._natoms, 3):
            raise TBLiteValueError("Dimension missmatch for position")
        library.update_geometry(self._mol, positions)

    def __del__(self):
        mol = getattr(self, "_mol", None)
        if mol is not None and mol.value:
            library.load().tblite_delete_structure(byref(mol))


class Result:
    """Calculation result and restart data (reference interface.py:175-380)."""

    _shapes = {
        "energy": (), "energies": ("nat",), "gradient": ("nat", 3), "virial": (3, 3),
        "charges": ("nat",), "bond-orders": ("nat", "nat"), "dipole": (3,), "quadrupole": (6,),
        "orbital-energies": ("nao",), "orbital-occupations": ("nao",),
        "orbital-coefficients": ("nao", "nao"), "density-matrix": ("nao", "nao"),
        "overlap-matrix": ("nao", "nao"), "hamiltonian-matrix": ("nao", "nao"),
    }

    def __init__(self, other: Optional["Result"] = None):
        lib = library.load()
        if other is not None:
            self._res = c_void_p(lib.tblite_copy_result(other._res))
        else:
            self._res = c_void_p(lib.tblite_new_result())

    def __del__(self):
        res = getattr(self, "_res", None)
        if res is not None and res.value:
            library.load().tblite_delete_result(byref(res))

    def get(self, attribute: str):
        if attribute == "natoms":
            return library.result_int(self._res, "number_of_atoms")
        if attribute == "gap":  # extension: HOMO, LUMO, error bound (spectral projection)
            return library.result_gap(self._res)
        if attribute == "norbitals":
            return library.result_int(self._res, "number_of_orbitals")
        if attribute == "shell-charges":  # extension: Mulliken shell charges
            return library.result_shell_charges(self._res)
        if attribute == "post-processing-dict":
            return library.post_processing_dict(self._res)
        if attribute not in self._shapes:
            raise TBLiteValueError(f"Attribute '{attribute}' is not available in this container")
        dims = {"nat": None, "nao": None}
        shape = self._shapes[attribute]
        if "nat" in shape:
            dims["nat"] = library.result_int(self._res, "number_of_atoms")
        if "nao" in shape:
            dims["nao"] = library.result_int(self._res, "number_of_orbitals")
        real = tuple(dims[s] if isinstance(s, str) else s for s in shape)
        name = attribute.replace("-", "_")
        if attribute == "bond-orders":
            nch = library.load().tblite_gb300_get_result_bond_order_channels(self._res)
            if nch == 2:  # open shell: (nat, nat, 2) total and magnetisation, column-major
                flat = library.result_array(self._res, name, (2 * real[0] * real[1],))
                return flat.reshape((real[0], real[1], 2), order="F")
        if attribute == "energy":
            return library.result_double(self._res, name)
        return library.result_array(self._res, name, real)

    def dict(self):
        out = {}
        for key in ("energy", "gradient", "virial", "charges", "dipole", "orbital-energies",
                    "orbital-occupations", "density-matrix"):
            try:
                out[key] = self.get(key)
            except TBLiteRuntimeError:
                pass
        return out


class Calculator(Structure):
    """Single point calculator (reference interface.py:382-685)."""

    _loader = {
        "GFN2-xTB": library.new_gfn2_calculator,
        "GFN1-xTB": library.new_gfn1_calculator,
        "IPEA1-xTB": library.new_ipea1_calculator,
    }

    def __init__(self, method: str, numbers, positions, charge: Optional[float] = None,
                 uhf: Optional[int] = None, lattice=None, periodic=None, xtb_config=None,
                 **context_kwargs):
        Structure.__init__(self, numbers, positions, charge, uhf, lattice, periodic)
        if isinstance(method, dict):  # a parameter set in the reference's TOML layout
            self._param = library.param_from_dict(method)
            self._ctx = library.new_context(**context_kwargs)
            self._calc = library.new_xtb_calculator(self._ctx, self._mol, self._param.h)
            self._method = "xTB"
            return
        if method not in self._loader:
            raise TBLiteValueError(f"Method '{method}' is not available for this calculator")
        self._ctx = library.new_context(**context_kwargs)
        self._calc = self._loader[method](self._ctx, self._mol)
        self._method = method

    def __del__(self):
        lib = library.load()
        calc = getattr(self, "_calc", None)
        if calc is not None and calc.value:
            lib.tblite_delete_calculator(byref(calc))
        ctx = getattr(self, "_ctx", None)
        if ctx is not None and ctx.value:
            lib.tblite_delete_context(byref(ctx))
        Structure.__del__(self)

    def set(self, attribute: str, value) -> None:
        lib = library.load()
        setters = {
            "accuracy": lambda v: lib.tblite_set_calculator_accuracy(self._ctx, self._calc, float(v)),
            "max-iter": lambda v: lib.tblite_set_calculator_max_iter(self._ctx, self._calc, int(v)),
            "mixer-damping": lambda v: lib.tblite_set_calculator_mixer_damping(self._ctx, self._calc,
                                                                               float(v)),
            "mixer-memory": lambda v: lib.tblite_set_calculator_mixer_memory(self._ctx, self._calc,
                                                                             int(v)),
            "temperature": lambda v: lib.tblite_set_calculator_temperature(self._ctx, self._calc,
                                                                           float(v)),
            "save-integrals": lambda v: lib.tblite_set_calculator_save_integrals(
                self._ctx, self._calc, int(bool(v))),
            "guess": lambda v: lib.tblite_set_calculator_guess(
                self._ctx, self._calc, {"sad": 0, "eeq": 1, "eeqbc": 2}.get(v, v)
                if isinstance(v, str) else int(v)),
            "annealing": lambda v: lib.tblite_set_calculator_temperature_annealing(
                self._ctx, self._calc, float(v[0]), int(v[1]), int(v[2])),
            "verbosity": lambda v: lib.tblite_set_context_verbosity(self._ctx, int(v)),
            # extension: "diagonalization" (default) or "purification" (purify.cu)
            "density-solver": lambda v: library.set_density_solver(self._ctx, self._calc, v),
        }
        if attribute not in setters:
            raise TBLiteValueError(f"Attribute '{attribute}' is not supported in this calculator")
        setters[attribute](value)
        library.context_check(self._ctx)

    def get(self, attribute: str):
        lib = library.load()
        if attribute in ("shell-map", "angular-momenta"):
            nsh = c_int(0)
            lib.tblite_get_calculator_shell_count(self._ctx, self._calc, byref(nsh))
            out = np.zeros(nsh.value, dtype=np.int32)
            fn = (lib.tblite_get_calculator_shell_map if attribute == "shell-map"
                  else lib.tblite_get_calculator_angular_momenta)
            fn(self._ctx, self._calc, library._ip(out))
            library.context_check(self._ctx)
            return out
        if attribute == "orbital-map":
            nao = c_int(0)
            lib.tblite_get_calculator_orbital_count(self._ctx, self._calc, byref(nao))
            out = np.zeros(nao.value, dtype=np.int32)
            lib.tblite_get_calculator_orbital_map(self._ctx, self._calc, library._ip(out))
            library.context_check(self._ctx)
            return out
        raise TBLiteValueError(f"Attribute '{attribute}' is not available in this calculator")

    _post_processing = {"bond-orders": "bond-orders", "molecular-multipoles": "molmom"}

    def add(self, interaction: str, *args) -> None:
        """Add an interaction or a post-processing step (reference interface.py:588-637).

        Interactions: ``"alpb-solvation"`` and ``"gbsa-solvation"`` with the solvent
        ``"water"`` and an optional solution state ``"gsolv"`` (default), ``"bar1mol"`` or
        ``"reference"`` (GFN2 parameters); ``"gbe-solvation"`` and ``"gb-solvation"`` with a
        dielectric constant and the Born kernel ``"still"`` or ``"p16"``; ``"electric-field"``
        with the three components of a homogeneous field (atomic units, GFN2-xTB form).
        Post-processing: ``"bond-orders"`` and ``"molecular-multipoles"`` (computed with every
        single point in the order added; without any, both are computed)."""
        cont = None
        if interaction == "alpb-solvation":
            cont = library.new_alpb_solvation(self._mol, *args, version=2)
        elif interaction == "gbsa-solvation":
            cont = library.new_gbsa_solvation(self._mol, *args, version=2)
        elif interaction == "electric-field":
            cont = library.new_electric_field(*args)
        elif interaction in ("gbe-solvation", "gb-solvation"):
            cont = library.new_gb_solvation_epsilon(self._mol, *args,
                                                    alpb=interaction == "gbe-solvation")
        if cont is not None:
            library.calculator_push_back(self._ctx, self._calc, cont)
            return
        if interaction in self._post_processing:
            library.post_processing_push_back(self._ctx, self._calc, self._mol,
                                              self._post_processing[interaction])
            return
        raise TBLiteValueError(f"Interaction '{interaction}' is not available in the GPU engine")

    def singlepoint(self, res: Optional[Result] = None, copy: bool = False) -> Result:
        if res is not None and not isinstance(res, Result):
            raise TBLiteTypeError("Restart data must be a Result object")
        _res = Result(res) if copy or res is None else res
        library.load().tblite_get_singlepoint(self._ctx, self._mol, self._calc, _res._res)
        library.context_check(self._ctx)
        return _res


def batch_singlepoint(calculators, results=None, verbosity: int = 0):
    """Energies and gradients of many molecules in one batched engine call.

    No counterpart in the reference (one molecule per ``singlepoint`` there).  Each
    ``Calculator`` keeps its own settings; ``results`` (optional, one per calculator) restart
    the molecules like ``Calculator.singlepoint(res)`` does.  Returns the list of ``Result``
    objects; density matrix and orbital coefficients are not kept by the batch.  Raises
    ``TBLiteRuntimeError`` listing every molecule that failed (the others keep their results).
    """
    lib = library.load()
    calcs = list(calculators)
    n = len(calcs)
    if results is None:
        results = [Result() for _ in range(n)]
    elif len(results) != n:
        raise TBLiteValueError("One result per calculator is required")
    mols = (c_void_p * n)(*[c._mol.value for c in calcs])
    hcalc = (c_void_p * n)(*[c._calc.value for c in calcs])
    hres = (c_void_p * n)(*[r._res.value for r in results])
    status = np.zeros(n, dtype=np.int32)
    ctx = library.new_context(verbosity=verbosity)
    try:
        lib.tblite_gb300_batch_singlepoint(ctx, n, mols, hcalc, hres, library._ip(status))
        library.context_check(ctx)
    finally:
        lib.tblite_delete_context(byref(ctx))
    return results


def batch_fallbacks() -> int:
    """Molecules of the last batch call that were evaluated by the one-molecule path."""
    return int(library.load().tblite_gb300_batch_last_fallbacks())
