"""ctypes binding of the C ABI in ``include/tblite.h`` (libtblite_gb300.so).

Mirrors the role of the reference's CFFI layer (python/tblite/library.py):
every wrapper checks the error handle / context after the call and raises
``TBLiteRuntimeError`` with the library's message.  The shared library is the
in-tree CUDA build; if it is missing or fails to load, importing the wrappers
raises -- there is no CPU implementation behind this module.
"""
from __future__ import annotations

import ctypes
import os
import threading
from ctypes import POINTER, byref, c_bool, c_char_p, c_double, c_int, c_void_p
from pathlib import Path

import numpy as np

from .exceptions import TBLiteRuntimeError, TBLiteValueError

_LIB = None
_dbl_p = POINTER(c_double)
_int_p = POINTER(c_int)


def library_path() -> Path:
    env = os.environ.get("TBLITE_GB300_LIBRARY")
    if env:
        return Path(env)
    return Path(__file__).resolve().parent / "lib" / "libtblite_gb300.so"


_SIGNATURES = {
    "tblite_get_version": (c_int, []),
    "tblite_get_feature": (c_int, [c_char_p]),
    "tblite_new_error": (c_void_p, []),
    "tblite_delete_error": (None, [POINTER(c_void_p)]),
    "tblite_check_error": (c_int, [c_void_p]),
    "tblite_clear_error": (None, [c_void_p]),
    "tblite_get_error": (None, [c_void_p, c_char_p, _int_p]),
    "tblite_set_error": (None, [c_void_p, c_char_p, _int_p]),
    "tblite_new_context": (c_void_p, []),
    "tblite_delete_context": (None, [POINTER(c_void_p)]),
    "tblite_check_context": (c_int, [c_void_p]),
    "tblite_get_context_error": (None, [c_void_p, c_char_p, _int_p]),
    "tblite_set_context_logger": (None, [c_void_p, c_void_p, c_void_p]),
    "tblite_set_context_color": (None, [c_void_p, c_int]),
    "tblite_set_context_verbosity": (None, [c_void_p, c_int]),
    "tblite_new_structure": (c_void_p, [c_void_p, c_int, _int_p, _dbl_p, _dbl_p, _int_p, _dbl_p,
                                        POINTER(c_bool)]),
    "tblite_delete_structure": (None, [POINTER(c_void_p)]),
    "tblite_update_structure_geometry": (None, [c_void_p, c_void_p, _dbl_p, _dbl_p]),
    "tblite_update_structure_charge": (None, [c_void_p, c_void_p, _dbl_p]),
    "tblite_update_structure_uhf": (None, [c_void_p, c_void_p, _int_p]),
    "tblite_new_result": (c_void_p, []),
    "tblite_copy_result": (c_void_p, [c_void_p]),
    "tblite_delete_result": (None, [POINTER(c_void_p)]),
    "tblite_new_gfn2_calculator": (c_void_p, [c_void_p, c_void_p, c_void_p]),
    "tblite_new_gfn1_calculator": (c_void_p, [c_void_p, c_void_p, c_void_p]),
    "tblite_delete_calculator": (None, [POINTER(c_void_p)]),
    "tblite_set_calculator_accuracy": (None, [c_void_p, c_void_p, c_double]),
    "tblite_set_calculator_max_iter": (None, [c_void_p, c_void_p, c_int]),
    "tblite_set_calculator_mixer_damping": (None, [c_void_p, c_void_p, c_double]),
    "tblite_set_calculator_mixer_memory": (None, [c_void_p, c_void_p, c_int]),
    "tblite_set_calculator_mixer": (None, [c_void_p, c_void_p, c_int]),
    "tblite_set_calculator_temperature_annealing": (None, [c_void_p, c_void_p, c_double, c_int,
                                                           c_int]),
    "tblite_set_calculator_guess": (None, [c_void_p, c_void_p, c_int]),
    "tblite_set_calculator_temperature": (None, [c_void_p, c_void_p, c_double]),
    "tblite_set_calculator_save_integrals": (None, [c_void_p, c_void_p, c_int]),
    "tblite_get_calculator_shell_count": (None, [c_void_p, c_void_p, _int_p]),
    "tblite_get_calculator_shell_map": (None, [c_void_p, c_void_p, _int_p]),
    "tblite_get_calculator_angular_momenta": (None, [c_void_p, c_void_p, _int_p]),
    "tblite_get_calculator_orbital_count": (None, [c_void_p, c_void_p, _int_p]),
    "tblite_get_calculator_orbital_map": (None, [c_void_p, c_void_p, _int_p]),
    "tblite_get_singlepoint": (None, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "tblite_new_alpb_solvation_solvent": (c_void_p, [c_void_p, c_void_p, c_char_p, c_int, c_int]),
    "tblite_new_gb_solvation_epsilon": (c_void_p, [c_void_p, c_void_p, c_double, c_int, c_int]),
    "tblite_new_electric_field": (c_void_p, [_dbl_p]),
    "tblite_calculator_push_back": (None, [c_void_p, c_void_p, POINTER(c_void_p)]),
    "tblite_delete_container": (None, [POINTER(c_void_p)]),
    # extensions (include/tblite_gb300_ext.h)
    "tblite_gb300_set_profiling": (None, [c_int]),
    "tblite_gb300_get_profile": (c_int, [_dbl_p, _int_p, c_int, _dbl_p, _int_p]),
    "tblite_gb300_get_launch_count": (ctypes.c_ulonglong, []),
    "tblite_gb300_get_split_gemm_flops": (ctypes.c_ulonglong, []),
    "tblite_gb300_get_result_bond_order_channels": (c_int, [c_void_p]),
    "tblite_gb300_set_calculator_parameter_gradient": (None, [c_void_p, c_void_p, c_int]),
    "tblite_gb300_get_calculator_shell_parameters": (
        None, [c_void_p, c_void_p, _dbl_p, _dbl_p, _dbl_p, _dbl_p]),
    "tblite_gb300_set_calculator_shell_parameters": (
        None, [c_void_p, c_void_p, _dbl_p, _dbl_p, _dbl_p, _dbl_p]),
    "tblite_gb300_get_result_parameter_gradient": (
        None, [c_void_p, c_void_p, _dbl_p, _dbl_p, _dbl_p, _dbl_p]),
    "tblite_gb300_get_kernel_profile": (c_int, [_dbl_p, _int_p, c_int]),
    "tblite_gb300_set_split_gemm": (None, [c_int]),
    "tblite_gb300_set_batch_streams": (None, [c_int]),
    "tblite_gb300_set_projection_threshold": (c_int, [c_int]),
    "tblite_gb300_set_small_tridiag": (None, [c_int]),
    "tblite_gb300_set_tridiag_ctas_per_sm": (None, [c_int]),
    "tblite_gb300_get_calculator_slater_exponents": (None, [c_void_p, c_void_p, _dbl_p]),
    "tblite_gb300_set_calculator_slater_exponents": (None, [c_void_p, c_void_p, _dbl_p]),
    "tblite_gb300_get_result_slater_gradient": (None, [c_void_p, c_void_p, _dbl_p]),
    "tblite_gb300_set_calculator_density_solver": (None, [c_void_p, c_void_p, c_int]),
    "tblite_gb300_split_gemm": (
        c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "tblite_gb300_set_pipelined_gemm": (None, [c_int]),
    "tblite_gb300_get_result_gap": (None, [c_void_p, c_void_p, _dbl_p]),
    "tblite_gb300_get_result_shell_charges": (None, [c_void_p, c_void_p, _dbl_p]),
    "tblite_get_post_processing_dict": (c_void_p, [c_void_p, c_void_p]),
    "tblite_get_n_entries_dict": (c_int, [c_void_p, c_void_p]),
    "tblite_get_array_size_index": (None, [c_void_p, c_void_p, _int_p, _int_p, _int_p, _int_p]),
    "tblite_get_array_entry_index": (None, [c_void_p, c_void_p, _int_p, _dbl_p]),
    "tblite_get_array_size_label": (None, [c_void_p, c_void_p, c_char_p, _int_p, _int_p,
                                           _int_p]),
    "tblite_get_array_entry_label": (None, [c_void_p, c_void_p, c_char_p, _dbl_p]),
    "tblite_get_label_entry_index": (None, [c_void_p, c_void_p, _int_p, c_char_p, _int_p]),
    "tblite_delete_double_dictionary": (None, [POINTER(c_void_p)]),
    "tblite_push_back_post_processing_str": (None, [c_void_p, c_void_p, c_void_p, c_char_p]),
    "tblite_save_result_wavefunction": (None, [c_void_p, c_void_p, c_char_p]),
    "tblite_load_result_wavefunction": (None, [c_void_p, c_void_p, c_char_p]),
    "tblite_gb300_density_matrix_noalloc": (
        c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tblite_gb300_density_matrix_noalloc_max": (c_int, []),
    "tblite_gb300_batch_singlepoint": (
        c_int, [c_void_p, c_int, POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p), _int_p]),
    "tblite_gb300_batch_last_fallbacks": (c_int, []),
    "tblite_gb300_set_batch_density_solver": (None, [c_int]),
    "tblite_gb300_set_calculator_fault": (None, [c_void_p, c_void_p, c_int]),
    "tblite_gb300_set_pipeline_wait_limit": (c_int, [c_int]),
    "tblite_gb300_get_pipe_batch_flops": (ctypes.c_ulonglong, []),
    "tblite_gb300_batch_last_projected": (c_int, []),
    "tblite_gb300_batch_last_modes": (c_int, [_int_p, c_int]),
    "tblite_gb300_batch_autotune": (c_int, [c_void_p, c_int, POINTER(c_void_p), POINTER(c_void_p),
                                            c_int]),
    "tblite_gb300_batch_schedule": (c_int, [c_char_p, c_int]),
    "tblite_gb300_batch_reset_schedule": (None, []),
    "tblite_gb300_set_batch_graphs": (None, [c_int]),
    "tblite_gb300_batch_last_graphs": (c_int, [_int_p, _int_p]),
    "tblite_gb300_batch_last_device_ms": (c_double, []),
    "tblite_gb300_batch_last_host_ms": (c_int, [POINTER(c_double), c_int]),
    "tblite_gb300_batch_last_iterations": (c_int, [_int_p, c_int]),
}
_c64p = POINTER(ctypes.c_int64)
_bp = POINTER(c_bool)
_SIGNATURES.update({
    "tblite_new_param": (c_void_p, []),
    "tblite_delete_param": (None, [POINTER(c_void_p)]),
    "tblite_load_param": (None, [c_void_p, c_void_p, c_void_p]),
    "tblite_dump_param": (None, [c_void_p, c_void_p, c_void_p]),
    "tblite_export_gfn2_param": (None, [c_void_p, c_void_p]),
    "tblite_export_gfn1_param": (None, [c_void_p, c_void_p]),
    "tblite_export_ipea1_param": (None, [c_void_p, c_void_p]),
    "tblite_new_xtb_calculator": (c_void_p, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "tblite_new_ipea1_calculator": (c_void_p, [c_void_p, c_void_p, c_void_p]),
    "tblite_push_back_post_processing_param": (None, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "tblite_new_table": (c_void_p, [c_void_p]),
    "tblite_delete_table": (None, [POINTER(c_void_p)]),
    "tblite_table_set_double": (None, [c_void_p, c_void_p, c_char_p, _dbl_p, c_int]),
    "tblite_table_set_int64_t": (None, [c_void_p, c_void_p, c_char_p, _c64p, c_int]),
    "tblite_table_set_bool": (None, [c_void_p, c_void_p, c_char_p, _bp, c_int]),
    "tblite_table_set_char": (None, [c_void_p, c_void_p, c_char_p, c_char_p, c_int]),
    "tblite_table_add_table": (c_void_p, [c_void_p, c_void_p, c_char_p]),
    "tblite_new_array": (c_void_p, []),
    "tblite_delete_array": (None, [POINTER(c_void_p)]),
    "tblite_array_push_back_double": (None, [c_void_p, c_void_p, c_double]),
    "tblite_array_push_back_int64_t": (None, [c_void_p, c_void_p, ctypes.c_int64]),
    "tblite_array_push_back_bool": (None, [c_void_p, c_void_p, c_bool]),
    "tblite_array_push_back_char": (None, [c_void_p, c_void_p, c_char_p]),
    "tblite_array_size": (c_int, [c_void_p, c_void_p]),
    "tblite_array_get_type": (c_int, [c_void_p, c_void_p, c_int]),
    "tblite_array_get_double": (None, [c_void_p, c_void_p, c_int, _dbl_p]),
    "tblite_array_get_int64_t": (None, [c_void_p, c_void_p, c_int, _c64p]),
    "tblite_array_get_bool": (None, [c_void_p, c_void_p, c_int, _bp]),
    "tblite_array_get_char": (None, [c_void_p, c_void_p, c_int, c_char_p, c_int]),
    "tblite_table_set_array": (None, [c_void_p, c_void_p, c_char_p, c_void_p]),
    "tblite_table_get_type": (c_int, [c_void_p, c_void_p, c_char_p]),
    "tblite_table_get_bool": (None, [c_void_p, c_void_p, c_char_p, _bp]),
    "tblite_table_get_int64_t": (None, [c_void_p, c_void_p, c_char_p, _c64p]),
    "tblite_table_get_double": (None, [c_void_p, c_void_p, c_char_p, _dbl_p]),
    "tblite_table_get_char": (None, [c_void_p, c_void_p, c_char_p, c_char_p, c_int]),
    "tblite_table_get_table": (c_void_p, [c_void_p, c_void_p, c_char_p]),
    "tblite_table_get_array": (c_void_p, [c_void_p, c_void_p, c_char_p]),
    "tblite_table_get_n_keys": (c_int, [c_void_p, c_void_p]),
    "tblite_table_get_key": (None, [c_void_p, c_void_p, c_int, c_char_p, c_int]),
    "tblite_dump_table": (None, [c_void_p, c_void_p, c_char_p]),
})
for _name in ("number_of_atoms", "number_of_shells", "number_of_orbitals", "number_of_spins"):
    _SIGNATURES[f"tblite_get_result_{_name}"] = (None, [c_void_p, c_void_p, _int_p])
for _name in ("energy", "energies", "gradient", "virial", "charges", "bond_orders", "dipole",
              "quadrupole", "orbital_energies", "orbital_occupations", "orbital_coefficients",
              "density_matrix", "overlap_matrix", "hamiltonian_matrix"):
    _SIGNATURES[f"tblite_get_result_{_name}"] = (None, [c_void_p, c_void_p, _dbl_p])


def load():
    """Load the CUDA engine; raises if the in-tree build is missing."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not path.exists():
            raise TBLiteRuntimeError(
                f"CUDA engine library not found at {path}; run tblite_gb300._build.build()")
        lib = ctypes.CDLL(str(path))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


PHASES = ("setup", "potential", "fock", "eigensolve", "density", "mulliken", "mixer",
          "gradient", "transfer")


def set_profiling(enable: bool) -> None:
    load().tblite_gb300_set_profiling(int(bool(enable)))


def set_batch_density_solver(solver: str) -> None:
    """Density solver of the batched SCF for closed shells of >= 96 orbitals (the projection
    threshold): "purification"
    (default, spectral projection on the tensor cores) or "diagonalization"."""
    code = DENSITY_SOLVERS.get(solver, solver) if isinstance(solver, str) else int(solver)
    if not isinstance(code, int):
        raise TBLiteValueError(f"Unknown density solver '{solver}'")
    load().tblite_gb300_set_batch_density_solver(code)


def batch_autotune(calculators, sample: int = 256) -> int:
    """Tune the batch schedule on a sample of these calculators' molecules (see
    tblite_gb300_batch_autotune); returns the number of timed calls."""
    lib = load()
    calcs = list(calculators)
    n = len(calcs)
    mols = (c_void_p * n)(*[c._mol.value for c in calcs])
    hcalc = (c_void_p * n)(*[c._calc.value for c in calcs])
    ctx = new_context(verbosity=0)
    try:
        rc = lib.tblite_gb300_batch_autotune(ctx, n, mols, hcalc, int(sample))
    finally:
        lib.tblite_delete_context(byref(ctx))
    if rc < 0:
        raise TBLiteRuntimeError("batch autotuning failed on its sample")
    return rc


def batch_schedule() -> str:
    """The current batch schedule as text."""
    buf = ctypes.create_string_buffer(512)
    load().tblite_gb300_batch_schedule(buf, 512)
    return buf.value.decode()


def set_batch_graphs(enable: bool) -> None:
    """Run the batched SCF iterations as CUDA graphs (default) or launch kernels directly."""
    load().tblite_gb300_set_batch_graphs(1 if enable else 0)


def batch_graphs():
    """(instantiations, graph launches) of the last batch call."""
    b, n = c_int(0), c_int(0)
    load().tblite_gb300_batch_last_graphs(byref(b), byref(n))
    return b.value, n.value


def batch_graphs_enabled() -> bool:
    """Whether batched SCF iterations run as CUDA graphs (the autotuner may switch them off)."""
    return bool(load().tblite_gb300_batch_last_graphs(None, None))


BATCH_HOST_PHASES = ("plans", "chunking", "staging", "unpacking", "one_molecule_path", "call")


def batch_host_ms() -> dict:
    """Host wall time (ms) of the last batch call by phase (the device time is
    ``tblite_gb300_batch_last_device_ms``)."""
    out = np.zeros(len(BATCH_HOST_PHASES), dtype=np.float64)
    load().tblite_gb300_batch_last_host_ms(_dp(out), out.size)
    return {k: float(v) for k, v in zip(BATCH_HOST_PHASES, out)}


def batch_projected() -> int:
    """Molecules of the last batch call whose SCF density came from the spectral projection."""
    return int(load().tblite_gb300_batch_last_projected())


def set_small_tridiag(full_storage: bool) -> None:
    """Small batch buckets: one-CTA full-storage tridiagonalisation (default) or the packed
    lower-triangle kernel."""
    load().tblite_gb300_set_small_tridiag(1 if full_storage else 0)


def set_batch_streams(count: int) -> None:
    """Streams a batch call spreads its size buckets over (1 serialises them)."""
    load().tblite_gb300_set_batch_streams(int(count))


def set_projection_threshold(nao: int) -> int:
    """Smallest orbital count of a closed shell that takes the spectral projection in the
    batch (0 only queries); returns the previous value."""
    return int(load().tblite_gb300_set_projection_threshold(int(nao)))


def set_tridiag_ctas_per_sm(count: int) -> None:
    """Schedule of the batched tridiagonalisation: 1 or 2 CTAs per SM."""
    load().tblite_gb300_set_tridiag_ctas_per_sm(int(count))


def set_split_gemm(enable: bool) -> None:
    """Batched GEMMs on the BF16 tensor cores with FP64-accurate splitting (default) or FP64."""
    load().tblite_gb300_set_split_gemm(int(bool(enable)))


def get_profile():
    """Per-phase device times (ms) of the last single point, from CUDA events."""
    lib = load()
    ms = np.zeros(len(PHASES))
    cnt = np.zeros(len(PHASES), dtype=np.int32)
    tot = c_double(0.0)
    it = c_int(0)
    lib.tblite_gb300_get_profile(_dp(ms), _ip(cnt), len(PHASES), byref(tot), byref(it))
    return {"phase_ms": dict(zip(PHASES, ms.tolist())), "phase_count": dict(zip(PHASES, cnt.tolist())),
            "total_ms": tot.value, "iterations": it.value}


KERNEL_SLOTS = ("tridiag", "multisect", "invit", "backtransform", "gemm", "fock", "mulliken",
                "pipe_products", "pipe_operands")


def get_kernel_profile():
    """Per-kernel device times (ms, summed over launches) and launch counts of the last single
    point, from CUDA events around each launch on the engine stream."""
    lib = load()
    ms = np.zeros(len(KERNEL_SLOTS))
    cnt = np.zeros(len(KERNEL_SLOTS), dtype=np.int32)
    lib.tblite_gb300_get_kernel_profile(_dp(ms), _ip(cnt), len(KERNEL_SLOTS))
    return {k: (float(t), int(c)) for k, t, c in zip(KERNEL_SLOTS, ms, cnt)}


def launch_count() -> int:
    return int(load().tblite_gb300_get_launch_count())


def pipe_batch_flops() -> int:
    """FP64-equivalent flop (2 m n K per output tile) of the batched projection squarings on the
    tensor cores since library load (counted on the device)."""
    return int(load().tblite_gb300_get_pipe_batch_flops())


def split_gemm_flops() -> int:
    """Algorithmic FP64 flop issued to the one-molecule split GEMM since library load."""
    return int(load().tblite_gb300_get_split_gemm_flops())


def exported_symbols():
    return list(_SIGNATURES)


# ----------------------------------------------------------------------------- helpers
def _dp(a):
    return a.ctypes.data_as(_dbl_p)


def _ip(a):
    return a.ctypes.data_as(_int_p)


class _Error:
    def __init__(self):
        self.lib = load()
        self.h = c_void_p(self.lib.tblite_new_error())

    def check(self):
        if self.lib.tblite_check_error(self.h):
            buf = ctypes.create_string_buffer(512)
            size = c_int(512)
            self.lib.tblite_get_error(self.h, buf, byref(size))
            self.lib.tblite_clear_error(self.h)
            raise TBLiteRuntimeError(buf.value.decode())

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.tblite_delete_error(byref(self.h))


_tls = threading.local()


def _thread_error() -> _Error:
    """One error handle per thread, reused by the result getters (``check`` clears it)."""
    err = getattr(_tls, "err", None)
    if err is None:
        err = _tls.err = _Error()
    return err


def context_check(ctx):
    lib = load()
    if lib.tblite_check_context(ctx):
        buf = ctypes.create_string_buffer(512)
        size = c_int(512)
        msgs = []
        while lib.tblite_check_context(ctx):
            lib.tblite_get_context_error(ctx, buf, byref(size))
            msgs.append(buf.value.decode())
        raise TBLiteRuntimeError("\n".join(msgs))


def new_context(verbosity: int = 0):
    lib = load()
    ctx = c_void_p(lib.tblite_new_context())
    lib.tblite_set_context_verbosity(ctx, int(verbosity))
    return ctx


def new_structure(numbers, positions, charge=None, uhf=None):
    lib = load()
    err = _Error()
    num = np.ascontiguousarray(numbers, dtype=np.int32)
    pos = np.ascontiguousarray(positions, dtype=np.float64)
    ch = None if charge is None else byref(c_double(float(charge)))
    u = None if uhf is None else byref(c_int(int(uhf)))
    mol = c_void_p(lib.tblite_new_structure(err.h, len(num), _ip(num), _dp(pos), ch, u, None, None))
    err.check()
    return mol


def update_geometry(mol, positions):
    lib = load()
    err = _Error()
    pos = np.ascontiguousarray(positions, dtype=np.float64)
    lib.tblite_update_structure_geometry(err.h, mol, _dp(pos), None)
    err.check()


def new_gfn2_calculator(ctx, mol):
    lib = load()
    calc = c_void_p(lib.tblite_new_gfn2_calculator(ctx, mol, None))
    context_check(ctx)
    return calc


def set_parameter_gradient(ctx, calc, enable=True):
    """Request dE/d(shell parameters) with the next single point (GFN2-xTB calculators)."""
    load().tblite_gb300_set_calculator_parameter_gradient(ctx, calc, 1 if enable else 0)
    context_check(ctx)


def new_xtb_calculator(ctx, mol, param):
    """Calculator from a parametrisation record handle (tblite_new_xtb_calculator)."""
    lib = load()
    calc = c_void_p(lib.tblite_new_xtb_calculator(ctx, mol, param, None))
    context_check(ctx)
    return calc


class Param:
    """A parametrisation record handle (tblite_param), freed with the object."""

    def __init__(self):
        self.h = c_void_p(load().tblite_new_param())

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            load().tblite_delete_param(byref(h))


class Table:
    """A data table handle (tblite_table), freed with the object."""

    def __init__(self, handle=None):
        self.h = c_void_p(handle if handle is not None else load().tblite_new_table(None))

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            load().tblite_delete_table(byref(h))


def _set_entry(lib, err, table, key: bytes, value):
    if isinstance(value, dict):
        sub = Table(lib.tblite_table_add_table(err.h, table, key))
        err.check()
        for k, v in value.items():
            _set_entry(lib, err, sub.h, str(k).encode(), v)
    elif isinstance(value, (list, tuple, np.ndarray)):
        arr = c_void_p(lib.tblite_new_array())
        try:
            for v in (value.tolist() if isinstance(value, np.ndarray) else value):
                if isinstance(v, (bool, np.bool_)):
                    lib.tblite_array_push_back_bool(err.h, arr, bool(v))
                elif isinstance(v, (int, np.integer)):
                    lib.tblite_array_push_back_int64_t(err.h, arr, int(v))
                elif isinstance(v, (float, np.floating)):
                    lib.tblite_array_push_back_double(err.h, arr, float(v))
                elif isinstance(v, str):
                    lib.tblite_array_push_back_char(err.h, arr, v.encode())
                else:
                    raise TBLiteValueError(f"Unsupported array entry {v!r}")
            lib.tblite_table_set_array(err.h, table, key, arr)
        finally:
            lib.tblite_delete_array(byref(arr))
    elif isinstance(value, (bool, np.bool_)):
        lib.tblite_table_set_bool(err.h, table, key, byref(c_bool(bool(value))), 0)
    elif isinstance(value, (int, np.integer)):
        lib.tblite_table_set_int64_t(err.h, table, key, byref(ctypes.c_int64(int(value))), 0)
    elif isinstance(value, (float, np.floating)):
        lib.tblite_table_set_double(err.h, table, key, byref(c_double(float(value))), 0)
    elif isinstance(value, str):
        lib.tblite_table_set_char(err.h, table, key, value.encode(), 0)
    else:
        raise TBLiteValueError(f"Unsupported value type {type(value)!r} for '{key.decode()}'")
    err.check()


def dict_to_table(data) -> Table:
    """A data table from a nested mapping (reference library.py dict_to_table)."""
    if not isinstance(data, dict):
        raise TBLiteValueError("Expected a dictionary for parametrization data")
    lib = load()
    err = _Error()
    table = Table()
    for k, v in data.items():
        _set_entry(lib, err, table.h, str(k).encode(), v)
    return table


def table_to_dict(table) -> dict:
    """A nested mapping from a data table handle."""
    lib = load()
    err = _Error()
    h = table.h if isinstance(table, Table) else table
    out = {}
    key = ctypes.create_string_buffer(512)
    for i in range(1, lib.tblite_table_get_n_keys(err.h, h) + 1):
        lib.tblite_table_get_key(err.h, h, i, key, 512)
        err.check()
        k = key.value
        kind = lib.tblite_table_get_type(err.h, h, k)
        if kind == 1:
            v = c_bool()
            lib.tblite_table_get_bool(err.h, h, k, byref(v))
            value = bool(v.value)
        elif kind == 2:
            v = ctypes.c_int64()
            lib.tblite_table_get_int64_t(err.h, h, k, byref(v))
            value = int(v.value)
        elif kind == 3:
            v = c_double()
            lib.tblite_table_get_double(err.h, h, k, byref(v))
            value = float(v.value)
        elif kind == 4:
            buf = ctypes.create_string_buffer(4096)
            lib.tblite_table_get_char(err.h, h, k, buf, 4096)
            value = buf.value.decode()
        elif kind == 5:
            arr = c_void_p(lib.tblite_table_get_array(err.h, h, k))
            try:
                value = []
                for j in range(1, lib.tblite_array_size(err.h, arr) + 1):
                    t = lib.tblite_array_get_type(err.h, arr, j)
                    if t == 1:
                        v = c_bool()
                        lib.tblite_array_get_bool(err.h, arr, j, byref(v))
                        value.append(bool(v.value))
                    elif t == 2:
                        v = ctypes.c_int64()
                        lib.tblite_array_get_int64_t(err.h, arr, j, byref(v))
                        value.append(int(v.value))
                    elif t == 3:
                        v = c_double()
                        lib.tblite_array_get_double(err.h, arr, j, byref(v))
                        value.append(float(v.value))
                    else:
                        buf = ctypes.create_string_buffer(4096)
                        lib.tblite_array_get_char(err.h, arr, j, buf, 4096)
                        value.append(buf.value.decode())
            finally:
                lib.tblite_delete_array(byref(arr))
        elif kind == 6:
            sub = Table(lib.tblite_table_get_table(err.h, h, k))
            value = table_to_dict(sub)
        else:
            raise TBLiteValueError(f"Unsupported table entry for key {k!r}")
        err.check()
        out[k.decode()] = value
    return out


def export_param(method: str) -> dict:
    """The parameters of a built-in method ("GFN2-xTB", "GFN1-xTB" or "IPEA1-xTB") as a nested
    mapping in the reference's TOML layout (tblite_export_*_param, tblite_dump_param)."""
    fn = {"GFN2-xTB": "tblite_export_gfn2_param", "GFN1-xTB": "tblite_export_gfn1_param",
          "IPEA1-xTB": "tblite_export_ipea1_param"}
    if method not in fn:
        raise TBLiteValueError(f"No parameters for method '{method}'")
    lib = load()
    err = _Error()
    p = Param()
    getattr(lib, fn[method])(err.h, p.h)
    err.check()
    t = Table()
    lib.tblite_dump_param(err.h, p.h, t.h)
    err.check()
    return table_to_dict(t)


def param_from_dict(data) -> Param:
    """A parametrisation record loaded from a nested mapping (tblite_load_param)."""
    lib = load()
    table = dict_to_table(data)
    err = _Error()
    p = Param()
    lib.tblite_load_param(err.h, p.h, table.h)
    err.check()
    return p


def new_gfn1_calculator(ctx, mol):
    lib = load()
    calc = c_void_p(lib.tblite_new_gfn1_calculator(ctx, mol, None))
    context_check(ctx)
    return calc


def new_ipea1_calculator(ctx, mol):
    lib = load()
    calc = c_void_p(lib.tblite_new_ipea1_calculator(ctx, mol, None))
    context_check(ctx)
    return calc


def result_array(res, name, shape):
    lib = load()
    err = _thread_error()
    out = np.zeros(shape, dtype=np.float64)
    getattr(lib, f"tblite_get_result_{name}")(err.h, res, _dp(out))
    err.check()
    return out


def post_processing_push_back(ctx, calc, mol, name: str):
    """Add a post-processing step ("bond-orders" or "molmom") to a calculator."""
    load().tblite_push_back_post_processing_str(ctx, calc, mol, name.encode("ascii"))
    context_check(ctx)


def post_processing_dict(res):
    """The post-processing arrays of a result by label (reference library.py:744-774); arrays
    keep the dictionary's dimensions in Fortran order."""
    lib = load()
    err = _Error()
    d = c_void_p(lib.tblite_get_post_processing_dict(err.h, res))
    err.check()
    out = {}
    try:
        for i in range(1, lib.tblite_get_n_entries_dict(err.h, d) + 1):
            idx = c_int(i)
            dims = [c_int(0), c_int(0), c_int(0)]
            lib.tblite_get_array_size_index(err.h, d, byref(idx), *[byref(x) for x in dims])
            err.check()
            shape = tuple(x.value for x in dims if x.value > 0)
            arr = np.zeros(int(np.prod(shape)), dtype=np.float64)
            lib.tblite_get_array_entry_index(err.h, d, byref(idx), _dp(arr))
            label = ctypes.create_string_buffer(512)
            size = c_int(512)
            lib.tblite_get_label_entry_index(err.h, d, byref(idx), label, byref(size))
            err.check()
            out[label.value.decode()] = arr.reshape(shape, order="F")
    finally:
        lib.tblite_delete_double_dictionary(byref(d))
    return out


def result_shell_charges(res):
    """Mulliken shell charges of the last single point (extension getter)."""
    lib = load()
    nsh = result_int(res, "number_of_shells")
    err = _Error()
    out = np.zeros(nsh, dtype=np.float64)
    lib.tblite_gb300_get_result_shell_charges(err.h, res, _dp(out))
    err.check()
    return out


def result_gap(res):
    """HOMO, LUMO and the bound on their errors certified by the spectral-projection solver."""
    lib = load()
    err = _Error()
    out = np.zeros(3, dtype=np.float64)
    lib.tblite_gb300_get_result_gap(err.h, res, _dp(out))
    err.check()
    return out


DENSITY_SOLVERS = {"diagonalization": 0, "diagonalisation": 0, "purification": 1}


def set_density_solver(ctx, calc, solver):
    """Density solver of the next single points: "diagonalization" (default, Fermi filling of
    the eigenvalues) or "purification" (spectral projection on the tensor cores, closed-shell
    systems with a gap of at least 80 kT)."""
    code = DENSITY_SOLVERS.get(solver, solver) if isinstance(solver, str) else int(solver)
    if not isinstance(code, int):
        raise ValueError(f"unknown density solver {solver!r}")
    load().tblite_gb300_set_calculator_density_solver(ctx, calc, code)
    context_check(ctx)


def result_double(res, name):
    lib = load()
    err = _thread_error()
    v = c_double(0.0)
    getattr(lib, f"tblite_get_result_{name}")(err.h, res, byref(v))
    err.check()
    return v.value


def result_int(res, name):
    lib = load()
    err = _thread_error()
    v = c_int(0)
    getattr(lib, f"tblite_get_result_{name}")(err.h, res, byref(v))
    err.check()
    return v.value


SOLUTION_STATES = {"gsolv": 1, "bar1mol": 2, "reference": 3}


def new_alpb_solvation(mol, solvent: str, state: str = "gsolv", version: int = 2):
    """ALPB container for a named solvent (model code 10 + version, as the reference's
    python/tblite/library.py:889-897 passes it)."""
    lib = load()
    if state not in SOLUTION_STATES:
        raise TBLiteValueError(f"Unknown solution state '{state}'")
    err = _Error()
    cont = c_void_p(lib.tblite_new_alpb_solvation_solvent(
        err.h, mol, solvent.encode("ascii"), 10 + int(version), SOLUTION_STATES[state]))
    err.check()
    return cont


def new_gbsa_solvation(mol, solvent: str, state: str = "gsolv", version: int = 2):
    """GBSA container for a named solvent (model code 20 + version, as the reference's
    python/tblite/library.py:900-908 passes it)."""
    return new_alpb_solvation(mol, solvent, state, version=10 + int(version))


BORN_KERNELS = {"still": 1, "p16": 2}


def new_gb_solvation_epsilon(mol, epsilon: float, born: str, alpb: bool):
    """Generalized Born container for a dielectric constant: model code 10 (GB-epsilon with
    the ALPB shape term, "gbe-solvation") or 20 ("gb-solvation"), Born kernel "still" or "p16"
    (python/tblite/library.py:911-922)."""
    lib = load()
    if born not in BORN_KERNELS:
        raise TBLiteValueError(f"Unknown Born kernel '{born}'")
    err = _Error()
    cont = c_void_p(lib.tblite_new_gb_solvation_epsilon(err.h, mol, float(epsilon),
                                                        10 if alpb else 20, BORN_KERNELS[born]))
    err.check()
    return cont


def new_electric_field(efield):
    """Container of a homogeneous electric field (three components, atomic units;
    tblite_new_electric_field)."""
    e = np.ascontiguousarray(efield, dtype=np.float64).reshape(3)
    cont = c_void_p(load().tblite_new_electric_field(_dp(e)))
    if not cont.value:
        raise TBLiteRuntimeError("Could not create the electric field container")
    return cont


def calculator_push_back(ctx, calc, cont):
    load().tblite_calculator_push_back(ctx, calc, byref(cont))
    context_check(ctx)
