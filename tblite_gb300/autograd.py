"""``torch.autograd`` bridge: GFN2-xTB energies differentiable in positions and shell parameters.

The energy is evaluated by the CUDA engine (``tblite_get_singlepoint``); the backward pass
returns the engine's analytic nuclear gradient and its parameter gradient
(``tblite_gb300_get_result_parameter_gradient``).  Because the SCF energy is stationary in
the density, both are explicit derivatives at the converged density: no response equations
are solved.

Differentiable shell parameters (one entry per shell of the calculator, in the calculator's
shell order): ``selfenergy`` (se0, Hartree), ``kcn`` (coordination-number shift of the self
energy), ``hubbard`` (chemical hardness), ``hubbard_deriv`` (third-order hardness
derivative) and ``slater`` (the shell's Slater exponent; the STO-nG expansion is redone for a
new value, and dE/dzeta comes from the exponent derivative of the overlap, H0 and multipole
integrals contracted with the converged densities).
"""
from __future__ import annotations

from typing import Dict, Optional, Sequence

import numpy as np

from . import library
from .interface import Calculator, Result

PARAMETERS = ("selfenergy", "kcn", "hubbard", "hubbard_deriv", "slater")
_LEVELS = PARAMETERS[:4]  # set and read together by one C call


def shell_count(calc: Calculator) -> int:
    return int(calc.get("shell-map").size)


def shell_parameters(calc: Calculator) -> Dict[str, np.ndarray]:
    """The calculator's current per-shell parameters."""
    nsh = shell_count(calc)
    out = {k: np.zeros(nsh) for k in PARAMETERS}
    lib = library.load()
    lib.tblite_gb300_get_calculator_shell_parameters(
        calc._ctx, calc._calc, *[library._dp(out[k]) for k in _LEVELS])
    lib.tblite_gb300_get_calculator_slater_exponents(calc._ctx, calc._calc,
                                                     library._dp(out["slater"]))
    library.context_check(calc._ctx)
    return out


def set_shell_parameters(calc: Calculator, **values) -> None:
    """Replace per-shell parameters (keys of ``PARAMETERS``; missing keys stay unchanged)."""
    nsh = shell_count(calc)
    arrays = {}
    for k in PARAMETERS:
        v = values.get(k)
        if v is None:
            continue
        a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1))
        if a.size != nsh:
            raise ValueError(f"{k}: expected {nsh} shell values, got {a.size}")
        arrays[k] = a
    lib = library.load()
    lib.tblite_gb300_set_calculator_shell_parameters(
        calc._ctx, calc._calc,
        *[library._dp(arrays[k]) if k in arrays else None for k in _LEVELS])
    library.context_check(calc._ctx)
    if "slater" in arrays:
        lib.tblite_gb300_set_calculator_slater_exponents(calc._ctx, calc._calc,
                                                         library._dp(arrays["slater"]))
        library.context_check(calc._ctx)


def parameter_gradient(res: Result, nsh: int) -> Dict[str, np.ndarray]:
    """dE/d(parameter) stored by a single point with the parameter gradient enabled."""
    out = {k: np.zeros(nsh) for k in PARAMETERS}
    err = library._Error()
    lib = library.load()
    lib.tblite_gb300_get_result_parameter_gradient(
        err.h, res._res, *[library._dp(out[k]) for k in _LEVELS])
    err.check()
    lib.tblite_gb300_get_result_slater_gradient(err.h, res._res, library._dp(out["slater"]))
    err.check()
    return out


def _torch():
    import torch

    return torch


def _function():
    torch = _torch()

    class GFN2Energy(torch.autograd.Function):
        """E(positions, selfenergy, kcn, hubbard, hubbard_deriv, slater) for one calculator."""

        @staticmethod
        def forward(ctx, calc, positions, selfenergy, kcn, hubbard, hubbard_deriv, slater):
            pos = positions.detach().to("cpu", torch.float64).numpy()
            calc.update(pos)
            set_shell_parameters(
                calc, **{k: t.detach().to("cpu", torch.float64).numpy()
                         for k, t in zip(PARAMETERS,
                                         (selfenergy, kcn, hubbard, hubbard_deriv, slater))})
            library.set_parameter_gradient(calc._ctx, calc._calc)
            res = calc.singlepoint()
            nsh = selfenergy.numel()
            pg = parameter_gradient(res, nsh)
            grads = [torch.from_numpy(res.get("gradient")).to(positions)]
            grads += [torch.from_numpy(pg[k]).to(selfenergy) for k in PARAMETERS]
            ctx.save_for_backward(*grads)
            return torch.tensor(res.get("energy"), dtype=torch.float64, device=positions.device)

        @staticmethod
        def backward(ctx, grad_e):
            g = ctx.saved_tensors
            return (None,) + tuple(grad_e * t for t in g)

    return GFN2Energy


_FN = None


def gfn2_energy(calc: Calculator, positions, selfenergy=None, kcn=None, hubbard=None,
                hubbard_deriv=None, slater=None):
    """Differentiable GFN2-xTB energy (Hartree) of ``calc``'s molecule at ``positions`` (Bohr,
    torch tensor [nat, 3]).  Parameters default to the calculator's current values."""
    global _FN
    torch = _torch()
    if _FN is None:
        _FN = _function()
    cur = shell_parameters(calc)
    vals = []
    for k, v in zip(PARAMETERS, (selfenergy, kcn, hubbard, hubbard_deriv, slater)):
        vals.append(v if v is not None else torch.tensor(cur[k], dtype=torch.float64))
    return _FN.apply(calc, positions, *vals)


def gfn2_energies(calcs: Sequence[Calculator], positions: Sequence, parameters:
                  Optional[Sequence[dict]] = None):
    """Energies of several molecules (one engine call each) as a list of 0-d tensors."""
    out = []
    for i, (calc, pos) in enumerate(zip(calcs, positions)):
        kw = parameters[i] if parameters is not None else {}
        out.append(gfn2_energy(calc, pos, **kw))
    return out


def _batch_function():
    torch = _torch()
    k = 1 + len(PARAMETERS)

    class GFN2EnergyBatch(torch.autograd.Function):
        """E_i(positions_i, parameters_i) for many calculators in one batched engine call
        (tblite_gb300_batch_singlepoint); the forces and dE/dtheta of every molecule come from
        the same call."""

        @staticmethod
        def forward(ctx, calcs, *tensors):
            from .interface import batch_singlepoint

            for i, calc in enumerate(calcs):
                pos, *prm = tensors[k * i:k * (i + 1)]
                calc.update(pos.detach().to("cpu", torch.float64).numpy())
                set_shell_parameters(
                    calc, **{name: t.detach().to("cpu", torch.float64).numpy()
                             for name, t in zip(PARAMETERS, prm)})
                library.set_parameter_gradient(calc._ctx, calc._calc)
            results = batch_singlepoint(list(calcs))
            grads, energies = [], []
            for i, res in enumerate(results):
                pos, sel = tensors[k * i], tensors[k * i + 1]
                pg = parameter_gradient(res, sel.numel())
                grads.append(torch.from_numpy(res.get("gradient")).to(pos))
                grads += [torch.from_numpy(pg[name]).to(sel) for name in PARAMETERS]
                energies.append(res.get("energy"))
            ctx.save_for_backward(*grads)
            ctx.nmol = len(results)
            return torch.tensor(energies, dtype=torch.float64, device=tensors[0].device)

        @staticmethod
        def backward(ctx, grad_e):
            g = ctx.saved_tensors
            out = [None]
            for i in range(ctx.nmol):
                out += [grad_e[i] * t for t in g[k * i:k * (i + 1)]]
            return tuple(out)

    return GFN2EnergyBatch


_FNB = None


def gfn2_energies_batch(calcs: Sequence[Calculator], positions: Sequence,
                        parameters: Optional[Sequence[dict]] = None):
    """Differentiable GFN2-xTB energies of many molecules, evaluated in one batched engine call;
    returns a tensor [nmol] whose backward pass gives every molecule's forces and dE/dtheta."""
    global _FNB
    torch = _torch()
    if _FNB is None:
        _FNB = _batch_function()
    flat = []
    for i, (calc, pos) in enumerate(zip(calcs, positions)):
        kw = parameters[i] if parameters is not None else {}
        cur = shell_parameters(calc)
        flat.append(pos)
        for name in PARAMETERS:
            v = kw.get(name)
            flat.append(v if v is not None else torch.tensor(cur[name], dtype=torch.float64))
    return _FNB.apply(tuple(calcs), *flat)
