"""Differentiation (needs a GPU): the torch.autograd bridge against central finite
differences of the engine's own energies.

Positions: step 0.5e-4 Bohr; parameters: relative step 1e-5.  The SCF is converged tightly
(accuracy 1e-5: |dE| < 1e-11 between iterations); with the relative parameter step of 1e-5
the finite differences then carry up to ~2e-6 of SCF noise, and the tolerances below are
set from that.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def built():
    from tblite_gb300 import _build

    _build.build()


def _calc(z, x):
    from tblite_gb300.interface import Calculator

    calc = Calculator("GFN2-xTB", z, x)
    calc.set("accuracy", 1e-5)
    return calc


def _energy(calc, x, **params):
    from tblite_gb300.autograd import gfn2_energy

    return float(gfn2_energy(calc, torch.tensor(x), **params))


def test_position_gradient_matches_fd():
    from tblite_gb300 import workloads
    from tblite_gb300.autograd import gfn2_energy

    z, x = workloads.alkane(3, seed=5)
    calc = _calc(z, x)
    pos = torch.tensor(x, requires_grad=True)
    e = gfn2_energy(calc, pos)
    e.backward()
    g = pos.grad.numpy()
    h = 0.5e-4
    for a, k in [(0, 0), (1, 2), (4, 1), (len(z) - 1, 0)]:
        xp, xm = x.copy(), x.copy()
        xp[a, k] += h
        xm[a, k] -= h
        fd = (_energy(calc, xp) - _energy(calc, xm)) / (2 * h)
        assert abs(fd - g[a, k]) < 2e-6, (a, k, fd, g[a, k])


@pytest.mark.parametrize("name", ["selfenergy", "kcn", "hubbard", "hubbard_deriv", "slater"])
def test_parameter_gradient_matches_fd(name):
    from tblite_gb300 import workloads
    from tblite_gb300.autograd import PARAMETERS, gfn2_energy, shell_parameters

    z, x = workloads.water_cluster_k(2, seed=9)
    calc = _calc(z, x)
    base = shell_parameters(calc)
    params = {k: torch.tensor(base[k], requires_grad=(k == name)) for k in PARAMETERS}
    e = gfn2_energy(calc, torch.tensor(x), **params)
    e.backward()
    g = params[name].grad.numpy()
    for s in range(len(base[name])):
        v0 = base[name][s]
        h = 1e-5 * max(abs(v0), 1e-2)
        vals = {k: base[k].copy() for k in PARAMETERS}
        vals[name][s] = v0 + h
        ep = _energy(calc, x, **{k: torch.tensor(v) for k, v in vals.items()})
        vals[name][s] = v0 - h
        em = _energy(calc, x, **{k: torch.tensor(v) for k, v in vals.items()})
        fd = (ep - em) / (2 * h)
        assert abs(fd - g[s]) <= 5e-6 + 1e-4 * abs(fd), (name, s, fd, g[s])
    # leave the calculator's parameters as they were
    from tblite_gb300.autograd import set_shell_parameters

    set_shell_parameters(calc, **base)


def test_batched_bridge_matches_one_molecule_path():
    """gfn2_energies_batch (one tblite_gb300_batch_singlepoint call, parameter gradient on the
    batched path) against gfn2_energy per molecule: energies, forces and all five parameter
    gradients at the parity bar."""
    from tblite_gb300 import workloads
    from tblite_gb300.autograd import (PARAMETERS, gfn2_energies_batch, gfn2_energy,
                                       shell_parameters)
    from tblite_gb300.interface import Calculator

    mols = workloads.alkane_batch(6, seed=7, nmin=3, nmax=14)
    single, batch_calcs = [], []
    for z, x in mols:
        calc = Calculator("GFN2-xTB", z, x)
        prm = {k: torch.tensor(v, requires_grad=True) for k, v in shell_parameters(calc).items()}
        pos = torch.tensor(x, requires_grad=True)
        e = gfn2_energy(calc, pos, **prm)
        e.backward()
        single.append((e.item(), pos.grad.numpy(), {k: prm[k].grad.numpy() for k in PARAMETERS}))
        batch_calcs.append(Calculator("GFN2-xTB", z, x))
    pos = [torch.tensor(x, requires_grad=True) for _, x in mols]
    prm = [{k: torch.tensor(v, requires_grad=True) for k, v in shell_parameters(c).items()}
           for c in batch_calcs]
    e = gfn2_energies_batch(batch_calcs, pos, prm)
    e.sum().backward()
    for i, (e1, g1, p1) in enumerate(single):
        assert abs(e[i].item() - e1) < 1e-7
        assert np.max(np.abs(pos[i].grad.numpy() - g1)) < 1e-6
        for k in PARAMETERS:
            assert np.max(np.abs(prm[i][k].grad.numpy() - p1[k])) < 1e-6, k
