"""Batched ensemble path vs the one-molecule path and the CPU oracle (needs a GPU).

The batch runs the same per-molecule arithmetic as tblite_get_singlepoint, except the
eigensolver's Cholesky and tridiagonalisation (one block cluster per molecule instead of a
grid-wide kernel), so the results agree with the plain path to rounding; the bar is the one of
the parity tests: |dE| <= 1e-7 Eh, charges <= 1e-6 e, gradient <= 1e-6 Eh/Bohr.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_TOL, Q_TOL, G_TOL, V_TOL = 1e-7, 1e-6, 1e-6, 1e-5


@pytest.fixture(scope="module", autouse=True)
def built():
    from tblite_gb300 import _build

    _build.build()


def _ensemble():
    from tblite_gb300 import workloads

    mols = []
    for k in (1, 2, 3, 5, 8, 13):
        mols.append(workloads.water_cluster_k(k, seed=100 + k))
    for n in (1, 2, 4, 7, 12, 20):
        mols.append(workloads.alkane(n, seed=200 + n))
    return mols


def _calc(z, x, method="GFN2-xTB", **settings):
    from tblite_gb300.interface import Calculator

    calc = Calculator(method, z, x)
    for k, v in settings.items():
        calc.set(k, v)
    return calc


def _compare(rb, rp):
    assert abs(rb.get("energy") - rp.get("energy")) <= E_TOL
    assert np.max(np.abs(rb.get("charges") - rp.get("charges"))) <= Q_TOL
    assert np.max(np.abs(rb.get("shell-charges") - rp.get("shell-charges"))) <= Q_TOL
    assert np.max(np.abs(rb.get("gradient") - rp.get("gradient"))) <= G_TOL
    assert np.max(np.abs(rb.get("virial") - rp.get("virial"))) <= V_TOL
    assert np.max(np.abs(rb.get("energies") - rp.get("energies"))) <= E_TOL
    assert np.max(np.abs(rb.get("dipole") - rp.get("dipole"))) <= 1e-6


def test_batch_matches_plain_path():
    from tblite_gb300.interface import batch_fallbacks, batch_singlepoint

    mols = _ensemble()
    calcs = [_calc(z, x) for z, x in mols]
    res_b = batch_singlepoint(calcs)
    assert batch_fallbacks() == 0
    for (z, x), rb in zip(mols, res_b):
        rp = _calc(z, x).singlepoint()
        _compare(rb, rp)
        occ_b, occ_p = rb.get("orbital-occupations"), rp.get("orbital-occupations")
        assert np.max(np.abs(occ_b - occ_p)) <= 1e-6


def test_batch_matches_oracle():
    from oracle import gfn2
    from tblite_gb300.interface import batch_singlepoint

    mols = _ensemble()[::3]
    res_b = batch_singlepoint([_calc(z, x) for z, x in mols])
    for (z, x), rb in zip(mols, res_b):
        ref = gfn2.singlepoint(gfn2.new_calc(gfn2.Molecule(np.asarray(z), np.asarray(x))), grad=True)
        assert abs(rb.get("energy") - ref.energy) <= E_TOL
        assert np.max(np.abs(rb.get("gradient") - ref.gradient)) <= G_TOL
        assert np.max(np.abs(rb.get("charges") - ref.qat)) <= Q_TOL
        assert np.max(np.abs(rb.get("shell-charges") - ref.qsh)) <= Q_TOL


def test_batch_per_molecule_settings_and_single_atom():
    from tblite_gb300 import workloads
    from tblite_gb300.interface import batch_singlepoint

    z, x = workloads.water_cluster_k(4, seed=7)
    o_atom = (np.array([8]), np.zeros((1, 3)))
    cases = [((z, x), {"accuracy": 0.01}), ((z, x), {"temperature": 3000 * 3.166808578545117e-6}),
             ((z, x), {"mixer-damping": 0.2}), (o_atom, {})]
    calcs = [_calc(mz, mx, **st) for (mz, mx), st in cases]
    res_b = batch_singlepoint(calcs)
    for ((mz, mx), st), rb in zip(cases, res_b):
        _compare(rb, _calc(mz, mx, **st).singlepoint())


def test_batch_restart_and_fallback():
    from tblite_gb300 import workloads
    from tblite_gb300.exceptions import TBLiteRuntimeError
    from tblite_gb300.interface import Result, batch_fallbacks, batch_singlepoint

    (z1, x1), (z2, x2) = workloads.water_cluster_k(6, seed=11), workloads.alkane(9, seed=12)
    first = batch_singlepoint([_calc(z1, x1), _calc(z2, x2)])
    again = batch_singlepoint([_calc(z1, x1), _calc(z2, x2)], [Result(r) for r in first])
    for a, b in zip(first, again):
        assert abs(a.get("energy") - b.get("energy")) <= E_TOL
    # a molecule that cannot converge in 3 iterations leaves the batch and fails like a plain call
    calcs = [_calc(z1, x1), _calc(z2, x2, **{"max-iter": 3})]
    with pytest.raises(TBLiteRuntimeError, match="Batch entry 1"):
        batch_singlepoint(calcs)
    assert batch_fallbacks() == 1


def test_batch_mixed_methods():
    """GFN1-xTB and GFN2-xTB molecules in one call: each method runs in its own chunk; both
    agree with their plain paths, and the GFN1 molecules with the GFN1 oracle."""
    from oracle import gfn1, gfn2
    from tblite_gb300.interface import batch_fallbacks, batch_singlepoint

    mols = _ensemble()
    methods = ["GFN1-xTB" if i % 2 == 0 else "GFN2-xTB" for i in range(len(mols))]
    res_b = batch_singlepoint([_calc(z, x, m) for (z, x), m in zip(mols, methods)])
    assert batch_fallbacks() == 0
    for (z, x), m, rb in zip(mols, methods, res_b):
        _compare(rb, _calc(z, x, m).singlepoint())
    for (z, x), m, rb in list(zip(mols, methods, res_b))[::4]:
        if m != "GFN1-xTB":
            continue
        ref = gfn1.singlepoint(gfn1.new_calc(gfn2.Molecule(np.asarray(z), np.asarray(x))))
        assert abs(rb.get("energy") - ref.energy) <= E_TOL
        assert np.max(np.abs(rb.get("gradient") - ref.gradient)) <= G_TOL


@pytest.mark.parametrize("method", ["GFN2-xTB", "GFN1-xTB"])
def test_batch_large_molecules(method):
    """Molecules above one CTA's shared memory (the cluster tridiagonalisation with packed
    lower-triangle storage; GFN1 water 64-mers have 512 orbitals) against the plain path."""
    from tblite_gb300 import workloads
    from tblite_gb300.interface import batch_fallbacks, batch_singlepoint

    mols = [workloads.water_cluster_k(40, seed=301), workloads.alkane(50, seed=302),
            workloads.water_cluster_k(64, seed=303), workloads.alkane(30, seed=304)]
    res_b = batch_singlepoint([_calc(z, x, method) for z, x in mols])
    assert batch_fallbacks() == 0
    for (z, x), rb in zip(mols, res_b):
        _compare(rb, _calc(z, x, method).singlepoint())


def test_split_gemm_matches_fp64_gemm():
    """The batched GEMMs on the BF16 tensor cores (FP64-accurate operand splitting) against the
    FP64 tile GEMMs on the same molecules: results agree at the parity bar."""
    from tblite_gb300 import library, workloads
    from tblite_gb300.interface import batch_singlepoint

    mols = [workloads.water_cluster_k(30, seed=401), workloads.alkane(40, seed=402),
            workloads.water_cluster_k(64, seed=403)]
    try:
        library.set_split_gemm(False)
        ref = batch_singlepoint([_calc(z, x) for z, x in mols])
    finally:
        library.set_split_gemm(True)
    res = batch_singlepoint([_calc(z, x) for z, x in mols])
    for a, b in zip(res, ref):
        _compare(a, b)


def test_projection_matches_diagonalisation():
    """Closed shells of >= 96 orbitals take the spectral projection in the batch (SP2 squarings
    on the tensor cores); the same molecules with the batched diagonalisation, and with the
    one-molecule path, agree at the parity bar, bond orders and orbital energies included."""
    from tblite_gb300 import library, workloads
    from tblite_gb300.interface import batch_fallbacks, batch_singlepoint

    # 96-126 orbitals (from the default threshold on) and 132-384
    mols = [workloads.water_cluster_k(k, seed=500 + k) for k in (16, 19, 21, 22, 31, 45, 64)]
    mols += [workloads.alkane(n, seed=520 + n) for n in (21, 33, 47, 60)]
    assert min(_calc(z, x).get("orbital-map").size for z, x in mols) >= 96
    res_p = batch_singlepoint([_calc(z, x) for z, x in mols])
    assert batch_fallbacks() == 0
    assert library.batch_projected() == len(mols)
    try:
        library.set_batch_density_solver("diagonalization")
        res_d = batch_singlepoint([_calc(z, x) for z, x in mols])
        assert library.batch_projected() == 0
    finally:
        library.set_batch_density_solver("purification")
    for (z, x), rp_, rd in zip(mols, res_p, res_d):
        _compare(rp_, rd)
        assert np.max(np.abs(rp_.get("bond-orders") - rd.get("bond-orders"))) <= 1e-6
        assert np.max(np.abs(rp_.get("orbital-energies") - rd.get("orbital-energies"))) <= 1e-6
        assert np.max(np.abs(rp_.get("orbital-occupations")
                             - rd.get("orbital-occupations"))) <= 1e-6
    for (z, x), rp_ in list(zip(mols, res_p))[::3]:
        _compare(rp_, _calc(z, x).singlepoint())


def test_projection_small_gap_leaves_the_batch():
    """A molecule whose final HOMO-LUMO gap is below 80 kT (here: a very high electronic
    temperature makes kT large) cannot use 0/2 occupations; it leaves the batch and the
    one-molecule path gives the reference's Fermi-smeared result."""
    from tblite_gb300 import library, workloads
    from tblite_gb300.interface import batch_fallbacks, batch_singlepoint

    z, x = workloads.alkane(30, seed=540)
    hot = {"temperature": 20000 * 3.166808578545117e-6}
    res = batch_singlepoint([_calc(z, x, **hot), _calc(z, x)])
    assert batch_fallbacks() == 1 and library.batch_projected() == 1
    _compare(res[0], _calc(z, x, **hot).singlepoint())
    _compare(res[1], _calc(z, x).singlepoint())


def test_autotuned_schedule_keeps_results():
    """The autotuner times candidate schedules on a sample and keeps the fastest; results
    under the tuned schedule agree with the one-molecule path."""
    from tblite_gb300 import library, workloads
    from tblite_gb300.interface import batch_singlepoint

    mols = workloads.mixed_ensemble(48, seed=77)
    calcs = [_calc(z, x) for z, x in mols]
    before = library.batch_schedule()
    try:
        assert library.batch_autotune(calcs, sample=24) > 0
        assert "autotuned on 24 molecules" in library.batch_schedule()
        res = batch_singlepoint(calcs)
        for (z, x), r in list(zip(mols, res))[::6]:
            _compare(r, _calc(z, x).singlepoint())
    finally:
        # back to the defaults for the other tests
        library.set_batch_streams(8)
        library.set_tridiag_ctas_per_sm(2)
        library.load().tblite_gb300_batch_reset_schedule()
    assert library.batch_schedule() == before


def test_scf_iterations_as_cuda_graphs():
    """The batched SCF iterations run as CUDA graphs (captured, updated in place, one launch
    per iteration and memory chunk); launching the kernels directly gives the same results."""
    from tblite_gb300 import library, workloads
    from tblite_gb300.interface import batch_singlepoint

    mols = workloads.mixed_ensemble(40, seed=88)
    library.set_profiling(False)
    res_g = batch_singlepoint([_calc(z, x) for z, x in mols])
    builds, launches = library.batch_graphs()
    assert launches > 0 and 0 < builds <= launches
    try:
        library.set_batch_graphs(False)
        res_d = batch_singlepoint([_calc(z, x) for z, x in mols])
        assert library.batch_graphs() == (0, 0)
    finally:
        library.set_batch_graphs(True)
    for a, b in zip(res_g, res_d):
        assert abs(a.get("energy") - b.get("energy")) <= 1e-12
        assert np.max(np.abs(a.get("gradient") - b.get("gradient"))) <= 1e-12


def test_packed_small_tridiagonalisation():
    """Small buckets tridiagonalised by the packed lower-triangle kernel (a cluster of one or two
    CTAs) instead of the one-CTA full-storage kernel: same results as the one-molecule path,
    from the smallest molecules (3 orbitals) up to the largest bucket the small kernel takes."""
    from tblite_gb300 import library, workloads
    from tblite_gb300.interface import batch_fallbacks, batch_singlepoint

    mols = _ensemble() + [workloads.water_cluster_k(26, seed=411),
                          workloads.alkane(25, seed=412)]  # 156 and 152 orbitals
    try:
        library.set_batch_density_solver("diagonalization")  # every bucket diagonalises
        library.set_small_tridiag(False)
        res = batch_singlepoint([_calc(z, x) for z, x in mols])
        assert batch_fallbacks() == 0
    finally:
        library.set_small_tridiag(True)
        library.set_batch_density_solver("purification")
    for (z, x), rb in zip(mols, res):
        _compare(rb, _calc(z, x).singlepoint())


def test_host_phases_and_projection_threshold():
    """The host phases of the last batch call add up to at most the whole call; the projection
    threshold setter returns the previous value and moves molecules between the solvers
    without changing their results beyond the parity bar."""
    from tblite_gb300 import library, workloads
    from tblite_gb300.interface import batch_singlepoint

    mols = [workloads.water_cluster_k(k, seed=560 + k) for k in (17, 20)]  # 102, 120 orbitals
    calcs = [_calc(z, x) for z, x in mols]
    old = library.set_projection_threshold(96)
    try:
        assert library.set_projection_threshold(0) == 96  # query only
        res_p = batch_singlepoint(calcs)
        host = library.batch_host_ms()
        assert set(host) == set(library.BATCH_HOST_PHASES)
        parts = sum(v for k, v in host.items() if k != "call")
        assert all(v >= 0.0 for v in host.values()) and parts <= host["call"] + 1e-6
        assert library.batch_projected() == 2
        assert library.set_projection_threshold(128) == 96
        res_d = batch_singlepoint(calcs)
        assert library.batch_projected() == 0
        for a, b in zip(res_p, res_d):
            _compare(a, b)
    finally:
        library.set_projection_threshold(old)
