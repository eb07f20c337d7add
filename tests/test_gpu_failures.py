"""Failure detection without a GPU fault (needs a GPU for the single points).

* A singular overlap (what coincident atoms produce) is injected on the host into a
  calculator's overlap factorisation: the single point fails with the reference's
  "(sygvd) failed to solve eigenvalue problem. info=n+1" (lapack/sygvd.f90:153-161) and its
  result is not reported; in a batch that molecule fails with the same message while the others
  complete.
* The pipelined split GEMM's pipeline waits are shortened to one poll, so they run out: the
  projection single point fails with an error naming the tensor-core pipeline, the batch hands
  its projected molecules to the one-molecule path (same results), and with the default limit
  restored the same calls succeed on the same context (the GPU stayed usable).
* Non-convergence within the iteration limit is an error with populated results (plain path:
  tests/test_gpu_parity.py; batch: tests/test_gpu_batch.py).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from tblite_gb300 import _build

    _build.build()


def _calc(z, x, **settings):
    from tblite_gb300.interface import Calculator

    c = Calculator("GFN2-xTB", z, x)
    for k, v in settings.items():
        c.set(k, v)
    return c


def test_singular_overlap_plain_and_batch():
    from tblite_gb300 import library, workloads
    from tblite_gb300.exceptions import TBLiteRuntimeError
    from tblite_gb300.interface import batch_singlepoint

    z, x = workloads.water_cluster_k(3, seed=21)
    bad = _calc(z, x)
    library.load().tblite_gb300_set_calculator_fault(bad._ctx, bad._calc, 1)
    n = bad.get("orbital-map").size
    with pytest.raises(TBLiteRuntimeError,
                       match=rf"\(sygvd\) failed to solve eigenvalue problem\. info={n + 1}"):
        bad.singlepoint()
    good = [workloads.alkane(5, seed=22), workloads.water_cluster_k(2, seed=23)]
    calcs = [_calc(*good[0]), bad, _calc(*good[1])]
    from tblite_gb300.interface import Result

    results = [Result() for _ in calcs]
    with pytest.raises(TBLiteRuntimeError, match=r"Batch entry 1: \(sygvd\) failed"):
        batch_singlepoint(calcs, results)
    for (gz, gx), r in zip(good, (results[0], results[2])):
        ref = _calc(gz, gx).singlepoint()
        assert abs(r.get("energy") - ref.get("energy")) < 1e-7
    with pytest.raises(TBLiteRuntimeError):
        results[1].get("energy")
    library.load().tblite_gb300_set_calculator_fault(bad._ctx, bad._calc, 0)
    assert np.isfinite(bad.singlepoint().get("energy"))


def test_pipeline_wait_runs_out():
    from tblite_gb300 import library, workloads
    from tblite_gb300.exceptions import TBLiteRuntimeError
    from tblite_gb300.interface import batch_fallbacks, batch_singlepoint

    lib = library.load()
    z, x = workloads.water_cluster((4, 4, 2), seed=0)  # 192 orbitals: projection on the pipe
    proj = _calc(z, x, **{"density-solver": "purification"})
    ref = proj.singlepoint().get("energy")
    mols = [workloads.alkane(30, seed=31), workloads.water_cluster_k(40, seed=32)]
    refs = [_calc(mz, mx).singlepoint().get("energy") for mz, mx in mols]
    assert lib.tblite_gb300_set_pipeline_wait_limit(1) == 0
    try:
        with pytest.raises(TBLiteRuntimeError, match="tensor-core"):
            proj.singlepoint()
        res = batch_singlepoint([_calc(mz, mx) for mz, mx in mols])
        assert batch_fallbacks() == len(mols)  # every projected molecule was handed off
        assert library.batch_projected() == 0
        for r, e in zip(res, refs):
            assert abs(r.get("energy") - e) < 1e-7
    finally:
        assert lib.tblite_gb300_set_pipeline_wait_limit(0) == 0
    assert abs(proj.singlepoint().get("energy") - ref) < 1e-9
    res = batch_singlepoint([_calc(mz, mx) for mz, mx in mols])
    assert batch_fallbacks() == 0 and library.batch_projected() == len(mols)
