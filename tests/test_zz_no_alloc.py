"""Density matrix through the allocation-free entry point (needs a GPU).

tblite_gb300_density_matrix_noalloc takes its workspace from a fixed device array inside the
library.  Its output is compared with the density matrix that tblite_get_singlepoint returns
for the same orbitals and occupations (the engine's own density step), on two calls in a
row, at |dP| <= 1e-12.  The file name sorts last so that the test also runs after every
other test in the session.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P_TOL = 1e-12


@pytest.fixture(scope="module")
def lib():
    from tblite_gb300 import _build, library

    _build.build()
    return library.load()


def _water_dimer():
    z = np.array([8, 1, 1, 8, 1, 1])
    x = np.array([
        [-1.551007, -0.114520, 0.000000],
        [-1.934259, 0.762503, 0.000000],
        [-0.599677, 0.040712, 0.000000],
        [1.350625, 0.111469, 0.000000],
        [1.680398, -0.373741, -0.758561],
        [1.680398, -0.373741, 0.758561],
    ]) * 1.8897261246257702
    return z, x


def _singlepoint():
    from tblite_gb300.interface import Calculator

    z, x = _water_dimer()
    res = Calculator("GFN2-xTB", z, x).singlepoint()
    return (res.get("orbital-coefficients"), res.get("orbital-occupations"),
            res.get("density-matrix"))


def _call(lib, n, k, c_dev, f_dev, p_dev, stream=None):
    import torch

    s = ctypes.c_void_p(stream if stream is not None else torch.cuda.current_stream().cuda_stream)
    return lib.tblite_gb300_density_matrix_noalloc(n, k, ctypes.c_void_p(c_dev.data_ptr()),
                                                   ctypes.c_void_p(f_dev.data_ptr()),
                                                   ctypes.c_void_p(p_dev.data_ptr()), s)


def test_matches_singlepoint_density_twice(lib):
    import torch

    cmat, occ, pmat = _singlepoint()
    n = occ.size
    assert cmat.shape == (n, n) and pmat.shape == (n, n)
    dev = torch.device("cuda:0")
    c_dev = torch.from_numpy(np.ascontiguousarray(cmat)).to(dev)
    f_dev = torch.from_numpy(np.ascontiguousarray(occ)).to(dev)
    k_occ = int(np.count_nonzero(occ > 0.0))
    for k in (n, k_occ):
        outs = []
        for _ in range(2):
            p_dev = torch.full((n, n), np.nan, dtype=torch.float64, device=dev)
            assert _call(lib, n, k, c_dev, f_dev, p_dev) == 0
            torch.cuda.synchronize()
            outs.append(p_dev.cpu().numpy())
        for p in outs:
            assert np.max(np.abs(p - pmat)) <= P_TOL
            assert np.array_equal(p, p.T)  # mirrored, not two roundings of one sum
        assert np.array_equal(outs[0], outs[1])
    # independent check: P = C^T diag(f) C in the row-major view of the column-major buffer
    ref = (cmat.T * occ) @ cmat
    assert np.max(np.abs(outs[0] - ref)) <= 1e-10


def test_no_device_memory_taken(lib):
    import torch

    cmat, occ, _ = _singlepoint()
    n = occ.size
    dev = torch.device("cuda:0")
    c_dev = torch.from_numpy(np.ascontiguousarray(cmat)).to(dev)
    f_dev = torch.from_numpy(np.ascontiguousarray(occ)).to(dev)
    p_dev = torch.empty((n, n), dtype=torch.float64, device=dev)
    assert _call(lib, n, n, c_dev, f_dev, p_dev) == 0  # first call: per-device set-up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(dev)[0]
    for _ in range(3):
        assert _call(lib, n, n, c_dev, f_dev, p_dev) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == free0


def test_rejects_oversized_and_invalid(lib):
    import torch

    cap = lib.tblite_gb300_density_matrix_noalloc_max()
    assert cap == 1 << 19
    dev = torch.device("cuda:0")
    buf = torch.zeros(4, dtype=torch.float64, device=dev)
    # n*k above the fixed workspace: rejected on the host, nothing launched
    n = 1024
    k = cap // n + 1
    assert _call(lib, n, k, buf, buf, buf) == -2
    assert _call(lib, 4, 5, buf, buf, buf) == -1  # k > n
    assert _call(lib, 0, 0, buf, buf, buf) == -1
    assert lib.tblite_gb300_density_matrix_noalloc(4, 2, None, None, None, None) == -1
