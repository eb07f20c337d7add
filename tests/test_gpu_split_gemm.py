"""Pipelined split GEMM (ozaki_pipe.cu) against an FP64 product (needs a GPU).

The kernel splits every FP64 operand into eight 7-bit slices and sums 36 exact BF16 slice
products on the tensor cores; the dropped and truncated terms are ~2^-52 of the row maximum of A
times the column maximum of B per k.
The test compares tblite_gb300_split_gemm (device pointers through the C ABI) with torch's FP64
matmul on shapes that are not multiples of the 128 x 64 tile or of the 32-wide k chunk, with k
over several 192-wide flush windows, rows and columns scaled over six orders of magnitude, and
the symmetric mode (lower tiles computed and mirrored).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# per element, relative to (|A| |B|): the dropped and truncated slice terms are ~2^-52 of
# (row max of A) (column max of B) per k, which for Gaussian entries is ~20 |a| |b|
REL = 2.0 ** -44


@pytest.fixture(scope="module")
def lib():
    from tblite_gb300 import _build, library

    _build.build()
    return library.load()


def _cm(torch, x):
    """numpy (r, c) -> CUDA tensor holding x column-major (shape (c, r), contiguous)."""
    return torch.from_numpy(np.ascontiguousarray(x.T)).cuda()


def _run(lib, a, b, sym=False):
    import torch

    m, k = a.shape
    n = b.shape[1]
    ta, tb = _cm(torch, a), _cm(torch, b)
    tc = torch.full((n, m), np.nan, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.tblite_gb300_split_gemm(m, n, k, ctypes.c_void_p(ta.data_ptr()),
                                     ctypes.c_void_p(tb.data_ptr()),
                                     ctypes.c_void_p(tc.data_ptr()), 1 if sym else 0, None)
    assert rc == 0
    c = tc.cpu().numpy().T
    ref = (torch.from_numpy(a).cuda() @ torch.from_numpy(b).cuda()).cpu().numpy()
    bound = (np.abs(a) @ np.abs(b)) * REL + 1e-300
    return c, ref, bound


@pytest.mark.parametrize("m,n,k", [(128, 64, 32), (200, 136, 300), (70, 50, 700), (257, 129, 17),
                                   (640, 320, 1000)])
def test_general(lib, m, n, k):
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    a = rng.standard_normal((m, k)) * 10.0 ** rng.uniform(-3, 3, size=(m, 1))
    b = rng.standard_normal((k, n)) * 10.0 ** rng.uniform(-3, 3, size=(1, n))
    c, ref, bound = _run(lib, a, b)
    assert np.all(np.isfinite(c))
    assert np.all(np.abs(c - ref) <= bound)


@pytest.mark.parametrize("n", [100, 384, 1000])
def test_symmetric(lib, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, n))
    x = 0.5 * (x + x.T)
    c, ref, bound = _run(lib, x, x, sym=True)
    assert np.array_equal(c, c.T)
    assert np.all(np.abs(c - ref) <= bound)


def test_zero_and_tiny(lib):
    """Zero rows, a zero matrix block and subnormal-range values."""
    rng = np.random.default_rng(5)
    a = rng.standard_normal((130, 70))
    a[3] = 0.0
    a[:, 10:20] *= 1e-300
    b = rng.standard_normal((70, 65))
    b[:, 7] = 0.0
    c, ref, bound = _run(lib, a, b)
    assert np.all(c[3] == 0.0) and np.all(c[:, 7] == 0.0)
    assert np.all(np.abs(c - ref) <= bound + 1e-290)


def test_bad_arguments(lib):
    assert lib.tblite_gb300_split_gemm(0, 4, 4, None, None, None, 0, None) == -1
    assert lib.tblite_gb300_split_gemm(4, 5, 4, ctypes.c_void_p(1), ctypes.c_void_p(1),
                                       ctypes.c_void_p(1), 1, None) == -1
