"""Products of two seeded random FP64 matrices on the pipelined split GEMM.

    python -m tblite_gb300.gemm_run [--n 4096] [--calls 2] [--sym]

Each call computes C = A B (or, with --sym, C = X X for a symmetric X) through
``tblite_gb300_split_gemm`` with n x n operands on the current GPU and prints the largest
deviation from torch's FP64 product relative to |A| |B|.  It is the fixed command behind the
kernel profiles of ``k_opipe``.
"""
from __future__ import annotations

import argparse
import ctypes
import sys
from pathlib import Path


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--calls", type=int, default=2)
    ap.add_argument("--sym", action="store_true")
    args = ap.parse_args(argv)
    root = Path(__file__).resolve().parents[1]
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))
    import torch

    from tblite_gb300 import _build, library

    _build.build()
    lib = library.load()
    n = args.n
    g = torch.Generator(device="cuda").manual_seed(7)
    a = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    if args.sym:
        a = 0.5 * (a + a.T)
        b = a
    else:
        b = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    c = torch.empty(n, n, dtype=torch.float64, device="cuda")
    # column-major views: the C ABI reads a.T's storage as A
    at, bt = a.T.contiguous(), b.T.contiguous()
    torch.cuda.synchronize()
    times = []
    for _ in range(args.calls):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(torch.cuda.default_stream())
        rc = lib.tblite_gb300_split_gemm(n, n, n, ctypes.c_void_p(at.data_ptr()),
                                         ctypes.c_void_p(bt.data_ptr()),
                                         ctypes.c_void_p(c.data_ptr()), 1 if args.sym else 0,
                                         None)
        e1.record(torch.cuda.default_stream())
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
        if rc != 0:
            print(f"split gemm returned {rc}")
            return 1
    ref = a @ b
    err = ((c.T - ref).abs() / (a.abs() @ b.abs())).max().item()
    flop = (n * (n + 1) * n if args.sym else 2 * n ** 3)
    best = min(times)
    print(f"n {n} calls {args.calls} sym {args.sym} max relative deviation "
          f"{err:.3e} best call {best:.3f} ms (split, allocation and product) "
          f"{flop / best / 1e9:.2f} TFLOP/s FP64-equivalent")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
