"""The CPU oracle over many molecules on all host cores.

TEST AND BASELINE INFRASTRUCTURE, not part of the product: used by the tests and by the CPU
legs of ``bench.py`` (the timed CPU baseline and the accuracy check of the GPU results).

An ensemble of independent molecules is spread over a process pool (``spawn`` start method, so
that a pool created after the GPU was used does not inherit a CUDA context), one molecule per
task, largest first, one BLAS/OpenMP thread per process: the highest throughput the oracle
reaches on an ensemble (a single small molecule cannot use many threads).
"""
from __future__ import annotations

import multiprocessing as mp
import os
import time

import numpy as np

_THREAD_VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")


def _init():
    from oracle import gfn2

    gfn2.lib()


def _one(task):
    method, z, x = task
    from oracle import gfn1, gfn2

    t0 = time.perf_counter()
    mol = gfn2.Molecule(np.asarray(z), np.asarray(x, dtype=np.float64))
    if method == "GFN1-xTB":
        r = gfn1.singlepoint(gfn1.new_calc(mol))
    else:
        r = gfn2.singlepoint(gfn2.new_calc(mol), grad=True)
    return {"energy": r.energy, "gradient": r.gradient, "qsh": r.qsh, "qat": r.qat,
            "seconds": time.perf_counter() - t0}


class OraclePool:
    """A pool of oracle processes (one thread each); ``run`` evaluates energy + gradient of a
    list of molecules and returns the results in input order and the wall time of the run."""

    def __init__(self, processes: int | None = None):
        self.processes = processes or os.cpu_count() or 1
        saved = {k: os.environ.get(k) for k in _THREAD_VARS}
        for k in _THREAD_VARS:
            os.environ[k] = "1"
        try:
            self._pool = mp.get_context("spawn").Pool(self.processes, initializer=_init)
            # start every worker (imports, oracle library) outside any timed region
            self._pool.map(_noop, range(4 * self.processes), chunksize=1)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    def run(self, mols, method="GFN2-xTB"):
        order = sorted(range(len(mols)), key=lambda i: -len(mols[i][0]))
        tasks = [(method, np.asarray(mols[i][0]), np.asarray(mols[i][1])) for i in order]
        t0 = time.perf_counter()
        out = self._pool.map(_one, tasks, chunksize=1)
        wall = time.perf_counter() - t0
        res = [None] * len(mols)
        for i, r in zip(order, out):
            res[i] = r
        return res, wall

    def close(self):
        self._pool.close()
        self._pool.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _noop(_):
    return None
