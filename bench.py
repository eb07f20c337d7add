"""Benchmark: GFN2-xTB energy + analytic gradient single points per second on one GB300.

Workload (default): the plain one-molecule-per-call path on C200H402 (602 atoms, 1202 AOs),
FP64, 300 K Fermi smearing, default SCF thresholds (accuracy 1), through the engine's
C ABI (tblite_get_singlepoint) -- the reference's own single-point entry point.

* value     evals/s of the device work of one single point (engine-internal CUDA events
            on the engine stream, first to last event), geometry already on the device
* e2e       evals/s of tblite_get_singlepoint called from host memory (host->device copy of
            the geometry and device->host copy of energy, gradient, charges, orbital data
            and density matrix inside the timed region)
* roofline  for the engine's dominant own kernel phase, from its per-launch event times
* cpu_baseline  the CPU oracle (plain C + numpy/LAPACK, all host threads) on one
            evaluation of the same molecule

``--impl reference`` times the CPU oracle instead (the reference itself cannot be built
here: no Fortran compiler).  Multi-GPU runs are independent replicas (one process per GPU,
no collective): value = total evaluations of all ranks / slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GFN2 energy+force evals/sec"
WORKLOADS = {"c200h402": "C200H402 GFN2-xTB energy+gradient single point (602 atoms, 1202 AOs)",
             "h2o32": "(H2O)32 GFN2-xTB energy+gradient single point (96 atoms, 192 AOs)",
             "c100h202": "C100H202 GFN2-xTB energy+gradient single point (302 atoms, 602 AOs)"}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return rank, ws


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([v.strip() for v in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        smax = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if len(s) > 4 + k and s[4 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(self.samples)}


def _peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text()), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def _fp64_peak(torch):
    """FP64 peak of this GPU, measured here: best of 5 cuBLAS DGEMMs (4096^3, CUDA events).
    The generated peaks file holds HBM and bf16 figures only."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    c = a @ b
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        c = a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b, c
    return 2.0 * 4096 ** 3 / (best / 1000.0) / 1e12


def _profile_traffic(name):
    """DRAM bytes per launch of a kernel from its committed ncu summary, or None."""
    path = ROOT / "profiles" / name
    try:
        for line in path.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def _roofline(kprof, n, ms_step, peaks, peak_kind, fp64_peak):
    """Roofline of the dominant own kernel (largest summed event time in the step).

    Algorithmic work per launch: Householder tridiagonalisation 4/3 n^3 flop; Fock assembly
    reads H, S, D(3), Q(6) and writes F = 12 n^2 doubles; Mulliken column sums read P, S, H,
    D(3), Q(6) = 12 n^2 doubles.  The other slots have data-dependent work and are listed
    with their times only."""
    kernels = {k: {"ms_per_launch": round(t / c, 4) if c else None, "launches": c,
                   "share_of_step": round(t / ms_step, 4) if ms_step else None}
               for k, (t, c) in kprof.items()}
    work = {"tridiag": ("fp64", 4.0 / 3.0 * n ** 3, "tridiag_smem_c200h402.md"),
            "fock": ("hbm", 12.0 * n * n * 8.0, None),
            "mulliken": ("hbm", 12.0 * n * n * 8.0, None)}
    dom = max(kprof, key=lambda k: kprof[k][0])
    pick = dom if dom in work else max(work, key=lambda k: kprof[k][0])
    t, c = kprof[pick]
    if not c:
        return None, kernels
    bound, units, prof_file = work[pick]
    ms = t / c
    if bound == "fp64":
        achieved = units / (ms / 1000.0) / 1e12
        peak, unit, src = fp64_peak, "TFLOP/s", "measured in this run (cuBLAS DGEMM 4096^3)"
    else:
        achieved = units / (ms / 1000.0) / 1e9
        peak, unit, src = peaks["hbm_gbs"], "GB/s", peak_kind
    roof = {"kernel": pick, "dominant_kernel": dom, "bound": bound, "achieved": round(achieved, 4),
            "peak": round(peak, 4), "unit": unit, "frac": round(achieved / peak, 4),
            "traffic": _profile_traffic(prof_file) if (prof_file and n == 1202) else None,
            "peak_source": src, "algorithmic_work_per_launch": units, "ms_per_launch": round(ms, 4),
            "launches_per_step": c}
    return roof, kernels


def _cpu_baseline(numbers, positions, sample_evals=1):
    """Time the CPU oracle (all host threads) on the same molecule."""
    from oracle import gfn2

    threads = os.cpu_count() or 1
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS"):
        os.environ.setdefault(var, str(threads))
    calc = gfn2.new_calc(gfn2.Molecule(numbers, positions))
    gfn2.lib()
    t0 = time.perf_counter()
    for _ in range(sample_evals):
        gfn2.singlepoint(calc, grad=True)
    dt = (time.perf_counter() - t0) / sample_evals
    return 1.0 / dt, threads


def _flush_l2(buf):
    if buf is not None:
        buf.fill_(1.0)


def run_gb300(args):
    import torch

    from tblite_gb300 import _build, library, workloads
    from tblite_gb300.interface import Calculator

    rank, ws = _dist()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    _build.build()
    numbers, positions = workloads.config(args.config)
    calc = Calculator("GFN2-xTB", numbers, positions)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    fp64_peak = _fp64_peak(torch)
    library.set_profiling(True)
    for _ in range(args.warmup):
        calc.singlepoint()
    torch.cuda.synchronize()
    n0 = library.launch_count()
    dev_ms, profiles = [], []
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    wall = 0.0
    with ClockSampler(dev) as clocks:
        for _ in range(args.steps):
            _flush_l2(flush)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = calc.singlepoint()          # host in, host out: the e2e measurement
            wall += time.perf_counter() - t0
            prof = library.get_profile()
            dev_ms.append(prof["total_ms"] - prof["phase_ms"]["transfer"])
            profiles.append(prof)
    torch.cuda.synchronize()
    launches = library.launch_count() - n0
    if ws > 1:
        t = torch.tensor([wall, sum(dev_ms)], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        wall, dev_sum = float(t[0]), float(t[1])
        torch.distributed.barrier()
    else:
        dev_sum = float(sum(dev_ms))
    if rank != 0:
        return None
    evals = args.steps * ws
    value = evals / (dev_sum / 1000.0)
    e2e = evals / wall
    nat, nao = len(numbers), res.get("norbitals")
    # phase breakdown (mean per single point) and roofline of the dominant own phase
    phases = {k: float(np.mean([p["phase_ms"][k] for p in profiles])) for k in profiles[0]["phase_ms"]}
    counts = {k: int(np.mean([p["phase_count"][k] for p in profiles])) for k in profiles[0]["phase_count"]}
    iters = int(np.mean([p["iterations"] for p in profiles]))
    peaks, peak_kind = _peaks()
    n = nao
    kprof = [library.get_kernel_profile() for _ in range(1)]  # last step's per-kernel events
    roofline, kernels = _roofline(kprof[0], n, dev_sum / args.steps, peaks, peak_kind, fp64_peak)
    cpu_val, cores = _cpu_baseline(numbers, positions) if not args.no_cpu else (None, None)
    h2d = positions.size * 8
    d2h = (1 + nat + 3 * nat + 9 + nat + 2 * n + n * n) * 8 + (res.get("norbitals") * 0)
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "evals/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_sum / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded geometry generator)",
        "config": {"workload": WORKLOADS[args.config], "atoms": nat, "orbitals": n,
                   "scf_iterations": iters, "path": "plain (one molecule per call)",
                   "l2": "flushed (256 MB write) before every step", "parallelism": f"replicas x{ws}"},
        "e2e": {"value": round(e2e, 4), "unit": "evals/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "kernels": kernels,
        "phase_ms": {k: round(v, 3) for k, v in phases.items()},
        "phase_launches": counts,
        "cpu_baseline": None if cpu_val is None else {
            "value": round(cpu_val, 5), "unit": "evals/s", "cores": cores, "kind": "port",
            "sample": f"1 evaluation of the same molecule, CPU oracle (C + numpy/LAPACK dsygvd)"},
        "clocks": clocks.summary(),
    }
    return line


def run_reference(args):
    from tblite_gb300 import workloads

    rank, ws = _dist()
    if rank != 0:
        return None
    numbers, positions = workloads.config(args.config)
    for _ in range(args.warmup):
        pass  # the oracle has no warm state worth priming beyond the first build
    from oracle import gfn2

    gfn2.lib()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    for _ in range(args.steps):
        calc = gfn2.new_calc(gfn2.Molecule(numbers, positions))
        gfn2.singlepoint(calc, grad=True)
    dt = time.perf_counter() - t0
    value = args.steps / dt
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 5), "unit": "evals/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * dt / args.steps, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.config]},
        "cpu_baseline": {"value": round(value, 5), "unit": "evals/s", "cores": threads,
                         "kind": "port", "sample": f"{args.steps} full evaluations"},
        "e2e": {"value": round(value, 5), "unit": "evals/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c200h402", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.impl == "reference":
        args.steps = min(args.steps, 3)
        line = run_reference(args)
    else:
        line = run_gb300(args)
    if line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
