"""Benchmark: GFN2-xTB energy + analytic gradient evaluations per second on one GB300.

Workload (default, ``--config ensemble4096``): 4096 molecules of uneven size (50 % water
clusters with k ~ log-uniform[1, 64] waters, 50 % alkanes CnH2n+2 with n ~ log-uniform[1, 60];
3-192 atoms, up to 384 AOs), FP64, 300 K Fermi smearing, default SCF thresholds, all evaluated
per step by one call of the batched entry point (tblite_gb300_batch_singlepoint).  The plain
one-molecule-per-call path (tblite_get_singlepoint, the reference's entry point) is timed on an
even sample of the same ensemble beside it.  ``--config c200h402`` / ``h2o32`` run the plain
path on one molecule (C200H402: 602 atoms, 1202 AOs; (H2O)32: 96 atoms, 192 AOs).

* value     evals/s from device time (CUDA events on the engine streams; the batch's uploads,
            read-back and host work excluded; for one molecule the events of the single point
            minus its result transfer)
* e2e       evals/s of the public call from host memory (geometry host->device, energies,
            gradients, charges, orbital data device->host inside the timed region)
* roofline  the dominant own kernel (Householder tridiagonalisation) against the FP64 peak
            measured in the same run (cuBLAS DGEMM), from its CUDA-event times
* cpu_baseline  the CPU oracle (plain C + numpy/LAPACK dsygvd, all host threads) on a bounded
            sample of the same workload

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

METRIC = "GFN2 energy+force evals/sec, batched vs plain GPU at |\u0394E|\u22641e-7 Eh, |\u0394F|\u22641e-6"
WORKLOADS = {"c200h402": "C200H402 GFN2-xTB energy+gradient single point (602 atoms, 1202 AOs)",
             "h2o32": "(H2O)32 GFN2-xTB energy+gradient single point (96 atoms, 192 AOs)",
             "c100h202": "C100H202 GFN2-xTB energy+gradient single point (302 atoms, 602 AOs)",
             "ensemble4096": "4096-molecule GFN2-xTB energy+gradient ensemble (50 % water clusters "
                             "k ~ log-uniform[1, 64], 50 % alkanes n ~ log-uniform[1, 60]; "
                             "3-192 atoms), batched",
             "ensemble512": "512-molecule subset of the same ensemble generator, batched",
             "h2o1000_alpb": "(H2O)1000 GFN2-xTB + ALPB(water) energy+gradient single point "
                             "(3000 atoms, 6000 AOs), density by spectral projection",
             "c200h402_sp2": "C200H402 GFN2-xTB energy+gradient single point (602 atoms, 1202 "
                             "AOs), density by spectral projection instead of diagonalisation",
             "autograd256": "256 alkanes CnH2n+2, n uniform in [4, 40] (seed 3), GFN2-xTB forces and "
                            "dE/d(shell self energy, CN shift, hardness, third-order derivative, "
                            "Slater exponent) through the torch.autograd bridge"}
ENSEMBLE_SIZE = {"ensemble4096": 4096, "ensemble512": 512}
GEOMETRY = {"h2o1000_alpb": "h2o1000", "c200h402_sp2": "c200h402"}  # -> workloads.config
SOLVATED = {"h2o1000_alpb"}
PURIFIED = {"h2o1000_alpb", "c200h402_sp2"}
LARGE = {"h2o1000_alpb"}  # one oracle evaluation takes tens of minutes: bounded CPU samples
SPLIT_SLICE_PRODUCTS = 36  # BF16 slice products per FP64 product in the split GEMM
# comparison legs of the ensemble: one seeded random order of the ensemble's molecules; the
# plain GPU leg takes its first 64, the CPU baseline its first 256 (with the accuracy check of
# the GPU results), the reference arm consecutive slices of REF_PER_STEP per step
SAMPLE_SEED = 4242
PLAIN_SAMPLE, CPU_SAMPLE, REF_PER_STEP = 64, 256, 128
BARS = {"energy_eh": 1e-7, "force_eh_per_bohr": 1e-6, "shell_charge_e": 1e-6}


def ensemble_order(count):
    """The seeded random order of the ensemble's molecules shared by the comparison legs."""
    return [int(i) for i in np.random.default_rng(SAMPLE_SEED).permutation(count)]


def _kinds(idx):
    """water clusters / alkanes among ensemble indices (the generator alternates them)."""
    w = sum(1 for i in idx if i % 2 == 0)
    return {"water_clusters": w, "alkanes": len(idx) - w}


def _accuracy(gpu_results, oracle_results, idx):
    """max |dE|, |dF|, |dq_sh|, |dq_at| of GPU results against the oracle's on the same
    molecules (ensemble indices idx)."""
    de = df = dqs = dqa = 0.0
    for i, ref in zip(idx, oracle_results):
        r = gpu_results[i]
        de = max(de, abs(r.get("energy") - ref["energy"]))
        df = max(df, float(np.max(np.abs(r.get("gradient") - ref["gradient"]))))
        dqs = max(dqs, float(np.max(np.abs(r.get("shell-charges") - ref["qsh"]))))
        dqa = max(dqa, float(np.max(np.abs(r.get("charges") - ref["qat"]))))
    out = {"molecules": len(idx), **_kinds(idx), "max_abs_dE_eh": float(f"{de:.3e}"),
           "max_abs_dF_eh_per_bohr": float(f"{df:.3e}"), "max_abs_dq_shell_e": float(f"{dqs:.3e}"),
           "max_abs_dq_atom_e": float(f"{dqa:.3e}"), "bars": BARS,
           "within_bars": bool(de <= BARS["energy_eh"] and df <= BARS["force_eh_per_bohr"]
                               and dqs <= BARS["shell_charge_e"]),
           "against": "CPU oracle (FP64, LAPACK dsygvd), same molecules and settings"}
    return out


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


def _roofline(kprof, n, ms_step, peaks, peak_kind, fp64_peak, split_flops=None):
    """Roofline of the dominant own kernel (largest summed event time in the step).

    Algorithmic work per launch: Householder tridiagonalisation 4/3 n^3 flop; Fock assembly
    reads H, S, D(3), Q(6) and writes F = 12 n^2 doubles; Mulliken column sums read P, S, H,
    D(3), Q(6) = 12 n^2 doubles; split GEMM (split_flops: FP64 flop of the step's products,
    counted by the library) 36 BF16 slice products per FP64 product on the tensor cores,
    against the sustained bf16 peak.  The other slots have data-dependent work and are listed
    with their times only."""
    kernels = {k: {"ms_per_launch": round(t / c, 4) if c else None, "launches": c,
                   "share_of_step": round(t / ms_step, 4) if ms_step else None}
               for k, (t, c) in kprof.items()}
    work = {"tridiag": ("fp64", 4.0 / 3.0 * n ** 3, "tridiag_smem_c200h402.md"),
            "fock": ("hbm", 12.0 * n * n * 8.0, None),
            "mulliken": ("hbm", 12.0 * n * n * 8.0, None)}
    if split_flops and kprof.get("gemm", (0, 0))[1]:
        work["gemm"] = ("tensor", SPLIT_SLICE_PRODUCTS * split_flops / kprof["gemm"][1], None)
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
    elif bound == "tensor":
        achieved = units / (ms / 1000.0) / 1e12
        peak = peaks.get("bf16_tflops_sustained", peaks["bf16_tflops"])
        unit, src = "TFLOP/s", f"{peak_kind} (bf16 sustained)"
    else:
        achieved = units / (ms / 1000.0) / 1e9
        peak, unit, src = peaks["hbm_gbs"], "GB/s", peak_kind
    roof = {"kernel": pick, "dominant_kernel": dom, "bound": bound, "achieved": round(achieved, 4),
            "peak": round(peak, 4), "unit": unit, "frac": round(achieved / peak, 4),
            "traffic": _profile_traffic(prof_file) if (prof_file and n == 1202) else None,
            "peak_source": src, "algorithmic_work_per_launch": units, "ms_per_launch": round(ms, 4),
            "launches_per_step": c}
    if bound == "tensor":
        roof["fp64_equivalent_tflops"] = round(units / SPLIT_SLICE_PRODUCTS / (ms / 1000.0) / 1e12,
                                               4)
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


def _eigensolve_seconds(numbers, positions):
    """One generalised eigensolve of the CPU oracle (LAPACK dsygvd on all host threads) of the
    molecule's H0 against S: (seconds, orbitals, threads)."""
    import scipy.linalg

    from oracle import gfn2

    threads = os.cpu_count() or 1
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS"):
        os.environ.setdefault(var, str(threads))
    calc = gfn2.new_calc(gfn2.Molecule(numbers, positions))
    gfn2.lib()
    st = gfn2.setup(calc)
    t0 = time.perf_counter()
    scipy.linalg.eigh(st["H"], st["S"], type=1, driver="gvd", lower=False)
    return time.perf_counter() - t0, st["S"].shape[0], threads


def _eigensolve_sample(dt, n, iterations):
    return (f"1 generalised eigensolve (n = {n}, dsygvd) of the CPU oracle per step, {dt:.1f} s, "
            f"times {iterations} SCF iterations; the rest of the oracle's SCF and gradient not "
            "counted (an upper bound on its evals/s)")


def _cpu_baseline_eigensolve(numbers, positions, iterations):
    """Bounded CPU sample for orbital counts where one oracle evaluation takes many minutes: the
    oracle's eigensolve of one SCF iteration times the SCF iterations of the GPU run."""
    dt, n, threads = _eigensolve_seconds(numbers, positions)
    return 1.0 / (dt * iterations), threads, _eigensolve_sample(dt, n, iterations)


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
    numbers, positions = workloads.config(GEOMETRY.get(args.config, args.config))
    calc = Calculator("GFN2-xTB", numbers, positions)
    if args.config in SOLVATED:
        calc.add("alpb-solvation", "water")
    purified = args.config in PURIFIED
    if purified:
        calc.set("density-solver", "purification")
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    fp64_peak = _fp64_peak(torch)
    library.set_profiling(True)
    for _ in range(args.warmup):
        calc.singlepoint()
    torch.cuda.synchronize()
    n0 = library.launch_count()
    f0 = library.split_gemm_flops()
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
    split_flops = (library.split_gemm_flops() - f0) / args.steps
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
    roofline, kernels = _roofline(kprof[0], n, dev_sum / args.steps, peaks, peak_kind, fp64_peak,
                                  split_flops)
    if args.no_cpu:
        cpu_val, cores, cpu_sample = None, None, None
    elif args.config in LARGE:
        cpu_val, cores, cpu_sample = _cpu_baseline_eigensolve(numbers, positions, iters)
    else:
        cpu_val, cores = _cpu_baseline(numbers, positions)
        cpu_sample = "1 evaluation of the same molecule, CPU oracle (C + numpy/LAPACK dsygvd)"
    h2d = positions.size * 8
    nsh = len(calc.get("shell-map"))
    # per step: P, bond orders, gradient, virial parts, charges and moments; C, e and f after
    # diagonalisation only
    d2h = (n * n + nat * nat + 3 * nat + 9 * nat + 9 + nsh + nat + 3 * nat + 6 * nat) * 8
    if not purified:
        d2h += (n * n + 2 * n) * 8
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "evals/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_sum / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded geometry generator)",
        "config": {"workload": WORKLOADS[args.config], "atoms": nat, "orbitals": n,
                   "scf_iterations": iters, "path": "plain (one molecule per call)",
                   "density_solver": "spectral projection (SP2)" if purified else
                   "diagonalisation (Fermi filling)", "solvation": "ALPB(water)" if
                   args.config in SOLVATED else None,
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
            "sample": cpu_sample},
        "clocks": clocks.summary(),
    }
    return line


def _ensemble_flops(mols_nao, mols_nel, iters, modes=None, pipe_flops=0.0):
    """Algorithmic FP64 work of the batched ensemble and of its tridiagonalisations.

    Diagonalised molecules: per SCF iteration the Cholesky-reduced eigensolve 16/3 n^3 and the
    density 2 n^2 k; once the Cholesky n^3/3 and the energy-weighted density 2 n^2 k; the
    tridiagonalisation 4/3 n^3 per iteration.  Projected molecules (mode 1): per iteration the
    reduction X^T F X (n^3 + n^3) and P = 2 X D X^T (n^3 + n^3), the squarings as counted on
    the device (pipe_flops, FP64-equivalent); once the Cholesky n^3/3, the final
    diagonalisation for the orbital energies 4/3 n^3 and W = P F P / 2 (4 n^3); k = occupied
    orbitals."""
    tot = tri = 0.0
    modes = modes if modes is not None else [0] * len(mols_nao)
    for n, nel, it, mode in zip(mols_nao, mols_nel, iters, modes):
        k = min(n, (nel + 1) // 2)
        if mode == 1:
            tot += it * 4.0 * n ** 3 + n ** 3 / 3.0 + 4.0 / 3.0 * n ** 3 + 4.0 * n ** 3
            tri += 4.0 / 3.0 * n ** 3
        else:
            tot += it * (16.0 / 3.0 * n ** 3 + 2.0 * n * n * k) + n ** 3 / 3.0 + 2.0 * n * n * k
            tri += it * 4.0 / 3.0 * n ** 3
    return tot + pipe_flops, tri


def _modes(count):
    from tblite_gb300 import library

    m = np.zeros(count, dtype=np.int32)
    library.load().tblite_gb300_batch_last_modes(library._ip(m), count)
    return m


def run_batch(args):
    """Batched ensemble: all molecules through tblite_gb300_batch_singlepoint per step."""
    import torch

    from tblite_gb300 import _build, library, workloads
    from tblite_gb300.interface import Calculator, batch_fallbacks, batch_singlepoint

    rank, ws = _dist()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    _build.build()
    count = ENSEMBLE_SIZE[args.config]
    mols = workloads.mixed_ensemble(count, seed=4 + 1000 * rank)
    calcs = [Calculator("GFN2-xTB", z, x) for z, x in mols]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    fp64_peak = _fp64_peak(torch)
    library.set_batch_graphs(not args.no_graphs)
    batch_singlepoint(calcs)  # first use: device memory, module loading
    tuned_calls = library.batch_autotune(calcs, sample=2048) if not args.no_tune else 0
    schedule = library.batch_schedule()
    library.set_profiling(False)  # the timed calls run their SCF iterations as CUDA graphs
    for _ in range(args.warmup):
        batch_singlepoint(calcs)
    torch.cuda.synchronize()
    n0 = library.launch_count()
    pf0 = library.pipe_batch_flops()
    if ws > 1:
        torch.distributed.barrier()
    wall = dev_ms = 0.0
    host = dict.fromkeys(library.BATCH_HOST_PHASES + ("python_call", "python_results"), 0.0)
    with ClockSampler(dev) as clocks:
        for _ in range(args.steps):
            _flush_l2(flush)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = batch_singlepoint(calcs)  # host in, host out
            t1 = time.perf_counter()
            energies = [r.get("energy") for r in res]
            t2 = time.perf_counter()
            wall += t2 - t0
            dev_ms += library.load().tblite_gb300_batch_last_device_ms()
            for k, v in library.batch_host_ms().items():
                host[k] += v
            host["python_call"] += 1e3 * (t1 - t0)
            host["python_results"] += 1e3 * (t2 - t1)
    launches = library.launch_count() - n0
    fallbacks = batch_fallbacks()
    projected = library.batch_projected()
    modes = _modes(count)
    pipe_flops_step = (library.pipe_batch_flops() - pf0) / args.steps
    graph_builds, graph_launches = library.batch_graphs()
    # per-kernel CUDA events: one more (untimed) call with the profiler on (kernels launched
    # directly, buckets on the side streams as in the timed calls)
    library.set_profiling(True)
    batch_singlepoint(calcs)
    kprof = library.get_kernel_profile()
    iters = np.zeros(count, dtype=np.int32)
    library.load().tblite_gb300_batch_last_iterations(library._ip(iters), count)
    if ws > 1:
        t = torch.tensor([wall, dev_ms], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        wall, dev_ms = float(t[0]), float(t[1])
        torch.distributed.barrier()
    if rank != 0:
        return None
    evals = args.steps * count * ws
    value = evals / (dev_ms / 1000.0)
    e2e = evals / wall
    nao = [c.get("orbital-map").size for c in calcs]
    nel = [int(round(sum({1: 1, 6: 4, 8: 6}[int(q)] for q in z))) for z, _ in mols]
    flops, tri_flops = _ensemble_flops(nao, nel, np.maximum(iters, 0), modes, pipe_flops_step)
    ms_step = dev_ms / args.steps
    kernels = {k: {"ms_per_step": round(t, 3), "launches": c, "share_of_step": round(t / ms_step, 4)}
               for k, (t, c) in kprof.items()}
    # roofline of the dominant kernel: the buckets share the GPU over 8 streams in the timed
    # steps, so an event pair there also spans other buckets' kernels; one more (untimed) call
    # with the buckets on one stream brackets every tridiagonalisation launch alone
    library.set_batch_streams(1)
    pf1 = library.pipe_batch_flops()
    batch_singlepoint(calcs)
    pipe_flops_s = library.pipe_batch_flops() - pf1
    kser = library.get_kernel_profile()
    library.set_batch_streams(8)
    iters_s = np.zeros(count, dtype=np.int32)
    library.load().tblite_gb300_batch_last_iterations(library._ip(iters_s), count)
    _, tri_flops_s = _ensemble_flops(nao, nel, np.maximum(iters_s, 0), _modes(count))
    t_tri, c_tri = kser["tridiag"]
    t_pipe, c_pipe = kser["pipe_products"]
    t_prep, c_prep = kser["pipe_operands"]
    peaks, peak_kind = _peaks()
    bf16 = peaks.get("bf16_tflops_sustained", peaks["bf16_tflops"])
    timing = ("CUDA events around each launch on its stream, one untimed call with the size "
              "buckets serialised on one stream")
    tri_roof = {"kernel": "tridiag (batched, one block cluster per molecule)", "bound": "fp64",
                "achieved": round(tri_flops_s / (t_tri / 1000.0) / 1e12, 4) if t_tri else None,
                "peak": round(fp64_peak, 4), "unit": "TFLOP/s",
                "frac": round(tri_flops_s / (t_tri / 1000.0) / 1e12 / fp64_peak, 4) if t_tri else None,
                "timing": timing, "traffic": 17577984,
                "traffic_note": "dram__bytes_read+write of one kb_tridiag launch (38 molecules, "
                                "288-384 orbitals; profiles/tridiag_cluster_ensemble512.md): each "
                                "matrix is read once, n^2 x 8 B per molecule",
                "peak_source": "measured in this run (cuBLAS DGEMM 4096^3)",
                "algorithmic_work_per_call": tri_flops_s, "ms_per_call": round(t_tri, 3),
                "launches_per_call": c_tri,
                "ms_per_launch": round(t_tri / c_tri, 4) if c_tri else None}
    pipe_roof = None
    if t_pipe and pipe_flops_s:
        ach = SPLIT_SLICE_PRODUCTS * pipe_flops_s / (t_pipe / 1000.0) / 1e12
        pipe_roof = {"kernel": "batched pipelined split GEMM on tcgen05 (projection squarings "
                               "kb_opipe_sq and product sites kb_opipe_site)",
                     "bound": "tensor", "achieved": round(ach, 4), "peak": round(bf16, 4),
                     "unit": "TFLOP/s", "frac": round(ach / bf16, 4), "timing": timing,
                     "traffic": _profile_traffic("pipe_sq_ensemble512.md"),
                     "traffic_note": "dram__bytes_read+write of one captured kb_opipe_sq launch "
                                     "(38 molecules of 288-384 orbitals; "
                                     "profiles/pipe_sq_ensemble512.md): each slice image read "
                                     "about once from DRAM, the tile re-reads served by L2",
                     "peak_source": f"{peak_kind} (bf16 sustained)",
                     "algorithmic_work_per_call": SPLIT_SLICE_PRODUCTS * pipe_flops_s,
                     "work_note": "36 BF16 slice products per FP64-equivalent flop; FP64-"
                                  "equivalent flop counted on the device (2 m n K per tile)",
                     "fp64_equivalent_tflops": round(pipe_flops_s / (t_pipe / 1000.0) / 1e12, 4),
                     "ms_per_call": round(t_pipe, 3), "launches_per_call": c_pipe,
                     "ms_per_launch": round(t_pipe / c_pipe, 4) if c_pipe else None,
                     "operands": {"kernels": "kb_sp2_slice, kb_pexp_site, kb_psplit_site "
                                             "(HBM-bound: slice images, exponents, partial "
                                             "sums)",
                                  "ms_per_call": round(t_prep, 3), "launches_per_call": c_prep}}
    if pipe_roof is not None and t_pipe >= t_tri:
        roofline, other = pipe_roof, tri_roof
    else:
        roofline, other = tri_roof, pipe_roof
    roofline = dict(roofline)
    roofline["secondary"] = other
    roofline["whole_step"] = {"algorithmic_flops": flops,
                              "achieved_tflops": round(flops / (ms_step / 1000.0) / 1e12, 4)}
    # the plain one-molecule GPU path on the first molecules of the seeded random order
    order = ensemble_order(count)
    sample = order[:PLAIN_SAMPLE]
    for i in sample:
        calcs[i].singlepoint()  # per-calculator workspace
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in sample:
        calcs[i].singlepoint()
    plain = len(sample) / (time.perf_counter() - t0)
    # the same ensemble with GFN1-xTB: one warm-up call, then the same number of timed steps
    calcs1 = [Calculator("GFN1-xTB", z, x) for z, x in mols]
    batch_singlepoint(calcs1)
    torch.cuda.synchronize()
    w1 = d1 = 0.0
    for _ in range(args.steps):
        _flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res1 = batch_singlepoint(calcs1)
        _ = [r.get("energy") for r in res1]
        w1 += time.perf_counter() - t0
        d1 += library.load().tblite_gb300_batch_last_device_ms()
    iters1 = np.zeros(count, dtype=np.int32)
    library.load().tblite_gb300_batch_last_iterations(library._ip(iters1), count)
    leave1 = {str(int(c)): int(np.sum(iters1 == c)) for c in np.unique(iters1[iters1 < 0])}
    gfn1 = {"value": round(args.steps * count / (d1 / 1000.0), 3), "unit": "evals/s",
            "e2e": round(args.steps * count / w1, 3), "fallbacks_to_plain": batch_fallbacks(),
            "fallback_reasons": leave1,
            "mean_scf_iterations": float(np.mean(iters1[iters1 > 0])) if np.any(iters1 > 0) else 0.0,
            "note": "same molecules and timing as the headline, GFN1-xTB Hamiltonian (D3 dispersion)"}
    cpu = accuracy = None
    if not args.no_cpu:
        # the CPU oracle on all host cores (a spawn pool: this process already uses the GPU),
        # on the first CPU_SAMPLE molecules of the same order; its results also check the GPU
        # results of those molecules from the last timed step (and of the GFN1 leg)
        from oracle.parallel import OraclePool

        cs = order[:CPU_SAMPLE]
        with OraclePool() as pool:
            refs, wall_cpu = pool.run([mols[i] for i in cs])
            refs1, _ = pool.run([mols[i] for i in cs[:PLAIN_SAMPLE]], method="GFN1-xTB")
            cores = pool.processes
        cpu = {"value": round(len(cs) / wall_cpu, 4), "unit": "evals/s", "cores": cores,
               "kind": "port",
               "sample": f"{len(cs)} molecules of the ensemble in a seeded random order "
                         f"(numpy default_rng({SAMPLE_SEED}).permutation; {_kinds(cs)}), CPU "
                         f"oracle (C + numpy/LAPACK dsygvd), one molecule per process on "
                         f"{cores} processes, evals/s of the sample"}
        accuracy = _accuracy(res, refs, cs)
        gfn1["accuracy"] = _accuracy(res1, refs1, cs[:PLAIN_SAMPLE])
    h2d = sum(m[1].size * 8 + m[0].size * 4 for m in mols)
    d2h = sum((1 + 5 * len(m[0]) + 9) * 8 for m in mols)
    return {
        "metric": METRIC, "value": round(value, 3), "unit": "evals/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded ensemble generator)",
        "config": {"workload": WORKLOADS[args.config], "molecules": count,
                   "max_orbitals": int(max(nao)),
                   "mean_scf_iterations": float(np.mean(iters[iters > 0])) if np.any(iters > 0) else 0.0,
                   "path": "batched (tblite_gb300_batch_singlepoint)",
                   "schedule": schedule, "autotune_calls": tuned_calls,
                   "projected_molecules": projected,
                   "scf_iteration_graphs": {"enabled": library.batch_graphs_enabled(),
                                            "instantiations": graph_builds,
                                            "launches": graph_launches,
                                            "note": "last timed call; each SCF iteration of a "
                                                    "memory chunk is one CUDA graph launch"},
                   "l2": "flushed (256 MB write) before every step", "parallelism": f"replicas x{ws}"},
        "e2e": {"value": round(e2e, 3), "unit": "evals/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "host_ms_per_step": {k: round(v / args.steps, 2) for k, v in host.items()},
                "host_note": "plans .. call: phases of the C call (host wall); python_call: "
                             "batch_singlepoint as Python sees it; python_results: the "
                             "energy getter over all results"},
        "batched_vs_plain": {"plain_gpu_evals_per_s": round(plain, 3),
                             "sample": f"first {len(sample)} molecules of the seeded random "
                                       f"order ({_kinds(sample)}), one per call",
                             "ratio_e2e": round(e2e / plain, 2)},
        "accuracy": accuracy,
        "fallbacks_to_plain": fallbacks,
        "gfn1": gfn1,
        "gpu_launches": int(launches),
        "roofline": roofline,
        "kernels": kernels,
        "kernels_serialised": {k: {"ms_per_call": round(t, 3), "launches": c}
                               for k, (t, c) in kser.items()},
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
    }


def run_autograd(args):
    """Differentiation: forces and parameter gradients of 256 alkanes through the
    torch.autograd bridge; finite-difference check on a sample; adjoint time per molecule."""
    import torch

    from tblite_gb300 import _build, library, workloads
    from tblite_gb300.autograd import (PARAMETERS, gfn2_energies_batch, gfn2_energy,
                                       shell_parameters)
    from tblite_gb300.interface import Calculator

    rank, ws = _dist()
    if rank != 0:
        return None
    _build.build()
    mols = workloads.alkane_batch(256, seed=3, nmin=4, nmax=40)
    calcs = [Calculator("GFN2-xTB", z, x) for z, x in mols]
    base = [shell_parameters(c) for c in calcs]

    def forward_backward(i):
        pos = torch.tensor(mols[i][1], requires_grad=True)
        prm = {k: torch.tensor(base[i][k], requires_grad=True) for k in PARAMETERS}
        e = gfn2_energy(calcs[i], pos, **prm)
        e.backward()
        return pos.grad, prm

    def batch_step():
        """all 256 molecules in one batched engine call: energies, then one backward pass"""
        pos = [torch.tensor(m[1], requires_grad=True) for m in mols]
        prm = [{k: torch.tensor(base[i][k], requires_grad=True) for k in PARAMETERS}
               for i in range(len(mols))]
        e = gfn2_energies_batch(calcs, pos, prm)
        e.sum().backward()
        return pos, prm

    for _ in range(max(args.warmup, 3)):
        batch_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batch_step()
    t_grad = (time.perf_counter() - t0) / args.steps
    # the same molecules through the one-molecule path (one engine call each)
    for i in range(min(args.warmup, 3)):
        forward_backward(i)
    t0 = time.perf_counter()
    for i in range(len(calcs)):
        forward_backward(i)
    t_loop = time.perf_counter() - t0
    # the same batched call without the parameter gradient: the adjoint pass is the difference
    from tblite_gb300.interface import batch_singlepoint

    for c in calcs:
        library.set_parameter_gradient(c._ctx, c._calc, False)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batch_singlepoint(calcs)
    t_plain = (time.perf_counter() - t0) / args.steps
    # central finite differences on three molecules (accuracy 1e-5): positions 0.5e-4 Bohr,
    # parameters 1e-5 relative
    errs = {"positions": 0.0, **{k: 0.0 for k in PARAMETERS}}
    for i in (0, 1, 2):
        c = calcs[i]
        c.set("accuracy", 1e-5)
        g, prm = forward_backward(i)
        x = mols[i][1]

        def energy(xx, **kw):
            vals = {k: torch.tensor(kw.get(k, base[i][k])) for k in PARAMETERS}
            return float(gfn2_energy(c, torch.tensor(xx), **vals))

        for a, k in [(0, 0), (1, 2)]:
            xp, xm = x.copy(), x.copy()
            xp[a, k] += 0.5e-4
            xm[a, k] -= 0.5e-4
            fd = (energy(xp) - energy(xm)) / 1e-4
            errs["positions"] = max(errs["positions"], abs(fd - float(g[a, k])))
        for k in PARAMETERS:
            v = base[i][k].copy()
            h = 1e-5 * max(abs(v[0]), 1e-2)
            v[0] += h
            ep = energy(x, **{k: v})
            v[0] -= 2 * h
            em = energy(x, **{k: v})
            errs[k] = max(errs[k], abs((ep - em) / (2 * h) - float(prm[k].grad[0])))
        c.set("accuracy", 1.0)
    count = len(calcs)
    return {
        "metric": "GFN2 energy+force+parameter-gradient evals/sec (torch.autograd bridge)",
        "value": round(count / t_grad, 3), "unit": "evals/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * t_grad, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded alkanes)",
        "config": {"workload": WORKLOADS[args.config], "molecules": count},
        "path": "batched (tblite_gb300_batch_singlepoint): one engine call for all molecules",
        "adjoint_ms_per_molecule": round(1000 * (t_grad - t_plain) / count, 4),
        "energy_force_ms_per_molecule": round(1000 * t_plain / count, 4),
        "one_molecule_path_evals_per_s": round(count / t_loop, 3),
        "fd_max_abs_error": {k: float(f"{v:.3e}") for k, v in errs.items()},
        "fd_sample": "molecules 0-2, accuracy 1e-5; positions 0.5e-4 Bohr, parameters 1e-5 relative "
                     "(first shell)",
    }


def run_reference(args):
    from tblite_gb300 import workloads

    rank, ws = _dist()
    if rank != 0:
        return None
    from oracle import gfn2

    gfn2.lib()
    threads = os.cpu_count() or 1
    if args.config in ENSEMBLE_SIZE or args.config == "autograd256":
        # a bounded sample per step on all host cores (one molecule per process): for the
        # ensemble, consecutive slices of the seeded random order the GPU arm's comparison legs
        # use (warm-up steps first, then the timed steps); for the alkanes, all 256 per step
        from oracle.parallel import OraclePool

        if args.config == "autograd256":
            mols = workloads.alkane_batch(256, seed=3, nmin=4, nmax=40)
            slices = [list(range(len(mols)))] * (args.warmup + args.steps)
            desc = "all 256 alkanes per step (energy + gradient)"
        else:
            count = ENSEMBLE_SIZE[args.config]
            mols = workloads.mixed_ensemble(count, seed=4)
            order = ensemble_order(count)
            slices = [[order[(s * REF_PER_STEP + j) % count] for j in range(REF_PER_STEP)]
                      for s in range(args.warmup + args.steps)]
            timed = [i for sl in slices[args.warmup:] for i in sl]
            desc = (f"{REF_PER_STEP} molecules of the ensemble per step, consecutive slices of "
                    f"its seeded random order (numpy default_rng({SAMPLE_SEED}).permutation) after "
                    f"{args.warmup} warm-up slices; timed: {len(set(timed))} distinct molecules, "
                    f"{_kinds(timed)}")
        with OraclePool() as pool:
            for sl in slices[:args.warmup]:
                pool.run([mols[i] for i in sl])
            wall = 0.0
            for sl in slices[args.warmup:]:
                _, w = pool.run([mols[i] for i in sl])
                wall += w
            cores = pool.processes
        evals = sum(len(sl) for sl in slices[args.warmup:])
        value = evals / wall
        return {
            "impl": "reference", "metric": METRIC, "value": round(value, 5), "unit": "evals/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000 * wall / args.steps, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.config]},
            "cpu_baseline": {"value": round(value, 5), "unit": "evals/s", "cores": cores,
                             "kind": "port", "sample": desc + f", {cores} processes"},
            "e2e": {"value": round(value, 5), "unit": "evals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
        }
    elif args.config in LARGE:
        # one oracle evaluation takes tens of minutes: each step times one generalised
        # eigensolve, scaled by the oracle's own SCF iteration count for this system
        numbers, positions = workloads.config(GEOMETRY[args.config])
        fixture = ROOT / "tests" / "golden" / "water1000_alpb.npz"
        iters = int(np.load(fixture)["iterations"]) if fixture.exists() else 1
        dts = []
        for _ in range(args.steps):
            dt, n, _ = _eigensolve_seconds(numbers, positions)
            dts.append(dt)
        desc = _eigensolve_sample(float(np.mean(dts)), n, iters)
        value = 1.0 / (float(np.mean(dts)) * iters)
        return {
            "impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": "evals/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000 * float(np.mean(dts)), 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.config]},
            "cpu_baseline": {"value": round(value, 6), "unit": "evals/s", "cores": threads,
                             "kind": "port", "sample": desc},
            "e2e": {"value": round(value, 6), "unit": "evals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
        }
    else:
        sample = [workloads.config(GEOMETRY.get(args.config, args.config))]
        sample_desc = "1 full evaluation per step"
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for numbers, positions in sample:
            calc = gfn2.new_calc(gfn2.Molecule(np.asarray(numbers), np.asarray(positions)))
            gfn2.singlepoint(calc, grad=True)
    dt = time.perf_counter() - t0
    value = args.steps * len(sample) / dt
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 5), "unit": "evals/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * dt / args.steps, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.config]},
        "cpu_baseline": {"value": round(value, 5), "unit": "evals/s", "cores": threads,
                         "kind": "port", "sample": sample_desc},
        "e2e": {"value": round(value, 5), "unit": "evals/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


# --------------------------------------------------------------------------------------------
# Fixed commands behind the kernel profiles (``--run``): one kind of engine call, no timing
# contract, no JSON line.
# --------------------------------------------------------------------------------------------
def profile_run_ensemble(args):
    """Batched energy + gradient calls over ``workloads.mixed_ensemble(molecules, seed=4)``;
    prints the molecules, the fallbacks to the one-molecule path and the energy sum."""
    from tblite_gb300 import _build, library, workloads
    from tblite_gb300.interface import Calculator, batch_fallbacks, batch_singlepoint

    _build.build()
    if args.tridiag_ctas:
        library.set_tridiag_ctas_per_sm(args.tridiag_ctas)
    mols = workloads.mixed_ensemble(args.molecules, seed=4)
    calcs = [Calculator(args.method, z, x) for z, x in mols]
    for _ in range(args.calls):
        res = batch_singlepoint(calcs)
        print(f"molecules {len(res)} fallbacks {batch_fallbacks()} "
              f"energy_sum {sum(r.get('energy') for r in res):.10f} "
              f"device_ms {library.load().tblite_gb300_batch_last_device_ms():.1f}")
    return 0


def profile_run_gemm(args):
    """Products of two seeded random FP64 n x n matrices (or X X for a symmetric X with
    ``--sym``) through ``tblite_gb300_split_gemm``; prints the largest deviation from torch's
    FP64 product relative to |A| |B| and the best call time."""
    import ctypes

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
    at, bt = a.T.contiguous(), b.T.contiguous()  # column-major views for the C ABI
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
    print(f"n {n} calls {args.calls} sym {args.sym} max relative deviation {err:.3e} best call "
          f"{best:.3f} ms (split, allocation and product) {flop / best / 1e9:.2f} TFLOP/s "
          "FP64-equivalent")
    return 0


def profile_run_single(args):
    """Plain-path single points (energy + gradient) of ``workloads.config(geometry)``, with
    ALPB(water) for ``--solvent`` and the density solver of ``--solver``."""
    from tblite_gb300 import _build, library, workloads
    from tblite_gb300.interface import Calculator

    _build.build()
    z, x = workloads.config(args.geometry)
    calc = Calculator(args.method, z, x)
    if args.solvent:
        calc.add("alpb-solvation", "water")
    calc.set("density-solver", args.solver)
    library.set_profiling(True)
    for _ in range(args.calls):
        res = calc.singlepoint()
        prof = library.get_profile()
        print(f"atoms {len(z)} energy {res.get('energy'):.10f} iterations {prof['iterations']}")
    return 0


PROFILE_RUNS = {"ensemble": profile_run_ensemble, "gemm": profile_run_gemm,
                "single": profile_run_single}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="ensemble4096", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch the batched SCF kernels directly instead of as CUDA graphs")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default batch schedule (no autotuning before the warm-up)")
    prof = ap.add_argument_group("fixed profiling commands (--run)")
    prof.add_argument("--run", choices=sorted(PROFILE_RUNS),
                      help="run one kind of engine call for a profiler instead of the benchmark")
    prof.add_argument("--molecules", type=int, default=512)
    prof.add_argument("--method", default="GFN2-xTB", choices=["GFN2-xTB", "GFN1-xTB"])
    prof.add_argument("--calls", type=int, default=1)
    prof.add_argument("--tridiag-ctas", type=int, default=0,
                      help="CTAs per SM of the batched tridiagonalisation (0: library default)")
    prof.add_argument("--n", type=int, default=4096)
    prof.add_argument("--sym", action="store_true")
    prof.add_argument("--geometry", default="h2o1000")
    prof.add_argument("--solvent", action="store_true")
    prof.add_argument("--solver", default="diagonalization",
                      choices=["diagonalization", "purification"])
    args = ap.parse_args()
    if args.run:
        raise SystemExit(PROFILE_RUNS[args.run](args))
    if args.impl == "reference":
        line = run_reference(args)
    else:
        if args.config == "autograd256":
            line = run_autograd(args)
        else:
            line = run_batch(args) if args.config in ENSEMBLE_SIZE else run_gb300(args)
    if line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
