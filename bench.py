"""Benchmark of the path-simulation hot path on GB300.

Workload (one "step" = one pass over one batch): Heston RQMC, S0=100,
v0=0.04, kappa=2, theta=0.04, xi=0.3, mu=0.03, rho=-0.7, T=1; full-truncation
Euler, 256 steps, 2^20 paths x 16 XOR-scrambled Sobol replicates (dimension
512, masks from seed 7), FP32 stepping, FP64 compensated reduction of
E[max(S_T-100, 0)], terminal-only output.  Synthetic, seeded inputs.

Default run: 1 GPU, --steps 10 --warmup 3.  Under torchrun (N>1) every rank
runs its own 16 replicates (replicate seeds offset by rank): weak scaling,
no data-path collective.

--impl reference times the CPU restatement of the sde-sim-rs algorithm (the
oracle: the Rust reference cannot be built here) on all host cores, on a
bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sde-sim-rs_gb300"))
sys.path.insert(0, ROOT)

HESTON = ["dv = (2 * (0.04 - max(v, 0))) * dt + (0.3 * max(v, 0)^0.5) * dW1",
          "dS = (0.03 * S) * dt + (-0.7 * max(v, 0)^0.5 * S) * dW1 + "
          "(0.714142842854285 * max(v, 0)^0.5 * S) * dW2"]
PAYOFF = "max(S - 100, 0)"
INIT = {"S": 100.0, "v": 0.04}
STEPS_T = 256
N_PATHS = 1 << 20
REPS = 16
SEED = 7
# transcendental (SFU) operations per path-step as written: two normals
# (log, sqrt, divide each) and sqrt(max(v, 0))
SFU_PER_PATH_STEP = 7
METRIC = "path-steps/s (fwd, Heston RQMC, FP32 stepping)"
WORKLOAD = "heston_rqmc_sobol_xor_2^20x16_256steps"


def times():
    return [i / STEPS_T for i in range(STEPS_T + 1)]


def dist_init(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return rank, world


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu_index: int):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = float(parts[2])
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(threads: int, paths: int):
    """Time the oracle on `paths` paths of replicate 0 (FP64, same equations,
    same scrambled Sobol inputs).  Returns (path-steps/s, seconds)."""
    from oracle import oracle as O
    O.build()
    u = O.Universe(HESTON)
    t0 = time.perf_counter()
    u.estimate(times(), INIT, 0, paths, PAYOFF, rng=O.SOBOL, scramble=O.XOR, seed=SEED,
               n_per_replicate=N_PATHS, threads=threads)
    dt = time.perf_counter() - t0
    return paths * STEPS_T / dt, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    paths = args.cpu_paths
    for _ in range(args.warmup):
        cpu_sample(threads, max(1024, paths // 16))
    vals = []
    for _ in range(args.steps):
        v, _ = cpu_sample(threads, paths)
        vals.append(v)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "path-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": paths * STEPS_T / value * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "paths": N_PATHS, "replicates": REPS, "steps": STEPS_T,
                       "sample_paths_per_step": paths},
            "cpu_baseline": {"value": value, "unit": "path-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{paths} paths x {STEPS_T} steps of replicate 0 per step "
                                       "(CPU restatement of the sde-sim-rs algorithm, FP64; the Rust "
                                       "reference cannot be built on this host)"},
            "e2e": {"value": value, "unit": "path-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_engine(args):
    import numpy as np
    import torch
    rank, world = dist_init(args.gpus)
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    import sde_sim_rs
    from sde_sim_rs import _native as N
    import ctypes as C

    npaths, reps = args.paths, args.reps
    plan = sde_sim_rs.Plan(HESTON, payoffs=[PAYOFF], rng="sobol", scramble="xor", precision="fp32",
                           output="none")
    T = times()
    stream = torch.cuda.current_stream()
    seed = SEED + rank * reps
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def one(p=plan, n=npaths):
        return p.run(T, INIT, n, replicates=reps, seed=seed, stream=stream)

    for _ in range(args.warmup):
        one().estimates()
    torch.cuda.synchronize()

    # device-timed region: CUDA events on the launching stream, L2 flushed
    # between steps (outside the events)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    results = []
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for k in range(args.steps):
            flush.fill_(k & 0xFF)
            ev[k][0].record(stream)
            results.append(one())
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = [a.elapsed_time(b) for a, b in ev]
    ms_step = sum(ms) / len(ms)
    if world > 1:
        t = torch.tensor([ms_step], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_step = float(t.item())
    path_steps = npaths * reps * STEPS_T
    value = path_steps * world / (ms_step * 1e-3)
    sums = results[-1].estimates()[0][:, 0]
    rep_means = sums / npaths
    price = float(rep_means.mean())
    price_se = float(rep_means.std(ddof=1) / math.sqrt(reps))

    # end to end through the public API: pinned H2D of the step's inputs,
    # kernel, D2H of the estimates, every step (host wall clock)
    h2d = (len(T) * 3 + 2 * (len(T) - 1)) * 8 + len(T) * (4 + 4) + 64
    e2e_t = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        one().estimates()
        e2e_t.append(time.perf_counter() - t0)
    e2e_val = path_steps / statistics.median(e2e_t)

    # the plain FP64 GPU path on the same scrambled inputs (a sample of the
    # paths): its throughput and the FP32 estimate's deviation from it
    fp64 = None
    if args.fp64_paths:
        p64 = sde_sim_rs.Plan(HESTON, payoffs=[PAYOFF], rng="sobol", scramble="xor", precision="fp64",
                              output="none")
        n64 = args.fp64_paths
        one(p64, n64).estimates()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r64 = one(p64, n64)
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        r32 = one(plan, n64)
        m64 = r64.estimates()[0][:, 0] / n64
        m32 = r32.estimates()[0][:, 0] / n64
        v64 = n64 * reps * STEPS_T / (ms64 * 1e-3)
        bias = float(np.abs(m32 - m64).max())
        se64 = float(m64.std(ddof=1) / math.sqrt(reps))
        fp64 = {"value": v64, "unit": "path-steps/s", "sample": f"{n64} paths x {reps} replicates",
                "estimate": float(m64.mean()),
                "fp32_minus_fp64_max_abs_per_replicate": bias, "rqmc_se_at_sample": se64,
                "equal_rmse_speedup": value / v64 * (1.0 if bias < se64 else (se64 / bias) ** 2)}

    # roofline: SFU bound; peak measured by a MUFU throughput probe
    peak = C.c_double()
    N.check(N.lib().sde_probe_sfu_peak(C.byref(peak)))
    sfu_ops = path_steps * SFU_PER_PATH_STEP
    achieved = sfu_ops / (ms_step * 1e-3)

    if rank == 0:
        cpu_v, cpu_s = cpu_sample(os.cpu_count() or 1, args.cpu_paths) if args.cpu_baseline else (None, 0)
        line = {
            "metric": METRIC, "value": value, "unit": "path-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Sobol XOR scrambles)",
            "config": {"workload": WORKLOAD if (npaths, reps) == (N_PATHS, REPS) else
                       f"heston_rqmc_sobol_xor_{npaths}x{reps}_256steps (reduced)",
                       "paths": npaths, "replicates": reps, "steps": STEPS_T,
                       "l2": "flushed (256 MiB write) between timed steps",
                       "estimate": price, "estimate_se_rqmc": price_se},
            "clocks": clk.summary(),
            "e2e": {"value": e2e_val, "unit": "path-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": reps * 16},
            "fp64_gpu": fp64,
            "gpu_launches": 3 * args.steps,
            "roofline": {"bound": "sfu", "achieved": achieved / 1e9, "peak": peak.value / 1e9,
                         "unit": "Gop/s", "frac": achieved / peak.value, "traffic": None,
                         "peak_source": "measured by sde_probe_sfu_peak (MUFU throughput probe)",
                         "algorithmic_ops_per_launch": sfu_ops},
            "cpu_baseline": {"value": cpu_v, "unit": "path-steps/s", "cores": os.cpu_count(),
                             "kind": "port",
                             "sample": f"{args.cpu_paths} paths x {STEPS_T} steps of replicate 0, FP64 "
                                       f"oracle ({cpu_s:.1f} s)"},
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--cpu-paths", type=int, default=1 << 17)
    ap.add_argument("--paths", type=int, default=N_PATHS)
    ap.add_argument("--reps", type=int, default=REPS)
    ap.add_argument("--fp64-paths", type=int, default=1 << 14)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
