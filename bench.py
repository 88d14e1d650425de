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
# transcendental (SFU) operations per path-step of the formula as written:
# two normals (log, sqrt, divide each) and sqrt(max(v, 0)); the algorithmic
# count (the kernel issues 6: a pair of normals shares one reciprocal)
SFU_PER_PATH_STEP = 7
METRIC = "path-steps/s (fwd, Heston RQMC, FP32 stepping)"
WORKLOAD = "heston_rqmc_sobol_xor_2^20x16_256steps"


def times():
    return [i / STEPS_T for i in range(STEPS_T + 1)]


# ---- 64-dimensional correlated basket --------------------------------------

def basket_equations(dim: int = 64, seed: int = 2024):
    """GBM basket in the reference grammar: sigma_i ~ U(0.1, 0.5), mu = 0.02,
    correlation 0.3 off the diagonal plus a 0.2-scaled random-orthogonal
    perturbation, projected to PSD (eigenvalues clipped, unit diagonal
    restored), FP64 Cholesky factor L.  Process i's diffusion terms are
    (L_ij sigma_i * S_i) * dW_j, j <= i."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sigma = rng.uniform(0.1, 0.5, dim)
    q, _ = np.linalg.qr(rng.standard_normal((dim, dim)))
    pert = q @ np.diag(rng.uniform(-1.0, 1.0, dim)) @ q.T
    np.fill_diagonal(pert, 0.0)
    corr = 0.3 * (np.ones((dim, dim)) - np.eye(dim)) + np.eye(dim) + 0.2 * pert
    w, v = np.linalg.eigh((corr + corr.T) / 2)
    corr = v @ np.diag(np.clip(w, 1e-6, None)) @ v.T
    d = np.sqrt(np.diag(corr))
    corr = corr / np.outer(d, d)
    L = np.linalg.cholesky(corr)
    eqs = []
    for i in range(dim):
        terms = [f"(0.02 * S{i + 1}) * dt"]
        for j in range(i + 1):
            terms.append(f"({float(L[i, j] * sigma[i])!r} * S{i + 1}) * dW{j + 1}")
        eqs.append(f"dS{i + 1} = " + " + ".join(terms))
    payoff = "max((" + " + ".join(f"S{i + 1}" for i in range(dim)) + f") / {dim} - 100, 0)"
    return eqs, payoff, sigma, L


def combine_ranks(ms_step: float, rep_means, world: int):
    """Weak-scaled replicas across ranks: the job's step time is the slowest
    rank's, and the replicate means of all ranks (disjoint replicate seeds)
    form one RQMC estimate.  Returns (ms_step, estimate, se, n_replicates).
    Works with any initialised torch.distributed backend (NCCL on the GPUs,
    gloo in the CPU test)."""
    import torch
    import torch.distributed as dist
    means = torch.as_tensor(rep_means, dtype=torch.float64).reshape(-1)
    if world > 1:
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([ms_step], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
        parts = [torch.zeros_like(means, device=dev) for _ in range(world)]
        dist.all_gather(parts, means.to(dev))
        means = torch.cat([p.cpu() for p in parts])
    n = means.numel()
    est = float(means.mean())
    se = float(means.std(unbiased=True) / math.sqrt(n)) if n > 1 else float("nan")
    return ms_step, est, se, n


def dist_init(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return rank, world


class Clocks:
    """nvidia-smi sampling during the timed region.  The default timed region
    of the Heston workload is under 100 ms, so the interval is short enough
    to take several samples inside it."""

    INTERVAL_MS = 25

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
                                          "--format=csv,noheader,nounits", "-lms", str(self.INTERVAL_MS)],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        # the timed region starts once nvidia-smi is sampling: its start-up
        # (NVML initialisation) otherwise lands inside a short timed region
        t0 = time.perf_counter()
        while self.proc is not None and time.perf_counter() - t0 < 3.0:
            if self.proc.poll() is not None or os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)
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
                "reasons": sorted(reasons), "samples": len(sm), "interval_ms": self.INTERVAL_MS}


# The oracle's RNG modes: the bench's XOR replicates (not a reference mode),
# the reference's own Sobol mode (point s+5 shifted by the scenario's ChaCha8
# doubles, src/rng/sobol.rs:35-79) and its default pseudo-random mode
# (ChaCha8 per scenario, src/rng/pseudo.rs:14-31).
CPU_MODES = ("sobol_xor", "sobol_shift", "pseudo")


def cpu_sample(threads: int, paths: int, mode: str = "sobol_xor"):
    """Time the oracle on `paths` paths of replicate 0 (FP64, same equations,
    same random inputs as the GPU arm in the XOR mode).  Returns
    (path-steps/s, seconds)."""
    from oracle import oracle as O
    O.build()
    u = O.Universe(HESTON)
    rng, scr = {"sobol_xor": (O.SOBOL, O.XOR), "sobol_shift": (O.SOBOL, O.SHIFT),
                "pseudo": (O.PSEUDO, O.SHIFT)}[mode]
    t0 = time.perf_counter()
    u.estimate(times(), INIT, 0, paths, PAYOFF, rng=rng, scramble=scr, seed=SEED,
               n_per_replicate=N_PATHS, threads=threads)
    dt = time.perf_counter() - t0
    return paths * STEPS_T / dt, dt


def cpu_rate(threads: int, paths: int, warmup: int, samples: int, mode: str = "sobol_xor"):
    """Warmed median of the oracle's throughput: `warmup` untimed runs on a
    sixteenth of the sample (library load, Sobol tables, thread start-up),
    then the median of `samples` timed runs.  Both arms use this sampler."""
    for _ in range(max(1, warmup)):
        cpu_sample(threads, max(1024, paths // 16), mode)
    vals = [cpu_sample(threads, paths, mode)[0] for _ in range(max(1, samples))]
    return statistics.median(vals)


def cpu_modes(threads: int, paths: int, samples: int = 3):
    """The oracle's rate in the reference's own RNG modes beside the XOR one."""
    return {m: cpu_rate(threads, paths, 1, samples, m) for m in CPU_MODES if m != "sobol_xor"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    paths = args.cpu_paths
    value = cpu_rate(threads, paths, args.warmup, args.steps)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "path-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": paths * STEPS_T / value * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "paths": N_PATHS, "replicates": REPS, "steps": STEPS_T,
                       "sample_paths_per_step": paths},
            "cpu_baseline": {"value": value, "unit": "path-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{paths} paths x {STEPS_T} steps of replicate 0 per step "
                                       "(CPU restatement of the sde-sim-rs algorithm, FP64; the Rust "
                                       "reference cannot be built on this host)",
                             "reference_modes": cpu_modes(threads, paths, min(3, args.steps)),
                             "note": "value: the XOR-scrambled Sobol inputs of the GPU arm; reference_modes: "
                                     "the same sample in the reference's own Sobol (shifted point s+5) and "
                                     "pseudo-random (ChaCha8) modes"},
            "e2e": {"value": value, "unit": "path-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def equal_rmse_speedup(thr32: float, thr64: float, bias: float, se: float):
    """Throughput ratio at equal estimator RMSE.  With RMSE^2 = se^2 N / N'
    + bias^2 (se: the FP64 estimator's standard error at N paths; bias: the
    FP32 estimate minus the FP64 one on the same random inputs), FP32 needs
    N' = N se^2 / (se^2 - bias^2) paths to match the FP64 RMSE at N, so the
    time ratio is (thr32 / thr64) (1 - bias^2 / se^2); 0 when the bias alone
    exceeds the FP64 error."""
    if not (se > 0 and math.isfinite(se)):
        return None
    f = 1.0 - (bias / se) ** 2
    return thr32 / thr64 * f if f > 0 else 0.0


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
    sums = results[-1].estimates()[0][:, 0]
    ms_step, price, price_se, _ = combine_ranks(sum(ms) / len(ms), sums / npaths, world)
    path_steps = npaths * reps * STEPS_T
    value = path_steps * world / (ms_step * 1e-3)

    # end to end through the public API: pinned H2D of the step's inputs,
    # kernel, D2H of the estimates, every step (host wall clock)
    h2d = (len(T) * 3 + 2 * (len(T) - 1)) * 8 + len(T) * (4 + 4) + 64
    e2e_t = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        one().estimates()
        e2e_t.append(time.perf_counter() - t0)
    e2e_val = path_steps / statistics.median(e2e_t)

    # the same workload on the reference's own Sobol mode (point s + 5 of
    # scenario s, shifted by the scenario's ChaCha8 doubles), FP32 stepping
    ps_plan = sde_sim_rs.Plan(HESTON, payoffs=[PAYOFF], rng="sobol", scramble="shift", precision="fp32",
                              output="none")
    one(ps_plan).estimates()
    ms_sh = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.fill_(1)
        e0.record(stream)
        r_sh = one(ps_plan)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_sh.append(e0.elapsed_time(e1))
    sh_price = float(r_sh.estimates()[0][:, 0].sum() / (npaths * reps))
    shift_leg = {"value": path_steps / (statistics.median(ms_sh) * 1e-3), "unit": "path-steps/s",
                 "ms": statistics.median(ms_sh), "estimate": sh_price,
                 "note": "the reference's Sobol mode: point s+5, ChaCha8 shift per scenario and dimension"}

    # the plain FP64 GPU path on the same scrambled inputs at the same size
    # (2^20 paths x 16 replicates), warmed and L2-flushed like the FP32 leg:
    # its throughput, the FP32 estimate's deviation from it, and the speedup
    # at equal RMSE with the RQMC standard error at full size
    fp64 = None
    if args.fp64_paths:
        p64 = sde_sim_rs.Plan(HESTON, payoffs=[PAYOFF], rng="sobol", scramble="xor", precision="fp64",
                              output="none")
        n64 = min(args.fp64_paths, npaths)
        one(p64, n64).estimates()
        ms64, r64 = _timed_runs(lambda: one(p64, n64), 2, stream, flush)
        m64 = r64[-1].estimates()[0][:, 0] / n64
        m32 = (sums / npaths if n64 == npaths else one(plan, n64).estimates()[0][:, 0] / n64)
        v64 = n64 * reps * STEPS_T / (statistics.median(ms64) * 1e-3)
        bias = float(np.mean(m32 - m64))
        se64 = float(m64.std(ddof=1) / math.sqrt(reps))
        fp64 = {"value": v64, "unit": "path-steps/s", "ms": statistics.median(ms64),
                "sample": f"{n64} paths x {reps} replicates (the FP32 leg's size)" if n64 == npaths
                else f"{n64} paths x {reps} replicates",
                "estimate": float(m64.mean()),
                "fp32_minus_fp64": bias,
                "fp32_minus_fp64_max_abs_per_replicate": float(np.abs(m32 - m64).max()),
                "rqmc_se": se64,
                "equal_rmse_speedup": equal_rmse_speedup(value / world, v64, bias, se64),
                "model": "RMSE^2 = se^2 N/N' + bias^2, se of the FP64 RQMC estimate at this size"}

    # the metric's forward+adjoint half: pathwise Greeks of GBM and Heston,
    # 2^20 paths x 365 steps, FP32 forward + reverse sweep, against the plain
    # FP64 GPU forward at the same size
    adjoint = adjoint_legs(args, stream, flush, min(npaths, 1 << 20)) if args.adjoint else None
    # the same Greeks through the reference's Runge-Kutta scheme (its cache
    # semantics), against the plain FP64 Runge-Kutta forward
    adjoint_rk = adjoint_legs(args, stream, flush, min(npaths, 1 << 20), scheme="runge-kutta") if args.adjoint else None
    # and the target's own configuration: the 4096 uneven instances, forward
    # and forward+adjoint in one graph-captured launch each, against 4096
    # per-instance FP64 forward launches
    batched = batched_legs(args, stream, flush) if args.batched else None
    # the reference's own configuration (GBM, 10,000 paths, FP64, full
    # filtration) and the memory-bound 64-dim basket, each as its own line
    others = {}
    if rank == 0 and args.others:
        others["gbm_full"] = collected(run_gbm_full, args)
        others["basket"] = collected(run_basket, args)

    # roofline: SFU bound; peak measured by a MUFU throughput probe
    peak = C.c_double()
    N.check(N.lib().sde_probe_sfu_peak(C.byref(peak)))
    sfu_ops = path_steps * SFU_PER_PATH_STEP
    achieved = sfu_ops / (ms_step * 1e-3)

    if rank == 0:
        threads = os.cpu_count() or 1
        cpu_v = cpu_rate(threads, args.cpu_paths, 1, 3) if args.cpu_baseline else None
        cpu_m = cpu_modes(threads, args.cpu_paths) if args.cpu_baseline else None
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
            "sobol_shift_fp32": shift_leg,
            "fwd_adjoint": adjoint,
            "fwd_adjoint_runge_kutta": adjoint_rk,
            "batched": batched,
            "other_configs": others or None,
            "gpu_launches": 3 * args.steps,
            "roofline": {"bound": "sfu", "achieved": achieved / 1e9, "peak": peak.value / 1e9,
                         "unit": "Gop/s", "frac": achieved / peak.value,
                         # ncu (1 pass, full size, 8 launches): 0.48 MB DRAM read
                         # per launch (the Sobol tables and masks), 0 B written
                         "traffic": 481.5e3,
                         "traffic_source": "profiles/bench_default_heston_rqmc_launch_list.md (full-size capture)",
                         "peak_source": "measured by sde_probe_sfu_peak (MUFU throughput probe)",
                         "algorithmic_ops_per_launch": sfu_ops},
            "cpu_baseline": {"value": cpu_v, "unit": "path-steps/s", "cores": threads,
                             "kind": "port",
                             "sample": f"{args.cpu_paths} paths x {STEPS_T} steps of replicate 0, FP64 "
                                       "oracle, median of 3 after a warm-up (the reference arm's sampler)",
                             "reference_modes": cpu_m},
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------
# Other configurations (not the default line): the reference's plain GBM,
# the batched instances, the pathwise adjoint and the 64-dim basket.
# ---------------------------------------------------------------------------

GBM = ["dX = (0.05 * X) * dt + (0.2 * X) * dW1"]
GBM_P = ["dX = (mu * X) * dt + (sigma * X) * dW1"]
OU_P = ["dX = (theta * (m - X)) * dt + (s) * dW1"]
HESTON_P = ["dv = (kappa * (theta - max(v, 0))) * dt + (xi * max(v, 0)^0.5) * dW1",
            "dS = (mu * S) * dt + (rho * max(v, 0)^0.5 * S) * dW1 + "
            "((1 - rho^2)^0.5 * max(v, 0)^0.5 * S) * dW2"]


def batched_instances(n=4096, seed=11, max_steps=1024, max_log2_paths=16):
    """Half GBM (mu ~ U(-0.05, 0.10), sigma ~ U(0.05, 0.6), X0 ~ U(50, 150)),
    half OU (theta ~ U(0.5, 5), m ~ N(0, 1), s ~ U(0.1, 1), X0 ~ N(0, 1));
    steps ~ U{16..max_steps}, paths = floor(2^U(8, max_log2_paths)), T = 1."""
    import numpy as np
    rng = np.random.default_rng(seed)
    half = n // 2
    tid = np.array([0] * half + [1] * (n - half), dtype=np.int32)
    steps = rng.integers(16, max_steps + 1, size=n)
    paths = np.floor(2.0 ** rng.uniform(8, max_log2_paths, size=n)).astype(np.uint64)
    params = np.zeros((n, 3))
    x0 = np.zeros((n, 1))
    params[:half, 0] = rng.uniform(-0.05, 0.10, half)
    params[:half, 1] = rng.uniform(0.05, 0.6, half)
    x0[:half, 0] = rng.uniform(50, 150, half)
    params[half:, 0] = rng.uniform(0.5, 5, n - half)
    params[half:, 1] = rng.normal(0, 1, n - half)
    params[half:, 2] = rng.uniform(0.1, 1, n - half)
    x0[half:, 0] = rng.normal(0, 1, n - half)
    seeds = np.arange(n, dtype=np.uint64) * np.uint64(1 << 20) + np.uint64(seed)
    return tid, steps, paths, seeds, x0, params


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {"hbm_gbs": 6800.0, "source": "fallback"}


def _timed_runs(fn, steps, stream, flush):
    """CUDA-event time of each of `steps` runs, L2 flushed before each
    (outside the events).  Only the latest run's result is kept alive: the
    one before it is released once the next is queued (its release waits for
    its own work only), so device memory holds at most two runs' buffers
    (a 64-dim basket run holds 17 GB).  Returns (ms list, [last result])."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    last = None
    torch.cuda.synchronize()
    for k in range(steps):
        flush.fill_(k & 0xFF)
        ev[k][0].record(stream)
        r = fn()
        ev[k][1].record(stream)
        last = r
        del r
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev], [last]


def _chacha_roofline(path_steps_per_s, blocks_per_path_step, note, traffic,
                     source="profiles/sde_batch_and_adjoint_pseudo.md (full-size one-pass capture)"):
    """Roofline of a pseudo-random kernel: the ChaCha8 blocks it consumes per
    second against the GPU's block rate measured by sde_probe_chacha8_rate
    (the reference's generator is the bound: ALU / issue)."""
    import ctypes as C
    from sde_sim_rs import _native as N
    peak = C.c_double()
    N.check(N.lib().sde_probe_chacha8_rate(C.byref(peak)))
    achieved = path_steps_per_s * blocks_per_path_step
    return {"bound": "alu (ChaCha8)", "achieved": achieved / 1e9, "peak": peak.value / 1e9, "unit": "Gblock/s",
            "frac": achieved / peak.value, "traffic": traffic,
            "traffic_source": source,
            "peak_source": "measured by sde_probe_chacha8_rate (every thread generates its own blocks)",
            "algorithmic_blocks_per_path_step": blocks_per_path_step, "note": note}


def _common(args, workload, metric, value, ms, dtype, clocks, e2e, launches, roofline, cpu, extra):
    line = {"metric": metric, "value": value, "unit": "path-steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": dict(workload=workload, l2="flushed (256 MiB write) between timed steps", **extra),
            "clocks": clocks, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
            "cpu_baseline": cpu}
    if getattr(args, "collect", None) is not None:
        args.collect.append(line)
    else:
        print(json.dumps(line), flush=True)


def collected(run, args):
    """Runs another configuration's bench and returns its line as a dict
    (nested in the default line) instead of printing it."""
    args.collect = []
    try:
        run(args)
        return args.collect[-1]
    finally:
        args.collect = None


def run_gbm_full(args):
    """The reference's plain configuration: GBM, Euler, 252 steps, 10,000
    paths, ChaCha8 seed 42, FP64, full filtration of 253 time points."""
    import numpy as np
    import torch
    import sde_sim_rs
    from oracle import oracle as O
    n, T = 10000, [i / 252 for i in range(253)]
    plan = sde_sim_rs.Plan(GBM, precision="fp64", output="full", chunked=args.chunked)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    one = lambda: plan.run(T, {"X": 100.0}, n, seed=42, stream=stream)
    for _ in range(args.warmup):
        one().wait()
    with Clocks(0) as clk:
        ms, res = _timed_runs(one, args.steps, stream, flush)
    ms_step = sum(ms) / len(ms)
    ps = n * 252
    xt = res[-1].values("device")[0, -1, 0]
    # the drop-in's first call lowers and loads the universe; later calls
    # with the same equations reuse it
    sde_sim_rs.simulate(GBM, T, n, {"X": 100.0}, "pseudo", "euler", seed=42, output_format="numpy")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fr = sde_sim_rs.simulate(GBM, T, n, {"X": 100.0}, "pseudo", "euler", seed=42, output_format="numpy")
    e2e_s = (time.perf_counter() - t0) / args.steps
    rows = len(fr["value"])
    nbytes = n * 253 * 8
    peak = _peaks()
    u = O.Universe(GBM)
    c0 = time.perf_counter()
    u.simulate(T, {"X": 100.0}, 0, n, seed=42, threads=os.cpu_count() or 1)
    cpu_s = time.perf_counter() - c0
    _common(args, "gbm_euler_fp64_10000x253_full", "path-steps/s (fwd, GBM full filtration, FP64)",
            ps / (ms_step * 1e-3), ms_step, "f64", clk.summary(),
            {"value": ps / e2e_s, "unit": "path-steps/s", "h2d_bytes_per_step": 253 * 28,
             "d2h_bytes_per_step": rows * 8, "through": "sde_sim_rs.simulate (long frame)",
             "note": "the value column is copied every call; the scenario, time and process columns "
                     "(16 B a row) are the shape's, copied once and shared by later calls of that shape"},
            2 * args.steps,
            {"bound": "hbm", "achieved": nbytes / (ms_step * 1e-3) / 1e9, "peak": peak["hbm_gbs"], "unit": "GB/s",
             "frac": nbytes / (ms_step * 1e-3) / 1e9 / peak["hbm_gbs"],
             # ncu of the chunked kernel at this size: 151 KB read; the 20 MB of
             # filtration writes are still in L2 when the kernel ends
             "traffic": 150530.0 if args.chunked != "off" else 106496.0,
             "traffic_source": "profiles/sde_step_euler_fp64_pseudo_gbm_c0.md (full-size capture)",
             "note": "not a bandwidth case: the chunked kernel is bound by the FP64 pipe (78% busy in ncu; "
                     "~119 FP64 lane-ops per path-step, the FP64 inverse CDF), one thread per path by latency"},
            {"value": ps / cpu_s, "unit": "path-steps/s", "cores": os.cpu_count(), "kind": "port",
             "sample": "full size (10,000 paths x 252 steps, full filtration)"},
            {"paths": n, "steps": 252, "chunked": args.chunked, "mean_XT": float(xt.mean()),
             "exact_mean": 100 * math.exp(0.05),
             "std_XT": float(xt.std()), "exact_std": 100 * math.exp(0.05) * math.sqrt(math.exp(0.04) - 1)})


def run_basket(args):
    """64-dim correlated GBM basket: Euler, 128 steps, 2^21 paths, XOR Sobol
    dimension 8192, FP32 filtration at 32 equally spaced checkpoints."""
    import numpy as np
    import torch
    import sde_sim_rs
    from oracle import oracle as O
    eqs, payoff, _, _ = basket_equations()
    n = args.paths if args.paths != N_PATHS else 1 << 21
    T = [i / 128 for i in range(129)]
    ck = list(range(4, 129, 4))
    init = {f"S{i + 1}": 100.0 for i in range(64)}
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    # the CUDA-core kernel (one FMA chain per process) and the tcgen05 one
    # (the 64 x 64 diffusion product as three FP16 MMAs per 16 indices and
    # 128 paths, FP32 accumulation)
    legs = {}
    for leg, tc in (("cuda_cores", False), ("tensor_cores_row", "row"), ("tensor_cores", True)):
        if tc and args.cuda_cores_only:
            continue
        plan = sde_sim_rs.Plan(eqs, payoffs=[payoff], rng="sobol", scramble="xor", precision="fp32",
                               output="checkpoints", tensor_cores=tc)
        one = lambda plan=plan: plan.run(T, init, n, seed=7, checkpoints=ck, stream=stream)
        for _ in range(args.warmup):
            one().wait()
        with Clocks(0) as clk:
            ms, res = _timed_runs(one, args.steps, stream, flush)
        s, q = res[-1].estimates()
        del res
        price = s[0, 0] / n
        legs[leg] = {"plan": plan, "one": one, "clk": clk, "ms": sum(ms) / len(ms), "price": price,
                     "se": math.sqrt(max(q[0, 0] / n - price ** 2, 0) / n), "tc": plan.uses_tensor_cores}
    main_leg = legs.get("tensor_cores", legs["cuda_cores"])
    one, clk, ms_step = main_leg["one"], main_leg["clk"], main_leg["ms"]
    price, se = main_leg["price"], main_leg["se"]
    ps = n * 128
    nbytes = n * 64 * 32 * 4
    peak = _peaks()
    # the compute fractions beside the HBM one: the lower-triangular K w is
    # 2,080 FMA = 4,160 flop per path-step (the tensor pipe executes three
    # split products of the full 64 x 64: 24,576 flop), against the measured
    # bf16 tensor peak; 64 normals x 3 SFU ops (lg2, rsqrt, rcp) per
    # path-step against the measured MUFU throughput
    from sde_sim_rs import _native as N
    import ctypes as C
    sfu_peak = C.c_double()
    N.check(N.lib().sde_probe_sfu_peak(C.byref(sfu_peak)))
    flop_alg = 4160.0 * ps
    sfu_ops = 192.0 * ps
    compute = {
        "tensor": {"achieved": flop_alg / (ms_step * 1e-3) / 1e12, "peak": peak.get("bf16_tflops"), "unit": "TFLOP/s",
                   "frac": (flop_alg / (ms_step * 1e-3) / 1e12 / peak["bf16_tflops"]) if peak.get("bf16_tflops") else None,
                   "algorithmic_flop_per_launch": flop_alg, "executed_flop_per_launch": 24576.0 * ps,
                   "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)"},
        "sfu": {"achieved": sfu_ops / (ms_step * 1e-3) / 1e9, "peak": sfu_peak.value / 1e9, "unit": "Gop/s",
                "frac": sfu_ops / (ms_step * 1e-3) / sfu_peak.value, "ops_per_launch": sfu_ops,
                "peak_source": "measured by sde_probe_sfu_peak (MUFU throughput probe)"}}
    t0 = time.perf_counter()
    for _ in range(2):
        one().estimates()
    e2e_s = (time.perf_counter() - t0) / 2
    # the basket price's error against FP64 on the same inputs: the plain FP64
    # GPU plan on the first n_s paths (XOR points 0..n_s-1, the timed run's
    # first paths), each FP32 leg on the same paths, per-path payoff
    # differences; and against the FP64 oracle on the CPU sample below
    n_s = min(n, 1 << 17)
    p64 = sde_sim_rs.Plan(eqs, rng="sobol", scramble="xor", precision="fp64", output="terminal")
    x64 = p64.run(T, init, n_s, seed=7, stream=stream).values()[0, :, -1, :]
    pay = lambda x: np.maximum(x.sum(axis=1) / 64 - 100.0, 0.0)
    pay64 = pay(x64)
    for v in legs.values():
        x32 = v["plan"].run(T, init, n_s, seed=7, checkpoints=[128], stream=stream).values()[0, :, -1, :]
        d = pay(x32) - pay64
        v["price_minus_fp64"] = float(d.mean())
        v["price_minus_fp64_se"] = float(d.std(ddof=1) / math.sqrt(n_s))
        v["max_abs_rel_terminal_vs_fp64"] = float(np.max(np.abs(x32 - x64) / np.abs(x64)))
        v["x32_head"] = x32[:512]
    u = O.Universe(eqs)
    cpu_n = 512
    c0 = time.perf_counter()
    xo = u.simulate(T, init, 0, cpu_n, rng=O.SOBOL, scramble=O.XOR, seed=7, n_per_replicate=n, full=False,
                    threads=os.cpu_count() or 1)
    cpu_s = time.perf_counter() - c0
    oracle_err = {k: {"price_minus_oracle": float((pay(v["x32_head"]) - pay(xo)).mean()),
                      "max_abs_rel_terminal_vs_oracle": float(np.max(np.abs(v.pop("x32_head") - xo) / np.abs(xo)))}
                  for k, v in legs.items()}
    _common(args, "basket64_euler_fp32_sobolxor_2^21x128_32ckpt", "path-steps/s (fwd, 64-dim basket, FP32)",
            ps / (ms_step * 1e-3), ms_step, "f32", clk.summary(),
            {"value": ps / e2e_s, "unit": "path-steps/s", "h2d_bytes_per_step": 129 * 28 + 64 * 8,
             "d2h_bytes_per_step": 16, "note": "filtration stays in HBM; the estimate is read back"},
            3 * args.steps,
            {"bound": "hbm", "achieved": nbytes / (ms_step * 1e-3) / 1e9, "peak": peak["hbm_gbs"], "unit": "GB/s",
             "frac": nbytes / (ms_step * 1e-3) / 1e9 / peak["hbm_gbs"],
             # ncu of the tensor-core kernel (1 pass, full size): 17.12 GB
             # written + 38.2 MB read
             "traffic": 17.12e9 + 38.16e6 if main_leg["tc"] else None,
             "traffic_source": "profiles/sde_step_basket64_tc_fp16.md (full-size capture)",
             "bytes_written_per_launch": nbytes},
            {"value": cpu_n * 128 / cpu_s, "unit": "path-steps/s", "cores": os.cpu_count(), "kind": "port",
             "sample": f"{cpu_n} paths x 128 steps, FP64 oracle, terminal values"},
            {"paths": n, "steps": 128, "checkpoints": 32, "price": price, "price_se": se,
             "price_minus_fp64": main_leg["price_minus_fp64"], "price_minus_fp64_se": main_leg["price_minus_fp64_se"],
             "fp64_error_sample": f"FP64 GPU plan on the first {n_s} paths (same XOR points), per-path payoff "
                                  f"differences; oracle: the first {cpu_n} paths",
             "oracle_error": oracle_err,
             "roofline_compute": compute,
             "kernel": "tcgen05 (3 x FP16 split, FP32 accumulate)" if main_leg["tc"] else "CUDA cores",
             "legs": {k: {"ms": v["ms"], "path_steps_per_s": ps / (v["ms"] * 1e-3), "price": v["price"],
                          "price_minus_fp64": v["price_minus_fp64"], "price_minus_fp64_se": v["price_minus_fp64_se"],
                          "max_abs_rel_terminal_vs_fp64": v["max_abs_rel_terminal_vs_fp64"],
                          "tensor_cores": v["tc"]} for k, v in legs.items()}})


def batched_legs(args, stream, flush):
    """4096 uneven GBM / OU instances in one persistent graph-captured launch
    (FP32): the forward batch, and the forward+adjoint batch (gradients of
    E[X_T] with respect to every parameter and X0), each against 4096 plain
    per-instance FP64 forward launches on the same paths."""
    import numpy as np
    import torch
    import sde_sim_rs
    from sde_sim_rs.batch import Batch
    tid, steps, paths, seeds, x0, params = batched_instances(n=args.instances)
    fwd_t = [sde_sim_rs.Plan(GBM_P, params=["mu", "sigma"], payoffs=["X"], precision="fp32", output="none"),
             sde_sim_rs.Plan(OU_P, params=["theta", "m", "s"], payoffs=["X"], precision="fp32", output="none")]
    adj_t = [sde_sim_rs.Plan(GBM_P, params=["mu", "sigma"], payoffs=["X"], grad_params=["mu", "sigma"],
                             grad_x0=["X"], precision="fp32", output="none"),
             sde_sim_rs.Plan(OU_P, params=["theta", "m", "s"], payoffs=["X"], grad_params=["theta", "m", "s"],
                             grad_x0=["X"], precision="fp32", output="none")]
    # baseline: plain per-instance FP64 forward launches
    pg = sde_sim_rs.Plan(GBM_P, params=["mu", "sigma"], payoffs=["X"], precision="fp64", output="none")
    po = sde_sim_rs.Plan(OU_P, params=["theta", "m", "s"], payoffs=["X"], precision="fp64", output="none")
    ps = int(np.sum(steps.astype(np.uint64) * paths))

    def fp64_launches(count=len(tid)):
        res = []
        for i in range(count):
            plan = pg if tid[i] == 0 else po
            res.append(plan.run(np.arange(steps[i] + 1) / steps[i], {"X": x0[i, 0]}, int(paths[i]),
                                seed=int(seeds[i]), params=params[i, :len(plan.params)], stream=stream))
        return res
    fp64_launches(64)[-1].wait()   # warm: both plans loaded (the first 64 instances)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = fp64_launches()
    torch.cuda.synchronize()
    fp64_s = time.perf_counter() - t0
    m64 = np.zeros(len(tid))
    se64 = np.zeros(len(tid))
    for i, r in enumerate(res):
        rs, rq = r.estimates()
        N = float(paths[i])
        m64[i] = rs[0, 0] / N
        se64[i] = math.sqrt(max(rq[0, 0] / N - m64[i] ** 2, 0) / N)
    thr64 = ps / fp64_s

    out = {}
    for leg, templates in (("forward", fwd_t), ("fwd_adjoint", adj_t)):
        t0 = time.perf_counter()
        job = Batch(templates).prepare(tid, steps, 1.0, paths, seeds, x0, params, autotune=True, stream=stream)
        prep_s = time.perf_counter() - t0
        for _ in range(args.warmup):
            job.run(stream).results()
        with Clocks(0) as clk:
            ms, _ = _timed_runs(lambda: job.run(stream), args.steps, stream, flush)
        ms_step = statistics.median(ms)
        s, q = job.results()
        t0 = time.perf_counter()
        for _ in range(3):
            job.run(stream).results()
        e2e_s = (time.perf_counter() - t0) / 3
        m32 = s[:, 0] / paths
        bias = m32 - m64
        z = np.abs(bias) / np.maximum(se64, 1e-300)
        thr = ps / (ms_step * 1e-3)
        # equal RMSE per instance (RMSE^2 = se^2 N/N' + bias^2), weighted by
        # each instance's share of the path-steps
        w = steps.astype(np.float64) * paths / ps
        frac = float(np.sum(w * np.clip(1.0 - (bias / np.maximum(se64, 1e-300)) ** 2, 0.0, None)))
        out[leg] = {"path_steps_per_s": thr, "ms": ms_step, "e2e_path_steps_per_s": ps / e2e_s, "prepare_s": prep_s,
                    "block": job.block, "paths_per_thread": job.paths_per_thread, "work_items": job.n_items,
                    "estimates_per_instance": job.n_payoffs, "clocks": clk.summary(),
                    "throughput_ratio_vs_fp64_launches": thr / thr64,
                    "equal_rmse_speedup_vs_fp64_launches": thr / thr64 * frac,
                    "fraction_within_3se_of_fp64": float(np.mean(z < 3)), "max_abs_z_vs_fp64": float(z.max())}
        if leg == "fwd_adjoint":
            # gradient of E[X_T] in X0 under Euler with n uniform steps:
            # (1 + mu/n)^n for GBM, (1 - theta/n)^n for OU (exact for the
            # discrete recursion; the OU one has no Monte Carlo error)
            g = tid == 0
            col = np.where(g, 3, 4)   # [payoff, (mu, sigma) | (theta, m, s), X0]
            rows = np.arange(len(tid))
            dx = s[rows, col] / paths
            dx_se = np.sqrt(np.maximum(q[rows, col] / paths - dx ** 2, 0) / paths)
            want = np.where(g, (1.0 + params[:, 0] / steps) ** steps, (1.0 - params[:, 0] / steps) ** steps)
            out[leg]["dX0_within_4se_of_discrete_closed_form"] = float(
                np.mean(np.abs(dx - want) <= 4 * dx_se + 1e-4 * np.abs(want)))
    out["fp64_per_instance_launches"] = {"path_steps_per_s": thr64, "seconds": fp64_s, "launches": int(len(tid))}
    out["config"] = {"instances": int(len(tid)), "path_steps": ps,
                     "adjoint": "gradients of E[X_T] in (mu, sigma, X0) for GBM and (theta, m, s, X0) for OU; "
                                "checkpoints every ceil(sqrt(steps)) steps, increments drawn again",
                     "path_steps_counted": "forward path-steps (paths x steps) for both legs"}
    return out


def run_batched(args):
    """4096 uneven GBM / OU instances in one persistent graph-captured launch
    (FP32), forward and forward+adjoint, against 4096 plain per-instance FP64
    forward launches."""
    import torch
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    out = batched_legs(args, stream, flush)
    f = out["forward"]
    clocks = f.pop("clocks")
    out["fwd_adjoint"].pop("clocks")
    _common(args, f"batched_{out['config']['instances']}_gbm_ou_fp32",
            f"path-steps/s (fwd, {out['config']['instances']} batched instances, FP32)",
            f["path_steps_per_s"], f["ms"], "f32", clocks,
            {"value": f["e2e_path_steps_per_s"], "unit": "path-steps/s", "h2d_bytes_per_step": 0,
             "d2h_bytes_per_step": out["config"]["instances"] * 16, "note": "graph replay + results read back"},
            2 * args.steps,
            # one Wiener index per instance: one u64 per path-step, 1/8 block
            _chacha_roofline(f["path_steps_per_s"], 1.0 / 8.0,
                             "each path-step draws one u64 of its scenario's ChaCha8 stream",
                             # ncu (1 pass, the full 4096 instances): 3.48 MB read, 0 B written
                             3.48e6),
            None, out)


ADJ_MODELS = (
    ("gbm", GBM_P, {"mu": 0.05, "sigma": 0.2}, ["mu", "sigma"], ["X"], {"X": 100.0}, "max(X - 100, 0)"),
    ("heston", HESTON_P, {"kappa": 2.0, "theta": 0.04, "xi": 0.3, "rho": -0.7, "mu": 0.03},
     ["kappa", "theta", "xi", "rho"], ["v"], {"S": 100.0, "v": 0.04}, "max(S - 100, 0)"))
ADJ_STEPS = 365


def adjoint_legs(args, stream, flush, n, scheme="euler"):
    """Pathwise Greeks of GBM (d/d mu, sigma, X0) and Heston (d/d kappa,
    theta, xi, rho, v0): 2^20 pseudo-random paths x 365 steps, checkpoints
    every 19 steps, FP32 forward + reverse sweep, L2 flushed between timed
    launches.  Beside it, on the same paths (same seeds): the plain FP64 GPU
    forward (timed the same way), and one FP64 adjoint run that gives every
    FP32 estimate and gradient its error against FP64."""
    import numpy as np
    import sde_sim_rs
    T = np.linspace(0.0, 1.0, ADJ_STEPS + 1)
    out = {}
    for name, eqs, params, gp, gx, init, pay in ADJ_MODELS:
        kw = dict(params=list(params), payoffs=[pay], scheme=scheme, output="none")
        adj = sde_sim_rs.Plan(eqs, grad_params=gp, grad_x0=gx, precision="fp32", **kw)
        f64 = sde_sim_rs.Plan(eqs, precision="fp64", **kw)
        a64 = sde_sim_rs.Plan(eqs, grad_params=gp, grad_x0=gx, precision="fp64", **kw)
        one_a = lambda: adj.run(T, init, n, seed=42, params=params, stream=stream)
        one_f = lambda: f64.run(T, init, n, seed=42, params=params, stream=stream)
        for _ in range(args.warmup):
            one_a().wait()
        one_f().wait()
        with Clocks(0) as clk:
            ms_a, ra = _timed_runs(one_a, args.steps, stream, flush)
        ms_f, rf = _timed_runs(one_f, 2, stream, flush)
        # end to end through the public API: the run (pinned H2D of the time
        # grid, parameters and initial values), the kernel, and the D2H of
        # the price and gradient sums, host wall clock
        e2e_t = []
        for _ in range(max(3, args.steps // 2)):
            t0 = time.perf_counter()
            one_a().estimates()
            e2e_t.append(time.perf_counter() - t0)
        s, q = ra[-1].estimates()
        m = s[0] / n
        se = np.sqrt(np.maximum(q[0] / n - m * m, 0) / n)
        s64, q64 = rf[-1].estimates()
        p64 = float(s64[0, 0] / n)
        se64 = float(math.sqrt(max(q64[0, 0] / n - p64 * p64, 0) / n))
        g64 = a64.run(T, init, n, seed=42, params=params, stream=stream).estimates()[0][0] / n
        ta, tf = statistics.median(ms_a), statistics.median(ms_f)
        thr_a, thr_f = n * ADJ_STEPS / (ta * 1e-3), n * ADJ_STEPS / (tf * 1e-3)
        # the same adjoint with its memory bounded by the checkpoints alone:
        # the reverse sweep draws the increments again instead of keeping
        # the forward pass's (N x steps x indices x 4 B) in device memory;
        # the same increments, so the same estimates bit for bit
        rec = sde_sim_rs.Plan(eqs, grad_params=gp, grad_x0=gx, precision="fp32", adjoint_recompute=True, **kw)
        one_r = lambda: rec.run(T, init, n, seed=42, params=params, stream=stream)
        one_r().wait()
        ms_r, rr = _timed_runs(one_r, max(3, args.steps // 2), stream, flush)
        same = bool(np.array_equal(rr[-1].estimates()[0], ra[-1].estimates()[0]))
        thr_r = n * ADJ_STEPS / (statistics.median(ms_r) * 1e-3)
        names = gp + gx
        out[name] = {"fwd_adjoint_path_steps_per_s": thr_a, "fp64_fwd_path_steps_per_s": thr_f,
                     "throughput_ratio_fp32_fwd_adj_vs_fp64_fwd": thr_a / thr_f,
                     "equal_rmse_speedup": equal_rmse_speedup(thr_a, thr_f, float(m[0]) - p64, se64),
                     "price_fp32": float(m[0]), "price_fp64": p64, "price_se": se64,
                     "price_fp32_minus_fp64": float(m[0]) - p64,
                     "gradients": dict(zip(names, [float(x) for x in m[1:]])),
                     "gradient_se": dict(zip(names, [float(x) for x in se[1:]])),
                     "gradient_fp32_minus_fp64": dict(zip(names, [float(x) for x in (m[1:] - g64[1:])])),
                     "ms": ta, "fp64_fwd_ms": tf,
                     "increments_kept_bytes": n * ADJ_STEPS * (len(eqs) + (scheme != "euler")) * 4,
                     "checkpoints_only": {"fwd_adjoint_path_steps_per_s": thr_r,
                                          "ms": statistics.median(ms_r),
                                          "throughput_ratio_vs_fp64_fwd": thr_r / thr_f,
                                          "equal_rmse_speedup": equal_rmse_speedup(thr_r, thr_f, float(m[0]) - p64,
                                                                                   se64),
                                          "checkpoint_bytes": n * ((ADJ_STEPS + 18) // 19) * len(eqs) *
                                          (1 if scheme == "euler" else 2) * 4,
                                          "estimates_equal_to_kept_increments": same},
                     "e2e_path_steps_per_s": n * ADJ_STEPS / statistics.median(e2e_t),
                     "clocks": clk.summary(), "n_estimates": 1 + len(names),
                     # the generator's roofline: one u64 per Wiener index and
                     # path-step; DRAM bytes per launch from the ncu launch
                     # list at 2^20 paths (Euler)
                     "roofline": _chacha_roofline(
                         thr_a, len(eqs) / 8.0, "forward draws plus the reverse sweep over stored increments",
                         {"gbm": 2.067e9 + 1.343e9, "heston": 4.671e9 + 2.922e9}[name] if scheme == "euler" else None,
                         "profiles/bench_default_heston_rqmc_launch_list.md (full-size one-pass capture)")}
    out["config"] = {"paths": n, "steps": ADJ_STEPS, "ckpt_every": 19, "rng": "pseudo (ChaCha8)",
                     "scheme": scheme, "l2": "flushed (256 MiB write) between timed launches",
                     "model": "equal_rmse_speedup: RMSE^2 = se^2 N/N' + bias^2 with the FP64 forward's se "
                              "at N and the FP32 price's bias against it on the same paths"}
    return out


def run_adjoint(args):
    """Pathwise adjoint Greeks, 2^20 paths, 365 steps, FP32 forward + reverse,
    checkpoints every 19 steps, against the plain FP64 GPU forward pass."""
    import torch
    n = args.paths if args.paths != N_PATHS else 1 << 20
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    out = adjoint_legs(args, stream, flush, n, scheme=args.scheme)
    g = out["gbm"]
    clocks = g.pop("clocks")
    out["heston"].pop("clocks")
    h2d = ((ADJ_STEPS + 1) * 3 + ADJ_STEPS * 2) * 8 + (ADJ_STEPS + 1) * (4 + 4) + 64
    e2e = {"value": g["e2e_path_steps_per_s"], "unit": "path-steps/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": g.pop("n_estimates") * 16,
           "through": "Plan.run(...).estimates() (price and gradient sums)"}
    out["heston"].pop("n_estimates")
    _common(args, f"adjoint_gbm_heston_2^20x365_{args.scheme}", f"path-steps/s (fwd+adjoint, GBM, FP32, {args.scheme})",
            g["fwd_adjoint_path_steps_per_s"], g["ms"], "f32", clocks, e2e, 2 * args.steps,
            _chacha_roofline(g["fwd_adjoint_path_steps_per_s"], 1.0 / 8.0,
                             "the forward pass draws one u64 per path-step; the reverse sweep reads the stored "
                             "increments back and adds the recompute and adjoint arithmetic",
                             # ncu (1 pass, GBM at 2^20 paths): 2.067 GB written (increments,
                             # checkpoints, segment spills) + 1.343 GB read
                             2.067e9 + 1.343e9),
            None, out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--cpu-paths", type=int, default=1 << 17)
    ap.add_argument("--paths", type=int, default=N_PATHS)
    ap.add_argument("--reps", type=int, default=REPS)
    ap.add_argument("--fp64-paths", type=int, default=N_PATHS,
                    help="heston_rqmc: paths per replicate of the FP64 GPU leg (default: the FP32 leg's)")
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-adjoint", dest="adjoint", action="store_false",
                    help="heston_rqmc: leave out the fwd+adjoint legs")
    ap.add_argument("--no-batched", dest="batched", action="store_false",
                    help="heston_rqmc: leave out the batched-instance legs")
    ap.add_argument("--no-others", dest="others", action="store_false",
                    help="heston_rqmc: leave out the GBM full-filtration and 64-dim basket lines")
    ap.add_argument("--scheme", default="euler", choices=["euler", "runge-kutta"],
                    help="adjoint: the scheme whose recursion the reverse sweep runs")
    ap.add_argument("--cuda-cores-only", action="store_true",
                    help="basket: time only the CUDA-core kernel (no tcgen05 leg)")
    ap.add_argument("--chunked", default="auto", choices=["auto", "on", "off"],
                    help="gbm_full: the FP64 kernel for few paths (auto: chosen by path count)")
    ap.add_argument("--workload", default="heston_rqmc",
                    choices=["heston_rqmc", "gbm_full", "basket", "batched", "adjoint"])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "heston_rqmc":
        run_engine(args)
    else:
        import torch
        torch.cuda.set_device(0)
        {"gbm_full": run_gbm_full, "basket": run_basket, "batched": run_batched,
         "adjoint": run_adjoint}[args.workload](args)


if __name__ == "__main__":
    main()
