"""GPU parity: the lowered sm_103a kernels through the C ABI against the CPU
oracle on the same seeded inputs.

Bars: integer RNG work (ChaCha8 words, Sobol points, scramble bits) is
bit-exact; FP64 paths agree within 1e-12 relative (|gpu-ref| <= 1e-12 *
max(|ref|, 1)); FP32 stepping is compared with the FP64 oracle on the same
random inputs, by per-path relative error (stated) and by estimator means
within 3 standard errors.
"""
import json
import math
import os

import numpy as np
import pytest

from conftest import EXAMPLE_GBM, EXAMPLE_PY, EXAMPLE_RS, GBM, GOLDEN, HESTON, OU

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-12
THREADS = os.cpu_count() or 1


def close64(gpu, ref):
    err = np.abs(gpu - ref) / np.maximum(np.abs(ref), 1.0)
    bad = ~(err <= FP64_RTOL) & ~(np.isnan(gpu) & np.isnan(ref))
    return float(np.nanmax(err)) if err.size else 0.0, int(bad.sum())


# A jump count (dN) is the first k with F(k) >= u on the inversion walk of
# src/proc/increment.rs:182-200.  The device's intensity or exp can differ
# from the oracle's in the last bit; the count then flips only when u sits
# within a few units of the last place of some F(k).  Every path that
# differs from the oracle must show exactly that at its first divergent
# step, in the oracle's own record of the draws there.
FLIP_ULPS = 16


def explain_jump_flips(oracle, eqs, gpu, ref, times, init, seed, n_per_replicate=0, **cfg):
    """Asserts that every path differing from the oracle by more than the
    FP64 bar diverges at a step where one of its Poisson draws lies within
    FLIP_ULPS units of the last place of a CDF value; returns the report
    [(path, step, ulps)]."""
    bad = np.abs(gpu - ref) > FP64_RTOL * np.maximum(np.abs(ref), 1.0)
    bad &= ~(np.isnan(gpu) & np.isnan(ref))
    u = oracle.Universe(eqs)
    report = []
    for path in np.unique(np.nonzero(bad)[0]):
        first_t = int(np.nonzero(bad[path].any(axis=-1))[0][0])
        step = first_t - 1
        assert step >= 0, (path, "differs at time 0")
        draws = [d for d in u.jump_trace(times, init, int(path), seed=seed, n_per_replicate=n_per_replicate, **cfg)
                 if d[0] == step]
        assert draws, (path, step, "no Poisson draw at the first divergent step")
        gap = min(oracle.poisson_boundary_ulps(d[2], d[3]) for d in draws)
        assert gap <= FLIP_ULPS, (path, step, gap, draws)
        report.append((int(path), step, gap))
    return report


# ---------------------------------------------------------------- KAT kernels

@pytest.mark.parametrize("seed", [0, 42, 2**63 + 11, 2**64 - 1])
def test_kat_chacha8_bit_exact(engine, oracle, seed):
    from sde_sim_rs import _native as N
    # the last two cross block 2^32, where the counter's high word turns on
    for first, n in ((0, 1000), (12345, 333), (2**35 - 4, 8), (2**40 + 3, 64)):
        out = np.zeros(n, dtype=np.uint64)
        N.check(N.lib().sde_kat_chacha8_u64(seed, first, n, out.ctypes.data))
        assert np.array_equal(out, oracle.chacha8_u64(seed, first, n))


def test_kat_sobol_bit_exact(engine, oracle):
    from sde_sim_rs import _native as N
    g = np.load(os.path.join(GOLDEN, "sobol_scipy.npz"))
    out = np.zeros((256, 64), dtype=np.uint32)
    N.check(N.lib().sde_kat_sobol_points(64, 0, 256, out.ctypes.data))
    assert np.array_equal(out, g["first256_d64"])
    out = np.zeros((64, 8), dtype=np.uint32)
    N.check(N.lib().sde_kat_sobol_points(8, 1000000, 64, out.ctypes.data))
    assert np.array_equal(out, g["at1e6_d8"])
    out = np.zeros((100, 8192), dtype=np.uint32)
    N.check(N.lib().sde_kat_sobol_points(8192, 2**20 - 50, 100, out.ctypes.data))
    assert np.array_equal(out, oracle.sobol_points(8192, 2**20 - 50, 100))


def test_kat_icdf(engine, oracle):
    from sde_sim_rs import _native as N
    with open(os.path.join(GOLDEN, "icdf.json")) as f:
        g = json.load(f)
    rng = np.random.default_rng(1)
    p = np.concatenate([np.array(g["p"]), rng.random(10000)])
    out = np.zeros_like(p)
    N.check(N.lib().sde_kat_icdf(p.ctypes.data, len(p), out.ctypes.data))
    ref = np.array([oracle.icdf_as26(float(x)) for x in p])
    # near p = 0.5 the formula cancels (t - ratio, both ~1.18): a one-ulp
    # difference of log() is an absolute, not a relative, error there
    assert np.max(np.abs(out - ref) / np.maximum(np.abs(ref), 1.0)) < 1e-14
    # the device logarithm (table-driven, within 0.52 ulp) and the C
    # library's differ by at most one ulp, and rarely: nearly every normal
    # is bit-identical
    assert np.mean(out == ref) > 0.98


# ---------------------------------------------------------------- FP64 parity

def test_c0_gbm_full_filtration(engine, oracle):
    """The reference's plain configuration: GBM, Euler, 252 steps, 10,000
    paths, pseudo-random seed 42, FP64, all 253 time points."""
    times = [i / 252 for i in range(253)]
    plan = engine.Plan(GBM, scheme="euler", rng="pseudo", precision="fp64", output="full")
    gpu = plan.run(times, {"X": 100.0}, 10000, seed=42).values("reference")[0]
    ref = oracle.Universe(GBM).simulate(times, {"X": 100.0}, 0, 10000, seed=42, threads=THREADS)
    err, nbad = close64(gpu, ref)
    assert nbad == 0, err
    xt = gpu[:, -1, 0]
    m, v = 100 * math.exp(0.05), 100 ** 2 * math.exp(0.1) * (math.exp(0.04) - 1)
    assert abs(xt.mean() - m) < 4 * math.sqrt(v / len(xt))
    assert abs(xt.std() / math.sqrt(v) - 1) < 0.05


CASES = {
    "gbm": (GBM, {"X": 100.0}),
    "example_rs": (EXAMPLE_RS, {"X1": 100.0, "X2": 0.0}),
    "example_py": (EXAMPLE_PY, {"X0": 0.5, "X1": 100.0, "X2": 0.0}),
    "example_gbm": (EXAMPLE_GBM, {"X1": 1.0}),
    "heston": (HESTON, {"S": 100.0, "v": 0.04}),
    "ou": (OU, {"X": 0.0}),
}
RNGS = {"pseudo": ("pseudo", "shift"), "sobol_shift": ("sobol", "shift"), "sobol_xor": ("sobol", "xor")}


def _oracle_cfg(oracle, scheme, rng, semantics):
    r, s = RNGS[rng]
    return dict(scheme=oracle.RK if scheme == "runge-kutta" else oracle.EULER,
                rng=oracle.SOBOL if r == "sobol" else oracle.PSEUDO,
                scramble=oracle.XOR if s == "xor" else oracle.SHIFT,
                semantics=oracle.TEXTBOOK if semantics == "textbook" else oracle.REFERENCE)


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("scheme", ["euler", "runge-kutta"])
@pytest.mark.parametrize("rng", list(RNGS))
@pytest.mark.parametrize("semantics", ["reference", "textbook"])
def test_fp64_paths_match_oracle(engine, oracle, case, scheme, rng, semantics):
    eqs, init = CASES[case]
    times = np.linspace(0.0, 2.0, 41) if case != "example_rs" else np.arange(0.0, 4.0, 0.1)
    n, seed = 300, 20240607
    r, s = RNGS[rng]
    plan = engine.Plan(eqs, scheme=scheme, rng=r, scramble=s, precision="fp64", semantics=semantics)
    gpu = plan.run(times, init, n, seed=seed).values("reference")[0]
    ref = oracle.Universe(eqs).simulate(times, init, 0, n, seed=seed, n_per_replicate=n,
                                        threads=THREADS, **_oracle_cfg(oracle, scheme, rng, semantics))
    err, nbad = close64(gpu, ref)
    if any("dN" in e for e in eqs):
        # a path may differ only through a jump count that flips at a CDF
        # boundary (explained draw by draw from the oracle's record)
        explain_jump_flips(oracle, eqs, gpu, ref, times, init, seed, n_per_replicate=n,
                           **_oracle_cfg(oracle, scheme, rng, semantics))
    else:
        assert nbad == 0, err


@pytest.mark.parametrize("name,eqs,init,times,scheme,rng", [
    # examples/example.rs: 100 time units at dt = 0.1, 10,000 scenarios
    ("example_rs", EXAMPLE_RS, {"X1": 100.0, "X2": 0.0},
     [i * 0.1 for i in range(1001)], "euler", "pseudo"),
    # examples/example.py: np.arange(0, 10, 0.01), 10,000 scenarios, RK
    ("example_py", EXAMPLE_PY, {"X0": 0.5, "X1": 100.0, "X2": 0.0},
     list(np.arange(0.0, 10.0, 0.01)), "runge-kutta", "pseudo"),
    # examples/example_gbm.py: np.arange(0, 10, 0.1), 10,000 scenarios, RK
    ("example_gbm", EXAMPLE_GBM, {"X1": 1.0}, list(np.arange(0.0, 10.0, 0.1)), "runge-kutta", "pseudo"),
    # the same with the reference's Sobol mode
    ("example_gbm_sobol", EXAMPLE_GBM, {"X1": 1.0}, list(np.arange(0.0, 10.0, 0.1)), "runge-kutta",
     "sobol_shift"),
])
def test_reference_examples_full_size(engine, oracle, name, eqs, init, times, scheme, rng):
    """The reference's example programs at their own sizes, every path and
    time point compared with the oracle."""
    n, seed = 10000, 777
    r, s = RNGS[rng]
    plan = engine.Plan(eqs, scheme=scheme, rng=r, scramble=s, precision="fp64")
    gpu = plan.run(times, init, n, seed=seed).values("reference")[0]
    ref = oracle.Universe(eqs).simulate(times, init, 0, n, seed=seed, threads=THREADS,
                                        **_oracle_cfg(oracle, scheme, rng, "reference"))
    if any("dN" in e for e in eqs):
        # every differing path is a jump count flipped at a CDF boundary
        report = explain_jump_flips(oracle, eqs, gpu, ref, times, init, seed,
                                    **_oracle_cfg(oracle, scheme, rng, "reference"))
        print(f"{name}: {len(report)} of {n} paths diverge through a flipped jump count", report)
    else:
        err, nbad = close64(gpu, ref)
        assert nbad == 0, (name, err)


def test_replicates_and_offsets_are_scenario_ranges(engine, oracle):
    times = np.linspace(0, 1, 17)
    plan = engine.Plan(EXAMPLE_PY, scheme="runge-kutta")
    init = {"X0": 0.5, "X1": 100.0}
    a = plan.run(times, init, 50, replicates=3, seed=5).values("reference")
    b = plan.run(times, init, 40, seed=5, path_offset=110).values("reference")[0]
    ref = oracle.Universe(EXAMPLE_PY).simulate(times, init, 0, 150, scheme=oracle.RK, seed=5)
    assert close64(a.reshape(150, 17, 3), ref)[1] == 0
    assert close64(b, ref[110:150])[1] == 0


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_shifted_sobol_offsets_and_high_indices(engine, oracle, precision):
    """Shifted Sobol takes point s + 5 for scenario s, so a warp's 32 points
    span two groups of 32 whose high parts the warp shares.  Path offsets
    that are not multiples of 32, replicates that start inside a warp, and
    point indices up to the 2^32 limit give the oracle's paths (FP64: bit
    level; FP32 from the same uniforms: FP32 accuracy)."""
    times = np.linspace(0, 1, 41)
    init = {"S": 100.0, "v": 0.04}
    plan = engine.Plan(HESTON, rng="sobol", precision=precision, chunked="off")
    u = oracle.Universe(HESTON)
    for offset, n, reps in [(77, 45, 3), (2**31 - 19, 64, 1), (2**32 - 5 - 200, 100, 2)]:
        gpu = plan.run(times, init, n, replicates=reps, seed=13, path_offset=offset).values("reference")
        ref = u.simulate(times, init, offset, offset + n * reps, rng=oracle.SOBOL, seed=13, threads=THREADS)
        gpu = gpu.reshape(n * reps, len(times), 2)
        if precision == "fp64":
            assert close64(gpu, ref)[1] == 0, offset
        else:
            scale = np.maximum(np.abs(ref), np.abs(ref).mean(axis=0, keepdims=True))
            rel = np.abs(gpu - ref) / scale
            # the same bar as the other FP32 paths against the FP64 oracle
            assert np.mean(rel < 1e-3) > 0.99, (offset, np.percentile(rel, [50, 99, 100]))
    with pytest.raises(Exception, match="beyond 2"):
        plan.run(times, init, 100, replicates=2, seed=13, path_offset=2**32 - 5 - 199)


def test_xor_replicates_match_oracle(engine, oracle):
    times = np.linspace(0, 1, 65)
    plan = engine.Plan(HESTON, rng="sobol", scramble="xor")
    gpu = plan.run(times, {"S": 100.0, "v": 0.04}, 96, replicates=4, seed=7).values("reference")
    ref = oracle.Universe(HESTON).simulate(times, {"S": 100.0, "v": 0.04}, 0, 4 * 96, rng=oracle.SOBOL,
                                           scramble=oracle.XOR, seed=7, n_per_replicate=96)
    assert close64(gpu.reshape(4 * 96, 65, 2), ref)[1] == 0


def test_output_modes_are_slices_of_full(engine):
    times = np.linspace(0, 1, 33)
    full = engine.Plan(HESTON).run(times, {"S": 100.0, "v": 0.04}, 200, seed=3).values("reference")
    ck = engine.Plan(HESTON, output="checkpoints").run(times, {"S": 100.0, "v": 0.04}, 200, seed=3,
                                                       checkpoints=[0, 8, 31, 32])
    assert ck.time_indices.tolist() == [0, 8, 31, 32]
    assert np.array_equal(ck.values("reference"), full[:, :, [0, 8, 31, 32], :])
    term = engine.Plan(HESTON, output="terminal").run(times, {"S": 100.0, "v": 0.04}, 200, seed=3)
    assert np.array_equal(term.values("reference")[:, :, 0, :], full[:, :, -1, :])
    dev = term.values("device")
    assert dev.shape == (1, 1, 2, 200)
    assert np.array_equal(dev[0, 0].T, full[0, :, -1, :])


def test_long_format_rows(engine, oracle):
    times = np.linspace(0, 1, 5)
    plan = engine.Plan(EXAMPLE_PY)
    res = plan.run(times, {"X0": 0.5, "X1": 100.0}, 7, seed=1, path_offset=3)
    cols = res.long()
    n = 7 * 5 * 3
    assert cols["scenario"].tolist() == [3 + s for s in range(7) for _ in range(5) for _ in range(3)]
    assert cols["time"].tolist() == [t for _ in range(7) for t in times for _ in range(3)]
    assert cols["process"].tolist() == [p for _ in range(7 * 5) for p in range(3)]
    ref = oracle.Universe(EXAMPLE_PY).simulate(times, {"X0": 0.5, "X1": 100.0}, 3, 10, seed=1)
    assert close64(cols["value"], ref.reshape(n))[1] == 0
    # the columns view pinned memory the result owns: read-only, and they
    # keep the result alive after the caller drops it
    assert not cols["value"].flags.writeable
    expect = cols["value"].copy()
    del res
    import gc
    gc.collect()
    for _ in range(3):  # recycle pool memory in between
        plan.run(times, {"X0": 1.5, "X1": 50.0}, 7, seed=9).long()
    assert np.array_equal(cols["value"], expect)
    # an empty run gives empty columns
    empty = plan.run(times, {"X0": 0.5, "X1": 100.0}, 0).long()
    assert all(len(c) == 0 for c in empty.values())


def test_long_index_columns_are_shared_by_shape(engine):
    """Results of one shape (replicates, paths, output times, processes,
    first scenario) share one pinned copy of the scenario, time and process
    columns; each has its own values.  Columns stay valid after the cache
    has moved on past its 8 shapes, and a different first scenario or time
    grid gets its own index."""
    times = np.linspace(0, 1, 9)
    plan = engine.Plan(HESTON)
    init = {"S": 100.0, "v": 0.04}
    a = plan.run(times, init, 50, seed=1).long()
    b = plan.run(times, init, 50, seed=2).long()
    for c in ("scenario", "time", "process"):
        assert a[c].__array_interface__["data"][0] == b[c].__array_interface__["data"][0]
    assert a["value"].__array_interface__["data"][0] != b["value"].__array_interface__["data"][0]
    assert not np.array_equal(a["value"], b["value"])
    shifted = plan.run(times, init, 50, seed=1, path_offset=7).long()
    assert shifted["scenario"][0] == 7 and a["scenario"][0] == 0
    regrid = plan.run(times * 2, init, 50, seed=1).long()
    assert regrid["time"][-1] == 2.0 and a["time"][-1] == 1.0
    keep = {c: a[c].copy() for c in a}
    for k in range(12):  # more shapes than the cache holds
        plan.run(times, init, 50 + k + 1, seed=3).long()
    for c in a:
        assert np.array_equal(a[c], keep[c])
    again = plan.run(times, init, 50, seed=1).long()
    for c in again:
        assert np.array_equal(again[c], keep[c])


@pytest.mark.parametrize("eqs,init", [(GBM, {"X": 100.0}), (HESTON, {"S": 100.0, "v": 0.04}),
                                      (EXAMPLE_RS, {"X1": 100.0}), (EXAMPLE_PY, {"X0": 0.5, "X1": 100.0})])
@pytest.mark.parametrize("scheme", ["euler", "runge-kutta"])
@pytest.mark.parametrize("rng", ["pseudo", "sobol"])
def test_chunked_kernel_is_bit_identical(engine, eqs, init, scheme, rng):
    """FP64 runs with few paths use the chunked kernel (8 warps draw a chunk
    of steps' increments, warp 0 steps through it); the paths are those of
    the one-thread-per-path kernel bit for bit, with a ragged last chunk
    (100 steps) and a ragged last CTA (1000 paths)."""
    times = np.linspace(0.0, 1.0, 101)
    on = engine.Plan(eqs, scheme=scheme, rng=rng, precision="fp64", chunked="on")
    off = engine.Plan(eqs, scheme=scheme, rng=rng, precision="fp64", chunked="off")
    a = on.run(times, init, 1000, seed=17, replicates=2).values()
    b = off.run(times, init, 1000, seed=17, replicates=2).values()
    assert np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("ppt,block", [(2, 0), (4, 0), (2, 64), (1, 512)])
@pytest.mark.parametrize("precision,rng,scramble", [("fp64", "pseudo", "shift"), ("fp64", "sobol", "shift"),
                                                    ("fp32", "sobol", "xor"), ("fp32", "pseudo", "shift")])
def test_paths_per_thread_and_block_are_bit_identical(engine, ppt, block, precision, rng, scramble):
    """Paths per thread and CTA size change only which thread steps a path:
    the full filtration (1000 paths: a ragged last CTA and, with several
    paths per thread, threads whose later paths are past the end) and the
    estimator are those of one path per thread, bit for bit."""
    times = np.linspace(0.0, 1.0, 41)
    init = {"S": 100.0, "v": 0.04}
    payoff = ["max(S - 100, 0)"]
    kw = dict(rng=rng, scramble=scramble, precision=precision, payoffs=payoff)
    base = engine.Plan(HESTON, **kw)
    alt = engine.Plan(HESTON, paths_per_thread=ppt, block_size=block, **kw)
    a = alt.run(times, init, 1000, seed=23, replicates=3)
    b = base.run(times, init, 1000, seed=23, replicates=3)
    assert np.array_equal(a.values(), b.values(), equal_nan=True)
    ta = engine.Plan(HESTON, paths_per_thread=ppt, block_size=block, output="none", **kw)
    tb = engine.Plan(HESTON, output="none", **kw)
    sa, qa = ta.run(times, init, 5000, seed=23, replicates=3).estimates()
    sb, qb = tb.run(times, init, 5000, seed=23, replicates=3).estimates()
    # sums over the same path values; only the order of the FP64 additions differs
    assert np.allclose(sa, sb, rtol=1e-12) and np.allclose(qa, qb, rtol=1e-12)


def test_automatic_wide_kernel(engine):
    """FP32 XOR-Sobol plans with automatic paths per thread launch the
    two-paths-per-thread kernel on large runs (here 2^16 paths x 16
    replicates) and the one-path kernel on small ones; both give the
    filtration of a plan fixed at one path per thread, bit for bit.  On a
    grid of equal steps the two-path kernel's twin takes dt and sqrt(dt)
    from the launch arguments; an uneven grid runs the general one."""
    uniform = np.linspace(0.0, 1.0, 9)
    uneven = np.cumsum(np.concatenate([[0.0], np.random.default_rng(4).uniform(0.05, 0.2, 8)]))
    init = {"S": 100.0, "v": 0.04}
    kw = dict(rng="sobol", scramble="xor", precision="fp32", payoffs=["max(S - 100, 0)"], output="terminal")
    auto = engine.Plan(HESTON, **kw)
    one = engine.Plan(HESTON, paths_per_thread=1, **kw)
    for times, n, reps, kernel in [(uniform, (1 << 16) - 3, 16, "wide"), (uneven, (1 << 16) - 3, 16, "wide"),
                                   (uniform, 5000, 2, "forward")]:
        a = auto.run(times, init, n, seed=9, replicates=reps)
        b = one.run(times, init, n, seed=9, replicates=reps)
        info = a.launch_info()
        assert info["kernel"] == kernel, info
        assert info["block"] == (128 if kernel == "wide" else info["block"])
        assert info["paths_per_block"] == (256 if kernel == "wide" else info["block"])
        assert b.launch_info()["kernel"] == "forward"
        assert np.array_equal(a.values(), b.values())
        sa, qa = a.estimates()
        sb, qb = b.estimates()
        assert np.allclose(sa, sb, rtol=1e-12) and np.allclose(qa, qb, rtol=1e-12)


def test_drop_in_simulate_frame(engine, oracle):
    times = [i / 252 for i in range(253)]
    fr = engine.simulate(GBM, times, 100, {"X": 100.0}, "pseudo", "euler", seed=42, output_format="numpy")
    ref = oracle.Universe(GBM).simulate(times, {"X": 100.0}, 0, 100, seed=42)
    assert len(fr) == 100 * 253
    assert set(fr.keys()) == {"scenario", "time", "process_name", "value"}
    assert fr["scenario"].dtype == np.int32 and fr["time"].dtype == np.float64
    assert list(fr["process_name"][:3]) == ["X", "X", "X"]
    assert close64(fr["value"], ref.reshape(-1))[1] == 0
    # an unknown rng_method falls back to pseudo, as in the reference
    fr2 = engine.simulate(GBM, times, 100, {"X": 100.0}, "quasi?", "euler", seed=42, output_format="numpy")
    assert np.array_equal(fr2["value"], fr["value"])
    fr3 = engine.simulate(GBM, times, 50, {"X": 100.0}, "sobol", "runge-kutta", seed=42, output_format="numpy")
    ref3 = oracle.Universe(GBM).simulate(times, {"X": 100.0}, 0, 50, seed=42, rng=oracle.SOBOL,
                                         scheme=oracle.RK)
    assert close64(fr3["value"], ref3.reshape(-1))[1] == 0
    # the name column: one name for one process (a read-only view), the
    # names cycling in universe order for several
    assert not fr["process_name"].flags.writeable and len(fr["process_name"]) == 100 * 253
    fr4 = engine.simulate(HESTON, times[:5], 3, {"S": 100.0, "v": 0.04}, "pseudo", "euler", seed=1,
                          output_format="numpy")
    assert list(fr4["process_name"]) == ["v", "S"] * 15 and not fr4["process_name"].flags.writeable


def test_estimators_fp64_match_oracle(engine, oracle):
    times = np.linspace(0, 1, 51)
    plan = engine.Plan(HESTON, payoffs=["max(S - 100, 0)", "S", "v"], output="none")
    s, q = plan.run(times, {"S": 100.0, "v": 0.04}, 5000, replicates=2, seed=11).estimates()
    u = oracle.Universe(HESTON)
    for r in range(2):
        for k, pay in enumerate(["max(S - 100, 0)", "S", "v"]):
            rs, rq = u.estimate(times, {"S": 100.0, "v": 0.04}, r * 5000, (r + 1) * 5000, pay, seed=11,
                                threads=THREADS)
            assert abs(s[r, k] - rs) <= 1e-10 * max(abs(rs), 1)
            assert abs(q[r, k] - rq) <= 1e-10 * max(abs(rq), 1)


# ---------------------------------------------------------------- FP32 stepping

@pytest.mark.parametrize("case", ["gbm", "heston", "ou", "example_py"])
@pytest.mark.parametrize("scheme", ["euler", "runge-kutta"])
@pytest.mark.parametrize("rng", list(RNGS))
def test_fp32_against_fp64_oracle(engine, oracle, case, scheme, rng):
    eqs, init = CASES[case]
    times = np.linspace(0.0, 1.0, 65)
    n, seed = 4000, 99
    r, s = RNGS[rng]
    plan = engine.Plan(eqs, scheme=scheme, rng=r, scramble=s, precision="fp32", output="terminal")
    gpu = plan.run(times, init, n, seed=seed).values("reference")[0, :, 0, :]
    ref = oracle.Universe(eqs).simulate(times, init, 0, n, seed=seed, n_per_replicate=n, full=False,
                                        threads=THREADS, **_oracle_cfg(oracle, scheme, rng, "reference"))
    scale = np.maximum(np.abs(ref), np.abs(ref).mean(axis=0, keepdims=True))
    rel = np.abs(gpu - ref) / scale
    # same random inputs: nearly every path agrees to FP32 accuracy
    assert np.mean(rel < 1e-3) > 0.99, np.percentile(rel, [50, 99, 100])
    for p in range(gpu.shape[1]):
        se = ref[:, p].std() / math.sqrt(n)
        assert abs(gpu[:, p].mean() - ref[:, p].mean()) <= 3 * se + 1e-12


def test_heston_rqmc_estimator_fp32(engine, oracle):
    """The Heston RQMC configuration at reduced size: XOR-scrambled Sobol,
    16 replicates, FP32 stepping, FP64 estimator reduction."""
    times = np.linspace(0.0, 1.0, 257)
    n, reps = 4096, 16
    plan = engine.Plan(HESTON, payoffs=["max(S - 100, 0)"], rng="sobol", scramble="xor",
                       precision="fp32", output="none")
    s, q = plan.run(times, {"S": 100.0, "v": 0.04}, n, replicates=reps, seed=7).estimates()
    est = s[:, 0] / n
    u = oracle.Universe(HESTON)
    ref = []
    for r in range(reps):
        rs, _ = u.estimate(times, {"S": 100.0, "v": 0.04}, r * n, (r + 1) * n, "max(S - 100, 0)",
                           rng=oracle.SOBOL, scramble=oracle.XOR, seed=7, n_per_replicate=n,
                           threads=THREADS)
        ref.append(rs / n)
    ref = np.array(ref)
    se = ref.std(ddof=1) / math.sqrt(reps)
    # per replicate, same scrambled points: FP32 bias far below the RQMC error
    assert np.max(np.abs(est - ref)) < 0.05 * se + 1e-4
    assert abs(est.mean() - ref.mean()) < 3 * se


# ---------------------------------------------------------------- edge cases

def test_edge_cases(engine):
    plan = engine.Plan(GBM, payoffs=["X"])
    r = plan.run([0.0, 1.0], {"X": 1.0}, 0)
    assert r.values().shape == (1, 0, 2, 1)
    assert r.estimates()[0].tolist() == [[0.0]]
    one = plan.run([0.5], {"X": 2.0}, 3).values()
    assert one.shape == (1, 3, 1, 1) and np.all(one == 2.0)
    rk = engine.Plan(["dX = (0.1 * X) * dt"], scheme="runge-kutta")
    with pytest.raises(ValueError, match="RNG Index 0 out of bounds"):
        rk.run([0.0, 1.0], {"X": 1.0}, 4)
    assert rk.run([0.0], {"X": 1.0}, 4).values().shape == (1, 4, 1, 1)
    with pytest.raises(ValueError, match="strictly increasing"):
        plan.run([0.0, 1.0, 1.0], {"X": 1.0}, 4)
    unknown = plan.run([0.0, 1.0], {"X": 1.0, "Q": 3.0}, 2).values()
    missing = plan.run([0.0, 1.0], {}, 2).values()
    assert np.all(missing == 0.0) and unknown.shape == (1, 2, 2, 1)


def test_caller_owned_device_buffer(engine):
    torch = pytest.importorskip("torch")
    times = np.linspace(0, 1, 9)
    plan = engine.Plan(HESTON, precision="fp32")
    buf = torch.zeros(9 * 2 * 128, dtype=torch.float32, device="cuda")
    r = plan.run(times, {"S": 100.0, "v": 0.04}, 128, seed=2, device_out=buf.data_ptr(),
                 device_out_bytes=buf.numel() * 4)
    ptr, elem = r.device_pointer()
    assert ptr == buf.data_ptr() and elem == 4
    r.wait()
    ref = plan.run(times, {"S": 100.0, "v": 0.04}, 128, seed=2).values("device")[0]
    assert np.array_equal(buf.cpu().numpy().reshape(9, 2, 128), ref.astype(np.float32))
    with pytest.raises(ValueError, match="smaller than the filtration"):
        plan.run(times, {"S": 100.0, "v": 0.04}, 128, device_out=buf.data_ptr(), device_out_bytes=16)


@pytest.mark.parametrize("rng", list(RNGS))
def test_accurate_icdf_option(engine, oracle, rng):
    times = np.linspace(0.0, 1.0, 33)
    r, s = RNGS[rng]
    eqs, init = CASES["heston"]
    p64 = engine.Plan(eqs, rng=r, scramble=s, precision="fp64", icdf="accurate")
    gpu = p64.run(times, init, 300, seed=5).values("reference")[0]
    ref = oracle.Universe(eqs).simulate(times, init, 0, 300, seed=5, n_per_replicate=300, icdf=1,
                                        **_oracle_cfg(oracle, "euler", rng, "reference"))
    assert close64(gpu, ref)[1] == 0
    p32 = engine.Plan(eqs, rng=r, scramble=s, precision="fp32", icdf="accurate", output="terminal")
    g32 = p32.run(times, init, 2000, seed=5).values("reference")[0, :, 0, :]
    r32 = oracle.Universe(eqs).simulate(times, init, 0, 2000, seed=5, n_per_replicate=2000, icdf=1, full=False,
                                        **_oracle_cfg(oracle, "euler", rng, "reference"))
    rel = np.abs(g32 - r32) / np.maximum(np.abs(r32), 1.0)
    assert np.mean(rel < 1e-3) > 0.99


def test_roofline_probes(engine):
    """The two roofline denominators the bench measures in its own run: the
    SFU (MUFU) throughput and the ChaCha8 block rate, positive and within
    what one GB300 can do (16 SFU ops and at most one 16-word block per
    SM and clock)."""
    import ctypes as C
    from sde_sim_rs import _native as N
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    ops, blocks = C.c_double(), C.c_double()
    N.check(N.lib().sde_probe_sfu_peak(C.byref(ops)))
    N.check(N.lib().sde_probe_chacha8_rate(C.byref(blocks)))
    clock = 2.2e9  # above the part's top SM clock
    assert 0 < ops.value <= 16 * sms * clock
    assert 0 < blocks.value <= sms * clock


@pytest.mark.parametrize("dim", [4, 8, 16, 32])
@pytest.mark.parametrize("ppt", [1, 2])
def test_shifted_sobol_chunk_loop_widths(engine, oracle, dim, ppt):
    """The FP32 kernel on the reference's shifted Sobol points walks
    32-dimension chunks with rolled inner step groups for 1, 2, 4, ..., 32
    stochastic indices: correlated baskets of 4 to 32 indices (8 to 1 steps
    per chunk), one and two paths per thread, a path offset inside a warp,
    against the FP64 oracle on the same points and shifts."""
    from bench import basket_equations
    eqs, _, _, _ = basket_equations(dim)
    init = {f"S{i + 1}": 100.0 for i in range(dim)}
    times = np.linspace(0.0, 1.0, 21)
    n, offset, seed = 300, 37, 9
    plan = engine.Plan(eqs, rng="sobol", scramble="shift", precision="fp32", paths_per_thread=ppt)
    gpu = plan.run(times, init, n, seed=seed, path_offset=offset).values()[0]
    ref = oracle.Universe(eqs).simulate(times, init, offset, offset + n, rng=oracle.SOBOL, seed=seed,
                                        threads=THREADS)
    rel = np.abs(gpu - ref) / np.abs(ref)
    assert np.mean(rel < 1e-3) > 0.99, np.percentile(rel, [50, 99, 100])
    assert rel.max() < 1e-2
