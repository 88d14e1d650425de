"""tcgen05 lowering of correlated GBM baskets (every dW coefficient is a
constant times its own process).  The tensor-core kernel draws the same
increments as the CUDA-core FP32 kernel and differs from it only by the
rounding of its product (three FP16 products of hi / lo splits, FP32
accumulation); against the FP64 oracle it meets the bar of the other FP32
kernels."""
import math

import numpy as np
import pytest

from bench import basket_equations

pytestmark = pytest.mark.gpu

THREADS = 8
RNGS = {"pseudo": ("pseudo", "shift"), "sobol_xor": ("sobol", "xor"), "sobol_shift": ("sobol", "shift")}


def _init(dim):
    return {f"S{i + 1}": 100.0 for i in range(dim)}


@pytest.mark.parametrize("dim,layout", [(4, "auto"), (20, "auto"), (64, "auto"), (64, "row"), (40, "auto")])
@pytest.mark.parametrize("rng", list(RNGS))
def test_tensor_core_paths_match_cuda_core_kernel(engine, dim, layout, rng):
    """4 and 20 dimensions: one thread per path; 64 and 40: two threads per
    path ("row" forces one); 40 pads N and K to 64 with a half-empty second
    half."""
    eqs, payoff, _, _ = basket_equations(dim)
    r, s = RNGS[rng]
    times = np.linspace(0.0, 1.0, 33)
    n, reps = 1000, 2  # 1000 = 7 full CTAs of 128 paths and a ragged one
    tc = engine.Plan(eqs, payoffs=[payoff], precision="fp32", rng=r, scramble=s, tensor_cores=layout)
    cc = engine.Plan(eqs, payoffs=[payoff], precision="fp32", rng=r, scramble=s)
    assert tc.uses_tensor_cores and not cc.uses_tensor_cores
    a = tc.run(times, _init(dim), n, replicates=reps, seed=5)
    b = cc.run(times, _init(dim), n, replicates=reps, seed=5)
    va, vb = a.values(), b.values()
    assert va.shape == vb.shape == (reps, n, len(times), dim)
    assert np.all(np.isfinite(va))
    rel = np.abs(va - vb) / np.abs(vb)
    # the split product keeps about FP32 accuracy per step; 32 steps of GBM
    assert rel.max() < 2e-5, np.percentile(rel, [50, 99, 100])
    sa, qa = a.estimates()
    sb, qb = b.estimates()
    assert np.allclose(sa, sb, rtol=2e-5) and np.allclose(qa, qb, rtol=4e-5)


def _sparse_universe(P, NI, seed):
    """P GBM-like processes driven by NI Wiener indices through random sparse
    constant loadings (each process sees 3..8 of the indices, each index is
    used): dS_i = (mu_i S_i) dt + sum_j (c_ij S_i) dW_j."""
    rng = np.random.default_rng(seed)
    eqs = []
    used = set()
    for i in range(P):
        js = sorted(rng.choice(NI, size=int(rng.integers(3, 9)), replace=False).tolist())
        if i == P - 1:  # every index appears somewhere (the registry numbers them in order of appearance)
            js = sorted(set(js) | (set(range(NI)) - used))
        used |= set(js)
        terms = [f"({float(rng.uniform(0.0, 0.05))!r} * S{i + 1}) * dt"]
        terms += [f"({float(rng.uniform(-0.2, 0.2))!r} * S{i + 1}) * dW{j + 1}" for j in js]
        eqs.append(f"dS{i + 1} = " + " + ".join(terms))
    return eqs


@pytest.mark.parametrize("P,NI", [(32, 48), (48, 32), (33, 40)])
@pytest.mark.parametrize("rng", ["pseudo", "sobol_xor"])
def test_tensor_core_non_square_universes(engine, P, NI, rng):
    """Processes and Wiener indices padded and split independently: more
    indices than processes, fewer, and sizes just past a multiple of 32."""
    eqs = _sparse_universe(P, NI, seed=P * 100 + NI)
    r, s = RNGS[rng]
    times = np.linspace(0.0, 1.0, 25)
    init = {f"S{i + 1}": 50.0 + i for i in range(P)}
    payoff = "max((" + " + ".join(f"S{i + 1}" for i in range(P)) + f") / {P} - 60, 0)"
    tc = engine.Plan(eqs, payoffs=[payoff], precision="fp32", rng=r, scramble=s, tensor_cores=True)
    cc = engine.Plan(eqs, payoffs=[payoff], precision="fp32", rng=r, scramble=s)
    assert tc.uses_tensor_cores and tc.n_stochastic == NI
    a = tc.run(times, init, 700, seed=4).values()
    b = cc.run(times, init, 700, seed=4).values()
    assert np.max(np.abs(a - b) / np.abs(b)) < 2e-5
    sa, _ = tc.run(times, init, 700, seed=4).estimates()
    sb, _ = cc.run(times, init, 700, seed=4).estimates()
    assert np.allclose(sa, sb, rtol=2e-5)


@pytest.mark.parametrize("rng", ["pseudo", "sobol_xor"])
def test_tensor_core_basket_against_fp64_oracle(engine, oracle, rng):
    dim = 8
    eqs, _, _, _ = basket_equations(dim)
    r, s = RNGS[rng]
    times = np.linspace(0.0, 1.0, 17)
    n, seed = 640, 11
    plan = engine.Plan(eqs, precision="fp32", rng=r, scramble=s, output="terminal", tensor_cores=True)
    assert plan.uses_tensor_cores
    gpu = plan.run(times, _init(dim), n, seed=seed).values("reference")[0, :, 0, :]
    cfg = dict(rng=oracle.PSEUDO) if r == "pseudo" else dict(rng=oracle.SOBOL, scramble=oracle.XOR)
    ref = oracle.Universe(eqs).simulate(times, _init(dim), 0, n, seed=seed, n_per_replicate=n, full=False,
                                        threads=THREADS, **cfg)
    rel = np.abs(gpu - ref) / np.abs(ref)
    # the same random inputs: every path agrees to FP32 accuracy
    assert np.mean(rel < 1e-3) > 0.99, np.percentile(rel, [50, 99, 100])
    for p in range(dim):
        se = ref[:, p].std() / math.sqrt(n)
        assert abs(gpu[:, p].mean() - ref[:, p].mean()) <= 3 * se


def test_tensor_core_checkpoint_output_and_no_steps(engine):
    dim = 16
    eqs, payoff, _, _ = basket_equations(dim)
    tc = engine.Plan(eqs, payoffs=[payoff], precision="fp32", rng="sobol", scramble="xor",
                     output="checkpoints", tensor_cores=True)
    cc = engine.Plan(eqs, payoffs=[payoff], precision="fp32", rng="sobol", scramble="xor",
                     output="checkpoints")
    times = np.linspace(0.0, 2.0, 65)
    ck = [0, 16, 32, 64]
    a = tc.run(times, _init(dim), 4096, seed=3, checkpoints=ck).values()
    b = cc.run(times, _init(dim), 4096, seed=3, checkpoints=ck).values()
    assert np.max(np.abs(a - b) / np.abs(b)) < 4e-5
    # a single time point: no step, no MMA issued, tensor memory still freed
    one = tc.run([0.0], _init(dim), 300, seed=3, checkpoints=[0]).values()
    assert np.all(one == 100.0)


def test_static_scratch_entry_refuses_tensor_core_plans(engine):
    from sde_sim_rs import _native as N
    eqs, payoff, _, _ = basket_equations(4)
    tc = engine.Plan(eqs, payoffs=[payoff], precision="fp32", tensor_cores=True)
    times = np.linspace(0.0, 1.0, 5)
    x0 = np.full(4, 100.0)
    hs = np.zeros(1)
    hq = np.zeros(1)
    rc = N.lib().sde_run_estimates_static(tc._h, times.ctypes.data, len(times), x0.ctypes.data, 4, None, 0,
                                          256, 1, 1, None, hs.ctypes.data, hq.ctypes.data)
    assert rc == N.SDE_ERR_UNSUPPORTED


@pytest.mark.parametrize("tc", [False, True], ids=["cuda_cores", "tensor_cores"])
def test_basket64_checkpoints_against_fp64_oracle(engine, oracle, tc):
    """The 64-dimensional correlated basket at its own dimension: Euler,
    XOR-scrambled Sobol (dimension 8192), 128 steps, FP32 output at 32
    equally spaced checkpoints, against the FP64 oracle on the same points
    (the per-term Euler sum of src/sim/euler.rs:15-28).  Every checkpoint
    value of every path is compared."""
    dim, n, seed = 64, 2048, 7
    eqs, payoff, _, _ = basket_equations(dim)
    times = np.linspace(0.0, 1.0, 129)
    ck = list(range(4, 129, 4))
    plan = engine.Plan(eqs, payoffs=[payoff], precision="fp32", rng="sobol", scramble="xor",
                       output="checkpoints", tensor_cores=tc)
    assert plan.uses_tensor_cores == tc
    res = plan.run(times, _init(dim), n, seed=seed, checkpoints=ck)
    gpu = res.values()[0]                                   # [path, checkpoint, process]
    assert gpu.shape == (n, len(ck), dim)
    u = oracle.Universe(eqs)
    ref = u.simulate(times, _init(dim), 0, n, rng=oracle.SOBOL, scramble=oracle.XOR, seed=seed,
                     n_per_replicate=n, full=True, threads=THREADS)[:, ck, :]
    rel = np.abs(gpu - ref) / np.abs(ref)
    # FP32 stepping against FP64 on the same inputs: 99% of all 4.2M values
    # within 1e-3 relative (the FP32 bar); in practice all of them far inside
    assert np.mean(rel < 1e-3) >= 0.99, np.percentile(rel, [50, 99, 100])
    assert rel.max() < 1e-2, rel.max()
    # per-process terminal means within 3 standard errors of the oracle's
    for p in range(dim):
        se = ref[:, -1, p].std() / math.sqrt(n)
        assert abs(gpu[:, -1, p].mean() - ref[:, -1, p].mean()) <= 3 * se
    # the basket call: the run's FP64 estimator against the oracle's payoff
    # over the same paths
    pay = u.payoff(payoff, 1.0, ref[:, -1, :])
    s, q = res.estimates()
    price = s[0, 0] / n
    se = pay.std() / math.sqrt(n)
    assert abs(price - pay.mean()) <= max(3 * se * 1e-2, 1e-4 * abs(pay.mean())) + 1e-12, (price, pay.mean(), se)


def test_tensor_core_wait_that_runs_out_is_reported(engine):
    """The A-ready wait of the two-threads-per-path step, given a budget of
    four clocks (polling, no suspend), gives up at some step of some CTA.
    That CTA stops stepping, waits with the full budget for its copies and
    product in flight, frees its tensor memory and sets the status word:
    the run reports SDE_ERR_DEVICE.  The next run on the same plan, with the
    default budget, matches the CUDA-core kernel.  Nothing faults: every wait
    is bounded."""
    from sde_sim_rs import _native as N
    dim = 64
    eqs, payoff, _, _ = basket_equations(dim)
    tc = engine.Plan(eqs, payoffs=[payoff], precision="fp32", rng="sobol", scramble="xor", tensor_cores=True)
    cc = engine.Plan(eqs, payoffs=[payoff], precision="fp32", rng="sobol", scramble="xor")
    times = np.linspace(0.0, 1.0, 33)
    tc.run(times, _init(dim), 256, seed=5).wait()
    N.check(N.lib().sde_debug_tc_wait_cycles(4))
    try:
        with pytest.raises(N.SdeError) as e:
            tc.run(times, _init(dim), 256, seed=5).wait()
        assert e.value.code == N.SDE_ERR_DEVICE and "timed out" in str(e.value)
    finally:
        N.check(N.lib().sde_debug_tc_wait_cycles(0))
    a = tc.run(times, _init(dim), 1000, replicates=2, seed=5).values()
    b = cc.run(times, _init(dim), 1000, replicates=2, seed=5).values()
    assert np.max(np.abs(a - b) / np.abs(b)) < 2e-5
