"""Batched uneven instances (GPU): half GBM, half Ornstein-Uhlenbeck, uneven
step and path counts, one persistent graph-captured launch with FP32
stepping, compared instance by instance with plain per-instance FP64 runs on
the same random inputs (means within 3 standard errors), and the FP64 batch
with the per-instance FP64 runs to 1e-10."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GBM_T = ["dX = (mu * X) * dt + (sigma * X) * dW1"]
OU_T = ["dX = (theta * (m - X)) * dt + (s) * dW1"]


def make_instances(n, seed, max_steps=1024, max_log2_paths=16):
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


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_matches_per_instance_runs(engine, precision):
    from sde_sim_rs.batch import Batch
    n = 48
    tid, steps, paths, seeds, x0, params = make_instances(n, 11, max_steps=200, max_log2_paths=12)
    tg = engine.Plan(GBM_T, params=["mu", "sigma"], payoffs=["X", "max(X - 100, 0)"], precision=precision,
                     output="none")
    to = engine.Plan(OU_T, params=["theta", "m", "s"], payoffs=["X"], precision=precision, output="none")
    job = Batch([tg, to]).prepare(tid, steps, 1.0, paths, seeds, x0, params)
    s, q = job.run().results()
    assert s.shape == (n, 2)
    # plain per-instance FP64 launches on the same streams
    pg = engine.Plan(GBM_T, params=["mu", "sigma"], payoffs=["X", "max(X - 100, 0)"], precision="fp64",
                     output="none")
    po = engine.Plan(OU_T, params=["theta", "m", "s"], payoffs=["X"], precision="fp64", output="none")
    for i in range(n):
        plan = pg if tid[i] == 0 else po
        np_ = len(plan.params)
        times = np.arange(steps[i] + 1) / steps[i]
        rs, rq = plan.run(times, {"X": x0[i, 0]}, int(paths[i]), seed=int(seeds[i]),
                          params=params[i, :np_]).estimates()
        for k in range(plan.n_payoffs):
            N = int(paths[i])
            m_ref = rs[0, k] / N
            se = math.sqrt(max(rq[0, k] / N - m_ref ** 2, 0.0) / N)
            m = s[i, k] / N
            if precision == "fp64":
                assert abs(m - m_ref) <= 1e-10 * max(1.0, abs(m_ref)), (i, k, m, m_ref)
            else:
                assert abs(m - m_ref) <= 3 * se + 1e-6 * max(1.0, abs(m_ref)), (i, k, m, m_ref, se)
        if tid[i] == 1:
            assert s[i, 1] == 0.0   # the OU template has one payoff


def test_batch_autotune_and_replay(engine):
    from sde_sim_rs.batch import Batch
    n = 256
    tid, steps, paths, seeds, x0, params = make_instances(n, 5, max_steps=256, max_log2_paths=13)
    tg = engine.Plan(GBM_T, params=["mu", "sigma"], payoffs=["X"], precision="fp32", output="none")
    to = engine.Plan(OU_T, params=["theta", "m", "s"], payoffs=["X"], precision="fp32", output="none")
    b = Batch([tg, to])
    job = b.prepare(tid, steps, 1.0, paths, seeds, x0, params, autotune=True)
    assert job.block in (128, 256) and job.paths_per_thread in (1, 2, 4)
    assert job.path_steps == int(np.sum(steps.astype(np.uint64) * paths))
    a = job.run().results()[0].copy()
    c = job.run().results()[0]
    assert np.array_equal(a, c)   # deterministic replay
    fixed = b.prepare(tid, steps, 1.0, paths, seeds, x0, params, autotune=False).run().results()[0]
    # another block shape only regroups paths: same per-path values,
    # compensated sums agree to rounding
    assert np.allclose(a, fixed, rtol=1e-9, atol=1e-9)
    # GBM mean against the exact lognormal mean X0 exp(mu)
    g = tid == 0
    m = a[g, 0] / paths[g]
    exact = x0[g, 0] * np.exp(params[g, 0])
    sd = x0[g, 0] * np.exp(params[g, 0]) * np.sqrt(np.exp(params[g, 1] ** 2) - 1)
    z = (m - exact) / (sd / np.sqrt(paths[g]))
    assert np.mean(np.abs(z) < 4) > 0.97


# ---- batched forward + adjoint ------------------------------------------------
# Adjoint plans as templates: every instance returns its payoffs and the
# pathwise gradients of payoff 0, as the template's own runs do (one
# universe per call in the reference, src/sim/mod.rs:20-92).  The batched
# template checkpoints every ceil(sqrt(steps)) steps instead of the plan's
# spacing, and its time grid is t * (t_end / steps): the gradients agree with
# per-instance adjoint runs to rounding.

HESTON_P = ["dv = (kappa * (theta - max(v, 0))) * dt + (xi * max(v, 0)^0.5) * dW1",
            "dS = (mu * S) * dt + (rho * max(v, 0)^0.5 * S) * dW1 + "
            "((1 - rho^2)^0.5 * max(v, 0)^0.5 * S) * dW2"]


def _adjoint_templates(engine, precision):
    tg = engine.Plan(GBM_T, params=["mu", "sigma"], payoffs=["max(X - 100, 0)", "X"], grad_params=["mu", "sigma"],
                     grad_x0=["X"], precision=precision, output="none")
    to = engine.Plan(OU_T, params=["theta", "m", "s"], payoffs=["X"], grad_params=["theta", "m", "s"],
                     grad_x0=["X"], precision=precision, output="none")
    th = engine.Plan(HESTON_P, params=["kappa", "theta", "xi", "rho", "mu"], payoffs=["max(S - 100, 0)"],
                     grad_params=["kappa", "xi", "rho"], grad_x0=["v"], precision=precision, output="none",
                     scheme="runge-kutta")
    return [tg, to, th]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batched_adjoint_matches_per_instance_adjoint_runs(engine, precision):
    from sde_sim_rs.batch import Batch
    n = 30
    tid, steps, paths, seeds, x0, params = make_instances(n, 23, max_steps=300, max_log2_paths=11)
    tid[::3] = 2                                   # every third instance: Heston, Runge-Kutta
    hx0 = np.tile([0.04, 100.0], (n, 1))
    hpar = np.tile([2.0, 0.04, 0.3, -0.7, 0.03], (n, 1))
    X0 = np.where((tid == 2)[:, None], hx0, np.pad(x0, ((0, 0), (0, 1))))
    PAR = np.where((tid == 2)[:, None], hpar, np.pad(params, ((0, 0), (0, 2))))
    templates = _adjoint_templates(engine, precision)
    job = Batch(templates).prepare(tid, steps, 1.0, paths, seeds, X0, PAR)
    s, q = job.run().results()
    assert s.shape == (n, 5)   # the widest templates: GBM 2 payoffs + 3 gradients, OU and Heston 1 + 4
    for i in range(n):
        plan = templates[tid[i]]
        times = np.arange(steps[i] + 1) / steps[i]
        init = {nm: X0[i, plan.index(nm)] for nm in plan.process_names}
        rs, rq = plan.run(times, init, int(paths[i]), seed=int(seeds[i]),
                          params=PAR[i, :len(plan.params)]).estimates()
        N = float(paths[i])
        for k in range(plan.n_payoffs):
            m, m_ref = s[i, k] / N, rs[0, k] / N
            sd = math.sqrt(max(rq[0, k] / N - m_ref ** 2, 0.0))
            if precision == "fp64":
                assert abs(m - m_ref) <= 1e-9 * max(1.0, abs(m_ref), sd), (i, k, m, m_ref)
            else:
                # FP32: another checkpoint spacing and time arithmetic move
                # each path by rounding only
                assert abs(m - m_ref) <= 1e-4 * max(1.0, abs(m_ref), sd), (i, k, m, m_ref)
        assert np.all(s[i, plan.n_payoffs:] == 0.0)


def test_batched_adjoint_greeks_and_limits(engine):
    """GBM instances of the batch against Black-Scholes delta / vega (Euler
    at 365 steps, 2^16 paths each), and the step limit of the template."""
    from sde_sim_rs.adjoint import black_scholes_call
    from sde_sim_rs.batch import Batch
    tg = engine.Plan(GBM_T, params=["mu", "sigma"], payoffs=["max(X - 100, 0)"], grad_params=["mu", "sigma"],
                     grad_x0=["X"], precision="fp32", output="none")
    sig = np.array([0.1, 0.2, 0.35, 0.5])
    mu = np.array([0.0, 0.05, 0.02, -0.03])
    n = len(sig)
    b = Batch([tg])
    job = b.prepare(np.zeros(n, np.int32), 365, 1.0, 1 << 16, np.arange(n, dtype=np.uint64) * 7919,
                    np.full((n, 1), 100.0), np.stack([mu, sig], axis=1))
    s, q = job.run().results()
    N = float(1 << 16)
    m = s / N
    se = np.sqrt(np.maximum(q / N - m * m, 0) / N)
    for i in range(n):
        price, delta, vega, dmu = black_scholes_call(100.0, 100.0, sig[i], mu[i], 1.0)
        for got, want, e in ((m[i, 0], price, se[i, 0]), (m[i, 3], delta, se[i, 3]), (m[i, 2], vega, se[i, 2]),
                             (m[i, 1], dmu, se[i, 1])):
            assert abs(got - want) < 4 * e + 5e-3 * abs(want), (i, got, want, e)
    with pytest.raises(Exception, match="at most 4096 steps"):
        b.prepare(np.zeros(1, np.int32), 4097, 1.0, 256, np.zeros(1, np.uint64), np.full((1, 1), 100.0),
                  np.array([[0.05, 0.2]]))


@pytest.mark.parametrize("adjoint", [False, True], ids=["forward", "fwd_adjoint"])
def test_every_launch_shape_gives_the_same_instances(engine, adjoint):
    """Each candidate (block, paths per thread) shape the autotuner may pick
    only regroups paths: per-instance estimates agree with the first shape's
    to rounding of the compensated sums, forward and forward+adjoint (whose
    template steps a thread's paths one after another)."""
    from sde_sim_rs.batch import Batch
    n = 40
    tid, steps, paths, seeds, x0, params = make_instances(n, 31, max_steps=150, max_log2_paths=11)
    kw = dict(precision="fp32", output="none")
    if adjoint:
        tg = engine.Plan(GBM_T, params=["mu", "sigma"], payoffs=["max(X - 100, 0)"], grad_params=["mu", "sigma"],
                         grad_x0=["X"], **kw)
        to = engine.Plan(OU_T, params=["theta", "m", "s"], payoffs=["X"], grad_params=["theta", "m", "s"],
                         grad_x0=["X"], scheme="runge-kutta", **kw)
    else:
        tg = engine.Plan(GBM_T, params=["mu", "sigma"], payoffs=["max(X - 100, 0)"], **kw)
        to = engine.Plan(OU_T, params=["theta", "m", "s"], payoffs=["X"], **kw)
    b = Batch([tg, to])
    out = []
    for shape in range(len(Batch.SHAPES)):
        job = b.prepare(tid, steps, 1.0, paths, seeds, x0, params, shape=shape)
        assert (job.block, job.paths_per_thread) == Batch.SHAPES[shape]
        out.append(job.run().results())
    for s, q in out[1:]:
        np.testing.assert_allclose(s, out[0][0], rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(q, out[0][1], rtol=1e-9, atol=1e-9)
    with pytest.raises(Exception, match="no such candidate"):
        b.prepare(tid, steps, 1.0, paths, seeds, x0, params, shape=len(Batch.SHAPES))
