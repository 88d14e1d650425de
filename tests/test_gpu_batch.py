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
