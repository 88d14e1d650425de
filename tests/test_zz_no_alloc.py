"""The estimator entry point that allocates no device memory
(sde_run_estimates_static), called through the C ABI.

It serves callers that cannot call cudaMalloc: their device memory comes from
an arena or budget they do not control, or an allocation's implicit
synchronisation is not acceptable where they call.  Its scratch is one static
device array of the library, shared by every call; these tests check that
two calls in a row on that shared array give the same estimates as the
ordinary sde_run path (the second with other inputs than the first), on
the default and on a created stream, and that an oversized run is refused.  The file is
collected last, so a stop-at-first-failure run has already run the others.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HESTON = ["dv = (2 * (0.04 - max(v, 0))) * dt + (0.3 * max(v, 0)^0.5) * dW1",
          "dS = (mu * S) * dt + (-0.7 * max(v, 0)^0.5 * S) * dW1 + "
          "(0.714142842854285 * max(v, 0)^0.5 * S) * dW2"]


def _static(N, plan, times, x0, params, n_paths, reps, seed, stream=None):
    K = plan.n_payoffs
    s = np.full((reps, K), np.nan)
    q = np.full((reps, K), np.nan)
    rc = N.lib().sde_run_estimates_static(plan._h, times.ctypes.data, len(times), x0.ctypes.data, len(x0),
                                          params.ctypes.data, len(params), n_paths, reps, seed, stream,
                                          s.ctypes.data, q.ctypes.data)
    N.check(rc)
    return s, q


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_static_scratch_matches_sde_run(engine, precision):
    from sde_sim_rs import _native as N
    plan = engine.Plan(HESTON, params=["mu"], payoffs=["max(S - 100, 0)", "S", "v"], precision=precision,
                       output="none")
    # the second call differs in every input (a shorter, uneven grid, other
    # seed, parameter, initial values, paths and replicates), so a piece of
    # scratch it failed to rewrite would show up as a mismatch
    cases = [(np.linspace(0.0, 1.0, 97), {"S": 100.0, "v": 0.04}, 0.03, 6000, 3, 11),
             (np.array([0.0, 0.1, 0.25, 0.3, 0.55, 0.8]), {"S": 90.0, "v": 0.09}, -0.02, 1500, 2, 12345)]
    for times, init, mu, n, reps, seed in cases:
        ref_s, ref_q = plan.run(times, init, n, replicates=reps, seed=seed, params={"mu": mu}).estimates()
        s, q = _static(N, plan, times, plan.x0(init), np.array([mu]), n, reps, seed)
        np.testing.assert_allclose(s, ref_s, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(q, ref_q, rtol=1e-12, atol=1e-12)


def test_static_scratch_on_a_stream_and_without_paths(engine):
    torch = pytest.importorskip("torch")
    from sde_sim_rs import _native as N
    plan = engine.Plan(HESTON, params=["mu"], payoffs=["S"], precision="fp32", output="none")
    times = np.linspace(0.0, 0.5, 33)
    init = {"S": 100.0, "v": 0.04}
    st = torch.cuda.Stream()
    ref_s, ref_q = plan.run(times, init, 2500, replicates=2, seed=3, params={"mu": 0.01}).estimates()
    s, q = _static(N, plan, times, plan.x0(init), np.array([0.01]), 2500, 2, 3, stream=st.cuda_stream)
    np.testing.assert_allclose(s, ref_s, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(q, ref_q, rtol=1e-12, atol=1e-12)
    s, q = _static(N, plan, times, plan.x0(init), np.array([0.01]), 0, 2, 3, stream=st.cuda_stream)
    assert np.all(s == 0.0) and np.all(q == 0.0)


def test_static_scratch_limit(engine):
    from sde_sim_rs import _native as N
    plan = engine.Plan(HESTON, params=["mu"], payoffs=["S"], precision="fp32", output="none")
    times = np.linspace(0.0, 1.0, 9)
    x0 = plan.x0({"S": 100.0, "v": 0.04})
    # 2^24 paths x 4 replicates -> 2^18 blocks of partial sums: above 4 MiB
    with pytest.raises(ValueError, match="static scratch holds 4194304 bytes"):
        _static(N, plan, times, x0, np.array([0.03]), 1 << 24, 4, 1)
    # Sobol plans keep their tables in engine-allocated memory: refused
    sob = engine.Plan(HESTON, params=["mu"], payoffs=["S"], rng="sobol", scramble="xor", output="none")
    with pytest.raises(Exception, match="pseudo-random plans"):
        _static(N, sob, times, x0, np.array([0.03]), 64, 1, 1)
