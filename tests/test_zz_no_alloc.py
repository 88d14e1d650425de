"""The estimator entry point that allocates no device memory
(sde_run_estimates_static), called through the C ABI.

It serves callers that cannot call cudaMalloc: their device memory comes from
an arena or budget they do not control, or an allocation's implicit
synchronisation is not acceptable where they call.  Its scratch is one static
device array of the library, shared by every call; these tests check that
two calls in a row on that shared array give the same estimates as the
ordinary sde_run path, and that an oversized run is refused.  The file is
collected last, so a stop-at-first-failure run has already run the others.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HESTON = ["dv = (2 * (0.04 - max(v, 0))) * dt + (0.3 * max(v, 0)^0.5) * dW1",
          "dS = (mu * S) * dt + (-0.7 * max(v, 0)^0.5 * S) * dW1 + "
          "(0.714142842854285 * max(v, 0)^0.5 * S) * dW2"]


def _static(N, plan, times, x0, params, n_paths, reps, seed):
    K = plan.n_payoffs
    s = np.full((reps, K), np.nan)
    q = np.full((reps, K), np.nan)
    rc = N.lib().sde_run_estimates_static(plan._h, times.ctypes.data, len(times), x0.ctypes.data, len(x0),
                                          params.ctypes.data, len(params), n_paths, reps, seed, None,
                                          s.ctypes.data, q.ctypes.data)
    N.check(rc)
    return s, q


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_static_scratch_matches_sde_run(engine, precision):
    from sde_sim_rs import _native as N
    plan = engine.Plan(HESTON, params=["mu"], payoffs=["max(S - 100, 0)", "S", "v"], precision=precision,
                       output="none")
    times = np.linspace(0.0, 1.0, 97)
    x0 = plan.x0({"S": 100.0, "v": 0.04})
    params = np.array([0.03])
    ref_s, ref_q = plan.run(times, {"S": 100.0, "v": 0.04}, 6000, replicates=3, seed=11,
                            params={"mu": 0.03}).estimates()
    for _ in range(2):   # the second call reuses the scratch the first one left
        s, q = _static(N, plan, times, x0, params, 6000, 3, 11)
        np.testing.assert_allclose(s, ref_s, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(q, ref_q, rtol=1e-12, atol=1e-12)


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
