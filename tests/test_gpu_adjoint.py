"""Pathwise adjoint Greeks (GPU): checked against closed-form Black-Scholes
delta / vega / d(mu), against central finite differences of the FP64
forward estimator with common random numbers (h = 1e-4 relative), and
through torch.autograd."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GBM_P = ["dX = (mu * X) * dt + (sigma * X) * dW1"]
HESTON_P = ["dv = (kappa * (theta - max(v, 0))) * dt + (xi * max(v, 0)^0.5) * dW1",
            "dS = (mu * S) * dt + (rho * max(v, 0)^0.5 * S) * dW1 + "
            "((1 - rho^2)^0.5 * max(v, 0)^0.5 * S) * dW2"]
TIMES = np.linspace(0.0, 1.0, 366)   # 365 Euler steps, T = 1


def _adjoint(engine, eqs, params, gp, gx, init, n, seed, ckpt=19, **kw):
    plan = engine.Plan(eqs, params=list(params), payoffs=["max(%s - 100, 0)" % ("S" if "S" in init else "X")],
                       grad_params=gp, grad_x0=gx, precision="fp32", output="none", ckpt_every=ckpt, **kw)
    s, q = plan.run(TIMES, init, n, seed=seed, params=params).estimates()
    mean = s[0] / n
    se = np.sqrt(np.maximum(q[0] / n - mean ** 2, 0) / n)
    return mean, se


def _fd(engine, eqs, params, init, n, seed, name, h=1e-4, is_x0=False, **kw):
    payoff = "max(%s - 100, 0)" % ("S" if "S" in init else "X")
    plan = engine.Plan(eqs, params=list(params), payoffs=[payoff], precision="fp64", output="none", **kw)
    vals = []
    for sgn in (+1, -1):
        p, x = dict(params), dict(init)
        if is_x0:
            x[name] = init[name] * (1 + sgn * h)
        else:
            p[name] = params[name] * (1 + sgn * h)
        s, _ = plan.run(TIMES, x, n, seed=seed, params=p).estimates()
        vals.append(s[0, 0] / n)
    base = init[name] if is_x0 else params[name]
    return (vals[0] - vals[1]) / (2 * h * base)


def test_gbm_greeks_closed_form_and_fd(engine):
    from sde_sim_rs.adjoint import black_scholes_call
    params = {"mu": 0.05, "sigma": 0.2}
    n = 1 << 20
    mean, se = _adjoint(engine, GBM_P, params, ["mu", "sigma"], ["X"], {"X": 100.0}, n, seed=42)
    price, d_mu, d_sigma, delta = mean
    bs = black_scholes_call(100.0, 100.0, 0.2, 0.05, 1.0)
    # Euler (dt = 1/365) and the AS 26.2.23 normals bias the estimate by
    # well under 0.5%; the MC error is se
    for got, want, s in ((price, bs[0], se[0]), (delta, bs[1], se[3]), (d_sigma, bs[2], se[2]),
                         (d_mu, bs[3], se[1])):
        assert abs(got - want) < 4 * s + 5e-3 * abs(want), (got, want, s)
    # FD with common random numbers differentiates the same estimator
    fd_delta = _fd(engine, GBM_P, params, {"X": 100.0}, n, 42, "X", is_x0=True)
    fd_sigma = _fd(engine, GBM_P, params, {"X": 100.0}, n, 42, "sigma")
    fd_mu = _fd(engine, GBM_P, params, {"X": 100.0}, n, 42, "mu")
    for got, fd in ((delta, fd_delta), (d_sigma, fd_sigma), (d_mu, fd_mu)):
        assert abs(got - fd) < 2e-3 * abs(fd) + 1e-4, (got, fd)


def test_heston_greeks_against_fd(engine):
    params = {"kappa": 2.0, "theta": 0.04, "xi": 0.3, "rho": -0.7, "mu": 0.03}
    init = {"S": 100.0, "v": 0.04}
    n = 1 << 18
    mean, se = _adjoint(engine, HESTON_P, params, ["kappa", "theta", "xi", "rho"], ["v"], init, n, seed=7)
    names = ["kappa", "theta", "xi", "rho", "v"]
    for k, name in enumerate(names):
        fd = _fd(engine, HESTON_P, params, init, n, 7, name, is_x0=(name == "v"))
        got = mean[1 + k]
        # same paths, same normals: FD and the pathwise adjoint estimate the
        # same derivative; FP32 stepping and O(h^2) set the tolerance
        assert abs(got - fd) < 5e-3 * abs(fd) + 2e-3 + 0.2 * se[1 + k], (name, got, fd, se[1 + k])


def test_checkpoint_spacing_does_not_change_gradients(engine):
    params = {"mu": 0.05, "sigma": 0.2}
    a, _ = _adjoint(engine, GBM_P, params, ["mu", "sigma"], ["X"], {"X": 100.0}, 1 << 14, seed=3, ckpt=19)
    b, _ = _adjoint(engine, GBM_P, params, ["mu", "sigma"], ["X"], {"X": 100.0}, 1 << 14, seed=3, ckpt=1)
    c, _ = _adjoint(engine, GBM_P, params, ["mu", "sigma"], ["X"], {"X": 100.0}, 1 << 14, seed=3, ckpt=64)
    assert np.allclose(a, b, rtol=1e-5) and np.allclose(a, c, rtol=1e-5)


@pytest.mark.parametrize("scheme", ["euler", "runge-kutta"])
@pytest.mark.parametrize("rng", ["pseudo", "sobol"])
def test_stored_increments_match_recompute(engine, rng, scheme):
    """The reverse sweep reads the forward pass's increments from device
    memory (default) or draws them again (adjoint_recompute=True): the same
    increments, so the same estimates bit for bit.  Heston has two Wiener
    indices; the jump universe has a Wiener and a Poisson index."""
    params = {"kappa": 2.0, "theta": 0.04, "xi": 0.3, "rho": -0.7, "mu": 0.03}
    jumps = ["dX = (mu * X) * dt + (sigma * X) * dW1 + (0.05 * X) * dN1(lam)"]
    cases = [(HESTON_P, params, ["kappa", "xi", "rho"], ["v", "S"], {"S": 100.0, "v": 0.04}, "max(S - 100, 0)"),
             (jumps, {"mu": 0.05, "sigma": 0.2, "lam": 0.7}, ["mu", "sigma"], ["X"], {"X": 100.0},
              "max(X - 100, 0)")]
    for eqs, prm, gp, gx, init, pay in cases:
        out = []
        for recompute in (False, True):
            plan = engine.Plan(eqs, params=list(prm), payoffs=[pay], grad_params=gp, grad_x0=gx, rng=rng,
                               precision="fp32", output="none", ckpt_every=23, adjoint_recompute=recompute,
                               scheme=scheme)
            out.append(plan.run(TIMES, init, 3000, replicates=2, seed=11, params=prm).estimates())
        assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("scheme,semantics", [("euler", "reference"), ("runge-kutta", "reference"),
                                              ("runge-kutta", "textbook")])
@pytest.mark.parametrize("rng,scramble", [("sobol", "xor"), ("sobol", "shift"), ("pseudo", "shift")])
def test_adjoint_forward_pass_uses_the_forward_kernels_inputs(engine, rng, scramble, scheme, semantics):
    """The adjoint kernel draws a step's inputs by random access (a
    segment's steps again in the recompute); its price, the forward pass's
    payoff sum, is the forward kernel's on the same inputs to FP32
    accuracy.  Different inputs (another Sobol point or scramble) would
    move it by the Monte Carlo error, far more than this bar."""
    params = {"kappa": 2.0, "theta": 0.04, "xi": 0.3, "rho": -0.7, "mu": 0.03}
    init = {"S": 100.0, "v": 0.04}
    times = np.linspace(0.0, 1.0, 101)
    kw = dict(params=list(params), payoffs=["max(S - 100, 0)"], rng=rng, scramble=scramble, precision="fp32",
              output="none", scheme=scheme, semantics=semantics)
    adj = engine.Plan(HESTON_P, grad_params=["kappa", "xi"], grad_x0=["S"], ckpt_every=17, **kw)
    fwd = engine.Plan(HESTON_P, **kw)
    for n, reps in [(3000, 2), (1000, 3)]:
        a = adj.run(times, init, n, replicates=reps, seed=21, params=params).estimates()[0][:, 0]
        b = fwd.run(times, init, n, replicates=reps, seed=21, params=params).estimates()[0][:, 0]
        assert np.allclose(a, b, rtol=2e-5), (a, b)


def test_torch_autograd_function(engine):
    torch = pytest.importorskip("torch")
    from sde_sim_rs.adjoint import PathwisePricer
    plan = engine.Plan(GBM_P, params=["mu", "sigma"], payoffs=["max(X - 100, 0)"], grad_params=["mu", "sigma"],
                       grad_x0=["X"], precision="fp32", output="none")
    pricer = PathwisePricer(plan, TIMES, {"X": 100.0}, 1 << 16, seed=5)
    x0 = torch.tensor([100.0], dtype=torch.float64, device="cuda", requires_grad=True)
    th = torch.tensor([0.05, 0.2], dtype=torch.float64, device="cuda", requires_grad=True)
    price = pricer(x0, th)
    (2.0 * price).backward()
    assert math.isclose(price.item(), pricer.last["price"], rel_tol=1e-12)
    assert np.allclose(th.grad.cpu().numpy(), 2.0 * pricer.last["grad"][:2])
    assert np.allclose(x0.grad.cpu().numpy(), 2.0 * pricer.last["grad"][2:])


def test_adjoint_plan_validation(engine):
    with pytest.raises(ValueError, match="not a declared parameter"):
        engine.Plan(GBM_P, params=["mu", "sigma"], payoffs=["X"], grad_params=["nu"])
    with pytest.raises(Exception, match="algebraic"):
        engine.Plan(GBM_P + ["Y = max(X - 100, 0)"], params=["mu", "sigma"], payoffs=["X"], grad_params=["mu"],
                    scheme="runge-kutta")
    with pytest.raises(ValueError, match="needs a payoff"):
        engine.Plan(GBM_P, params=["mu", "sigma"], grad_params=["mu"])


# ---- Runge-Kutta (src/sim/runge_kutta.rs:17-97) ------------------------------
# The reverse sweep runs the two-stage recursion backwards with the step's
# sign sk held fixed.  In the reference's semantics the stage-1 coefficients
# read the cache the previous step left at its probe (src/func.rs:32-42), so
# the cache is part of the state; in textbook semantics they read the state.
# This scheme adds about (1 + sqrt(2/pi)) sigma^2 / 2 to the GBM drift (its
# probe takes the same normal as the step and sk = sign of that normal), so
# no closed form applies: central differences of the FP64 forward estimator
# with common random numbers differentiate the same discrete estimator.

@pytest.mark.parametrize("semantics", ["reference", "textbook"])
def test_rk_gbm_greeks_against_fd(engine, semantics):
    params = {"mu": 0.05, "sigma": 0.2}
    n = 1 << 18
    kw = dict(scheme="runge-kutta", semantics=semantics)
    mean, se = _adjoint(engine, GBM_P, params, ["mu", "sigma"], ["X"], {"X": 100.0}, n, seed=42, **kw)
    _, d_mu, d_sigma, delta = mean
    fd_delta = _fd(engine, GBM_P, params, {"X": 100.0}, n, 42, "X", is_x0=True, **kw)
    fd_sigma = _fd(engine, GBM_P, params, {"X": 100.0}, n, 42, "sigma", **kw)
    fd_mu = _fd(engine, GBM_P, params, {"X": 100.0}, n, 42, "mu", **kw)
    for got, fd in ((delta, fd_delta), (d_sigma, fd_sigma), (d_mu, fd_mu)):
        assert abs(got - fd) < 2e-3 * abs(fd) + 1e-4, (semantics, got, fd)


@pytest.mark.parametrize("semantics", ["reference", "textbook"])
def test_rk_heston_greeks_against_fd(engine, semantics):
    params = {"kappa": 2.0, "theta": 0.04, "xi": 0.3, "rho": -0.7, "mu": 0.03}
    init = {"S": 100.0, "v": 0.04}
    n = 1 << 18
    kw = dict(scheme="runge-kutta", semantics=semantics)
    mean, se = _adjoint(engine, HESTON_P, params, ["kappa", "theta", "xi", "rho"], ["v", "S"], init, n, seed=7, **kw)
    for k, name in enumerate(["kappa", "theta", "xi", "rho", "v", "S"]):
        fd = _fd(engine, HESTON_P, params, init, n, 7, name, is_x0=(name in init), **kw)
        got = mean[1 + k]
        assert abs(got - fd) < 5e-3 * abs(fd) + 2e-3 + 0.2 * se[1 + k], (semantics, name, got, fd, se[1 + k])


@pytest.mark.parametrize("semantics", ["reference", "textbook"])
def test_rk_checkpoint_spacing_does_not_change_gradients(engine, semantics):
    """In the reference's semantics a segment restarts from the checkpointed
    state and cache; a cache left out of the checkpoint would move every
    gradient when the spacing changes."""
    params = {"kappa": 2.0, "theta": 0.04, "xi": 0.3, "rho": -0.7, "mu": 0.03}
    init = {"S": 100.0, "v": 0.04}
    out = [_adjoint(engine, HESTON_P, params, ["kappa", "xi", "rho"], ["v", "S"], init, 1 << 14, seed=3, ckpt=c,
                    scheme="runge-kutta", semantics=semantics)[0] for c in (19, 1, 64)]
    assert np.allclose(out[0], out[1], rtol=1e-5) and np.allclose(out[0], out[2], rtol=1e-5), out
