"""Pathwise Greeks as a torch.autograd.Function.

``PathwisePricer`` wraps an adjoint plan (``Plan(..., grad_params=...,
grad_x0=...)``): calling it with tensors of initial values and parameters
returns the Monte Carlo estimate of E[payoffs[0]] as a 0-d float64 tensor,
and backward() hands back the pathwise derivatives that the same GPU launch
computed by its reverse sweep (FP32 per path, FP64 compensated reduction).
The reference has no derivatives; this is an addition on top of its
simulate path.
"""
from __future__ import annotations

import math
from typing import Mapping, Sequence

import numpy as np
import torch

from . import Plan


class _PathwiseFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, params, pricer):
        price, grads = pricer._run(x0.detach().double().cpu().numpy(),
                                   params.detach().double().cpu().numpy())
        gp = torch.as_tensor(grads[: len(pricer.plan.grad_params)], dtype=params.dtype, device=params.device)
        gx = torch.as_tensor(grads[len(pricer.plan.grad_params):], dtype=x0.dtype, device=x0.device)
        ctx.save_for_backward(gx, gp)
        return torch.tensor(price, dtype=torch.float64, device=x0.device)

    @staticmethod
    def backward(ctx, g):
        gx, gp = ctx.saved_tensors
        return g.to(gx.dtype) * gx, g.to(gp.dtype) * gp, None


class PathwisePricer:
    """E[payoff] and its pathwise gradient through one adjoint launch.

    x0 tensor: values of ``plan.grad_x0`` processes (other processes take
    ``initial_values``).  params tensor: values of ``plan.grad_params``
    (other declared parameters take ``fixed_params``).
    """

    def __init__(self, plan: Plan, times: Sequence[float], initial_values: Mapping[str, float],
                 n_paths: int, *, fixed_params: Mapping[str, float] | None = None, seed: int = 0,
                 replicates: int = 1, stream=None):
        if not plan.adjoint:
            raise ValueError("PathwisePricer needs a plan created with grad_params / grad_x0")
        self.plan = plan
        self.times = np.ascontiguousarray(times, dtype=np.float64)
        self.initial_values = dict(initial_values)
        self.fixed_params = dict(fixed_params or {})
        self.n_paths = int(n_paths)
        self.seed = seed
        self.replicates = replicates
        self.stream = stream
        self.last = None

    def _run(self, x0_vals, param_vals):
        init = dict(self.initial_values)
        for name, v in zip(self.plan.grad_x0, x0_vals):
            init[name] = float(v)
        params = dict(self.fixed_params)
        for name, v in zip(self.plan.grad_params, param_vals):
            params[name] = float(v)
        res = self.plan.run(self.times, init, self.n_paths, replicates=self.replicates, seed=self.seed,
                            params=params, stream=self.stream)
        s, q = res.estimates()
        n = self.n_paths * self.replicates
        mean = s.sum(axis=0) / n
        var = np.maximum(q.sum(axis=0) / n - mean ** 2, 0.0)
        se = np.sqrt(var / n)
        K = len(self.plan.payoffs)
        self.last = {"mean": mean, "se": se, "price": mean[0], "price_se": se[0],
                     "grad": mean[K:], "grad_se": se[K:]}
        return float(mean[0]), mean[K:].copy()

    def __call__(self, x0: torch.Tensor, params: torch.Tensor) -> torch.Tensor:
        return _PathwiseFn.apply(x0, params, self)


def black_scholes_call(s0, k, sigma, mu, t):
    """E[max(S_T - K, 0)] for dS = mu S dt + sigma S dW and its derivatives
    (undiscounted): returns price, d/dS0, d/dsigma, d/dmu."""
    from math import erf, exp, log, pi, sqrt
    d1 = (log(s0 / k) + (mu + 0.5 * sigma * sigma) * t) / (sigma * sqrt(t))
    d2 = d1 - sigma * sqrt(t)
    N = lambda x: 0.5 * (1.0 + erf(x / sqrt(2.0)))
    phi = lambda x: exp(-0.5 * x * x) / sqrt(2.0 * pi)
    growth = exp(mu * t)
    price = s0 * growth * N(d1) - k * N(d2)
    delta = growth * N(d1)
    vega = s0 * growth * phi(d1) * sqrt(t)
    dmu = t * s0 * growth * N(d1)
    return price, delta, vega, dmu
