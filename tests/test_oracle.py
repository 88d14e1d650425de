"""The oracle pinned against golden vectors and closed forms (CPU only)."""
import json
import math
import os

import numpy as np
import pytest

from conftest import EXAMPLE_GBM, EXAMPLE_PY, EXAMPLE_RS, GBM, GOLDEN, HESTON


def test_chacha20_core_matches_cryptography(oracle):
    with open(os.path.join(GOLDEN, "chacha.json")) as f:
        g = json.load(f)
    for case in g["chacha20"]:
        for b, blk in enumerate(case["blocks"]):
            got = oracle.chacha_block(case["key_words"], case["counter"] + b, 0, rounds=20)
            assert got.tolist() == blk


def test_chacha8_published_vector(oracle):
    with open(os.path.join(GOLDEN, "chacha.json")) as f:
        tc1 = json.load(f)["chacha8_tc1"]
    got = oracle.chacha_block(tc1["key_words"], tc1["counter"], 0, rounds=8)
    assert got.tolist() == tc1["block"]


def test_chacha8_stream_u64_pairs(oracle):
    # u64 k of the stream = words 2k (low) and 2k+1 (high) of the blocks
    key = oracle.seed_from_u64(42)
    words = np.concatenate([oracle.chacha_block(key, b, 0, 8) for b in range(3)]).astype(np.uint64)
    u = oracle.chacha8_u64(42, 0, 24)
    assert np.array_equal(u, words[0::2] | (words[1::2] << np.uint64(32)))
    # random access agrees with sequential reads
    assert np.array_equal(oracle.chacha8_u64(42, 5, 11), u[5:16])


def test_seed_from_u64_pcg32(oracle):
    # rand_core's PCG32 expansion, restated independently in Python
    def pcg(seed):
        MUL, INC, M = 6364136223846793005, 11634580027462260723, 2**64
        out = []
        s = seed
        for _ in range(8):
            s = (s * MUL + INC) % M
            xs = (((s >> 18) ^ s) >> 27) & 0xFFFFFFFF
            rot = s >> 59
            out.append(((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF)
        return out
    for seed in (0, 1, 42, 2**63 + 5, 2**64 - 1):
        assert oracle.seed_from_u64(seed).tolist() == pcg(seed)


def test_sobol_matches_scipy_golden(oracle):
    g = np.load(os.path.join(GOLDEN, "sobol_scipy.npz"))
    assert np.array_equal(oracle.sobol_points(64, 0, 256), g["first256_d64"])
    assert np.array_equal(oracle.sobol_points(8, 1000000, 64), g["at1e6_d8"])


def test_sobol_matches_scipy_live(oracle):
    qmc = pytest.importorskip("scipy.stats.qmc")
    s = qmc.Sobol(d=700, scramble=False, bits=32)
    pts = (s.random(128) * 2.0 ** 32).astype(np.uint64).astype(np.uint32)
    assert np.array_equal(oracle.sobol_points(700, 0, 128), pts)


def test_icdf_golden(oracle):
    with open(os.path.join(GOLDEN, "icdf.json")) as f:
        g = json.load(f)
    for p, x in zip(g["p"], g["x"]):
        assert oracle.icdf_as26(p) == x


def test_icdf_accuracy_bound(oracle):
    sp = pytest.importorskip("scipy.special")
    p = np.linspace(1e-6, 1 - 1e-6, 2001)
    got = np.array([oracle.icdf_as26(float(x)) for x in p])
    assert np.max(np.abs(got - sp.ndtri(p))) < 4.6e-4   # AS 26.2.23 bound


def test_poisson_inverse_cdf(oracle):
    from scipy.stats import poisson
    for lam in (0.0, -1.0, 0.05, 1.0, 3.5, 20.0):
        for u in (0.0, 0.1, 0.5, 0.9, 0.999):
            k = oracle.poisson(u, lam)
            if lam <= 0:
                assert k == 0
            else:
                # smallest k with F(k) >= u (ties at float precision aside)
                assert poisson.cdf(k, lam) >= u - 1e-12
                assert k == 0 or poisson.cdf(k - 1, lam) < u + 1e-12
    assert oracle.poisson(1.0, 500.0) == 200   # the reference's cap


def test_parse_example_fixtures(oracle):
    u = oracle.Universe(EXAMPLE_RS)
    assert u.process_names == ["X1", "X2"] and u.is_levy == [True, False]
    assert u.stochastic_tokens == ["dW1", "dN1(0.5 * cos(t))"]
    u = oracle.Universe(EXAMPLE_PY)
    assert u.process_names == ["X0", "X1", "X2"]
    assert u.stochastic_tokens == ["dN1(X0)", "dW1"]   # order of first appearance
    u = oracle.Universe(EXAMPLE_GBM)
    assert u.process_names == ["X1"] and u.stochastic_tokens == ["dW1"]
    u = oracle.Universe(HESTON)
    assert u.process_names == ["v", "S"] and u.stochastic_tokens == ["dW1", "dW2"]


@pytest.mark.parametrize("eq,msg", [
    ("dX = (0.1 * X) * dt = 3", "Missing '='"),
    ("dX = (0.1 * X * dt", "Unbalanced parentheses in coefficient"),
    ("dX = (0.1 * X) * dZ1", "Unknown incrementor type: dZ1"),
    ("dX = (0.1 * ) * dt", "Math error in coefficient"),
    ("dX = (0.1) * dN1(X", "Unbalanced parentheses in dN intensity"),
])
def test_parse_errors(oracle, eq, msg):
    with pytest.raises(ValueError, match=msg.replace("(", r"\(").replace(")", r"\)")):
        oracle.Universe([eq])


def test_gbm_lognormal_moments(oracle):
    times = [i / 252 for i in range(253)]
    u = oracle.Universe(GBM)
    full = u.simulate(times, {"X": 100.0}, 0, 10000, seed=42, threads=os.cpu_count() or 1)
    xt = full[:, -1, 0]
    m, v = 100 * math.exp(0.05), 100 ** 2 * math.exp(0.1) * (math.exp(0.04) - 1)
    se = math.sqrt(v / len(xt))
    assert abs(xt.mean() - m) < 4 * se
    assert abs(xt.std() / math.sqrt(v) - 1) < 0.05


def test_threads_do_not_change_paths(oracle):
    times = np.linspace(0, 1, 33)
    u = oracle.Universe(EXAMPLE_PY)
    init = {"X0": 0.5, "X1": 100.0, "X2": 0.0}
    a = u.simulate(times, init, 0, 64, scheme=oracle.RK, seed=3, threads=1)
    b = u.simulate(times, init, 0, 64, scheme=oracle.RK, seed=3, threads=5)
    assert np.array_equal(a, b)
    # a scenario range is the same paths as the prefix run
    c = u.simulate(times, init, 10, 20, scheme=oracle.RK, seed=3)
    assert np.array_equal(c, a[10:20])


def test_rk_sign_uses_index0_uniform(oracle):
    # With no drift and one Wiener term, RK's probe adds sk*sqrt(dt)*c with
    # sk = sign(u0 - 0.5): the same uniform as dW1, so k2 differs from k1 by
    # a deterministic amount and the path stays finite.
    u = oracle.Universe(["dX = (X) * dW1"])
    f = u.simulate([0.0, 0.5, 1.0], {"X": 1.0}, 0, 4, scheme=oracle.RK, seed=9)
    assert np.all(np.isfinite(f))


def test_rk_without_stochastic_index_fails_like_reference(oracle):
    u = oracle.Universe(["dX = (0.1 * X) * dt"])
    with pytest.raises(oracle.OracleError, match="RNG Index 0 out of bounds"):
        u.simulate([0.0, 1.0], {"X": 1.0}, 0, 2, scheme=oracle.RK)


def test_missing_initial_value_is_zero(oracle):
    u = oracle.Universe(["dX = (1.0) * dt", "dY = (X) * dt"])
    f = u.simulate([0.0, 1.0, 2.0], {"X": 1.0, "nope": 5.0}, 0, 1)
    assert f[0, 0].tolist() == [1.0, 0.0]
    assert f[0, 2].tolist() == [3.0, 3.0]


def test_icdf_accurate_option(oracle):
    sp = pytest.importorskip("scipy.special")
    p = np.concatenate([np.logspace(-300, -1, 60), np.linspace(0.01, 0.99, 99), 1 - np.logspace(-16, -1, 30)])
    got = np.array([oracle.icdf_accurate(float(x)) for x in p])
    want = sp.ndtri(p)
    assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1.0)) < 2e-15


def test_jump_trace_and_cdf_boundaries(oracle):
    """The oracle's record of Poisson draws: one draw per dN term and step in
    the reference's order, each count the inversion walk's; a draw on a CDF
    value is 0 units of the last place from it, and there a last-bit change
    of lambda * dt moves the count, while typical draws sit far away."""
    times = np.arange(0.0, 3.0, 0.1)
    u = oracle.Universe(EXAMPLE_PY)
    tr = u.jump_trace(times, {"X0": 0.5, "X1": 100.0, "X2": 0.0}, 5, scheme=oracle.RK, seed=9)
    # dN1 appears in two terms (X0 and X1): two draws per step, same uniform
    assert len(tr) == 2 * (len(times) - 1)
    for (t, idx, uu, lam, k), (t2, _, uu2, _, _) in zip(tr[0::2], tr[1::2]):
        assert idx == 0 and t == t2 and uu == uu2
        assert k == oracle.poisson(uu, lam)
    gaps = [oracle.poisson_boundary_ulps(d[2], d[3]) for d in tr]
    assert min(gaps) > 1e6
    # a uniform placed on F(1): the walk stops at k = 1 for lambda and moves
    # to 2 when lambda shrinks by a few units of its last place
    lam = 0.37
    f1 = math.exp(-lam) * (1.0 + lam)
    assert oracle.poisson_boundary_ulps(f1, lam) <= 1.0
    counts = {oracle.poisson(f1, lam * (1 + j * 2.0 ** -52)) for j in range(-8, 9)}
    assert counts == {1, 2}
