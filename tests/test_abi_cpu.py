"""Host side of the engine without a GPU: the C ABI library, the equation
front end, the lowering (NVRTC compiles for sm_103a on the CPU) and the
error behaviour of the drop-in."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import EXAMPLE_GBM, EXAMPLE_PY, EXAMPLE_RS, GBM, HESTON, OU, ROOT


def _declared_symbols():
    with open(os.path.join(ROOT, "include", "sdegpu.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sde_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(engine):
    from sde_sim_rs import _native as N
    lib = C.CDLL(N.LIB_PATH)
    names = _declared_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    # and the binding declares a signature for each of them
    assert set(names) == set(N.SIGNATURES)
    assert lib.sde_abi_version() == 1


def test_struct_sizes_match_header(engine):
    from sde_sim_rs import _native as N
    o = N.Options()
    N.lib().sde_options_init(C.byref(o))
    assert o.struct_size == C.sizeof(N.Options)
    a = N.RunArgs()
    N.lib().sde_run_args_init(C.byref(a))
    assert a.struct_size == C.sizeof(N.RunArgs) and a.n_replicates == 1


@pytest.mark.parametrize("eqs", [GBM, EXAMPLE_RS, EXAMPLE_PY, EXAMPLE_GBM, HESTON, OU])
def test_front_end_matches_oracle(engine, oracle, eqs):
    p = engine.Plan(eqs)
    u = oracle.Universe(eqs)
    assert p.process_names == u.process_names
    assert p.stochastic_tokens == u.stochastic_tokens


@pytest.mark.parametrize("scheme", ["euler", "runge-kutta"])
@pytest.mark.parametrize("rng,scramble", [("pseudo", "shift"), ("sobol", "shift"), ("sobol", "xor")])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("semantics", ["reference", "textbook"])
def test_lowering_compiles(engine, scheme, rng, scramble, precision, semantics):
    p = engine.Plan(EXAMPLE_PY, scheme=scheme, rng=rng, scramble=scramble, precision=precision,
                    semantics=semantics, payoffs=["max(X1 - 100, 0)", "X0"])
    src = p.source
    assert "__global__" in src and "sde_step_" in src
    if precision == "fp32":
        # FP32 stepping: no double arithmetic in the step body
        body = re.split(r"for \(int t[01] = 0;", src)[1].split("double fs[")[0]
        assert "double" not in body


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_degenerate_universes_compile(engine, precision):
    # no stochastic term (RK panics only once a step runs), no Levy term,
    # only algebraic processes, a process with no terms
    for scheme in ("euler", "runge-kutta"):
        engine.Plan(["dX = (0.1 * X) * dt"], scheme=scheme, precision=precision)
        engine.Plan(["Y = 2 * t"], scheme=scheme, precision=precision)
        engine.Plan(["dX = 3", "Y = X + 1"], scheme=scheme, precision=precision)
    f = engine.Frame(a=np.arange(3))
    assert len(f) == 3 and f.height == 3 and len(engine.Frame()) == 0


def test_fasteval_operators_compile(engine):
    # '=' may not appear in an equation (the reference splits on it), so the
    # comparisons that contain one are exercised through a payoff
    expr = ("(abs(X) + sign(X) + int(X) + ceil(X) + floor(X) + round(X) + round(0.5, X) + log(X)"
            " + log(2, X) + e() + pi() + sin(X) + cos(X) + tan(X) + atan(X) + sinh(X) + tanh(X)"
            " + (X > 1) + (X < 1) + (X && 1)"
            " + (X || 0) + !X + X % 3 + X ^ 1.5 + -X ^ 2 + min(X, 1, 2) + max(X, t) + sqrt(X) + exp(-X))")
    for prec in ("fp64", "fp32"):
        engine.Plan([f"dX = {expr} * dt + (0.1) * dW1"], precision=prec,
                    payoffs=["(X >= 1) + (X <= 1) + (X == 1) + (X != 1)"])
    with pytest.raises(ValueError, match="Missing '='"):
        engine.Plan(["dX = (X == 1) * dt"])


@pytest.mark.parametrize("eq,msg", [
    ("dX = (0.1 * X) * dt = 3", "Missing '='"),
    ("dX = (0.1 * X * dt", "Unbalanced parentheses in coefficient"),
    ("dX = (0.1 * X) * dZ1", "Unknown incrementor type: dZ1"),
    ("dX = (0.1 * ) * dt", "Math error in coefficient"),
    ("dX = (0.1) * dN1(X", "Unbalanced parentheses in dN intensity"),
    ("dX = (0.1 * Y) * dt", "Unknown variable 'Y'"),
])
def test_parse_errors_raise_value_error(engine, eq, msg):
    with pytest.raises(ValueError, match=re.escape(msg)):
        engine.Plan([eq])


def test_simulate_argument_errors(engine):
    with pytest.raises(ValueError, match="scenarios must be a positive integer"):
        engine.simulate(GBM, [0.0, 1.0], 0, {"X": 1.0})
    with pytest.raises(ValueError, match="unknown scheme"):
        engine.simulate(GBM, [0.0, 1.0], 1, {"X": 1.0}, scheme="milstein")
    with pytest.raises(ValueError, match="Failed to parse equations"):
        engine.simulate(["dX = (X * dt"], [0.0, 1.0], 1, {"X": 1.0})


def test_params_are_declared_names(engine):
    p = engine.Plan(["dX = (mu * X) * dt + (sigma * X) * dW1"], params=["mu", "sigma"])
    assert "PR0" in p.source and "PR1" in p.source
    with pytest.raises(ValueError, match="name of a process"):
        engine.Plan(["dX = (X) * dt"], params=["X"])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("rng,scramble", [("pseudo", "shift"), ("sobol", "shift"), ("sobol", "xor")])
def test_adjoint_lowering_compiles(engine, precision, rng, scramble):
    eqs = ["dv = (kappa * (theta - max(v, 0))) * dt + (xi * max(v, 0)^0.5) * dW1",
           "dS = (mu * S) * dt + (rho * max(v, 0)^0.5 * S) * dW1 + ((1 - rho^2)^0.5 * max(v, 0)^0.5 * S) * dW2"]
    p = engine.Plan(eqs, params=["kappa", "theta", "xi", "rho", "mu"], payoffs=["max(S - 100, 0)", "v"],
                    grad_params=["kappa", "theta", "xi", "rho"], grad_x0=["v", "S"], precision=precision,
                    rng=rng, scramble=scramble, output="none")
    assert p.n_payoffs == 2 + 4 + 2
    assert "sde_adjoint_euler" in p.source
    # Runge-Kutta in both semantics: the reference's carries the cache (the
    # previous step's probe) as state, checkpointed beside the processes
    for sem in ("reference", "textbook"):
        q = engine.Plan(eqs, params=["kappa", "theta", "xi", "rho", "mu"], payoffs=["max(S - 100, 0)"],
                        grad_params=["kappa", "rho"], grad_x0=["v"], precision=precision, rng=rng,
                        scramble=scramble, output="none", scheme="runge-kutta", semantics=sem)
        assert "sde_adjoint_rk" in q.source and ("LC0" in q.source) == (sem == "reference")
    # jump terms are held fixed in the reverse sweep; algebraic processes
    # are not differentiated
    engine.Plan(["dX = (mu * X) * dt + (0.1 * X) * dN1(2.0)"], params=["mu"], payoffs=["X"],
                grad_params=["mu"], precision=precision, scheme="runge-kutta")
    with pytest.raises(Exception, match="algebraic"):
        engine.Plan(["dX = (mu * X) * dt + (0.1) * dW1", "Y = X"], params=["mu"], payoffs=["X"],
                    grad_params=["mu"])


def test_symbolic_derivatives(engine):
    """The lowering differentiates with the same rules the adjoint uses;
    spot-check them numerically through a compiled FP64 plan's source."""
    p = engine.Plan(["dX = (a * X^3 + sin(X) / (1 + X^2) + max(X, 0.5)^0.5) * dt + (0.1) * dW1"],
                    params=["a"], payoffs=["X"], grad_params=["a"], grad_x0=["X"])
    assert "sde_mul0" in p.source and "sde_rsqrt" in p.source


def test_host_sobol_directions_match_oracle(engine, oracle):
    from sde_sim_rs import _native as N
    dims = 21201
    V = np.zeros((dims, 32), dtype=np.uint32)
    N.check(N.lib().sde_sobol_directions(dims, V.ctypes.data))
    assert np.array_equal(V, oracle.sobol_directions(dims))


def test_sobol_dimension_limit_message(engine):
    p = engine.Plan(GBM, rng="sobol")
    # 21201 dimensions is the Joe-Kuo table: one more step than that fails
    # before touching a device
    with pytest.raises(Exception, match="Joe-Kuo table has 21201"):
        p.run(np.arange(21203, dtype=np.float64), {"X": 1.0}, 4)


def test_batch_lowering_compiles(engine):
    from sde_sim_rs.batch import Batch
    tg = engine.Plan(["dX = (mu * X) * dt + (sigma * X) * dW1"], params=["mu", "sigma"], payoffs=["X"],
                     precision="fp32", output="none")
    to = engine.Plan(["dX = (theta * (m - X)) * dt + (s) * dW1"], params=["theta", "m", "s"],
                     payoffs=["X", "X^2"], precision="fp32", output="none", scheme="runge-kutta")
    Batch([tg, to])
    # adjoint plans are templates too (Euler and Runge-Kutta), beside forward ones
    ag = engine.Plan(["dX = (mu * X) * dt + (sigma * X) * dW1"], params=["mu", "sigma"], payoffs=["X"],
                     grad_params=["mu", "sigma"], grad_x0=["X"], precision="fp32", output="none")
    ar = engine.Plan(["dX = (theta * (m - X)) * dt + (s) * dW1"], params=["theta", "m", "s"], payoffs=["X"],
                     grad_params=["theta"], precision="fp32", output="none", scheme="runge-kutta")
    Batch([tg, ag, ar])
    with pytest.raises(Exception, match="pseudo-random"):
        Batch([engine.Plan(["dX = (0.1) * dW1"], payoffs=["X"], rng="sobol")])
    with pytest.raises(ValueError, match="share one precision"):
        Batch([tg, engine.Plan(["dX = (0.1) * dW1"], payoffs=["X"], precision="fp64")])


@pytest.mark.parametrize("rng,scramble", [("pseudo", "shift"), ("sobol", "xor"), ("sobol", "shift")])
def test_tensor_core_lowering(engine, rng, scramble):
    """Correlated GBM baskets lower to tcgen05 (3 FP16 MMAs per 16 Wiener
    indices, 128 paths per CTA); other universes keep the CUDA-core kernel."""
    from bench import basket_equations
    eqs, payoff, _, _ = basket_equations(20)
    p = engine.Plan(eqs, payoffs=[payoff], precision="fp32", rng=rng, scramble=scramble, tensor_cores=True)
    assert p.uses_tensor_cores
    src = p.source
    assert "_tc(const sde_args a)" in src and "__launch_bounds__(128, 4)" in src
    # K = 20 padded to 32 = 2 chunks of 16, 3 MMAs each, per unrolled step
    n_mma = src.count("sde_mma_f16(")
    assert n_mma > 0 and n_mma == 6 * src.count("sde_mma_commit(")
    assert "sde_idesc_f16(128, 32)" in src                # N = 20 processes padded to 32
    assert "sde_mbar_wait_bounded" in src and "sde_tmem_dealloc" in src
    # the B image: rows of K = diag(sigma) L scaled by 2^e (largest entry in
    # [2^12, 2^13)), FP16 hi + lo, in the K-major core-matrix layout
    _, _, sigma, L = basket_equations(20)
    words = re.search(r"_kmat\[(\d+)\] = \{([^}]*)\}", src)
    img = np.array([int(w, 16) for w in words.group(2).replace(",", " ").split()], dtype=np.uint16)
    NP, KP = 32, 32
    assert int(words.group(1)) == img.size == 2 * NP * KP
    half = img.view(np.float16).astype(np.float64)
    n, k = np.meshgrid(np.arange(NP), np.arange(KP), indexing="ij")
    at = (n // 8) * (8 * KP) + (k // 8) * 64 + (n % 8) * 8 + k % 8
    hi, lo = half[at], half[NP * KP + at]
    K = np.zeros((NP, KP))
    K[:20, :20] = L * sigma[:, None]
    e = np.array([13 - np.frexp(np.abs(r).max())[1] if np.abs(r).max() > 0 else 0 for r in K])
    kf = (K * np.ldexp(1.0, e)[:, None]).astype(np.float32)
    assert np.array_equal(hi, kf.astype(np.float16).astype(np.float64))
    assert np.array_equal(lo, (kf - kf.astype(np.float16).astype(np.float32)).astype(np.float16).astype(np.float64))
    assert np.all(np.abs(hi[:20]).max(axis=1) < 2 ** 13) and np.all(np.abs(hi[:20]).max(axis=1) >= 2 ** 12)
    # two threads per path from 32 processes and 32 indices with linear drifts
    eqs32, pay32, _, _ = basket_equations(32)
    assert "__launch_bounds__(256, 3)" in engine.Plan(eqs32, payoffs=[pay32], precision="fp32",
                                                      tensor_cores=True).source
    assert "__launch_bounds__(128, 4)" in engine.Plan(eqs32, payoffs=[pay32], precision="fp32",
                                                      tensor_cores="row").source
    cross = list(eqs32)
    cross[0] = cross[0].replace("(0.02 * S1) * dt", "(0.02 * S2) * dt")
    q = engine.Plan(cross, payoffs=[pay32], precision="fp32", tensor_cores=True)
    assert q.uses_tensor_cores and "__launch_bounds__(128, 4)" in q.source
    with pytest.raises(ValueError):
        engine.Plan(eqs32, precision="fp32", tensor_cores="sometimes")
    # a coefficient of 1 * X and a folded constant are eligible too
    q = engine.Plan(["dA = (0.01 * A) * dt + A * dW1 + ((0.5 * 0.2) * A) * dW2",
                     "dB = (0.3 * B) * dW2"], payoffs=["A + B"], precision="fp32", tensor_cores=True)
    assert q.uses_tensor_cores
    # not eligible: state-dependent diffusion, FP64, Runge-Kutta, a cross term,
    # an algebraic process, several paths per thread
    for eqs2, kw in [(HESTON, {}), (EXAMPLE_GBM, {"precision": "fp64"}), (EXAMPLE_GBM, {"scheme": "runge-kutta"}),
                     (["dA = (0.2 * B) * dW1", "dB = (0.1 * B) * dW1"], {}),
                     (["dA = (0.2 * A) * dW1", "B = max(A - 1, 0)"], {}),
                     (EXAMPLE_GBM, {"paths_per_thread": 2}),
                     (["dA = (s * A) * dW1"], {"params": ["s"]})]:
        kw.setdefault("precision", "fp32")
        r = engine.Plan(eqs2, tensor_cores=True, **kw)
        assert not r.uses_tensor_cores, (eqs2, kw)
        assert "_tc(" not in r.source


def test_chunked_kernel_lowering_and_options(engine):
    """FP64 pseudo / shifted-Sobol plans with 1, 2, 4 or 8 stochastic indices
    carry the chunked kernel for runs with few paths; others do not; option
    values are checked."""
    for eqs, rng, want in [(GBM, "pseudo", True), (HESTON, "sobol", True), (EXAMPLE_RS, "pseudo", True),
                           (["dX = (0.1) * dW1 + (0.1) * dW2 + (0.1) * dW3"], "pseudo", False)]:
        src = engine.Plan(eqs, rng=rng, precision="fp64").source
        assert ("_chunked(const sde_args a)" in src) == want, (eqs, rng)
    for kw in [dict(precision="fp32"), dict(rng="sobol", scramble="xor"), dict(paths_per_thread=2)]:
        assert "_chunked(" not in engine.Plan(GBM, **kw).source, kw
    src = engine.Plan(GBM, precision="fp64").source
    assert "__shared__ double SW[2048]" in src        # 64 steps x 1 index x 32 paths
    with pytest.raises(ValueError):
        engine.Plan(GBM, chunked="sometimes")
    from sde_sim_rs import _native as N
    import ctypes as C
    for field, bad in (("chunked", 7), ("adjoint_recompute", 2), ("tensor_cores", 5)):
        opts = N.Options()
        N.lib().sde_options_init(C.byref(opts))
        setattr(opts, field, bad)
        h = C.c_void_p()
        rc = N.lib().sde_plan_create(N.cstrs(GBM), 1, N.cstrs([]), 0, N.cstrs([]), 0, C.byref(opts), C.byref(h))
        assert rc == N.SDE_ERR_INVALID, field


def test_wide_kernel_lowering(engine):
    """FP32 XOR-Sobol plans with automatic paths per thread (the default)
    also carry a two-paths-per-thread kernel in CTAs of 128; a set
    paths_per_thread or block_size, FP64, other streams, adjoint and
    tensor-core plans do not."""
    wide = "sde_step_euler_fp32_sobolxor_ppt2(const sde_args a)"
    src = engine.Plan(HESTON, precision="fp32", rng="sobol", scramble="xor").source
    assert wide in src and "sde_step_euler_fp32_sobolxor(const sde_args a)" in src
    assert "__launch_bounds__(128) sde_step_euler_fp32_sobolxor_ppt2" in src
    # its twin for grids of equal steps takes dt and sqrt(dt) from the
    # argument block and reads neither per-step table
    ug = src[src.index("sde_step_euler_fp32_sobolxor_ppt2_ug(const sde_args a)"):]
    assert "__launch_bounds__(128) sde_step_euler_fp32_sobolxor_ppt2_ug" in src
    assert "const float dt = a.udt_f;" in ug and "const float sdt = a.usdt_f;" in ug
    assert "a.dts_f[" not in ug and "a.sqrt_dts_f[" not in ug
    general = src[src.index("sde_step_euler_fp32_sobolxor_ppt2(const sde_args a)"):
                  src.index("sde_step_euler_fp32_sobolxor_ppt2_ug(const sde_args a)")]
    assert "a.dts_f[" in general and "a.udt_f" not in general
    from bench import basket_equations
    for eqs, kw in [(HESTON, dict(paths_per_thread=1)), (HESTON, dict(block_size=256)),
                    (HESTON, dict(precision="fp64")), (HESTON, dict(scramble="shift")),
                    (HESTON, dict(rng="pseudo", scramble="shift")),
                    (GBM, dict(payoffs=["X"], grad_x0=["X"])),
                    (basket_equations(8)[0], dict(tensor_cores=True))]:
        args = dict(precision="fp32", rng="sobol", scramble="xor")
        args.update(kw)
        assert "_ppt2(" not in engine.Plan(eqs, **args).source, kw


@pytest.mark.parametrize("ppt", [2, 4])
def test_paths_per_thread_lowering(engine, ppt):
    from sde_sim_rs import _native as N
    import ctypes as C
    p = engine.Plan(["dv = (2 * (0.04 - max(v, 0))) * dt + (0.3 * max(v, 0)^0.5) * dW1",
                     "dS = (0.03 * S) * dt + (-0.7 * max(v, 0)^0.5 * S) * dW1"], payoffs=["S"],
                    rng="sobol", scramble="xor", precision="fp32", output="terminal", paths_per_thread=1)
    src = p.source
    assert "X1_1" not in src
    opts = N.Options()
    N.lib().sde_options_init(C.byref(opts))
    opts.paths_per_thread = ppt
    h = C.c_void_p()
    N.check(N.lib().sde_plan_create(N.cstrs(["dX = (0.1 * X) * dW1"]), 1, N.cstrs([]), 0, N.cstrs(["X"]), 1,
                                    C.byref(opts), C.byref(h)))
    N.lib().sde_plan_destroy(h)


def test_lowering_choices_of_the_measured_variants(engine):
    """Each kernel family carries the variant measured faster on GB300:
    * tensor-core XOR step: LO words bulk-copied (cp.async.bulk + mbarrier
      expect_tx) into two buffers, drained on an early exit; Sobol high parts
      by the unrolled loader; one reciprocal per normal;
    * CUDA-core XOR kernels: high parts by set bits; a pair of normals
      shares one reciprocal; full step groups without the bound check;
    * ChaCha8 kernels: one copy of the step group (bound-checked)."""
    from bench import basket_equations
    eqs, pay, _, _ = basket_equations(16)
    tc = engine.Plan(eqs, payoffs=[pay], rng="sobol", scramble="xor", precision="fp32", tensor_cores=True).source
    assert "sde_bulk_g2s(" in tc and "sde_mbar_arrive_expect_tx(" in tc
    assert "for (int s_ = lb_waited + 1; s_ <= lb_issued; ++s_)" in tc
    assert "sde_sobol_hi_unrolled(" in tc and "sde_normal_xor2<false>(" in tc
    fwd = engine.Plan(HESTON, payoffs=["max(S - 100, 0)"], rng="sobol", scramble="xor", precision="fp32",
                      output="none").source
    assert "= sde_sobol_hi(a.sobol_vt" in fwd and "sde_sobol_hi_unrolled(" not in fwd
    assert "sde_normal_xor2(" in fwd and "<false>" not in fwd
    assert "if (t0 + 16 <= n_steps) {" in fwd
    pseudo = engine.Plan(GBM, payoffs=["X"], precision="fp32", output="none").source
    assert "<= n_steps) {" not in pseudo and "if (t < n_steps) {" in pseudo


def test_register_budgets_of_the_measured_kernels(engine):
    """The kernels keep the register counts their measured occupancy rests
    on (ptxas, as NVRTC compiles the plan), and none spills.  A lowering
    change that crosses a budget moves the kernel to another occupancy class
    and needs measuring again."""
    from bench import PAYOFF, basket_equations
    eqs, pay, _, _ = basket_equations(64)
    budgets = {
        "sde_step_euler_fp32_sobolxor_ppt2_ug": 48,   # Heston RQMC headline, CTAs of 128
        "sde_step_euler_fp32_sobolxor_ppt2": 56,
        "sde_step_euler_fp32_sobolxor": 32,           # one path per thread, CTAs of 256
        "sde_step_euler_fp32_sobolshift": 64,
        "sde_step_euler_fp64_pseudo_chunked": 64,
        "sde_step_euler_fp64_pseudo": 64,
        "sde_step_euler_fp32_sobolxor_tc": 80,
        "sde_adjoint_euler_fp32_pseudo": 40,
        "sde_step_euler_fp32_pseudo": 40,
    }
    plans = [
        engine.Plan(HESTON, payoffs=[PAYOFF], rng="sobol", scramble="xor", precision="fp32", output="none"),
        engine.Plan(HESTON, payoffs=[PAYOFF], rng="sobol", scramble="shift", precision="fp32", output="none"),
        engine.Plan(GBM, precision="fp64"),
        engine.Plan(eqs, payoffs=[pay], rng="sobol", scramble="xor", precision="fp32", tensor_cores=True,
                    output="none"),
        engine.Plan(GBM, payoffs=["max(X - 1, 0)"], grad_x0=["X"], precision="fp32", output="none"),
    ]
    seen = {}
    for p in plans:
        for m in re.finditer(r"Function properties for (\w+)\n.*?(\d+) bytes spill stores.*?\n"
                             r"ptxas info    : Used (\d+) registers", p.compile_log, re.S):
            seen[m.group(1)] = (int(m.group(2)), int(m.group(3)))
    assert set(budgets) <= set(seen), set(budgets) - set(seen)
    for name, cap in budgets.items():
        spill, regs = seen[name]
        assert spill == 0, name
        assert regs <= cap, (name, regs, cap)


def test_rust_shim_declarations_match_header():
    """The extern block of the Rust shim declares each function with the
    header's parameter count (sde-sim-rs_gb300/rust/src/gpu.rs, which has
    no compiler here)."""
    with open(os.path.join(ROOT, "sde-sim-rs_gb300", "rust", "src", "gpu.rs")) as f:
        rs = f.read()
    block = re.search(r'unsafe extern "C" \{(.*?)\n\}', rs, re.S).group(1)
    rust = {m.group(1): [a for a in m.group(2).split(",") if a.strip()]
            for m in re.finditer(r"fn (sde_\w+)\((.*?)\)\s*->", block, re.S)}
    with open(os.path.join(ROOT, "include", "sdegpu.h")) as f:
        hdr = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
    assert set(rust) == {"sde_simulate", "sde_result_shape", "sde_result_copy_long", "sde_result_destroy",
                         "sde_last_error"}
    for name, args in rust.items():
        decl = re.search(r"\b" + name + r"\s*\((.*?)\);", hdr, re.S).group(1)
        assert len(args) == len([a for a in decl.split(",") if a.strip()]), name
