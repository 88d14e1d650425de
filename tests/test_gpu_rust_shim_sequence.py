"""The call sequence of the Rust shim (sde-sim-rs_gb300/rust/src/gpu.rs),
made through ctypes: sde_simulate -> sde_result_shape ->
sde_result_copy_long -> sde_result_destroy, and sde_last_error on failure.
The rows are the reference's long frame (src/filtration.rs:81-116 per
scenario, concatenated in scenario order, src/sim/mod.rs:91), checked
against the oracle."""
import ctypes as C

import numpy as np
import pytest

from conftest import EXAMPLE_RS, GBM

pytestmark = pytest.mark.gpu


def _cstrs(strs):
    arr = (C.c_char_p * max(1, len(strs)))()
    for i, s in enumerate(strs):
        arr[i] = s.encode()
    return arr


def _shim_simulate(lib, eqs, times, init, n, scheme, rng, seed=None):
    """What gpu::simulate does, step for step; returns the four columns."""
    t = np.ascontiguousarray(times, dtype=np.float64)
    names = list(init)
    vals = np.array([init[k] for k in names] or [0.0], dtype=np.float64)
    r = C.c_void_p()
    dp = C.POINTER(C.c_double)
    rc = lib.sde_simulate(_cstrs(eqs), len(eqs), t.ctypes.data_as(dp), len(t), _cstrs(names),
                          vals.ctypes.data_as(dp), len(names), n, scheme.encode(), rng.encode(),
                          0 if seed is None else seed, 0 if seed is None else 1, C.byref(r))
    if rc != 0:
        buf = C.create_string_buffer(4096)
        lib.sde_last_error(buf, len(buf))
        assert not r.value
        return rc, buf.value.decode()
    try:
        n_paths, n_out, n_proc, n_rep = C.c_uint64(), C.c_int32(), C.c_int32(), C.c_int32()
        assert lib.sde_result_shape(r, C.byref(n_paths), C.byref(n_out), C.byref(n_proc), C.byref(n_rep)) == 0
        rows = n_paths.value * n_out.value * n_proc.value * n_rep.value
        cols = (np.zeros(rows, np.int32), np.zeros(rows, np.float64), np.zeros(rows, np.int32),
                np.zeros(rows, np.float64))
        assert lib.sde_result_copy_long(r, *[c.ctypes.data for c in cols]) == 0
    finally:
        assert lib.sde_result_destroy(r) == 0
    return 0, cols


@pytest.mark.parametrize("eqs,init,scheme", [(GBM, {"X": 100.0}, "euler"),
                                             (EXAMPLE_RS, {"X1": 100.0, "X2": 0.0}, "runge-kutta")])
@pytest.mark.parametrize("rng", ["pseudo", "sobol"])
def test_shim_sequence_rows_match_oracle(engine, oracle, eqs, init, scheme, rng):
    from sde_sim_rs import _native as N
    lib = N.lib()
    times = [i / 50 for i in range(51)]
    n = 300
    rc, (scen, tm, proc, val) = _shim_simulate(lib, eqs, times, init, n, scheme, rng, seed=42)
    assert rc == 0
    u = oracle.Universe(eqs)
    P = u.n_processes
    ref = u.simulate(times, init, 0, n, scheme=oracle.RK if scheme == "runge-kutta" else oracle.EULER,
                     rng=oracle.SOBOL if rng == "sobol" else oracle.PSEUDO, seed=42, threads=8)
    # row order (scenario, time, process)
    assert len(val) == n * len(times) * P
    np.testing.assert_array_equal(scen, np.repeat(np.arange(n), len(times) * P))
    np.testing.assert_array_equal(tm, np.tile(np.repeat(times, P), n))
    np.testing.assert_array_equal(proc, np.tile(np.arange(P), n * len(times)))
    got = val.reshape(n, len(times), P)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)
    # jump counts may flip on a last-bit intensity difference at a CDF
    # boundary (one path at most here); every other value to 1e-12
    bad = np.unique(np.nonzero(rel > 1e-12)[0])
    assert len(bad) <= (1 if "dN" in "".join(eqs) else 0), bad


def test_shim_sequence_os_seed_and_errors(engine):
    from sde_sim_rs import _native as N
    lib = N.lib()
    rc, cols = _shim_simulate(lib, GBM, [0.0, 0.5, 1.0], {"X": 100.0}, 64, "euler", "pseudo")
    assert rc == 0 and len(cols[3]) == 64 * 3 and np.all(np.isfinite(cols[3]))
    rc, msg = _shim_simulate(lib, ["dX = (0.05 * X * dt"], [0.0, 1.0], {"X": 1.0}, 4, "euler", "pseudo")
    assert rc == N.SDE_ERR_PARSE and msg
    rc, msg = _shim_simulate(lib, GBM, [0.0, 1.0], {"X": 1.0}, 4, "milstein", "pseudo")
    assert rc == N.SDE_ERR_INVALID and "milstein" in msg
