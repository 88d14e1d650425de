"""ctypes front end of the CPU oracle (oracle/sde_oracle.c).

TEST INFRASTRUCTURE ONLY.  The oracle: what the GPU engine's parity tests
compare with, and the timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / reference arm import it; the product package never does.

The oracle restates the sde-sim-rs hot path (src/sim, src/proc, src/rng,
src/filtration, src/func.rs) in plain C; see sde_oracle.h for the list of
reference functions and the pins.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libsde_oracle.so")

EULER, RK = 0, 1
PSEUDO, SOBOL = 0, 1
SHIFT, XOR = 0, 1
REFERENCE, TEXTBOOK = 0, 1


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, portable flags)."""
    src = os.path.join(HERE, "sde_oracle.c")
    hdr = os.path.join(HERE, "sde_oracle.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O3", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-shared", "-pthread", "-D_GNU_SOURCE", src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class _Cfg(C.Structure):
    _fields_ = [("scheme", C.c_int), ("rng", C.c_int), ("scramble", C.c_int),
                ("semantics", C.c_int), ("seed", C.c_uint64),
                ("n_paths_per_replicate", C.c_uint64),
                ("sobol_v", C.POINTER(C.c_uint32)), ("sobol_dims", C.c_int), ("icdf", C.c_int)]


class _Jump(C.Structure):
    _fields_ = [("t", C.c_int32), ("idx", C.c_int32), ("u", C.c_double), ("lam", C.c_double),
                ("k", C.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_parse.argtypes = [C.POINTER(C.c_char_p), C.c_int, C.POINTER(C.c_char_p),
                                C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_void_p),
                                C.c_char_p, C.c_size_t]
        L.orc_free.argtypes = [C.c_void_p]
        for f in ("orc_n_processes", "orc_n_stochastic"):
            getattr(L, f).argtypes = [C.c_void_p]
        L.orc_process_name.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_size_t]
        L.orc_stochastic_token.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_size_t]
        L.orc_process_is_levy.argtypes = [C.c_void_p, C.c_int]
        L.orc_process_index.argtypes = [C.c_void_p, C.c_char_p]
        L.orc_simulate.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int,
                                   C.POINTER(C.c_double), C.c_uint64, C.c_uint64,
                                   C.POINTER(_Cfg), C.c_void_p, C.c_void_p, C.c_int,
                                   C.c_char_p, C.c_size_t]
        L.orc_estimate.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int,
                                   C.POINTER(C.c_double), C.c_uint64, C.c_uint64,
                                   C.POINTER(_Cfg), C.c_char_p, C.c_int,
                                   C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   C.c_char_p, C.c_size_t]
        L.orc_eval_payoff.argtypes = [C.c_void_p, C.c_char_p, C.c_double, C.c_void_p,
                                      C.c_int64, C.c_void_p, C.c_char_p, C.c_size_t]
        L.orc_chacha_block.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int, C.c_void_p]
        L.orc_seed_from_u64.argtypes = [C.c_uint64, C.c_void_p]
        L.orc_chacha8_u64.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p]
        L.orc_u64_to_f64.argtypes = [C.c_uint64]
        L.orc_u64_to_f64.restype = C.c_double
        L.orc_xor_mask.argtypes = [C.c_uint64, C.c_int, C.c_int]
        L.orc_xor_mask.restype = C.c_uint32
        L.orc_sobol_directions.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        L.orc_sobol_points.argtypes = [C.c_void_p, C.c_int, C.c_uint64, C.c_uint64, C.c_void_p]
        L.orc_icdf_as26.argtypes = [C.c_double]
        L.orc_icdf_as26.restype = C.c_double
        L.orc_icdf_accurate.argtypes = [C.c_double]
        L.orc_icdf_accurate.restype = C.c_double
        L.orc_jump_trace.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double),
                                     C.c_uint64, C.POINTER(_Cfg), C.POINTER(_Jump), C.c_int,
                                     C.POINTER(C.c_int), C.c_char_p, C.c_size_t]
        L.orc_poisson.argtypes = [C.c_double, C.c_double]
        L.orc_poisson.restype = C.c_uint64
        _lib = L
    return _lib


def _cstrs(strs):
    arr = (C.c_char_p * max(1, len(strs)))()
    for i, s in enumerate(strs):
        arr[i] = s.encode()
    return arr


class OracleError(RuntimeError):
    pass


_JK = None


def joe_kuo_table():
    """(poly, vinit) of the Joe-Kuo D6 21201-dimension table, read from the
    copy scipy ships (the same published data the sobol crate embeds)."""
    global _JK
    if _JK is None:
        import scipy.stats as st
        path = os.path.join(os.path.dirname(st.__file__), "_sobol_direction_numbers.npz")
        d = np.load(path)
        _JK = (np.ascontiguousarray(d["poly"], dtype=np.int64),
               np.ascontiguousarray(d["vinit"], dtype=np.int64))
    return _JK


_V = {}


def sobol_directions(dims: int) -> np.ndarray:
    if dims not in _V:
        poly, vinit = joe_kuo_table()
        if dims > len(poly):
            raise OracleError(f"Sobol table has {len(poly)} dimensions, {dims} requested")
        V = np.zeros((dims, 32), dtype=np.uint32)
        rc = lib().orc_sobol_directions(poly.ctypes.data, vinit.ctypes.data, dims, V.ctypes.data)
        if rc:
            raise OracleError("bad Joe-Kuo row")
        _V[dims] = V
    return _V[dims]


def sobol_points(dims: int, first: int, n: int) -> np.ndarray:
    V = sobol_directions(dims)
    out = np.zeros((n, dims), dtype=np.uint32)
    lib().orc_sobol_points(V.ctypes.data, dims, first, n, out.ctypes.data)
    return out


def chacha_block(key, counter: int, stream: int = 0, rounds: int = 8) -> np.ndarray:
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(16, dtype=np.uint32)
    lib().orc_chacha_block(k.ctypes.data, counter, stream, rounds, out.ctypes.data)
    return out


def seed_from_u64(seed: int) -> np.ndarray:
    k = np.zeros(8, dtype=np.uint32)
    lib().orc_seed_from_u64(seed & (2**64 - 1), k.ctypes.data)
    return k


def chacha8_u64(seed: int, first: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.uint64)
    lib().orc_chacha8_u64(seed & (2**64 - 1), first, n, out.ctypes.data)
    return out


def u64_to_f64(x: np.ndarray) -> np.ndarray:
    return (np.asarray(x, dtype=np.uint64) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def xor_mask(seed: int, replicate: int, dim: int) -> int:
    return int(lib().orc_xor_mask(seed, replicate, dim))


def icdf_accurate(p: float) -> float:
    return lib().orc_icdf_accurate(p)


def icdf_as26(p: float) -> float:
    return lib().orc_icdf_as26(p)


def poisson(u: float, lam: float) -> int:
    return int(lib().orc_poisson(u, lam))


def poisson_boundary_ulps(u: float, lam: float) -> float:
    """Distance, in units of the last place of u, from the uniform u to the
    nearest cumulative probability F(k) that the reference's inversion walk
    (src/proc/increment.rs:182-200) compares it with: F(0) = exp(-lam),
    F(k) = F(k-1) + p(k-1) lam / k, up to one past the count it returns.  A
    count that flips on a last-bit difference of lam (or of exp) has u
    within a few units of the last place of one of them."""
    import math
    if lam <= 0.0:
        return math.inf
    k_end = poisson(u, lam) + 1
    p = math.exp(-lam)
    f = p
    best = abs(u - f)
    for k in range(1, min(k_end, 200) + 1):
        p *= lam / k
        f += p
        best = min(best, abs(u - f))
    return best / math.ulp(max(u, 1e-300))


class Universe:
    """Parsed equations (src/proc/util.rs:52-166)."""

    def __init__(self, equations, params=None):
        params = dict(params or {})
        names = list(params.keys())
        vals = (C.c_double * max(1, len(names)))(*[float(params[k]) for k in names])
        err = C.create_string_buffer(1024)
        h = C.c_void_p()
        rc = lib().orc_parse(_cstrs(equations), len(equations), _cstrs(names), vals, len(names),
                             C.byref(h), err, len(err))
        if rc:
            raise ValueError(err.value.decode())
        self._h = h
        self.params = params
        L = lib()
        self.n_processes = L.orc_n_processes(h)
        self.n_stochastic = L.orc_n_stochastic(h)
        buf = C.create_string_buffer(512)
        self.process_names = []
        self.is_levy = []
        for i in range(self.n_processes):
            L.orc_process_name(h, i, buf, len(buf))
            self.process_names.append(buf.value.decode())
            self.is_levy.append(bool(L.orc_process_is_levy(h, i)))
        self.stochastic_tokens = []
        for i in range(self.n_stochastic):
            L.orc_stochastic_token(h, i, buf, len(buf))
            self.stochastic_tokens.append(buf.value.decode())

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_free(self._h)
            self._h = None

    def index(self, name: str) -> int:
        return lib().orc_process_index(self._h, name.encode())

    def x0(self, initial_values) -> np.ndarray:
        """Time-0 row: unknown names ignored, missing values 0.0
        (src/filtration.rs:42-50)."""
        x = np.zeros(max(1, self.n_processes), dtype=np.float64)
        for k, v in dict(initial_values).items():
            i = self.index(k)
            if i >= 0:
                x[i] = float(v)
        return x

    def _cfg(self, scheme, rng, scramble, semantics, seed, n_per_rep, sobol_dims_needed, icdf=0):
        cfg = _Cfg()
        cfg.scheme, cfg.rng, cfg.scramble, cfg.semantics = scheme, rng, scramble, semantics
        cfg.icdf = icdf
        cfg.seed = seed & (2**64 - 1)
        cfg.n_paths_per_replicate = n_per_rep
        self._keep = None
        if rng == SOBOL:
            V = sobol_directions(max(1, sobol_dims_needed))
            self._keep = V
            cfg.sobol_v = V.ctypes.data_as(C.POINTER(C.c_uint32))
            cfg.sobol_dims = V.shape[0]
        return cfg

    def simulate(self, times, initial_values, path_begin, path_end, *, scheme=EULER, rng=PSEUDO,
                 scramble=SHIFT, semantics=REFERENCE, seed=0, n_per_replicate=0, full=True,
                 threads=1, icdf=0):
        times = np.ascontiguousarray(times, dtype=np.float64)
        T, P = len(times), self.n_processes
        n = path_end - path_begin
        x0 = self.x0(initial_values)
        cfg = self._cfg(scheme, rng, scramble, semantics, seed, n_per_replicate or n,
                        (T - 1) * self.n_stochastic, icdf)
        full_arr = np.zeros((n, T, P), dtype=np.float64) if full else None
        term = np.zeros((n, P), dtype=np.float64)
        err = C.create_string_buffer(1024)
        rc = lib().orc_simulate(self._h, times.ctypes.data_as(C.POINTER(C.c_double)), T,
                                x0.ctypes.data_as(C.POINTER(C.c_double)), path_begin, path_end,
                                C.byref(cfg), full_arr.ctypes.data if full else None,
                                term.ctypes.data, threads, err, len(err))
        if rc:
            raise OracleError(err.value.decode())
        return full_arr if full else term

    def estimate(self, times, initial_values, path_begin, path_end, payoff, *, scheme=EULER,
                 rng=PSEUDO, scramble=SHIFT, semantics=REFERENCE, seed=0, n_per_replicate=0,
                 threads=1, icdf=0):
        times = np.ascontiguousarray(times, dtype=np.float64)
        T = len(times)
        x0 = self.x0(initial_values)
        n = path_end - path_begin
        cfg = self._cfg(scheme, rng, scramble, semantics, seed, n_per_replicate or n,
                        (T - 1) * self.n_stochastic, icdf)
        s, q = C.c_double(), C.c_double()
        err = C.create_string_buffer(1024)
        rc = lib().orc_estimate(self._h, times.ctypes.data_as(C.POINTER(C.c_double)), T,
                                x0.ctypes.data_as(C.POINTER(C.c_double)), path_begin, path_end,
                                C.byref(cfg), payoff.encode(), threads, C.byref(s), C.byref(q),
                                err, len(err))
        if rc:
            raise OracleError(err.value.decode())
        return s.value, q.value

    def jump_trace(self, times, initial_values, scenario, *, scheme=EULER, rng=PSEUDO, scramble=SHIFT,
                   semantics=REFERENCE, seed=0, n_per_replicate=0, icdf=0, max_draws=0):
        """Every Poisson draw of one scenario in draw order: a list of
        (step, stochastic index, uniform, lambda * dt, count)."""
        times = np.ascontiguousarray(times, dtype=np.float64)
        T = len(times)
        x0 = self.x0(initial_values)
        cfg = self._cfg(scheme, rng, scramble, semantics, seed, n_per_replicate or (scenario + 1),
                        (T - 1) * self.n_stochastic, icdf)
        max_draws = max_draws or 64 * max(1, T - 1)
        buf = (_Jump * max_draws)()
        n = C.c_int()
        err = C.create_string_buffer(1024)
        rc = lib().orc_jump_trace(self._h, times.ctypes.data_as(C.POINTER(C.c_double)), T,
                                  x0.ctypes.data_as(C.POINTER(C.c_double)), scenario, C.byref(cfg), buf,
                                  max_draws, C.byref(n), err, len(err))
        if rc:
            raise OracleError(err.value.decode())
        return [(buf[i].t, buf[i].idx, buf[i].u, buf[i].lam, buf[i].k) for i in range(n.value)]

    def payoff(self, expr, t, rows):
        rows = np.ascontiguousarray(rows, dtype=np.float64)
        out = np.zeros(rows.shape[0], dtype=np.float64)
        err = C.create_string_buffer(1024)
        rc = lib().orc_eval_payoff(self._h, expr.encode(), float(t), rows.ctypes.data,
                                   rows.shape[0], out.ctypes.data, err, len(err))
        if rc:
            raise ValueError(err.value.decode())
        return out
