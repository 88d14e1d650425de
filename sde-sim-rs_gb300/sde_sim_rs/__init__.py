"""sde_sim_rs -- GB300 (sm_103a) engine for the sde-sim-rs path-simulation hot
path, with the reference's Python API as a drop-in.

``simulate`` keeps the signature of the reference's binding
(src/py_binding.rs:10-18, python/sde_sim_rs/sde_sim_rs.pyi:6-13) and returns
the same long/tidy frame: one row per (scenario, time, process) with columns
scenario:i32, time:f64, process_name:str, value:f64
(src/filtration.rs:81-116).  ``Plan`` exposes the engine directly: compiled
once per process universe, run many times, with FP32 stepping, Sobol XOR
replicates, checkpointed / terminal output and payoff estimators.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Mapping, Sequence

import numpy as np

from . import _native as N
from ._native import SdeError

__all__ = ["simulate", "Plan", "Result", "SdeError", "Frame"]


def _stream_handle(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream"))


class Frame(dict):
    """Column mapping returned when neither polars nor pyarrow is importable:
    name -> numpy array, in the reference's row order."""

    @property
    def height(self) -> int:
        return len(next(iter(self.values()))) if dict.__len__(self) else 0

    def __len__(self):
        return self.height


class _HostColumn:
    """A column of engine-owned pinned memory as a numpy array interface;
    numpy keeps this object (and with it the result owning the memory)
    alive for as long as the array lives."""

    def __init__(self, owner, ptr: int, n: int, typestr: str):
        self._owner = owner
        self.__array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, True), "version": 3}


class Result:
    """One run: the filtration (on the device until copied) and estimators."""

    def __init__(self, handle, plan: "Plan | None", process_names, times):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle
        self._plan = plan  # keeps the plan alive while the run may execute
        self.process_names = list(process_names)
        self._times = np.asarray(times, dtype=np.float64)
        n, no, P, R = C.c_uint64(), C.c_int32(), C.c_int32(), C.c_int32()
        N.check(N.lib().sde_result_shape(self._h, C.byref(n), C.byref(no), C.byref(P), C.byref(R)))
        self.n_paths, self.n_out, self.n_processes, self.n_replicates = n.value, no.value, P.value, R.value
        ti = np.zeros(max(1, self.n_out), dtype=np.int32)
        N.check(N.lib().sde_result_time_indices(self._h, ti.ctypes.data))
        self.time_indices = ti[: self.n_out]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and N._lib is not None:
            N._lib.sde_result_destroy(h)
            self._h = C.c_void_p()

    def wait(self) -> "Result":
        N.check(N.lib().sde_result_wait(self._h))
        return self

    @property
    def output_times(self) -> np.ndarray:
        return self._times[self.time_indices]

    def values(self, layout: str = "reference") -> np.ndarray:
        """Filtration as f64: "reference" -> [rep, path, time, process]
        (the reference's row order), "device" -> [rep, time, process, path]."""
        shape_dev = (self.n_replicates, self.n_out, self.n_processes, self.n_paths)
        shape_ref = (self.n_replicates, self.n_paths, self.n_out, self.n_processes)
        out = np.zeros(shape_ref if layout == "reference" else shape_dev, dtype=np.float64)
        if out.size:
            lay = N.LAYOUT_REFERENCE if layout == "reference" else N.LAYOUT_DEVICE
            N.check(N.lib().sde_result_copy_values(self._h, out.ctypes.data, lay))
        return out

    def device_pointer(self):
        """(device pointer, bytes per element) of the [rep][time][process][path]
        filtration."""
        p, e = C.c_void_p(), C.c_int32()
        N.check(N.lib().sde_result_device_values(self._h, C.byref(p), C.byref(e)))
        return p.value, e.value

    def long(self) -> dict:
        """Long columns in reference row order (scenario, time, process):
        read-only views of pinned host memory that this result owns (the
        arrays keep it alive), so nothing is copied on the host."""
        ptrs = [C.c_void_p() for _ in range(4)]
        n = C.c_uint64()
        N.check(N.lib().sde_result_long_host(self._h, *[C.byref(p) for p in ptrs], C.byref(n)))
        cols = {}
        for name, p, typestr in zip(("scenario", "time", "process", "value"), ptrs, ("<i4", "<f8", "<i4", "<f8")):
            if n.value == 0:
                cols[name] = np.zeros(0, dtype=np.dtype(typestr))
            else:
                cols[name] = np.asarray(_HostColumn(self, p.value, n.value, typestr))
        return cols

    KERNELS = {0: "none", 1: "forward", 2: "chunked", 3: "wide", 4: "tensor_cores", 5: "adjoint"}

    def launch_info(self) -> dict:
        """The step kernel this run launched ("forward", "chunked": 8 warps
        per 32 paths, "wide": two paths per thread, "tensor_cores",
        "adjoint"), its CTA size and the paths one CTA steps."""
        k, b, pb = C.c_int32(), C.c_int32(), C.c_int32()
        N.check(N.lib().sde_result_launch_info(self._h, C.byref(k), C.byref(b), C.byref(pb)))
        return {"kernel": self.KERNELS[k.value], "block": b.value, "paths_per_block": pb.value}

    def estimates(self):
        """(sum, sumsq) arrays [replicates, payoffs] of the payoff estimators."""
        K = self._plan.n_payoffs if self._plan is not None else 0
        s = np.zeros((self.n_replicates, max(1, K)), dtype=np.float64)
        q = np.zeros_like(s)
        N.check(N.lib().sde_result_estimates(self._h, s.ctypes.data, q.ctypes.data))
        return s[:, :K], q[:, :K]

    def frame(self, fmt: str = "auto"):
        """The reference's long/tidy frame: polars if importable, else pyarrow,
        else a Frame of numpy columns."""
        cols = self.long()
        if fmt in ("auto", "polars"):
            try:
                import polars as pl  # noqa: F401
                import pyarrow as pa
                return pl.from_arrow(_arrow_table(cols, self.process_names, pa))
            except ImportError:
                if fmt == "polars":
                    raise
        if fmt in ("auto", "arrow"):
            try:
                import pyarrow as pa
                return _arrow_table(cols, self.process_names, pa)
            except ImportError:
                if fmt == "arrow":
                    raise
        # rows cycle through the processes in order (src/filtration.rs:87-91),
        # so the name column is the name list tiled: fixed-width unicode, no
        # per-row Python objects and no gather.  One process: a read-only
        # zero-stride view of the one name (like the other columns, which
        # are read-only views of pinned memory), no copy at all
        ustr = np.asarray(list(self.process_names) or [""], dtype=str)
        P = max(1, self.n_processes)
        if P == 1:
            names = np.broadcast_to(ustr[:1], (len(cols["process"]),))
        else:
            names = np.tile(ustr[:P], len(cols["process"]) // P)
            names.flags.writeable = False
        return Frame(scenario=cols["scenario"], time=cols["time"], process_name=names, value=cols["value"])


def _arrow_table(cols, process_names, pa):
    dictionary = pa.array(list(process_names), type=pa.string())
    pname = pa.DictionaryArray.from_arrays(pa.array(cols["process"], type=pa.int32()), dictionary)
    return pa.table({"scenario": pa.array(cols["scenario"], type=pa.int32()),
                     "time": pa.array(cols["time"], type=pa.float64()),
                     "process_name": pname.cast(pa.string()),
                     "value": pa.array(cols["value"], type=pa.float64())})


class Plan:
    """A process universe lowered to one sm_103a kernel (parse_equations,
    src/proc/util.rs:52-66, plus NVRTC lowering of every coefficient)."""

    def __init__(self, equations: Sequence[str], *, params: Sequence[str] = (),
                 payoffs: Sequence[str] = (), scheme: str = "euler", rng: str = "pseudo",
                 scramble: str = "shift", precision: str = "fp64", semantics: str = "reference",
                 output: str = "full", block_size: int = 0, grad_params: Sequence[str] | None = None,
                 grad_x0: Sequence[str] | None = None, ckpt_every: int = 0, paths_per_thread: int = 0,
                 icdf: str = "as26", tensor_cores: bool | str = False, adjoint_recompute: bool = False,
                 chunked: str = "auto"):
        """grad_params / grad_x0 make an adjoint plan: each run also returns
        the pathwise derivatives of E[payoffs[0]] with respect to those
        parameters and initial values (Euler-Maruyama or Runge-Kutta in
        either semantics, checkpoints every ckpt_every steps, default 19);
        the forward pass's increments are kept in device memory for the
        reverse sweep when they fit in a quarter of the free memory
        (adjoint_recompute=True draws them again instead).
        tensor_cores=True lowers the dW
        terms of an FP32 Euler universe whose diffusions are constant * own
        process (correlated GBM) to one tcgen05 product per 128 paths, with
        two threads per path for wide universes ("row": always one);
        ``uses_tensor_cores`` says whether the universe was eligible.
        chunked ("auto" | "on" | "off") picks the FP64 kernel for runs with
        few paths, where 8 warps per 32 paths draw the increments.
        paths_per_thread 1, 2 or 4 fixes how many paths a thread steps; 0
        (default) lets FP32 XOR-Sobol plans take two on large runs."""
        if scheme not in N.SCHEME:
            raise ValueError(f"unknown scheme '{scheme}'")
        opts = N.Options()
        N.lib().sde_options_init(C.byref(opts))
        opts.scheme = N.SCHEME[scheme]
        opts.rng = N.RNG[rng]
        opts.scramble = N.SCRAMBLE[scramble]
        opts.precision = N.PRECISION[precision]
        opts.semantics = N.SEMANTICS[semantics]
        opts.output = N.OUTPUT[output]
        opts.block_size = block_size
        opts.ckpt_every = ckpt_every
        opts.adjoint_recompute = 1 if adjoint_recompute else 0
        if chunked not in N.CHUNKED:
            raise ValueError(f"unknown chunked {chunked!r}")
        opts.chunked = N.CHUNKED[chunked]
        opts.paths_per_thread = paths_per_thread
        opts.icdf = N.ICDF[icdf]
        if tensor_cores not in N.TENSOR_CORES:
            raise ValueError(f"unknown tensor_cores {tensor_cores!r}")
        opts.tensor_cores = N.TENSOR_CORES[tensor_cores]
        self.equations = list(equations)
        self.params = list(params)
        self.payoffs = list(payoffs)
        self.precision = precision
        self.grad_params = list(grad_params or [])
        self.grad_x0 = list(grad_x0 or [])
        self.adjoint = grad_params is not None or grad_x0 is not None
        h = C.c_void_p()
        if self.adjoint:
            N.check(N.lib().sde_plan_create_adjoint(
                N.cstrs(self.equations), len(self.equations), N.cstrs(self.params), len(self.params),
                N.cstrs(self.payoffs), len(self.payoffs), N.cstrs(self.grad_params),
                len(self.grad_params), N.cstrs(self.grad_x0), len(self.grad_x0), C.byref(opts),
                C.byref(h)))
        else:
            N.check(N.lib().sde_plan_create(N.cstrs(self.equations), len(self.equations),
                                            N.cstrs(self.params), len(self.params),
                                            N.cstrs(self.payoffs), len(self.payoffs),
                                            C.byref(opts), C.byref(h)))
        self._h = h
        n = C.c_int32()
        N.check(N.lib().sde_plan_n_estimates(h, C.byref(n)))
        self.n_payoffs = n.value
        N.check(N.lib().sde_plan_n_processes(h, C.byref(n)))
        self.n_processes = n.value
        N.check(N.lib().sde_plan_n_stochastic(h, C.byref(n)))
        self.n_stochastic = n.value
        N.check(N.lib().sde_plan_tensor_cores(h, C.byref(n)))
        self.uses_tensor_cores = bool(n.value)
        buf = C.create_string_buffer(4096)
        self.process_names = []
        for i in range(self.n_processes):
            N.check(N.lib().sde_plan_process_name(h, i, buf, len(buf)))
            self.process_names.append(buf.value.decode())
        self.stochastic_tokens = []
        for i in range(self.n_stochastic):
            N.check(N.lib().sde_plan_stochastic_token(h, i, buf, len(buf)))
            self.stochastic_tokens.append(buf.value.decode())

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and N._lib is not None:
            N._lib.sde_plan_destroy(h)
            self._h = C.c_void_p()

    @property
    def source(self) -> str:
        need = C.c_size_t()
        N.check(N.lib().sde_plan_source(self._h, None, 0, C.byref(need)))
        buf = C.create_string_buffer(need.value)
        N.check(N.lib().sde_plan_source(self._h, buf, need.value, None))
        return buf.value.decode()

    @property
    def compile_log(self) -> str:
        """NVRTC / ptxas output of the lowering (registers, spills)."""
        need = C.c_size_t()
        N.check(N.lib().sde_plan_compile_log(self._h, None, 0, C.byref(need)))
        buf = C.create_string_buffer(need.value)
        N.check(N.lib().sde_plan_compile_log(self._h, buf, need.value, None))
        return buf.value.decode(errors="replace")

    def index(self, name: str) -> int:
        idx = C.c_int32()
        N.check(N.lib().sde_plan_process_index(self._h, name.encode(), C.byref(idx)))
        return idx.value

    def x0(self, initial_values: Mapping[str, float]) -> np.ndarray:
        """Time-0 row: unknown names are ignored and missing processes start at
        0.0, as ScenarioFiltration::new does (src/filtration.rs:42-50)."""
        x = np.zeros(max(1, self.n_processes), dtype=np.float64)
        for k, v in dict(initial_values).items():
            i = self.index(k)
            if i >= 0:
                x[i] = float(v)
        return x

    def run(self, times: Sequence[float], initial_values: Mapping[str, float], n_paths: int, *,
            replicates: int = 1, seed: int = 0, params: Mapping[str, float] | Sequence[float] | None = None,
            checkpoints: Sequence[int] | None = None, path_offset: int = 0, stream=None,
            device_out: int | None = None, device_out_bytes: int = 0) -> Result:
        times_a = np.ascontiguousarray(times, dtype=np.float64)
        x0 = self.x0(initial_values)
        if params is None:
            pv = np.zeros(max(1, len(self.params)), dtype=np.float64)
            if self.params:
                raise ValueError(f"values for parameters {self.params} are required")
        elif isinstance(params, Mapping):
            missing = [p for p in self.params if p not in params]
            if missing:
                raise ValueError(f"missing parameter values {missing}")
            pv = np.array([float(params[p]) for p in self.params] or [0.0], dtype=np.float64)
        else:
            pv = np.ascontiguousarray(params, dtype=np.float64).reshape(-1)
            if len(pv) != len(self.params):
                raise ValueError("parameter count does not match the plan")
            if len(pv) == 0:
                pv = np.zeros(1, dtype=np.float64)
        ck = np.ascontiguousarray(checkpoints if checkpoints is not None else [0], dtype=np.int32)
        a = N.RunArgs()
        N.lib().sde_run_args_init(C.byref(a))
        a.times = times_a.ctypes.data_as(C.POINTER(C.c_double))
        a.n_times = len(times_a)
        a.x0 = x0.ctypes.data_as(C.POINTER(C.c_double))
        a.n_x0 = self.n_processes
        a.params = pv.ctypes.data_as(C.POINTER(C.c_double))
        a.n_params = len(self.params)
        a.n_paths = int(n_paths)
        a.n_replicates = int(replicates)
        a.seed = int(seed) & (2**64 - 1)
        a.path_offset = int(path_offset)
        a.checkpoints = ck.ctypes.data_as(C.POINTER(C.c_int32))
        a.n_checkpoints = len(checkpoints) if checkpoints is not None else 0
        a.stream = _stream_handle(stream)
        a.device_out = device_out
        a.device_out_bytes = int(device_out_bytes)
        h = C.c_void_p()
        N.check(N.lib().sde_run(self._h, C.byref(a), C.byref(h)))
        return Result(h, self, self.process_names, times_a)


def simulate(processes_equations: Sequence[str], time_steps: Sequence[float], scenarios: int,
             initial_values: Mapping[str, float], rng_method: str = "pseudo",
             scheme: str = "euler", *, seed: int | None = None, output_format: str = "auto"):
    """Drop-in for sde_sim_rs.simulate (src/py_binding.rs:10-56).

    Runs on the GPU: FP64, the reference's Euler / Runge-Kutta semantics and
    RNG streams, full filtration.  ``seed`` is an addition (the reference
    draws it from the OS, src/sim/mod.rs:28-29; ``None`` keeps that).
    Errors: scenarios <= 0 and malformed equations raise ValueError; an
    unknown scheme raises ValueError (the reference panics); an unknown
    rng_method falls back to pseudo, as in the reference.
    """
    if int(scenarios) <= 0:
        raise ValueError("scenarios must be a positive integer")
    if scheme not in N.SCHEME:
        raise ValueError(f"unknown scheme '{scheme}'")
    eqs = [str(e) for e in processes_equations]
    times = np.ascontiguousarray(time_steps, dtype=np.float64)
    names = list(initial_values.keys())
    vals = np.array([float(initial_values[k]) for k in names] or [0.0], dtype=np.float64)
    h = C.c_void_p()
    rc = N.lib().sde_simulate(N.cstrs(eqs), len(eqs), times.ctypes.data_as(C.POINTER(C.c_double)),
                              len(times), N.cstrs(names), vals.ctypes.data_as(C.POINTER(C.c_double)),
                              len(names), int(scenarios), scheme.encode(), str(rng_method).encode(),
                              0 if seed is None else int(seed) & (2**64 - 1),
                              0 if seed is None else 1, C.byref(h))
    if rc == N.SDE_ERR_PARSE:
        raise ValueError(f"Failed to parse equations: {N.last_error()}")
    N.check(rc)
    # process names in universe order come from a plan-free parse of the
    # equations' left-hand sides (src/proc/util.rs:78-80)
    pnames = []
    for e in eqs:
        lhs = e.split("=")[0].strip()
        pnames.append(lhs[1:] if lhs.startswith("d") else lhs)
    res = Result(h, None, pnames, times)
    return res.frame(output_format)
