"""ctypes binding of libsdegpu.so (include/sdegpu.h).

The library is built in-tree by ``__graft_entry__.build()`` (or
``python sde-sim-rs_gb300/csrc/build.py``).  There is no CPU fallback:
importing the engine without the library raises.
"""
from __future__ import annotations

import ctypes as C
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libsdegpu.so")

SDE_OK = 0
SDE_ERR_PARSE = 1
SDE_ERR_INVALID = 2
SDE_ERR_COMPILE = 3
SDE_ERR_CUDA = 4
SDE_ERR_OOM = 5
SDE_ERR_RNG_INDEX = 6
SDE_ERR_UNSUPPORTED = 7
SDE_ERR_DEVICE = 8

SCHEME = {"euler": 0, "runge-kutta": 1}
RNG = {"pseudo": 0, "sobol": 1}
SCRAMBLE = {"shift": 0, "xor": 1}
PRECISION = {"fp64": 0, "fp32": 1}
SEMANTICS = {"reference": 0, "textbook": 1}
OUTPUT = {"full": 0, "checkpoints": 1, "terminal": 2, "none": 3}
ICDF = {"as26": 0, "reference": 0, "accurate": 1}
TENSOR_CORES = {False: 0, True: 1, "off": 0, "auto": 1, "row": 2}
CHUNKED = {"auto": 0, "on": 1, "off": 2}
LAYOUT_REFERENCE, LAYOUT_DEVICE = 0, 1


class Options(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("scheme", C.c_int32), ("rng", C.c_int32),
                ("scramble", C.c_int32), ("precision", C.c_int32), ("semantics", C.c_int32),
                ("output", C.c_int32), ("block_size", C.c_int32), ("ckpt_every", C.c_int32),
                ("paths_per_thread", C.c_int32), ("icdf", C.c_int32), ("tensor_cores", C.c_int32),
                ("adjoint_recompute", C.c_int32), ("chunked", C.c_int32), ("reserved", C.c_int32 * 2)]


class RunArgs(C.Structure):
    _fields_ = [("struct_size", C.c_uint32),
                ("times", C.POINTER(C.c_double)), ("n_times", C.c_int32),
                ("x0", C.POINTER(C.c_double)), ("n_x0", C.c_int32),
                ("params", C.POINTER(C.c_double)), ("n_params", C.c_int32),
                ("n_paths", C.c_uint64), ("n_replicates", C.c_int32),
                ("seed", C.c_uint64), ("path_offset", C.c_uint64),
                ("checkpoints", C.POINTER(C.c_int32)), ("n_checkpoints", C.c_int32),
                ("stream", C.c_void_p), ("device_out", C.c_void_p),
                ("device_out_bytes", C.c_uint64)]


class BatchInstances(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("n_instances", C.c_int32),
                ("template_id", C.c_void_p), ("n_steps", C.c_void_p), ("t_end", C.c_void_p),
                ("n_paths", C.c_void_p), ("seed", C.c_void_p), ("x0", C.c_void_p),
                ("x0_stride", C.c_int32), ("params", C.c_void_p), ("param_stride", C.c_int32)]


class SdeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


# exported symbol -> (argtypes, restype); the ABI surface of include/sdegpu.h
SIGNATURES = {
    "sde_abi_version": ([], C.c_int32),
    "sde_last_error": ([C.c_char_p, C.c_size_t], C.c_int),
    "sde_debug_tc_wait_cycles": ([C.c_uint64], C.c_int),
    "sde_options_init": ([C.POINTER(Options)], None),
    "sde_run_args_init": ([C.POINTER(RunArgs)], None),
    "sde_plan_create": ([C.POINTER(C.c_char_p), C.c_int32, C.POINTER(C.c_char_p), C.c_int32,
                         C.POINTER(C.c_char_p), C.c_int32, C.POINTER(Options),
                         C.POINTER(C.c_void_p)], C.c_int),
    "sde_plan_create_adjoint": ([C.POINTER(C.c_char_p), C.c_int32, C.POINTER(C.c_char_p), C.c_int32,
                                 C.POINTER(C.c_char_p), C.c_int32, C.POINTER(C.c_char_p), C.c_int32,
                                 C.POINTER(C.c_char_p), C.c_int32, C.POINTER(Options),
                                 C.POINTER(C.c_void_p)], C.c_int),
    "sde_plan_n_estimates": ([C.c_void_p, C.POINTER(C.c_int32)], C.c_int),
    "sde_plan_destroy": ([C.c_void_p], C.c_int),
    "sde_plan_n_processes": ([C.c_void_p, C.POINTER(C.c_int32)], C.c_int),
    "sde_plan_n_stochastic": ([C.c_void_p, C.POINTER(C.c_int32)], C.c_int),
    "sde_plan_process_name": ([C.c_void_p, C.c_int32, C.c_char_p, C.c_size_t], C.c_int),
    "sde_plan_process_index": ([C.c_void_p, C.c_char_p, C.POINTER(C.c_int32)], C.c_int),
    "sde_plan_stochastic_token": ([C.c_void_p, C.c_int32, C.c_char_p, C.c_size_t], C.c_int),
    "sde_plan_source": ([C.c_void_p, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)], C.c_int),
    "sde_plan_compile_log": ([C.c_void_p, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)], C.c_int),
    "sde_plan_tensor_cores": ([C.c_void_p, C.POINTER(C.c_int32)], C.c_int),
    "sde_probe_chacha8_rate": ([C.POINTER(C.c_double)], C.c_int),
    "sde_result_launch_info": ([C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)],
                               C.c_int),
    "sde_result_long_host": ([C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                              C.POINTER(C.c_void_p), C.POINTER(C.c_uint64)], C.c_int),
    "sde_run": ([C.c_void_p, C.POINTER(RunArgs), C.POINTER(C.c_void_p)], C.c_int),
    "sde_simulate": ([C.POINTER(C.c_char_p), C.c_int32, C.POINTER(C.c_double), C.c_int32,
                      C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.c_int32, C.c_uint64,
                      C.c_char_p, C.c_char_p, C.c_uint64, C.c_int32, C.POINTER(C.c_void_p)],
                     C.c_int),
    "sde_result_destroy": ([C.c_void_p], C.c_int),
    "sde_result_wait": ([C.c_void_p], C.c_int),
    "sde_result_shape": ([C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_int32),
                          C.POINTER(C.c_int32), C.POINTER(C.c_int32)], C.c_int),
    "sde_result_time_indices": ([C.c_void_p, C.c_void_p], C.c_int),
    "sde_result_device_values": ([C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int32)], C.c_int),
    "sde_result_copy_values": ([C.c_void_p, C.c_void_p, C.c_int32], C.c_int),
    "sde_result_copy_long": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "sde_result_estimates": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "sde_run_estimates_static": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                  C.c_int32, C.c_uint64, C.c_int32, C.c_uint64, C.c_void_p, C.c_void_p,
                                  C.c_void_p], C.c_int),
    "sde_batch_create": ([C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)], C.c_int),
    "sde_batch_destroy": ([C.c_void_p], C.c_int),
    "sde_batch_prepare": ([C.c_void_p, C.POINTER(BatchInstances), C.c_int32, C.c_void_p,
                           C.POINTER(C.c_void_p)], C.c_int),
    "sde_batch_job_run": ([C.c_void_p, C.c_void_p], C.c_int),
    "sde_batch_job_results": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "sde_batch_job_info": ([C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                            C.POINTER(C.c_int32), C.POINTER(C.c_uint64), C.POINTER(C.c_int32)], C.c_int),
    "sde_batch_job_destroy": ([C.c_void_p], C.c_int),
    "sde_kat_chacha8_u64": ([C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p], C.c_int),
    "sde_kat_sobol_points": ([C.c_int32, C.c_uint64, C.c_uint64, C.c_void_p], C.c_int),
    "sde_kat_icdf": ([C.c_void_p, C.c_uint64, C.c_void_p], C.c_int),
    "sde_sobol_directions": ([C.c_int32, C.c_void_p], C.c_int),
    "sde_probe_sfu_peak": ([C.POINTER(C.c_double)], C.c_int),
}

_lib = None


def lib():
    """Load libsdegpu.so; raises if it was not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"libsdegpu.so not found at {LIB_PATH}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(8192)
    lib().sde_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int) -> None:
    if rc != SDE_OK:
        msg = last_error()
        if rc in (SDE_ERR_PARSE, SDE_ERR_INVALID, SDE_ERR_RNG_INDEX):
            err = ValueError(msg)
            err.code = rc
            raise err
        raise SdeError(rc, msg)


def cstrs(strs):
    arr = (C.c_char_p * max(1, len(strs)))()
    for i, s in enumerate(strs):
        arr[i] = s.encode()
    return arr
