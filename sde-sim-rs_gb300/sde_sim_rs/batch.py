"""Many independent SDE instances in one persistent, graph-captured launch.

The reference simulates one process universe per call
(src/sim/mod.rs:20-92).  ``Batch`` takes a few plans as templates
(e.g. one GBM and one Ornstein-Uhlenbeck universe written with named
parameters) and runs thousands of instances of them -- each with its own
uniform step count, horizon, path count, seed, initial values and parameter
values -- as one work-queue kernel.  ``prepare`` picks the block shape and
paths per thread by timing the candidates on the actual instances, then
captures the launch in a CUDA graph; ``BatchJob.run`` replays it.
Adjoint plans (``Plan(..., grad_params=..., grad_x0=...)``) are templates
too: their instances also return the gradients of payoff 0 (at most 4096
steps each).
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import Plan
from . import _native as N


def _lib():
    return N.lib()


def _stream(stream):
    if stream is None:
        return None
    return stream if isinstance(stream, int) else int(stream.cuda_stream)


class BatchJob:
    def __init__(self, handle, batch: "Batch", n_instances: int):
        self._h = handle
        self._batch = batch
        self.n_instances = n_instances
        b, p, ni, K = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        ps = C.c_uint64()
        N.check(_lib().sde_batch_job_info(self._h, C.byref(b), C.byref(p), C.byref(ni), C.byref(ps),
                                          C.byref(K)))
        self.block, self.paths_per_thread, self.n_items = b.value, p.value, ni.value
        self.path_steps, self.n_payoffs = ps.value, K.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and N._lib is not None:
            N._lib.sde_batch_job_destroy(h)
            self._h = C.c_void_p()

    def run(self, stream=None) -> "BatchJob":
        N.check(_lib().sde_batch_job_run(self._h, _stream(stream)))
        return self

    def results(self):
        """(sum, sumsq) arrays [instances, payoffs] over each instance's paths."""
        s = np.zeros((self.n_instances, self.n_payoffs), dtype=np.float64)
        q = np.zeros_like(s)
        N.check(_lib().sde_batch_job_results(self._h, s.ctypes.data, q.ctypes.data))
        return s, q


class Batch:
    def __init__(self, templates: Sequence[Plan]):
        self.templates = list(templates)
        arr = (C.c_void_p * len(self.templates))(*[t._h.value for t in self.templates])
        h = C.c_void_p()
        N.check(_lib().sde_batch_create(arr, len(self.templates), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and N._lib is not None:
            N._lib.sde_batch_destroy(h)
            self._h = C.c_void_p()

    # the candidate (block, paths per thread) shapes, in the engine's order
    SHAPES = ((128, 1), (256, 1), (128, 2), (256, 2), (128, 4))

    def prepare(self, template_id, n_steps, t_end, n_paths, seed, x0, params, *, autotune: bool = True,
                shape: int | None = None, stream=None) -> BatchJob:
        """x0: [n, x0_stride] initial values by process index of the
        instance's template; params: [n, param_stride] by parameter index.
        shape (an index into SHAPES) fixes the launch shape instead of
        timing the candidates."""
        tid = np.ascontiguousarray(template_id, dtype=np.int32)
        n = len(tid)
        steps = np.ascontiguousarray(np.broadcast_to(n_steps, (n,)), dtype=np.int32)
        tend = np.ascontiguousarray(np.broadcast_to(t_end, (n,)), dtype=np.float64)
        npaths = np.ascontiguousarray(np.broadcast_to(n_paths, (n,)), dtype=np.uint64)
        seeds = np.ascontiguousarray(np.broadcast_to(seed, (n,)), dtype=np.uint64)
        x0a = np.ascontiguousarray(np.asarray(x0, dtype=np.float64).reshape(n, -1))
        pa = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(n, -1))
        ins = N.BatchInstances()
        ins.struct_size = C.sizeof(N.BatchInstances)
        ins.n_instances = n
        ins.template_id, ins.n_steps, ins.t_end = tid.ctypes.data, steps.ctypes.data, tend.ctypes.data
        ins.n_paths, ins.seed = npaths.ctypes.data, seeds.ctypes.data
        ins.x0, ins.x0_stride = x0a.ctypes.data, x0a.shape[1]
        ins.params, ins.param_stride = pa.ctypes.data, pa.shape[1]
        h = C.c_void_p()
        mode = -1 - int(shape) if shape is not None else (1 if autotune else 0)
        N.check(_lib().sde_batch_prepare(self._h, C.byref(ins), mode, _stream(stream), C.byref(h)))
        return BatchJob(h, self, n)
