"""The multi-GPU path of bench.py (weak-scaled replicas, one process per GPU)
on CPU: two gloo ranks with fake per-rank timings and replicate means."""
import math
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    means = np.arange(4, dtype=np.float64) + 10 * rank   # disjoint replicates
    ms, est, se, n = bench.combine_ranks(5.0 + rank, means, world)
    out.put((rank, ms, est, se, n))
    dist.destroy_process_group()


def test_combine_ranks_gloo_world2():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    allm = np.concatenate([np.arange(4) + 0.0, np.arange(4) + 10.0])
    for rank, ms, est, se, n in res:
        assert ms == 6.0                      # slowest rank
        assert n == 8 and est == pytest.approx(allm.mean())
        assert se == pytest.approx(allm.std(ddof=1) / math.sqrt(8))


def test_combine_ranks_single():
    import bench
    ms, est, se, n = bench.combine_ranks(3.0, [1.0, 2.0, 3.0], 1)
    assert (ms, est, n) == (3.0, 2.0, 3) and se == pytest.approx(1.0 / math.sqrt(3))
