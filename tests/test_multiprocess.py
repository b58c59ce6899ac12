"""The replicas path of bench.py with world_size 2 on CPU (gloo).

Every rank runs the whole workload on its own device and the job reports
all ranks' work over the slowest rank's time; nothing but the timings is
exchanged. Here each rank times the oracle on its own inputs and the ranks
agree on the max and on the aggregate value.
"""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import numpy as np

        import bench
        import oracle

        rng = np.random.default_rng(rank)
        x = (rng.standard_normal((64, 1000)) + 1j * rng.standard_normal((64, 1000))).astype(np.complex64)
        _, secs = oracle.cfft1d(x, "forward", nthreads=1, timing=True)
        local = [secs + 0.01 * rank, 1.0 + rank]
        reduced = bench.reduce_max(local, world)
        out[rank] = (local, reduced, bench.aggregate_value(world, reduced[0]))
    finally:
        dist.destroy_process_group()


def test_replicas_reduce_max_gloo():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    (l0, r0, v0), (l1, r1, v1) = out[0], out[1]
    assert r0 == r1 == [max(l0[0], l1[0]), max(l0[1], l1[1])]
    assert v0 == pytest.approx(v1)
    import bench

    assert v0 == pytest.approx(2 * bench.TOTAL_FLOPS / r0[0] / 1e9)
