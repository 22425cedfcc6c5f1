"""Replica (N > 1) host logic of bench.py on CPU: two gloo ranks, max-over-ranks timing."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        ms = bench.max_over_ranks(1.0 + rank, torch.device("cpu"))  # rank 1 is the slow one
        value = bench.replica_throughput(world, 1.0e9, ms)
        out[rank] = (ms, value)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_max_and_weak_scaling_value():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1]
    ms, value = out[0]
    assert ms == pytest.approx(2.0)
    assert value == pytest.approx(2 * 1.0e9 / 2.0e-3 / 1e9)
