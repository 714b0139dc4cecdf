"""The multi-GPU path of bench.py is replicas only: every rank runs its own grid and the ranks meet
only for a barrier and the max-over-ranks time. This checks that path with two gloo ranks on CPU:
the slowest rank's time sets the job time and the value counts every rank's cells."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        ms = 100.0 if rank == 0 else 250.0        # the second replica is slower
        worst = bench.max_over_ranks(ms, world)
        out[rank] = (worst, bench.replica_value(1_000_000, 10, worst, world))
        bench.barrier(world)
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    assert out[0][0] == out[1][0] == 250.0
    # 2 replicas x 1e6 cells x 10 steps in 0.25 s
    assert out[0][1] == pytest.approx(2 * 1e6 * 10 / 0.25 / 1e9)
