"""The N > 1 path of bench.py (independent replicas, one per rank): two gloo ranks on the CPU
agree on the max of their step times, which the job reports over the world size."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, times, out):
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.replica_time(times[rank], world, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_time_two_gloo_ranks():
    world = 2
    times = [0.0123, 0.0150]
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), times, out), nprocs=world, join=True)
        got = dict(out)
    assert got == {0: max(times), 1: max(times)}
    assert max(times) / world == pytest.approx(0.0075)


def test_replica_time_single_rank():
    import bench
    assert bench.replica_time(0.5, 1) == 0.5
