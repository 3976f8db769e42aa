"""Multi-process path of bench.py on CPU (gloo, world size 2): each rank is an
independent replica (the CTMRG path does not shard within one iPEPS on this
hardware), the job's time is the slowest rank's and the throughput counts the
moves of every rank."""

import os
import socket

import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, times, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        total_max, value = bench.aggregate(times[rank], 8, world)
        out[rank] = (total_max, value)
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_takes_slowest_rank():
    world = 2
    times = [2.0, 3.0]
    # a spawned manager: forking a process that already runs threads (torch,
    # the reference's import) can deadlock the child
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.spawn(_worker, args=(world, _free_port(), times, out), nprocs=world, join=True)
    for rank in range(world):
        total_max, value = out[rank]
        assert total_max == 3.0
        assert abs(value - world * 8 / 3.0) < 1e-12


def test_single_process_aggregation():
    total_max, value = bench.aggregate(4.0, 8, 1)
    assert total_max == 4.0 and value == 2.0
