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


def _replica_worker(rank, world, port, out):
    """One replica of the path per rank (the oracle on the host: there is no
    GPU here), timed between barriers as bench.py times its ranks."""
    import time

    import numpy as np

    from oracle import ctm_oracle as orc
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        st = orc.random_state(2, 8, seed=100 + rank)
        cfg = dict(projectors="half-system", svd_type="rsvd", rsvd_oversampling=2, rsvd_niter=2,
                   svd_cutoff=1e-12)
        dist.barrier()
        t0 = time.perf_counter()
        orc.ctmrg(st, cfg, orc.OmegaStream(7 + rank), steps=2)
        dist.barrier()
        elapsed = time.perf_counter() - t0
        total_max, value = bench.aggregate(elapsed, 16, world)
        spec = np.linalg.svd(st[(0, 0)]["C"][0], compute_uv=False)
        ref_line = bench.run_reference(type("A", (), {"steps": 1, "warmup": 0, "gpus": world})(),
                                       rank) if rank else None
        out[rank] = (elapsed, total_max, value, spec.tolist(), ref_line)
    finally:
        dist.destroy_process_group()


def test_replicas_run_independent_paths():
    """Each rank's replica equals the same replica run alone (no exchange
    between ranks), the job time is the slowest rank's, the throughput
    counts every rank's moves, and the reference arm does no work on ranks
    other than 0."""
    import numpy as np

    from oracle import ctm_oracle as orc
    world = 2
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.spawn(_replica_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    slowest = max(out[r][0] for r in range(world))
    cfg = dict(projectors="half-system", svd_type="rsvd", rsvd_oversampling=2, rsvd_niter=2,
               svd_cutoff=1e-12)
    for rank in range(world):
        elapsed, total_max, value, spec, ref_line = out[rank]
        assert total_max == slowest
        assert abs(value - world * 16 / slowest) < 1e-9
        st = orc.random_state(2, 8, seed=100 + rank)
        orc.ctmrg(st, cfg, orc.OmegaStream(7 + rank), steps=2)
        alone = np.linalg.svd(st[(0, 0)]["C"][0], compute_uv=False)
        assert np.allclose(spec, alone, rtol=1e-12, atol=0)
        if rank:
            assert ref_line is None
