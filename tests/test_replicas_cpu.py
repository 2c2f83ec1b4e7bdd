"""The multi-GPU contract of bench.py on CPU: a grid does not shard, so N ranks
run N independent replicas; the job's time is the slowest rank's (max over
ranks, one all-reduce of the timing only, no data-path collective) and the
value counts every rank's cell-steps.  Two gloo ranks on 127.0.0.1; the
reference arm does its work on rank 0 only."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms_local = [40.0, 55.0][rank]
    ms, value = bench.replicas_value(ms_local, world, cells=1000, steps=10, dist=dist, device="cpu")
    # the reference arm: ranks other than 0 leave without work
    assert bench.dist_env() == (rank, world, rank)
    if rank != 0:
        assert bench.run_reference(None) is None
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank(tmp_path):
    world = 2
    port = _free_port()
    out = mp.get_context("spawn").Manager().dict()   # no fork of this (threaded) process
    mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    for r in range(world):
        ms, value = out[r]
        assert ms == 55.0
        assert value == pytest.approx(world * 1000 * 10 / (55.0e-3) / 1e9)


def test_single_rank_needs_no_process_group():
    import bench
    ms, value = bench.replicas_value(20.0, 1, cells=500, steps=4)
    assert ms == 20.0 and value == pytest.approx(500 * 4 / 20e-3 / 1e9)
