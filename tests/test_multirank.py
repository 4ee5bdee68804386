"""The benchmark's multi-rank path (replicas, no data-path collective) on CPU with gloo, world size 2."""

import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    # each rank integrates its own batch (different seed) and times it
    w = bench.initial_vorticity(2, seed=bench.SEED + rank)
    ms = 100.0 + 50.0 * rank
    ms_max = bench.max_over_ranks(ms, dist)
    value = bench.job_throughput(2 * bench.N * bench.N * bench.TIME_STEPS, world, ms_max)
    out[rank] = (float(w.sum()), ms_max, value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_timing_is_the_max_and_inputs_differ():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    s0, m0, v0 = out[0]
    s1, m1, v1 = out[1]
    assert m0 == m1 == 150.0
    assert v0 == v1 == pytest.approx(world * 2 * 256 * 256 * 1000 / 0.150)
    assert s0 != s1  # replicas integrate different samples
