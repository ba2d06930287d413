"""Replica path of bench.py on CPU: two gloo ranks (no GPU), the job time is
the slowest replica's and the throughput sums the replicas' work."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 1.0 + rank  # rank 1 is the slow replica
    out[rank] = bench.max_over_ranks(ms, world, device="cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_time():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    assert dict(out) == {0: 2.0, 1: 2.0}


def test_replica_throughput_sums_work_over_the_slowest_time():
    # 2 replicas x 1 GB per step in 2 ms (slowest) -> 1000 GB/s for the job
    assert bench.replica_throughput(1e9, 2.0, 2) == pytest.approx(1000.0)
    assert bench.max_over_ranks(3.5, 1) == 3.5
