"""The replica path of bench.py on CPU: two gloo ranks, the job time is the slowest
rank's, and the whole-job throughput is the per-replica throughput times the ranks."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(1.0 + rank, "cpu")     # rank 1 is the slow one
        value = bench.replica_value(1000.0 / ms, world)
        out[rank] = (ms, value)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    with mp.get_context("spawn").Manager() as man:  # no fork of a threaded process
        out = man.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (2.0, 1000.0)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, "cpu") == 3.5
    assert bench.replica_value(10.0, 1) == 10.0
