"""Replica runs of bench.py (one process per GPU, no data-path collective): the
step time every rank reports is the slowest rank's, and the job value counts
every rank's units.  Two gloo ranks on CPU."""

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


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    dist.barrier()
    ms = bench.max_over_ranks(1.0 + rank, world)  # rank 1 is the slower
    out[rank] = ms
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world = 2
    out = mp.get_context("spawn").Manager().dict()  # no fork: the test process may hold a CUDA context
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    assert dict(out) == {0: 2.0, 1: 2.0}


def test_replica_value_counts_every_rank():
    import bench

    assert bench.replica_value(1e9, 2.0, 1) == pytest.approx(5e11)
    assert bench.replica_value(1e9, 2.0, 4) == pytest.approx(2e12)
    assert bench.max_over_ranks(3.5, 1) == 3.5
