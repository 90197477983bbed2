"""The N > 1 path of bench.py: independent replicas, one per rank, no data-path collective; the
slowest rank's time and the whole job's throughput come from one max-reduction.  Run as two gloo
ranks on the CPU (the same reduction bench.py makes over NCCL)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [10.0, 12.5][rank]  # each replica's own timed region
        got = bench.replica_throughput(ms, faces=1000, steps=4, world=world, dist=dist,
                                       device="cpu")
        out[rank] = got
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_summed_work():
    world, port = 2, _free_port()
    out = mp.get_context("spawn").Manager().dict()  # no fork of this multi-threaded process
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        ms, value = out[r]
        assert ms == 12.5  # max over ranks
        assert value == pytest.approx(world * 1000 * 4 / 12.5e-3 / 1e9)


def test_single_replica_needs_no_process_group():
    ms, value = bench.replica_throughput(8.0, faces=500, steps=2, world=1, dist=None,
                                         device="cpu")
    assert ms == 8.0 and value == pytest.approx(500 * 2 / 8e-3 / 1e9)
