"""The multi-GPU path of bench.py is replicas only (one independent Louvain run
per GPU, no data-path collective): its timing is the slowest rank's and its
throughput the sum over replicas.  The reduction runs here on two gloo ranks
on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
    slowest = bench.max_over_ranks(dist, torch, ms, "cpu")
    dist.barrier()
    out[rank] = (slowest, bench.replica_throughput(world, 1000, slowest))
    dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    mgr = torch.multiprocessing.get_context("spawn").Manager()
    out = mgr.dict()
    torch.multiprocessing.start_processes(_rank, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    assert out[0] == out[1]
    slowest, value = out[0]
    assert slowest == 15.0
    assert value == 2 * 1000 / 0.015
