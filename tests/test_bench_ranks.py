"""The bench's whole-job figures over N replicas (one rank per GPU): successors summed over the
ranks, times the max over them -- checked with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    gen, dev, wall, total = 1000.0 * (rank + 1), 0.5 + rank, 0.7 + rank, 1.0 + 2 * rank
    out[rank] = bench.combine_ranks(gen, dev, wall, total, dist, "cpu")
    dist.destroy_process_group()


def test_combine_ranks_two_gloo_ranks():
    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        assert out[r] == (3000.0, 1.5, 1.7, 3.0)


def test_combine_ranks_single_process():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.combine_ranks(5.0, 1.0, 2.0, 3.0, None, "cpu") == (5.0, 1.0, 2.0, 3.0)
