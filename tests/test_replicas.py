"""The benchmark's multi-process path on CPU: two `gloo` ranks (127.0.0.1) reduce their
per-step timings with bench.max_over_ranks, as the GPU ranks do over NCCL; every rank
gets the slowest replica's value of each timing."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, values, out):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    dist.barrier()
    out[rank] = bench.max_over_ranks(values[rank], dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    values = [[58.5, 160.0], [61.0, 157.0]]
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, _free_port(), values, out), nprocs=2, join=True)
        got = dict(out)
    assert got[0] == got[1] == [61.0, 160.0]


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([1, 2.5], None, "cpu") == [1.0, 2.5]
