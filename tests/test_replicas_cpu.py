"""bench.py --gpus N runs N independent replicas of the contraction (the path
is not split across GPUs); the step time is the maximum over ranks. The
reduction is exercised here with world_size 2 over gloo on the CPU."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from conftest import ROOT  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys

    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    assert bench.dist_env() == (world, rank, 0)
    got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.25 * rank])
    out[rank] = got
    dist.barrier()
    dist.destroy_process_group()


def test_step_time_is_the_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
        assert out[0] == out[1] == [2.0, 10.0, 0.25]
