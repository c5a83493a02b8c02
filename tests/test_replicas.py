"""Multi-process host logic of bench.py on CPU (gloo, world size 2): every
rank runs its own replica and only the step time is reduced (max over
ranks); rank 0 alone prints."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w = bench.dist_env()
    v = bench.max_over_ranks(10.0 + rank, w)
    out.put((r, w, v))
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    tmp.start_processes(_worker, args=(2, port, q), nprocs=2, join=True, start_method="spawn")
    got = sorted(q.get(timeout=60) for _ in range(2))
    assert got == [(0, 2, 11.0), (1, 2, 11.0)]


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
