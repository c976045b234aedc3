"""Replica timing and aggregation of bench.py across ranks (gloo, world size 2, CPU).

One problem never spans GPUs; N GPUs run N independent replicas.  Each rank
reports its own time, the job takes the slowest rank and counts every rank's
applications, and only rank 0 prints.  These tests run that host logic over a
real two-process gloo group."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist          # noqa: E402
import torch.multiprocessing as mp        # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        r, w, local = bench.dist_env()
        # per-rank seconds differ; every rank must see the slowest one
        t_max = bench.reduce_max(1.0 + rank, w)
        value = bench.replicas_value(100, w, t_max)
        out[rank] = (r, w, local, t_max, value)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replicas_max_over_ranks():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for rank, (r, w, local, t_max, value) in res.items():
        assert (r, w, local) == (rank, world, rank)
        assert t_max == 2.0                        # the slowest rank's time on every rank
        assert value == pytest.approx(100 * world / 2.0)   # all ranks' units / slowest time


def test_single_rank_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(3.5, 1) == 3.5
    assert bench.replicas_value(10, 1, 2.0) == 5.0
