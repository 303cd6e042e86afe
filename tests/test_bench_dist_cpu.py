"""The benchmark's multi-rank reduction on two CPU ranks (gloo): every rank gets the largest time of
any rank, and a single process keeps its own."""
import os
import socket
import sys

import torch.distributed as dist
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, REPO)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.max_over_ranks(1.5 + 2.0 * rank, dist, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        assert dict(out) == {0: 3.5, 1: 3.5}


def test_single_process_keeps_its_value():
    sys.path.insert(0, REPO)
    import bench

    assert bench.max_over_ranks(2.25, None, "cpu") == 2.25
