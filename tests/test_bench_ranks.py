"""The N > 1 host path of bench.py on CPU: two gloo ranks reduce their
replica figures to the slowest time and the summed collisions and parcels."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    out = bench.reduce_ranks(10.0 + rank, 1000 * (rank + 1), 500 + rank, dist, "cpu")
    q.put((rank, out))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_time_and_totals():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert res[r] == (11.0, 3000.0, 1001.0)


def test_single_rank_passes_through():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_ranks(3.5, 7, 11, None, "cpu") == (3.5, 7.0, 11.0)
