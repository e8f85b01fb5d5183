"""bench.py's multi-GPU mode runs independent replicas: the timed region is
the max over ranks, the work the sum.  Checked with 2 gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, work = bench.aggregate(10.0 + 5.0 * rank, 1000 * (rank + 1))
    q.put((rank, ms, work))
    dist.destroy_process_group()


def test_replica_aggregation_gloo():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, work in res:
        assert ms == pytest.approx(15.0)
        assert work == pytest.approx(3000.0)


def test_single_process_aggregate_is_identity():
    import bench

    assert bench.aggregate(3.0, 7) == (3.0, 7)
