"""Multi-rank host logic on CPU (gloo, world size 2): the job time is the
maximum over ranks, the work the sum of the replicas."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from tiledarray_gb300.replicas import aggregate
    ms, fl, ws = aggregate(10.0 + rank * 5.0, 1e12 * (rank + 1), dist)
    q.put((rank, ms, fl, ws))
    dist.destroy_process_group()


def test_aggregate_gloo_two_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(2))
    for rank, ms, fl, ws in res:
        assert ws == 2 and ms == 15.0 and fl == 3e12


def test_aggregate_single_process():
    from tiledarray_gb300.replicas import aggregate
    assert aggregate(3.0, 7.0) == (3.0, 7.0, 1)
