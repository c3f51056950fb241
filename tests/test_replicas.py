"""The N-GPU path: replicas reported as (sum of work, max of time) over ranks,
checked with two gloo ranks on the CPU."""
import os
import socket

import pytest

from entropical_gb300.replicas import aggregate, shard


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units, ms = aggregate(100.0 * (rank + 1), 10.0 + rank, dist)
    out.put((rank, units, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 300.0, 11.0), (1, 300.0, 11.0)]


def test_single_process_identity():
    assert aggregate(5.0, 2.0) == (5.0, 2.0)


def test_shard_covers_everything_once():
    for n in (0, 1, 7, 2016):
        for w in (1, 2, 3, 8):
            parts = [list(shard(n, r, w)) for r in range(w)]
            flat = [i for p in parts for i in p]
            assert flat == list(range(n))
