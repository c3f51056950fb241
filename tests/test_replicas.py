"""The N-GPU path, checked with two gloo ranks on the CPU: the report as (sum
of work, max of time) over ranks, and one all-pairs MI split over ranks (a
stand-in entropy function in place of the GPU batch) giving the same matrix
as one rank."""
import os
import socket

import pytest

import numpy as np

from entropical_gb300.replicas import aggregate, mi_all_pairs_sharded, mi_instances, shard


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


def _fake_entropies(batch):
    # any deterministic function of each instance stands in for the GPU batch
    return [float(np.sum(x.astype(np.float64) ** 2) * float(np.prod(h))) + x.shape[0]
            for x, h in batch]


def _mi_worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    x = np.random.default_rng(4).standard_normal((6, 50)).astype(np.float32)
    h = [0.3, 0.4, 0.5, 0.6, 0.7, 0.8]
    mi, hx = mi_all_pairs_sharded(_fake_entropies, x, h, dist)
    out.put((rank, mi.tolist(), hx.tolist()))
    dist.barrier()
    dist.destroy_process_group()


def test_mi_split_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_mi_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    x = np.random.default_rng(4).standard_normal((6, 50)).astype(np.float32)
    h = [0.3, 0.4, 0.5, 0.6, 0.7, 0.8]
    mi1, hx1 = mi_all_pairs_sharded(_fake_entropies, x, h)
    for _, mi, hx in res:
        assert np.array_equal(np.array(mi), mi1) and np.array_equal(np.array(hx), hx1)
    assert len(mi_instances(64)) == 64 + 2016
