"""The N-GPU path, checked with two gloo ranks on the CPU: the report as (sum
of work, max of time) over ranks, and one all-pairs MI split over ranks (a
stand-in entropy function in place of the GPU batch) giving the same matrix
as one rank."""
import os
import socket

import pytest

import numpy as np

from entropical_gb300.replicas import (WEIGHTS, aggregate, deal, densities_split, mi_assemble,
                                       mi_instances, shard, split_entropies, te_assemble,
                                       te_instances)


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


def _fake_entropies(items):
    # any deterministic function of each item stands in for the GPU batch
    return [np.sin(1.0 + float(i)) * 3.0 + 0.01 * float(i) for i in items]


def _split_worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = [WEIGHTS[len(c)] for c in mi_instances(6)]
    H = split_entropies(_fake_entropies, w, dist)
    mi, hx = mi_assemble(6, H)
    wt = [WEIGHTS[{1: 1, 2: 2, 3: 2, 4: 3}[k]] for _, k, _, _ in te_instances(4, 2)]
    te = te_assemble(4, 2, split_entropies(_fake_entropies, wt, dist))
    out.put((rank, mi.tolist(), hx.tolist(), te.tolist()))
    dist.barrier()
    dist.destroy_process_group()


def test_split_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_split_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    w = [WEIGHTS[len(c)] for c in mi_instances(6)]
    mi1, hx1 = mi_assemble(6, split_entropies(_fake_entropies, w))
    wt = [WEIGHTS[{1: 1, 2: 2, 3: 2, 4: 3}[k]] for _, k, _, _ in te_instances(4, 2)]
    te1 = te_assemble(4, 2, split_entropies(_fake_entropies, wt))
    for _, mi, hx, te in res:
        assert np.array_equal(np.array(mi), mi1) and np.array_equal(np.array(hx), hx1)
        assert np.array_equal(np.array(te), te1)
    assert len(mi_instances(64)) == 64 + 2016


def test_deal_covers_everything_once_and_balances():
    inst = mi_instances(64)
    w = [WEIGHTS[len(c)] for c in inst]
    for world in (1, 2, 3, 8):
        shares = deal(w, world)
        flat = sorted(int(i) for s in shares for i in s)
        assert flat == list(range(len(inst)))
        loads = [sum(w[int(i)] for i in s) for s in shares]
        assert max(loads) - min(loads) <= max(w)
        # the cheap marginals do not all land on one rank
        if world > 1:
            assert all(any(int(i) < 64 for i in s) for s in shares[:2]) or world > 64


def test_te_assemble_formula():
    M, T = 3, 2
    inst = te_instances(M, T)
    H = np.arange(len(inst), dtype=np.float64) * 0.5 + 1.0
    te = te_assemble(M, T, H)
    idx = {v: k for k, v in enumerate(inst)}
    for q in range(T):
        for i in range(M):
            for j in range(M):
                if i == j:
                    assert te[q, i, j] == 0
                    continue
                a, b = min(i, j), max(i, j)
                ref = (H[idx[(q, 3, a, b)]] + H[idx[(q, 2, i, i)]] - H[idx[(q, 4, i, j)]]
                       - H[idx[(q, 1, i, i)]])
                assert te[q, i, j] == ref


class _FakeShareContext:
    """Stands in for the GPU call: writes share `part` of a fixed density
    vector through the pointer it is given (host memory here)."""
    def __init__(self, p):
        self.p = p

    def combined_densities_part_device(self, d_coords, n_rows, n_cols, i_cols, h, tau, part,
                                       n_parts, d_out):
        import ctypes as C
        n = len(self.p)
        lo, hi = n * part // n_parts, n * (part + 1) // n_parts
        out = np.ctypeslib.as_array((C.c_double * n).from_address(d_out))
        out[lo:hi] = self.p[lo:hi]
        return n, float(np.sum(np.log(self.p[lo:hi])))


def _dens_worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    p = np.random.default_rng(6).uniform(0.1, 2.0, 1001)
    dens, H = densities_split(_FakeShareContext(p), 0, 1001, 1, [0], [0.3], None, dist,
                              device="cpu")
    out.put((rank, dens.tolist(), H))
    dist.barrier()
    dist.destroy_process_group()


def test_density_split_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_dens_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = np.random.default_rng(6).uniform(0.1, 2.0, 1001)
    for _, dens, H in res:
        assert np.array_equal(np.array(dens), ref)
        assert abs(H - (-np.mean(np.log(ref)))) < 1e-12
