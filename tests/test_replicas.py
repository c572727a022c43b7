"""Replica bookkeeping over torch.distributed with two gloo ranks on the CPU:
view partitioning, max over ranks, whole-job throughput."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from taichi_three_gb300 import replicas


def test_partition_views_covers_all():
    for n in (0, 1, 5, 64, 65):
        for k in (1, 2, 3, 8):
            parts = [replicas.partition_views(n, k, r) for r in range(k)]
            flat = [v for p in parts for v in p]
            assert flat == list(range(n))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1


def _worker(rank, port, q):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=2)
    try:
        views = replicas.partition_views(7, 2, rank)
        t = 1.0 + rank  # rank 1 is the slowest
        q.put((rank, views, replicas.max_over_ranks(t), replicas.aggregate_rate(len(views), t),
               replicas.world()))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def test_two_gloo_ranks():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict()
    for _ in range(2):
        rank, views, tmax, rate, w = q.get(timeout=120)
        out[rank] = (views, tmax, rate, w)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][0] + out[1][0] == list(range(7))
    assert out[0][1] == out[1][1] == 2.0
    assert out[0][2] == out[1][2] == pytest.approx(7 / 2.0)
    assert out[0][3] == (2, 0) and out[1][3] == (2, 1)


def test_single_process_defaults():
    assert replicas.world() == (1, 0)
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.aggregate_rate(10, 2.0) == 5.0
