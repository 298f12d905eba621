"""Replica sharding on CPU ranks (gloo, world size 2): balanced shards, film
row-slab gather and gradient sum on the host."""
import os
import socket

import numpy as np
import pytest

from woodenpbrengine_gb300 import replicas


def test_shard_covers_every_unit_once():
    for n in (0, 1, 7, 1080, 1081):
        for world in (1, 2, 3, 8):
            ranges = [replicas.shard(n, world, r) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            for (a, b), (c, d) in zip(ranges, ranges[1:]):
                assert b == c
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)


def test_shard_scenes_balances_cost():
    costs = [5.0, 1.0, 1.0, 1.0, 1.0, 1.0]
    parts = replicas.shard_scenes(costs, 2)
    assert sorted(sum(parts, [])) == list(range(6))
    assert parts == [[0], [1, 2, 3, 4, 5]]


def _film(rows, W):
    y = np.arange(rows[0], rows[1], dtype=np.float32)[:, None, None]
    x = np.arange(W, dtype=np.float32)[None, :, None]
    return (y * 1000 + x + np.array([0.25, 0.5, 0.75], np.float32)).astype(np.float32)


def _worker(rank, world, port, H, W, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rows = replicas.shard(H, world, rank)
        full = replicas.gather_rows(_film(rows, W), H, dist)
        g = np.full(5, rank + 1, np.float32)
        s = replicas.allreduce_sum(g, dist)
        q.put((rank, None if full is None else full.tobytes(), s.tolist()))
    finally:
        dist.destroy_process_group()


def test_gather_and_reduce_on_two_gloo_ranks():
    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    H, W, world = 37, 5, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, H, W, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res = {r: (f, s) for r, f, s in out}
    full = np.frombuffer(res[0][0], np.float32).reshape(H, W, 3)
    assert np.array_equal(full, _film((0, H), W))
    assert res[1][0] is None
    assert res[0][1] == res[1][1] == [3.0] * 5
