"""Replica sharding host logic with two gloo ranks on CPU: disjoint, complete
shards; distinct seeds; sharded processing equals unsharded processing (each
rank transforms its own images with the oracle, results gathered); the
timing reduction takes the slowest rank; no collective carries image data
except this test's own result check."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from glscv_gb300 import replicas


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist

    from oracle import oracle as orc
    from glscv_gb300 import workloads as wl
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n = 10
        mine = list(replicas.shard(n, rank, world))
        shards = [None] * world
        dist.all_gather_object(shards, mine)
        seeds = [None] * world
        dist.all_gather_object(seeds, replicas.seeds_for(rank, 3))
        # each rank transforms its own images (oracle on CPU, 16 x 16)
        outs = {i: orc.fft2d(wl.complex_uniform(16, 16, 500 + i), 0, 0) for i in mine}
        gathered = [None] * world
        dist.all_gather_object(gathered, {i: v.tobytes() for i, v in outs.items()})
        slowest = replicas.max_over_ranks(1.0 + rank, dist)
        q.put((rank, shards, seeds, gathered, slowest))
    finally:
        dist.destroy_process_group()


def test_shard_cover_and_balance():
    for n in (0, 1, 7, 64, 512):
        for world in (1, 2, 3, 8):
            parts = [replicas.shard(n, r, world) for r in range(world)]
            flat = [i for p in parts for i in p]
            assert flat == list(range(n))
            sizes = [len(p) for p in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def test_aggregate_and_single_rank():
    assert replicas.aggregate_rate(64, 4, 0.5) == 512
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.seeds_for(1, 3) == [1003, 1004, 1005]


def test_two_gloo_ranks_match_unsharded(oracle):
    import multiprocessing as mp
    from glscv_gb300 import workloads as wl
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    for rank, shards, seeds, gathered, slowest in res:
        assert shards == [[0, 1, 2, 3, 4], [5, 6, 7, 8, 9]]
        flat_seeds = [s for part in seeds for s in part]
        assert len(set(flat_seeds)) == len(flat_seeds)
        assert slowest == 2.0
        merged = {}
        for part in gathered:
            assert not (set(part) & set(merged))
            merged.update(part)
        assert sorted(merged) == list(range(10))
        for i, b in merged.items():
            ref = oracle.fft2d(wl.complex_uniform(16, 16, 500 + i), 0, 0)
            assert np.array_equal(np.frombuffer(b, dtype=np.complex64).reshape(16, 16), ref)
