"""Multi-GPU form on CPU: two gloo ranks exercise the replica aggregation
bench.py uses at N > 1 (max of per-rank step times, sums of counts) and the
round-robin sharding of independent scenarios. No GPU, no data-path
collective."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        mine = bench.shard(10, rank, world)
        got = bench.reduce_over_ranks(
            dist, {"ms": 3.0 + rank, "cells": 100.0 * (rank + 1), "n": len(mine), "lo": 7.0 - rank},
            {"ms": "max", "cells": "sum", "n": "sum", "lo": "min"})
        q.put((rank, mine, got))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_and_sharding_on_two_gloo_ranks():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q))
             for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    shards = [r[1] for r in res]
    assert sorted(shards[0] + shards[1]) == list(range(10))
    assert not set(shards[0]) & set(shards[1])
    for _, _, got in res:
        assert got == {"ms": 4.0, "cells": 300.0, "n": 10.0, "lo": 6.0}


def test_single_process_is_identity():
    import bench
    assert bench.reduce_over_ranks(None, {"a": 2.0}, {"a": "max"}) == {"a": 2.0}
    assert bench.shard(5, 0, 1) == [0, 1, 2, 3, 4]

