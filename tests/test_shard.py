"""Replicas-only sharding across ranks, exercised with two gloo processes on CPU."""

import os
import socket

import numpy as np
import pytest

from braincell_gb300.shard import balanced_shards, shard_range


def test_shard_range_partitions():
    for n in (0, 1, 7, 10000):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = shard_range(n, r, world)
                seen.extend(range(lo, hi))
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def test_balanced_shards_cover_and_balance():
    w = np.random.default_rng(0).lognormal(size=1000)
    g = balanced_shards(w, 4)
    allidx = np.sort(np.concatenate(g))
    assert np.array_equal(allidx, np.arange(1000))
    loads = [w[x].sum() for x in g]
    assert max(loads) / min(loads) < 1.01


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from braincell_gb300 import workloads as W
        from braincell_gb300.shard import gather_objects, reduce_max, shard_range

        lo, hi = shard_range(40, rank, world)
        descs = W.uneven(indices=range(lo, hi))
        b = W.descs_to_batch(descs)
        local = {"rank": rank, "cells": list(range(lo, hi)), "ncv": int(b.n_cv)}
        t = reduce_max(1.0 + rank)
        got = gather_objects(local)
        q.put((rank, t, got))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_sharding():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, tmax, got in res:
        assert tmax == 2.0
        cells = sorted(c for g in got for c in g["cells"])
        assert cells == list(range(40))
        from braincell_gb300 import workloads as W

        total = W.descs_to_batch(W.uneven(indices=range(40))).n_cv
        assert sum(g["ncv"] for g in got) == total
