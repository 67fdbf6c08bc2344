"""Multi-process sharding on CPU (gloo, world size 2): each rank runs its cost-
balanced range of a batch through the oracle (standing in for its GPU) and
rank 0 gathers the outputs in pair order; the result equals the unsharded run.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from ncollide_gb300 import shard as S
from ncollide_gb300 import workloads as W


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b = W.mixed_convex(4096, seed=51)
        mine, rng = S.shard(b, world, rank)
        r = O.query(mine, O.CONTACT, O.F32, param=0.0, threads=1)
        out = S.gather({"tag": r.tag, "value": r.value, "dir": r.dir}, rng, b.n_pairs)
        if rank == 0:
            q.put(out)
    finally:
        dist.destroy_process_group()


def test_shard_ranges_cover_and_balance():
    b = W.mixed_convex(1 << 15, seed=50)
    c = S.pair_cost(b)
    for world in (1, 2, 3, 8):
        rs = S.shard_ranges(c, world)
        assert rs[0][0] == 0 and rs[-1][1] == b.n_pairs
        assert all(rs[i][1] == rs[i + 1][0] for i in range(world - 1))
        loads = np.array([c[a:z].sum() for a, z in rs])
        assert loads.max() <= 1.05 * loads.mean() + c.max()


def test_two_rank_gloo_gather_matches_single_process():
    from oracle import oracle as O
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    b = W.mixed_convex(4096, seed=51)
    want = O.query(b, O.CONTACT, O.F32, param=0.0, threads=1)
    assert np.array_equal(got["tag"], want.tag)
    assert np.array_equal(got["value"], want.value)
    assert np.array_equal(got["dir"], want.dir)
