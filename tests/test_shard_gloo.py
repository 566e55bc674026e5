"""Sharded execution over 2 ranks (gloo, CPU): the multi-GPU logic without GPUs.

Each rank takes its balanced list range, computes with the C oracle what its
GPU would compute (sum / argmax reductions and combinations offsets + carry),
rebases offsets and indices, and rank 0 checks that the concatenated shards
equal the single-process result bit for bit.  Rendezvous on 127.0.0.1.
"""

import os
import socket

import numpy as np
import pytest

import oracle
from awkward_gb300 import shard


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _data():
    rng = np.random.default_rng(21)
    L = np.minimum(rng.poisson(6, 20_000), 40)
    L[rng.random(len(L)) < 0.02] = 0
    L[123] = 3000
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    x = rng.standard_normal(int(off[-1]))
    return off, x


def _compute(off, x):
    lib = oracle.load()
    n = len(off) - 1
    s = np.zeros(n)
    oracle.call(lib, "awkward_reduce_sum_float64_float64_64", toptr=s, fromptr=x, offsets=off,
                outlength=n)
    a = np.zeros(n, np.int64)
    oracle.call(lib, "awkward_reduce_argmax_float64_64", toptr=a, fromptr=x, offsets=off,
                starts=off[:-1].copy(), outlength=n)
    tot = np.zeros(1, np.int64)
    too = np.zeros(n + 1, np.int64)
    oracle.call(lib, "awkward_ListArray64_combinations_length_64", totallen=tot, tooffsets=too,
                n=2, replacement=False, starts=off[:-1].copy(), stops=off[1:].copy(), length=n)
    rows = [np.zeros(max(int(tot[0]), 1), np.int64) for _ in range(2)]
    oracle.call(lib, "awkward_ListArray64_combinations_64", tocarry=rows,
                toindex=np.zeros(2, np.int64), fromindex=np.zeros(2, np.int64), n=2,
                replacement=False, starts=off[:-1].copy(), stops=off[1:].copy(), length=n)
    return s, a, too, [r[: int(tot[0])] for r in rows]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        off, x = _data()
        loff, lx, l0, e0 = shard.local_shard(off, x, rank, world)
        s, a, too, rows = _compute(loff, lx)
        a = np.where(a >= 0, a + e0, a)  # global element indices
        too = shard.rebase_offsets(too)
        rows = [r + e0 for r in rows]
        q.put((rank, l0, s, a, too, rows))
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_equal_single_process():
    import multiprocessing as mp

    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in range(world)], key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    off, x = _data()
    s, a, too, rows = _compute(off, x)
    np.testing.assert_array_equal(np.concatenate([r[2] for r in res]), s)
    np.testing.assert_array_equal(np.concatenate([r[3] for r in res]), a)
    glued = np.concatenate([res[0][4][:-1], res[1][4]])
    np.testing.assert_array_equal(glued, too)
    for k in range(2):
        np.testing.assert_array_equal(np.concatenate([r[5][k] for r in res]), rows[k])


def test_shard_bounds_balance_and_cover():
    off, _x = _data()
    for world in (1, 2, 3, 8):
        b = shard.shard_bounds(off, world)
        assert b[0] == 0 and b[-1] == len(off) - 1 and np.all(np.diff(b) >= 0)
        items = np.diff(b) + np.diff(off[b])
        assert items.max() - items.min() <= 3000 + 2  # within one (giant) list
    with pytest.raises(IndexError):
        shard.local_shard(off, _x, 2, 2)
