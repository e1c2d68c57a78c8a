"""Host-side sharding of batched systems over ranks (CPU, gloo world_size 2)."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from sptrsv_gb300 import shard


def test_assign_covers_every_system_once_and_balances():
    rng = np.random.default_rng(0)
    w = rng.integers(1_000, 4_000_000, size=512)
    for world in (1, 2, 3, 4, 8):
        owned = shard.assign(w, world)
        flat = sorted(i for o in owned for i in o)
        assert flat == list(range(w.size))
        ld = shard.loads(w, world)
        assert max(ld) <= w.sum() / world + w.max()
        assert owned == shard.assign(w, world)          # deterministic
        for r in range(world):
            assert shard.shard_of(w, world, r) == owned[r]


def test_assign_edge_cases():
    assert shard.assign([], 2) == [[], []]
    assert shard.assign([5], 3) == [[0], [], []]
    assert shard.assign([1, 1, 1, 1], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        shard.assign([1, 2], 0)
    with pytest.raises(ValueError):
        shard.assign([1, -2], 2)
    with pytest.raises(ValueError):
        shard.shard_of([1, 2], 2, 2)


def test_rhs_columns_partition():
    for rhs in (0, 1, 7, 16, 64):
        for world in (1, 2, 3, 4, 8):
            cols = [shard.rhs_columns(rhs, world, r) for r in range(world)]
            assert cols[0][0] == 0 and cols[-1][1] == rhs
            assert all(cols[r][1] == cols[r + 1][0] for r in range(world - 1))
            widths = [b - a for a, b in cols]
            assert max(widths) - min(widths) <= 1
    with pytest.raises(ValueError):
        shard.rhs_columns(4, 2, 2)
    with pytest.raises(ValueError):
        shard.rhs_columns(-1, 2, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, weights, result_q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard.shard_of(weights, world, rank)
        # stand-in per-system result: the system index repeated over its size
        local = {k: np.full(3 + k % 5, float(k)) for k in mine}
        sol = shard.gather_solutions(local, len(weights))
        ok = all(np.all(v == k) and v.size == 3 + k % 5 for k, v in enumerate(sol))
        # a rank that claims a system twice is caught on every rank
        dup_err = False
        try:
            shard.gather_solutions({0: np.zeros(1)}, len(weights))
        except RuntimeError:
            dup_err = True
        # right-hand-side columns: every rank solves its slice of B with the
        # oracle (stand-in for the device solve) and the slices join to L^-1 B
        from oracle import oracle
        from sptrsv_gb300 import matgen
        m = matgen.poisson_band(200, 4.0, 50, seed=3)
        B = np.random.default_rng(4).standard_normal((m.n, 7))
        a, b = shard.rhs_columns(7, world, rank)
        blk = oracle.port().solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution,
                                  np.ascontiguousarray(B[:, a:b])).reshape(m.n, b - a)
        X = shard.gather_columns(blk, 7)
        full = oracle.port().solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, B).reshape(m.n, 7)
        cols_ok = bool(np.array_equal(X, full))
        result_q.put((rank, ok and cols_ok, len(mine), dup_err))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_gather():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    weights = list(np.random.default_rng(1).integers(10, 1000, size=37))
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, weights, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert all(ok for _, ok, _, _ in res)
    assert sum(c for _, _, c, _ in res) == 37
    assert all(dup for *_, dup in res)
