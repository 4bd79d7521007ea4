"""Replica sharding of independent solves (host logic; gloo ranks on CPU)."""
import os
import socket

import numpy as np
import pytest

from cppe_gb300 import shard


def _systems(k=7, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(k):
        n = 3 * (2 + i)
        a = rng.normal(size=(n, n))
        out.append((a @ a.T + n * np.eye(n), rng.normal(size=n)))
    return out


def _solve(item):
    a, b = item
    return np.linalg.solve(a, b)


def test_shard_round_robin_covers_every_item_once():
    for n in (0, 1, 5, 256):
        for world in (1, 2, 3, 8):
            got = sorted(i for r in range(world) for i in shard.shard(n, r, world))
            assert got == list(range(n))
    with pytest.raises(ValueError):
        shard.shard(4, 2, 2)


def test_local_without_process_group():
    items = _systems()
    res = shard.solve_sharded(items, _solve)
    assert sorted(res) == list(range(len(items)))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        items = _systems()
        mine = shard.solve_sharded(items, _solve, gather=False)
        full = shard.solve_sharded(items, _solve)
        q.put((rank, sorted(mine), {i: v.tolist() for i, v in full.items()}))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_solves_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    items = _systems()
    ref = [_solve(it) for it in items]
    owned = {rank: mine for rank, mine, _ in out}
    assert owned[0] == [0, 2, 4, 6] and owned[1] == [1, 3, 5]
    for _, _, full in out:
        assert sorted(full) == list(range(len(items)))
        for i, v in full.items():
            np.testing.assert_allclose(v, ref[i], rtol=1e-12)
