"""Sharding of independent light curves across ranks (host logic, CPU):
cost-balanced partition, local renumbering, and the gather of results with
world_size-2 gloo process groups (the per-rank magnifications are stood in for
by a function of the global point index; no GPU work)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from caustics_gb300 import shard


def curves(n=40, seed=0):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 50, n)
    cv = np.stack([np.ones(n), 10 ** rng.uniform(-4, 0, n)] + [np.zeros(n)] * 6, axis=1)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    return off, np.arange(off[-1], dtype=np.float64) * 0.5, cv


def test_partition_covers_every_curve_once_and_balances():
    off, t, cv = curves()
    parts = shard.partition(off, cv, 3)
    allc = np.sort(np.concatenate(parts))
    assert np.array_equal(allc, np.arange(len(cv)))
    cost = shard.curve_costs(off, cv)
    loads = [cost[p].sum() for p in parts]
    assert max(loads) - min(loads) <= cost.max() + 1e-9


def test_local_problem_renumbers():
    off, t, cv = curves(seed=1)
    idx = np.array([3, 7, 11])
    lo, lt, lc, gi = shard.local_problem(off, t, cv, idx)
    assert lo[-1] == len(lt) == len(gi)
    for k, c in enumerate(idx):
        assert np.array_equal(lt[lo[k]:lo[k + 1]], t[off[c]:off[c + 1]])
        assert np.array_equal(lc[k], cv[c])


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    off, t, cv = curves(seed=2)
    parts = shard.partition(off, cv, world)
    lo, lt, lc, gi = shard.local_problem(off, t, cv, parts[rank])
    local = 3.0 * lt + rank * 0.0  # stands in for this rank's magnifications
    out = shard.gather(local, gi, int(off[-1]))
    q.put((rank, out))
    dist.destroy_process_group()


def test_gather_world_size_2():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    off, t, cv = curves(seed=2)
    for r in (0, 1):
        assert np.array_equal(res[r], 3.0 * t)
