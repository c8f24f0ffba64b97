"""Multi-rank host logic on CPU: two gloo ranks shard an uneven ensemble, reduce times and gather rows."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from magex_gb300.replicas import gather_rows, max_over_ranks, shard_systems
from magex_gb300.workloads import film_ensemble


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, sizes, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard_systems(sizes, world, rank)
        # each rank "measures" its own time and produces one row per owned system
        t = max_over_ranks([1.0 + rank, 10.0 - rank], dist)
        rows = [[k, float(sizes[k]), k * 0.5] for k in mine]
        table = gather_rows(mine, rows, len(sizes), dist)
        q.put((rank, mine, t, table))
    finally:
        dist.destroy_process_group()


def test_two_rank_ensemble_sharding():
    sizes = [s["L"] ** 2 for s in film_ensemble(n=64, seed=2)]
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, sizes, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res.sort()
    owned = [set(r[1]) for r in res]
    assert owned[0].isdisjoint(owned[1]) and owned[0] | owned[1] == set(range(len(sizes)))
    loads = [sum(sizes[k] for k in o) for o in owned]
    assert abs(loads[0] - loads[1]) <= max(sizes)             # LPT balance
    for r in res:
        assert r[2] == [2.0, 10.0]                             # element-wise max over ranks
        np.testing.assert_array_equal(r[3][:, 0], np.arange(len(sizes)))
        np.testing.assert_array_equal(r[3][:, 1], np.asarray(sizes, float))


def test_single_process_fallbacks():
    assert shard_systems([5, 3, 2], 1, 0) == [0, 1, 2]
    assert max_over_ranks([1.5, 2.5]) == [1.5, 2.5]
    np.testing.assert_array_equal(gather_rows([1, 0], [[1.0], [0.0]], 2), [[0.0], [1.0]])
