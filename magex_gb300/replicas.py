"""Host logic for running on several GPUs: independent systems, no exchange on the data path.

The LLG step of one lattice needs no communication; an ensemble of independent systems (replicas,
temperature / field scans, uneven films) is split across ranks by system, each rank steps its share
with its own BatchedLLG, and only the per-system observables are gathered at the end.  This is the
GPU analogue of magex running one process per temperature or per replica.  One lattice too large
for one GPU is split into slabs with a halo exchange per Heun stage instead (magex/mpi_spin.py:160-174):
that path is ``magex_gb300.slab``.

All functions work with any torch.distributed backend (nccl on GPUs, gloo on CPU) or without one.
"""
from __future__ import annotations

import numpy as np


def shard_systems(sizes, world, rank):
    """Indices of the systems assigned to `rank` out of `world`, balancing total spins: systems are
    taken largest first and given to the least loaded rank (longest-processing-time rule), which is
    deterministic, so every rank computes the same partition without communicating."""
    sizes = np.asarray(sizes, np.int64)
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    load = np.zeros(world, np.int64)
    owner = np.empty(len(sizes), np.int64)
    for k in sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i)):
        r = int(np.argmin(load))
        owner[k] = r
        load[r] += sizes[k]
    return [k for k in range(len(sizes)) if owner[k] == rank]


def max_over_ranks(values, dist=None):
    """Element-wise maximum of a list of floats over all ranks (the timing rule: the slowest rank sets
    the time of the job)."""
    import torch
    t = torch.tensor(list(values), dtype=torch.float64)
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        if dist.get_backend() == "nccl":
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


def gather_rows(local_index, local_rows, nsys, dist=None):
    """Per-system rows (e.g. observables) from every rank, assembled in system order on all ranks."""
    local = (list(map(int, local_index)), np.asarray(local_rows, float).tolist())
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        parts = [None] * dist.get_world_size()
        dist.all_gather_object(parts, local)
    else:
        parts = [local]
    out = [None] * nsys
    for idx, rows in parts:
        for k, row in zip(idx, rows):
            out[k] = row
    if any(r is None for r in out):
        raise RuntimeError("some systems were not reported by any rank")
    return np.array(out)
