"""Replica parallelism across GPUs / processes.

Estimates are independent (one catalogue -> one data vector): the path has
no exchange step, so several GPUs run as replicas.  Each rank takes a
disjoint, balanced share of the units (mock catalogues or bin blocks), runs
them locally, and the small per-unit result vectors are gathered on rank 0.
No collective touches meshes or spectra.
"""
from __future__ import annotations

import numpy as np


def shard_units(n_units: int, rank: int, world: int, costs=None):
    """Indices of the units rank `rank` of `world` runs.

    Without `costs` units are dealt round-robin; with per-unit `costs`
    (e.g. particle counts of uneven mocks) a greedy longest-first
    assignment balances the total cost per rank.
    """
    if world < 1 or not 0 <= rank < world:
        raise ValueError("Invalid rank / world size.")
    if costs is None:
        return list(range(rank, n_units, world))
    costs = np.asarray(costs, dtype=float)
    if costs.shape != (n_units,):
        raise ValueError("`costs` must have one entry per unit.")
    load = np.zeros(world)
    owner = np.empty(n_units, dtype=int)
    for u in np.argsort(-costs, kind='stable'):
        r = int(np.argmin(load))
        owner[u] = r
        load[r] += costs[u]
    return [int(u) for u in np.flatnonzero(owner == rank)]


def gather_results(local: dict, n_units: int, group=None):
    """Gather {unit index: 1-D result array} from every rank onto rank 0.

    Uses ``torch.distributed`` object collectives on the given process
    group (any backend); returns the full list of length `n_units` on rank
    0 and None elsewhere.
    """
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    payload = {int(k): np.asarray(v) for k, v in local.items()}
    gathered = [None] * world if rank == 0 else None
    dist.gather_object(payload, gathered, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * n_units
    for part in gathered:
        for k, v in part.items():
            if out[k] is not None:
                raise RuntimeError(f"Unit {k} computed twice.")
            out[k] = v
    missing = [i for i, v in enumerate(out) if v is None]
    if missing:
        raise RuntimeError(f"Units never computed: {missing}.")
    return out
