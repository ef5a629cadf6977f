"""Replica sharding across ranks (host logic, gloo on CPU, world size 2)."""
import os
import socket

import numpy as np
import pytest

from triumvirate_gb300.replicas import gather_results, shard_units


def test_round_robin_covers_every_unit_once():
    for n, world in [(10, 3), (1, 4), (256, 8), (7, 1)]:
        got = sorted(u for r in range(world)
                     for u in shard_units(n, r, world))
        assert got == list(range(n))


def test_cost_balanced_sharding():
    rng = np.random.default_rng(0)
    costs = rng.integers(200_000, 2_000_000, 256)   # uneven mock sizes
    world = 8
    parts = [shard_units(256, r, world, costs) for r in range(world)]
    assert sorted(u for p in parts for u in p) == list(range(256))
    loads = np.array([costs[p].sum() for p in parts])
    assert loads.max() / loads.mean() < 1.01


def test_invalid_rank():
    with pytest.raises(ValueError):
        shard_units(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n_units, queue):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard_units(n_units, rank, world)
        # Each unit's "data vector" is a deterministic function of its index.
        local = {u: np.arange(4, dtype=float) + 10. * u for u in mine}
        out = gather_results(local, n_units)
        if rank == 0:
            queue.put([v.tolist() for v in out])
    finally:
        dist.destroy_process_group()


def test_gather_over_gloo_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    n_units = 7
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n_units, queue))
             for r in range(2)]
    for p in procs:
        p.start()
    result = queue.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    expected = [(np.arange(4, dtype=float) + 10. * u).tolist()
                for u in range(n_units)]
    assert result == expected
