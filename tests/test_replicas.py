"""Replicas on several ranks (CPU, gloo): each rank solves its shard of the
scenarios with the CPU oracle's Newton loop; the gathered result equals a
single-process solve of all scenarios, and the timing reduction is the max."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from phdthesis_albertojimenezruiz_gb300.replicas import gather_columns, max_over_ranks, shard

DIMS = (1, 2, 5)
SCENARIOS = 5


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _solve(indices):
    from oracle import oracle as O
    from phdthesis_albertojimenezruiz_gb300 import GMIN_STAGES, Plant, Symbolic

    p = Plant(*DIMS)
    sym = Symbolic(p.rowptr, p.colidx)
    port = O.Port(p.rowptr, p.colidx, sym.array("perm_amd"))
    cols = []
    for k in indices:
        g = 1000.0 - np.random.default_rng(100 + k).uniform(0.0, 500.0, p.n_panels)
        rc, _, _, _, x = port.newton(p, p.iph(g), p.flat_start(), GMIN_STAGES, 1e-9)
        assert rc == 0
        cols.append(x)
    return np.stack(cols, 1) if cols else np.zeros((p.n, 0))


def _worker(rank, world, port, out_path):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = _solve(shard(SCENARIOS, rank, world))
        full = gather_columns(local, dist)
        slowest = max_over_ranks(float(rank + 1), dist)
        if rank == 0:
            np.save(out_path, full)
            assert slowest == float(world)
    finally:
        dist.destroy_process_group()


def test_shard_covers_every_scenario_once():
    for total in (0, 1, 5, 512):
        for world in (1, 2, 3, 8):
            seen = [i for r in range(world) for i in shard(total, r, world)]
            assert seen == list(range(total))


@pytest.mark.parametrize("world", [2])
def test_replicas_gather_equals_single_process(tmp_path, world):
    out = tmp_path / "full.npy"
    mp.spawn(_worker, args=(world, _free_port(), str(out)), nprocs=world, join=True)
    assert np.array_equal(np.load(out), _solve(range(SCENARIOS)))
