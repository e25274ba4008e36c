"""Batch sharding across ranks (shard.py) on CPU: the plan is a balanced
partition that every rank computes identically, and a world-size-2 gloo run
in which each rank steps its own cases (with the oracle standing in for the
per-rank batch engine) and the host gather reproduces the single-rank result
bit for bit."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _shard():
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge
    pkg = ge.load_package()
    import importlib
    return importlib.import_module(pkg.__name__ + ".shard"), pkg


def test_plan_is_a_balanced_deterministic_partition():
    shard, _ = _shard()
    rng = np.random.default_rng(0)
    sizes = (64, 128, 256, 512)
    for world in (1, 2, 3, 4, 8):
        shapes = [tuple(int(v) for v in rng.choice(sizes, 2)) for _ in range(97)]
        costs = [shard.case_cost(nx, ny) for nx, ny in shapes]
        a = shard.plan(costs, world)
        assert a == shard.plan(costs, world)
        flat = sorted(c for part in a for c in part)
        assert flat == list(range(len(costs)))
        assert len(a) == world
        # list-scheduling bound: every rank's load <= mean + largest case
        bound = sum(costs) / world + max(costs)
        assert shard.makespan(costs, a) <= bound
    # the batch workload's 256 cases over 8 ranks stay within 5 % of the mean
    pkg = _shard()[1]
    cases = pkg.cases.droplet_batch(n_cases=256)
    costs = [shard.case_cost(c[0].nx, c[0].ny) for c in cases]
    a = shard.plan(costs, 8)
    assert shard.makespan(costs, a) <= 1.05 * sum(costs) / 8


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _cases(pkg, orc):
    out = []
    for p, C0, dt in pkg.cases.droplet_batch(n_cases=5, seed=21, sizes=(16, 24, 32), nsub=4):
        f = pkg.Fields.allocate(p)
        f.C[...] = C0
        orc.apply_vof_bc(p, f.C)
        orc.update_physical_properties(p, f)
        orc.compute_curvature_and_csf(p, f)
        out.append((p, f, dt))
    return out


def _steps(orc, p, f, dt, n):
    g = f.copy()
    for k in range(n):
        iu, ip, rr, st = orc.time_step(p, dt, k, g)
        assert st == 0
    return {name: getattr(g, name) for name in ("u", "v", "p", "C")}


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import __graft_entry__ as ge
    pkg = ge.load_package()
    orc = ge._load_oracle()
    import importlib
    shard = importlib.import_module(pkg.__name__ + ".shard")
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cases = _cases(pkg, orc)
        parts = shard.plan_params([c[0] for c in cases], world)
        mine = {c: _steps(orc, *cases[c], 2) for c in parts[rank]}
        merged = shard.gather(mine, world)
        ok = sorted(merged) == list(range(len(cases)))
        if rank == 0:
            for c, (p, f, dt) in enumerate(cases):
                ref = _steps(orc, p, f, dt, 2)
                ok = ok and all(np.array_equal(merged[c][k], ref[k]) for k in ref)
        q.put((rank, ok, [len(x) for x in parts]))
    finally:
        dist.destroy_process_group()


def test_sharded_steps_gather_equals_single_rank_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(o[1] for o in out), out
    # both ranks got work
    assert all(n > 0 for n in out[0][2])
