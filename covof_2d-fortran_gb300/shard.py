"""Batches of independent cases split across GPUs (one process per GPU).

The cases of a batch share nothing, so a multi-GPU run gives each rank a
subset and runs one batch per rank with no collective on the data path; the
host gathers the per-case statuses and statistics at the end.  This is the
only split of the hot path: a single case is never divided (the reference's
SP Poisson operator has no halo exchange, src/module_simulation.f90:
2668-2758, so a domain split would change its answer), and the reference's
own parallelism is the MPI domain decomposition of src/module_mesh.f90:96-143,
one case per job.

Assignment: each case's cost is estimated as cells x the longer side (the
work model of the batch engine's own team planner: Krylov iterations grow
with the longer side); cases go longest first to the rank with the least
assigned cost (greedy LPT), ties to the lower rank, so every rank computes
the same plan from the same case list.
"""
from __future__ import annotations

from typing import Sequence


def case_cost(nx: int, ny: int) -> int:
    """Estimated work of one case: cells x the longer side."""
    return int(nx) * int(ny) * max(int(nx), int(ny))


def plan(costs: Sequence[int], world: int) -> list[list[int]]:
    """Case indices per rank: longest first to the least-loaded rank.
    Within a rank the cases keep their original order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda c: (-int(costs[c]), c))
    load = [0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for c in order:
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(c)
        load[r] += int(costs[c])
    return [sorted(x) for x in out]


def plan_params(params: Sequence, world: int) -> list[list[int]]:
    """plan() over covof_params-like objects (fields nx, ny)."""
    return plan([case_cost(p.nx, p.ny) for p in params], world)


def makespan(costs: Sequence[int], assignment: list[list[int]]) -> int:
    """Largest per-rank cost of an assignment."""
    return max((sum(int(costs[c]) for c in part) for part in assignment), default=0)


def gather(local: dict, world: int) -> dict:
    """Merge every rank's {case index: record} on every rank (host-side
    object gather of torch.distributed; identity when world == 1)."""
    if world == 1:
        return dict(local)
    import torch.distributed as dist
    parts: list = [None] * world
    dist.all_gather_object(parts, local)
    out: dict = {}
    for part in parts:
        for k, v in part.items():
            if k in out:
                raise RuntimeError(f"case {k} reported by two ranks")
            out[k] = v
    return out
