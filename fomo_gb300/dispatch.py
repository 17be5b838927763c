"""Spreading render requests over several GPUs (one process per GPU).

Views, lines and requests are independent: nothing is exchanged between GPUs
while rendering.  Each rank renders its share of a request list on its own GPU
(every rank holds its own copy of the snapshots) and the cubes are gathered
on one rank afterwards.  This replaces the reference's loop over (l, b) views
(fomo-c/src/fomo-nearestneighbour.cpp:285-306) when the views are spread over
ranks; the reference itself has no multi-GPU path.

    shares = partition(costs, world)            # which requests each rank renders
    cubes  = render_distributed(reqs, render_share, group=None, dst=0)

``render_share(indices)`` renders the requests with those indices on the local
GPU (for example with ``Context.render_batch``) and returns their cubes in
that order.  The gather uses ``torch.distributed`` object collectives, so any
backend works (gloo for host tensors; the cubes are host arrays).
"""

from __future__ import annotations

import heapq
from typing import Callable, Sequence


def request_cost(nx: int, ny: int, nz: int, nlambda: int) -> float:
    """Work of one request: LOS samples, plus the lambda binning per sample."""
    return float(nx) * ny * nz * (1.0 + 0.02 * max(nlambda, 1))


def partition(costs: Sequence[float], world: int) -> list[list[int]]:
    """Request indices per rank, balancing the summed cost (longest first,
    each to the least loaded rank; ties to the lower rank).  Every index is
    assigned exactly once; each rank's list is in increasing index order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    shares: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in shares]


def render_distributed(costs: Sequence[float], render_share: Callable[[list[int]], list], group=None,
                       dst: int = 0):
    """Render request i on the rank that partition() assigns it to, then gather.

    Returns the list of all cubes in request order on rank ``dst`` and None on
    the other ranks.  Without an initialised process group it renders
    everything locally.
    """
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return list(render_share(list(range(len(costs)))))
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    shares = partition(costs, world)
    mine = shares[rank]
    # a failing rank still takes part in the gather (with its error), so that
    # no rank is left waiting in the collective
    err = None
    try:
        local = list(render_share(mine))
        if len(local) != len(mine):
            raise RuntimeError(f"render_share returned {len(local)} cubes for {len(mine)} requests")
        payload = ("ok", list(zip(mine, local)))
    except Exception as e:  # noqa: BLE001 - reported to every rank below
        err = f"rank {rank}: {e}"
        payload = ("error", err)
    gathered = [None] * world if rank == dst else None
    dist.gather_object(payload, gathered, dst=dst, group=group)
    if rank != dst:
        if err:
            raise RuntimeError(err)
        return None
    errors = [p[1] for p in gathered if p[0] == "error"]
    if errors:
        raise RuntimeError("; ".join(errors))
    out = [None] * len(costs)
    for _, part in gathered:
        for i, cube in part:
            out[i] = cube
    missing = [i for i, c in enumerate(out) if c is None]
    if missing:
        raise RuntimeError(f"requests never rendered: {missing[:8]}")
    return out
