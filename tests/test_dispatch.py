"""Spreading requests over ranks (fomo_gb300.dispatch): host logic, CPU only.

Two gloo ranks render disjoint shares of a request list with a stand-in
renderer (a deterministic function of the request) and rank 0 gathers the
cubes; the result must equal the single-process result, every request must be
rendered exactly once, and a rank that drops a cube must raise.
"""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from fomo_gb300 import dispatch


def test_partition_assigns_every_request_once_and_balances():
    costs = [dispatch.request_cost(nx, ny, nz, L) for nx, ny, nz, L in
             [(64, 64, 128, 16), (1024, 1024, 256, 1), (128, 128, 256, 64), (512, 512, 512, 128), (64, 64, 64, 1),
              (256, 256, 256, 16), (256, 256, 512, 64), (128, 128, 128, 128)]]
    for world in (1, 2, 3, 4, 8, 16):
        shares = dispatch.partition(costs, world)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in s) for s in shares]
        # longest-first greedy: no rank exceeds the mean by more than the largest request
        assert max(loads) <= sum(costs) / world + max(costs) + 1e-6
    assert dispatch.partition([], 3) == [[], [], []]
    with pytest.raises(ValueError):
        dispatch.partition([1.0], 0)


def _fake_cube(i):
    rng = np.random.default_rng(1000 + i)
    return rng.standard_normal((3 + i % 4, 5, 2)).astype(np.float32)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, costs, drop, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        def share(idx):
            cubes = [_fake_cube(i) for i in idx]
            return cubes[:-1] if (drop and rank == 1 and cubes) else cubes
        try:
            out = dispatch.render_distributed(costs, share)
            q.put((rank, "ok", None if out is None else [c.tolist() for c in out]))
        except RuntimeError as e:
            q.put((rank, "error", str(e)))
    finally:
        dist.destroy_process_group()


def _run(world, costs, drop=False):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, costs, drop, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
    return {r: (status, val) for r, status, val in res}


def test_two_gloo_ranks_render_disjoint_shares_and_gather_in_order():
    costs = [float(c) for c in (5, 1, 9, 3, 3, 7, 2)]
    res = _run(2, costs)
    status0, out = res[0]
    assert status0 == "ok" and res[1] == ("ok", None)
    assert len(out) == len(costs)
    for i, c in enumerate(out):
        np.testing.assert_array_equal(np.array(c, np.float32), _fake_cube(i))


def test_a_rank_that_drops_a_cube_raises_on_every_rank():
    res = _run(2, [float(c) for c in (4, 4, 4, 4)], drop=True)
    for r in (0, 1):
        assert res[r][0] == "error" and "rank 1: render_share returned" in res[r][1]
