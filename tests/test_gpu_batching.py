"""GPU: batched launches, CUDA-graph replay, the render server, and a
full-size parity sample.  Every result must equal the same request rendered
alone (one warp owns one ray, so mixing cannot change a ray's arithmetic)."""

import math
import threading

import numpy as np
import pytest

import fomo_gb300 as fg
import oracle
from fomo_gb300 import synth
from tests import _golden as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = fg.Context(0)
    yield c
    c.close()


def _mixed_requests(sid, tids, bb, rng, n):
    reqs = []
    for _ in range(n):
        kind = rng.integers(0, 3)
        nx = int(rng.choice([8, 16, 32, 48]))
        ny = int(rng.choice([8, 16, 24]))
        nz = int(rng.choice([7, 32, 64]))
        l, b = float(rng.uniform(0, math.pi)), float(rng.uniform(-0.6, 0.6))
        if kind == 0:
            reqs.append(fg.Context.request(sid, int(rng.choice(tids)), fg.METHOD_NN, nx, ny, nz,
                                           int(rng.choice([16, 64, 128])), l, b, 1.5e5))
        elif kind == 1:
            reqs.append(fg.Context.request(sid, bb, fg.METHOD_NN, nx, ny, nz, 1, l, b, 1e5))
        else:
            reqs.append(fg.Context.request(sid, int(rng.choice(tids)), fg.METHOD_NN, nx, ny, nz, 40, l, b, 9e4))
    return reqs


def test_graph_replay_equals_direct(ctx):
    import torch
    s = synth.loop_snapshot(20, seed=9)
    sid = ctx.snapshot(s)
    tids = [ctx.table(synth.line_table(peak_logT=p, lambda0=lam)) for p, lam in ((5.9, 171.0), (6.1, 195.0))]
    dev = torch.device("cuda", 0)
    for (l, b) in [(0.2, 0.1), (1.1, -0.4), (2.0, 0.3)]:  # same shape: captured once, replayed
        reqs = [ctx.request(sid, t, fg.METHOD_NN, 24, 20, 48, 32, l, b, 1.4e5) for t in tids]
        outs = [torch.empty((20, 24, 32), dtype=torch.float32, device=dev) for _ in reqs]
        ctx.render_batch_device(reqs, [o.data_ptr() for o in outs], graph=True)
        ctx.synchronize()
        for q, o in zip(reqs, outs):
            single, _, _ = ctx.render(q)
            np.testing.assert_array_equal(o.cpu().numpy(), single)
    ctx.drop_snapshot(sid)


def test_host_batch_downloads_in_chunks_same_as_alone(ctx):
    """About 1 GB of cubes: the batch marches in four chunks of views whose
    cubes download while the next chunk marches.  Every cube and view info must
    match the same request rendered alone, with lines of one view kept together
    even when the caller interleaves them."""
    s = synth.loop_snapshot(24, seed=21)
    sid = ctx.snapshot(s)
    tids = [ctx.table(synth.line_table(peak_logT=p, lambda0=lam)) for p, lam in ((5.9, 171.0), (6.2, 211.0))]
    bb = ctx.table(synth.broadband_table(171))
    views = [(0.15 * k, 0.05 * (k - 4)) for k in range(9)]
    reqs = []
    for tid in tids:  # line-major order: a view's two lines are far apart in the list
        for (l, b) in views:
            reqs.append(ctx.request(sid, tid, fg.METHOD_NN, 512, 512, 32, 64, l, b, 1.5e5))
    reqs.append(ctx.request(sid, bb, fg.METHOD_NN, 256, 128, 40, 1, 0.7, 0.2, 1e5))
    cubes, infos = ctx.render_batch(reqs)
    for q, c, inf in zip(reqs, cubes, infos):
        single, _, sinf = ctx.render(q)
        np.testing.assert_array_equal(c, single)
        assert inf.as_dict() == sinf.as_dict()
    ctx.drop_snapshot(sid)


def test_small_neighbour_buffer_marches_in_item_chunks(monkeypatch):
    """FOMO_NPOS_CAP bounds the march's neighbour buffer; a launch then marches
    in chunks of work items.  Neighbour indices and cubes must be the same bits
    as those of an unchunked render (the emission pass bins every ray from the
    buffer in sample order, with no atomics); a host batch (view ranges +
    chunks) as well."""
    s = synth.loop_snapshot(24, seed=5)
    t = synth.line_table()
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    views = [(0.3, 0.1), (1.0, -0.2), (1.7, 0.25)]

    def run(c):
        sid, tid = c.snapshot(s), c.table(t)
        cube, idx, info = c.render(c.request(sid, tid, fg.METHOD_NN, 48, 40, 96, 32, 0.6, -0.15, width),
                                   want_idx=True)
        cubes, infos = c.render_batch([c.request(sid, tid, fg.METHOD_NN, 40, 36, 80, 24, l, b, width)
                                       for (l, b) in views])
        return cube, idx, info, cubes, infos

    with fg.Context(0) as c1:
        ref = run(c1)
    monkeypatch.setenv("FOMO_NPOS_CAP", str(96 * 37))  # 37 work items per chunk
    with fg.Context(0) as c2:
        got = run(c2)
    np.testing.assert_array_equal(got[1], ref[1])
    np.testing.assert_array_equal(got[0], ref[0])
    assert got[2].as_dict() == ref[2].as_dict()
    for a, b, ia, ib in zip(got[3], ref[3], got[4], ref[4]):
        np.testing.assert_array_equal(a, b)
        assert ia.as_dict() == ib.as_dict()


def test_server_same_alone_and_in_mix():
    rng = np.random.default_rng(17)
    with fg.Server(0) as srv:
        c = srv.ctx
        s = synth.loop_snapshot(24, seed=3)
        sid = c.snapshot(s)
        tids = [c.table(synth.line_table(peak_logT=p, lambda0=lam)) for p, lam in ((5.8, 171.0), (6.2, 211.0))]
        bb = c.table(synth.broadband_table(171))
        reqs = _mixed_requests(sid, tids, bb, rng, 24)
        alone = []
        for q in reqs:
            out = np.empty(fg.Context.cube_shape(q), np.float32)
            st = srv.wait(srv.submit(q, out))
            assert st.status == fg.OK
            alone.append(out)
        # all at once, from several threads
        mixed = [np.empty(fg.Context.cube_shape(q), np.float32) for q in reqs]
        tickets = [None] * len(reqs)

        def sub(idx):
            for i in idx:
                tickets[i] = srv.submit(reqs[i], mixed[i])

        th = [threading.Thread(target=sub, args=(list(range(k, len(reqs), 4)),)) for k in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        stats = [srv.wait(t) for t in tickets]
        for a, m, st in zip(alone, mixed, stats):
            assert st.status == fg.OK and st.t_done >= st.t_submit
            np.testing.assert_array_equal(a, m)


def test_server_admission_rejects_oversized_request():
    with fg.Server(0, hbm_budget=64 << 20) as srv:
        sid = srv.ctx.snapshot(synth.loop_snapshot(8, seed=1))
        tid = srv.ctx.table(synth.line_table())
        big = fg.Context.request(sid, tid, fg.METHOD_NN, 1024, 1024, 64, 128, 0.0, 0.0, 1e5)  # 512 MB cube
        with pytest.raises(fg.FomoError) as ei:
            srv.submit(big, np.empty(1024 * 1024 * 128, np.float32))  # never touched: rejected at submit
        assert ei.value.code == fg.EADMISSION
        with pytest.raises(fg.FomoError) as ei:
            srv.submit(big, np.empty(1, np.float32))  # a result array smaller than the cube
        assert ei.value.code == fg.EINVAL
        ok = fg.Context.request(sid, tid, fg.METHOD_NN, 16, 16, 16, 16, 0.0, 0.0, 1e5)
        out = np.empty((16, 16, 16), np.float32)
        assert srv.wait(srv.submit(ok, out)).status == fg.OK


def test_unknown_ids_and_bad_arguments(ctx):
    with pytest.raises(fg.FomoError) as ei:
        ctx.render(ctx.request(12345, 0, fg.METHOD_NN, 8, 8, 8, 8))
    assert ei.value.code == fg.ENOTFOUND
    sid = ctx.snapshot(synth.loop_snapshot(6, seed=1))
    with pytest.raises(fg.FomoError) as ei:
        ctx.render(ctx.request(sid, 0, 7, 8, 8, 8, 8))
    assert ei.value.code == fg.EMETHOD
    with pytest.raises(fg.FomoError) as ei:
        ctx.render(ctx.request(sid, 0, fg.METHOD_THOMSON, 1, 8, 8, 1))
    assert ei.value.code == fg.EINVAL
    with pytest.raises(fg.FomoError) as ei:
        ctx.load_table("/nonexistent/table.dat")
    assert ei.value.code == fg.EIO
    ctx.drop_snapshot(sid)


def test_snapshot_from_device_arrays_renders_the_same(ctx):
    import torch
    s = synth.loop_snapshot(16, seed=12)
    t = synth.line_table()
    tid = ctx.table(t)
    dev = [torch.from_numpy(a.copy()).cuda() for a in s.arrays()]
    sid_h = ctx.snapshot(s)
    torch.cuda.synchronize()  # the arrays must be complete: the snapshot copies them on the context's stream
    sid_d = ctx.snapshot_device(s.npoints, [d.data_ptr() for d in dev])
    del dev  # the snapshot keeps its own copy
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    a, ia, _ = ctx.render(ctx.request(sid_h, tid, fg.METHOD_NN, 20, 16, 32, 16, 0.4, -0.2, width), want_idx=True)
    b, ib, _ = ctx.render(ctx.request(sid_d, tid, fg.METHOD_NN, 20, 16, 32, 16, 0.4, -0.2, width), want_idx=True)
    np.testing.assert_array_equal(ia, ib)
    np.testing.assert_array_equal(a, b)
    with pytest.raises(fg.FomoError) as ei:  # host arrays are refused by the device entry point
        ctx.snapshot_device(s.npoints, [a.ctypes.data for a in s.arrays()])
    assert ei.value.code == fg.EINVAL
