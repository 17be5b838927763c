"""GPU: failure handling, with every failure made on the host.

* a request cancelled while it waits in the server's queue, and one cancelled
  while it renders: both end FOMO_ECANCELLED and their result arrays are never
  written; the server goes on serving;
* a server stopped with work still queued drains it (every queued request is
  rendered and delivered) and a new server then renders the same bits;
* a device allocation that fails (FOMO_INJECT_ALLOC_FAILURE=k: the k-th
  allocation of the context fails as cudaMalloc would) in a snapshot upload, a
  table upload, an emissivity payload or a render's scratch: the call returns
  FOMO_ENOMEM, frees what it had taken, and the same context then renders the
  same bits as a fresh one.

The reference has no recovery at all: it exits (fomo-CHIANTI.cpp:27-29,126-128,
146-148; fomo-object.cpp:430-434).  No test here faults, traps or hangs the GPU.
"""

import time

import numpy as np
import pytest

import fomo_gb300 as fg
from fomo_gb300 import synth

pytestmark = pytest.mark.gpu

SENTINEL = -7.0


def _setup(ctx):
    sid = ctx.snapshot(synth.loop_snapshot(64, seed=1))
    tid = ctx.table(synth.line_table())
    return sid, tid


def _big(sid, tid):
    # about 2 G LOS samples: tens of milliseconds on the device
    return fg.Context.request(sid, tid, fg.METHOD_NN, 1024, 1024, 2048, 16, 0.3, 0.2, 1.5e5)


def _small(sid, tid, l=0.4):
    return fg.Context.request(sid, tid, fg.METHOD_NN, 32, 24, 64, 16, l, -0.1, 1.5e5)


def test_cancel_queued_request():
    with fg.Server(0, max_inflight=1) as srv:
        sid, tid = _setup(srv.ctx)
        warm = np.empty(fg.Context.cube_shape(_small(sid, tid)), np.float32)
        srv.wait(srv.submit(_small(sid, tid), warm))
        a = np.empty(fg.Context.cube_shape(_big(sid, tid)), np.float32)
        b = np.full(fg.Context.cube_shape(_small(sid, tid)), SENTINEL, np.float32)
        ta = srv.submit(_big(sid, tid), a)
        tb = srv.submit(_small(sid, tid), b)  # one request in flight at a time: this one waits
        srv.cancel(tb)
        with pytest.raises(fg.FomoError) as ei:
            srv.wait(tb)
        assert ei.value.code == fg.ECANCELLED
        assert (b == SENTINEL).all()
        assert srv.wait(ta).status == fg.OK
        # the server goes on, and renders what a context renders
        c = np.empty_like(warm)
        assert srv.wait(srv.submit(_small(sid, tid, 0.9), c)).status == fg.OK
        with pytest.raises(fg.FomoError) as ei:
            srv.cancel(123456789)
        assert ei.value.code == fg.ENOTFOUND
    with fg.Context(0) as ctx:
        sid, tid = _setup(ctx)
        ref, _, _ = ctx.render(_small(sid, tid, 0.9))
    np.testing.assert_array_equal(c, ref)


def test_cancel_running_request():
    """A running request that is cancelled ends FOMO_ECANCELLED, undelivered;
    its batch (no other request in it) is halted on the device, so it ends
    well before the same request rendered in full; the next batch on the
    same slot renders normally (its halt word cleared)."""
    with fg.Server(0, max_inflight=1) as srv:
        sid, tid = _setup(srv.ctx)
        warm = np.empty(fg.Context.cube_shape(_small(sid, tid)), np.float32)
        srv.wait(srv.submit(_small(sid, tid), warm))
        full = np.empty(fg.Context.cube_shape(_big(sid, tid)), np.float32)
        st = srv.wait(srv.submit(_big(sid, tid), full))
        t_full = st.t_done - st.t_start
        a = np.full(fg.Context.cube_shape(_big(sid, tid)), SENTINEL, np.float32)
        ta = srv.submit(_big(sid, tid), a)
        time.sleep(0.02)  # admitted at once and on the device by now
        srv.cancel(ta)
        with pytest.raises(fg.FomoError) as ei:
            srv.wait(ta)
        assert ei.value.code == fg.ECANCELLED
        assert (a == SENTINEL).all()  # the rendered cube is discarded, not delivered
        t_cancelled = ei.value.stats.t_done - ei.value.stats.t_start
        assert t_full > 0.05, t_full  # the full render takes long enough for the comparison
        assert t_cancelled < 0.6 * t_full, (t_cancelled, t_full)
        for _ in range(2):  # both slots have run since
            c = np.empty_like(warm)
            assert srv.wait(srv.submit(_small(sid, tid), c)).status == fg.OK
            np.testing.assert_array_equal(c, warm)
        again = np.empty_like(full)
        assert srv.wait(srv.submit(_big(sid, tid), again)).status == fg.OK
        np.testing.assert_array_equal(again, full)


def test_stopped_server_drains_its_queue_and_a_new_one_renders_the_same():
    reqs_l = [0.1 * k for k in range(6)]
    srv = fg.Server(0, max_inflight=1)
    sid, tid = _setup(srv.ctx)
    outs = [np.full(fg.Context.cube_shape(_small(sid, tid)), SENTINEL, np.float32) for _ in reqs_l]
    for l, o in zip(reqs_l, outs):
        srv.submit(_small(sid, tid, l), o)
    srv.close()  # stop: the scheduler renders what is queued, then exits
    for o in outs:
        assert not (o == SENTINEL).any()
    with fg.Server(0) as srv2:
        sid2, tid2 = _setup(srv2.ctx)
        for l, o in zip(reqs_l, outs):
            again = np.empty_like(o)
            assert srv2.wait(srv2.submit(_small(sid2, tid2, l), again)).status == fg.OK
            np.testing.assert_array_equal(again, o)


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6, 7, 8])
def test_injected_allocation_failure_leaves_a_usable_context(monkeypatch, k):
    s = synth.loop_snapshot(20, seed=4)
    t = synth.line_table()
    req = lambda sid, tid: fg.Context.request(sid, tid, fg.METHOD_NN, 24, 20, 48, 32, 0.5, 0.3, 1.5e5)  # noqa: E731
    with fg.Context(0) as fresh:
        ref, ref_idx, _ = fresh.render(req(fresh.snapshot(s), fresh.table(t)), want_idx=True)
    monkeypatch.setenv("FOMO_INJECT_ALLOC_FAILURE", str(k))
    with fg.Context(0) as ctx:
        failed = None
        try:
            sid = ctx.snapshot(s)
            tid = ctx.table(t)
            ctx.render(req(sid, tid))
        except fg.FomoError as e:
            failed = e
        if failed is not None:
            assert failed.code == fg.ENOMEM and "injected" in str(failed)
        if k <= 2:
            assert failed is not None  # the snapshot's first allocations
            assert ctx.memory()[0] == 0  # nothing kept from the failed upload
        # the same context, once more: everything works and gives the same bits
        sid = ctx.snapshot(s)
        tid = ctx.table(t)
        cube, idx, _ = ctx.render(req(sid, tid), want_idx=True)
        np.testing.assert_array_equal(idx, ref_idx)
        np.testing.assert_array_equal(cube, ref)
