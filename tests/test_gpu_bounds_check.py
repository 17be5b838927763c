"""GPU: the bounds-check build (libfomo_gpu_checked.so, FOMO_BOUNDS_CHECK=1).

compute-sanitizer is not available for these runs, so every gather and scatter
index of the kernels (points, cell ranges, LOS tables, the neighbour buffer,
the deferred and hard queues, the shared-memory candidate lists, the cubes, the
index build's scatter, the G(T) table, the projection's pixels) is checked in
this build: an index out of range would be recorded in a device error word and
the call would fail with FOMO_EDEVICE (the access itself is redirected inside
the buffer, so nothing faults).  These tests run the golden cases and the
paths with split, deferred, hard-sample, chunked, Thomson, projection and
no-allocation marches through that build: every call must succeed (no index
out of range) and give the regular build's results.
"""

import ctypes

import numpy as np
import pytest

import fomo_gb300 as fg
import oracle
from fomo_gb300 import synth
from tests import _golden as G

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.fixture(scope="module")
def ctxs():
    a = fg.Context(0, checked=True)
    b = fg.Context(0)
    yield a, b
    a.close()
    b.close()


def _both(ctxs, snap, table, reqf, want_idx=True):
    """Render with the checked and the regular build; both must succeed."""
    out = []
    for c in ctxs:
        sid = c.snapshot(snap)
        tid = c.table(table) if table is not None else 0
        out.append(c.render(reqf(sid, tid), want_idx=want_idx))
        c.drop_snapshot(sid)
    return out


@pytest.mark.parametrize("name", ["nn_spectro.npz", "nn_medium.npz", "nn_imaging.npz"])
def test_golden_nn_cases(ctxs, name):
    d = G.load(name)
    s, t = G.snapshot(d), G.table(d)
    nx, ny, nz, L = (int(v) for v in d["res"])
    for v, (l, b) in enumerate(d["views"]):
        width = d["meta"][v][4]
        (cc, ci, _), (rc, ri, _) = _both(ctxs, s, t, lambda sid, tid: fg.Context.request(
            sid, tid, fg.METHOD_NN, nx, ny, nz, L, l, b, width))
        np.testing.assert_array_equal(ci, ri)
        np.testing.assert_array_equal(cc, rc)
        assert G.norm_max_err(cc.ravel(), d["cube"][v]) <= TOL


def test_golden_thomson_and_edges(ctxs):
    d = G.load("thomson.npz")
    s = G.snapshot(d)
    nx, ny, nz, _ = (int(v) for v in d["res"])
    for l, b in d["views"]:
        (cc, ci, _), (rc, ri, _) = _both(ctxs, s, None, lambda sid, tid: fg.Context.request(
            sid, 0, fg.METHOD_THOMSON, nx, ny, nz, 1, l, b, 1e5))
        np.testing.assert_array_equal(ci, ri)
        np.testing.assert_array_equal(cc, rc)
    d = G.load("nn_edges.npz")
    s, t = G.snapshot(d), G.table(d)
    for suffix in ("_a", "_b"):
        nx, ny, nz, L = (int(v) for v in d["res" + suffix])
        for v, (l, b) in enumerate(d["views" + suffix]):
            width = d["meta" + suffix][v][4]
            (cc, ci, _), (rc, ri, _) = _both(ctxs, s, t, lambda sid, tid: fg.Context.request(
                sid, tid, fg.METHOD_NN, nx, ny, nz, L, l, b, width))
            np.testing.assert_array_equal(ci, ri)
            np.testing.assert_array_equal(cc, rc)


def test_dense_cells_wide_boxes_and_off_equator_thomson(ctxs):
    """Overflowing segments (march_split), deferred samples and whole-warp
    searches (march_hard) on a flux rope at 64 x 64 pixels; Thomson off the
    equator (wide boxes, far neighbours)."""
    s = synth.flux_rope_snapshot(512 * 1024, seed=20)
    t = synth.line_table()
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    for (l, b) in ((0.5, 0.2), (1.2, -0.3)):
        (cc, ci, _), (rc, ri, _) = _both(ctxs, s, t, lambda sid, tid: fg.Context.request(
            sid, tid, fg.METHOD_NN, 64, 64, 256, 16, l, b, width))
        np.testing.assert_array_equal(ci, ri)
        np.testing.assert_array_equal(cc, rc)
    ts = synth.thomson_snapshot(24, seed=7)
    (cc, ci, _), (rc, ri, _) = _both(ctxs, ts, None, lambda sid, tid: fg.Context.request(
        sid, 0, fg.METHOD_THOMSON, 48, 40, 96, 1, 0.4, 0.3, 1e5))
    np.testing.assert_array_equal(ci, ri)
    np.testing.assert_array_equal(cc, rc)


def test_chunked_batch_projection_and_no_allocation_paths(ctxs, monkeypatch):
    """A batch whose neighbour buffer is capped (item chunks and view ranges),
    a projection render, and the no-allocation entry point in several chunks."""
    import torch

    s = synth.loop_snapshot(24, seed=5)
    t = synth.line_table()
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    views = [(0.3, 0.1), (1.0, -0.2), (1.7, 0.25)]
    monkeypatch.setenv("FOMO_NPOS_CAP", str(80 * 37))
    with fg.Context(0, checked=True) as c:
        sid, tid = c.snapshot(s), c.table(t)
        got, _ = c.render_batch([c.request(sid, tid, fg.METHOD_NN, 40, 36, 80, 24, l, b, width) for l, b in views])
    monkeypatch.delenv("FOMO_NPOS_CAP")
    c, r = ctxs
    rsid, rtid = r.snapshot(s), r.table(t)
    ref, _ = r.render_batch([r.request(rsid, rtid, fg.METHOD_NN, 40, 36, 80, 24, l, b, width) for l, b in views])
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)
    # projection (a scatter into the cube)
    csid, ctid = c.snapshot(s), c.table(t)
    pc, _, _ = c.render(c.request(csid, ctid, fg.METHOD_PROJECTION, 30, 26, 40, 32, 0.6, 0.2, width))
    pr, _, _ = r.render(r.request(rsid, rtid, fg.METHOD_PROJECTION, 30, 26, 40, 32, 0.6, 0.2, width))
    assert G.norm_max_err(pc, pr) <= 1e-6  # atomics: FP32 summation order
    # the no-allocation entry point, 8 chunks of its static deferred queue
    req = c.request(csid, ctid, fg.METHOD_NN, 256, 256, 512, 32, 0.45, 0.3, width)
    ref_cube, _, _ = c.render(req)
    out = torch.empty(ref_cube.shape, dtype=torch.float32, device="cuda:0")
    rc = c._L.fomo_render_noalloc(c.h, ctypes.byref(req), ctypes.c_void_p(out.data_ptr()), None)
    assert rc == fg.OK, c._L.fomo_last_error(c.h).decode()
    c.synchronize()  # reads the error words of the bounds-check build
    assert G.norm_max_err(out.cpu().numpy(), ref_cube) <= TOL
    eps, w = c.emission(csid, ctid)
    oeps, ow = oracle.emission(s, t)
    np.testing.assert_array_equal(w, ow)
