"""fomo_render_noalloc: the render entry point for callers that must not
allocate device memory while they render (their working memory is a fixed
static device array inside the library).  Its cube must match the regular
render's, call after call.  Collected last on purpose (file name), so a run
that stops at the first failure has run every other test before it."""

import ctypes

import numpy as np
import pytest

import fomo_gb300 as fg
from fomo_gb300 import synth
from tests import _golden as G

pytestmark = pytest.mark.gpu

TOL = 1e-4  # normalised max error, as for every other render test


def test_noalloc_render_matches_regular_render_on_consecutive_calls():
    import torch

    with fg.Context(0) as ctx:
        lib = fg.lib()
        s = synth.loop_snapshot(24, seed=21)
        t = synth.line_table()
        sid = ctx.snapshot(s)
        tid = ctx.table(t)
        width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
        req = ctx.request(sid, tid, fg.METHOD_NN, 40, 36, 96, 64, 0.7, -0.35, width)
        # the regular entry point; it also makes this snapshot/table emissivity resident
        ref, _, _ = ctx.render(req)
        out = torch.empty(ref.shape, dtype=torch.float32, device="cuda:0")
        for _ in range(2):
            out.fill_(float("nan"))
            torch.cuda.synchronize()
            rc = lib.fomo_render_noalloc(ctx.h, ctypes.byref(req), ctypes.c_void_p(out.data_ptr()), None)
            assert rc == fg.OK, lib.fomo_last_error(ctx.h).decode()
            ctx.synchronize()
            got = out.cpu().numpy()
            assert np.isfinite(got).all()
            assert G.norm_max_err(got, ref) <= TOL

        # sizes beyond the static array are refused, not rendered
        big = ctx.request(sid, tid, fg.METHOD_NN, 16, 16, 5000, 16, 0.1, 0.2, width)
        rc = lib.fomo_render_noalloc(ctx.h, ctypes.byref(big), ctypes.c_void_p(out.data_ptr()), None)
        assert rc == fg.EINVAL
        assert "limits" in lib.fomo_last_error(ctx.h).decode()


def test_noalloc_one_lane_searches_match_warp_searches_on_dense_cells():
    """The no-allocation path has no hard-sample queue: every deferred sample is
    searched by one lane without a budget.  On a flux rope at 64 x 64 pixels
    (wide boxes, ~90-point cells) the regular render sends many samples to
    whole-warp searches instead; both must find the same neighbours, so the
    cubes differ only by the order of the deferred passes' atomic additions."""
    import torch

    with fg.Context(0) as ctx:
        lib = fg.lib()
        s = synth.flux_rope_snapshot(512 * 1024, seed=20)
        t = synth.line_table()
        sid = ctx.snapshot(s)
        tid = ctx.table(t)
        width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
        for (l, b) in ((0.5, 0.2), (1.2, -0.3)):
            req = ctx.request(sid, tid, fg.METHOD_NN, 64, 64, 256, 16, l, b, width)
            ref, _, _ = ctx.render(req)
            out = torch.empty(ref.shape, dtype=torch.float32, device="cuda:0")
            torch.cuda.synchronize()
            rc = lib.fomo_render_noalloc(ctx.h, ctypes.byref(req), ctypes.c_void_p(out.data_ptr()), None)
            assert rc == fg.OK, lib.fomo_last_error(ctx.h).decode()
            ctx.synchronize()
            assert G.norm_max_err(out.cpu().numpy(), ref) <= 1e-5


@pytest.mark.parametrize("nx,ny,nz,nlam", [(256, 256, 512, 32), (64, 64, 4096, 16)])
def test_noalloc_render_in_several_chunks_matches_regular_render(nx, ny, nz, nlam):
    """The static deferred-sample queue holds 65,536 segment records (one per 64
    LOS samples of a ray), so a render with more segments marches its rays in
    chunks: 65,536 rays x 8 segments in 8 chunks, and 4,096 rays x 64 segments
    in 4 chunks of 1,024 rays.  Each chunk clears the work counters and starts
    its rays from its own first work item; the cube must still match the
    regular render's, on two calls in a row."""
    import torch

    with fg.Context(0) as ctx:
        lib = fg.lib()
        s = synth.loop_snapshot(32, seed=4)
        t = synth.line_table()
        sid = ctx.snapshot(s)
        tid = ctx.table(t)
        width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
        req = ctx.request(sid, tid, fg.METHOD_NN, nx, ny, nz, nlam, 0.45, 0.3, width)
        ref, _, _ = ctx.render(req)
        out = torch.empty(ref.shape, dtype=torch.float32, device="cuda:0")
        for _ in range(2):
            out.fill_(float("nan"))
            torch.cuda.synchronize()
            rc = lib.fomo_render_noalloc(ctx.h, ctypes.byref(req), ctypes.c_void_p(out.data_ptr()), None)
            assert rc == fg.OK, lib.fomo_last_error(ctx.h).decode()
            ctx.synchronize()
            got = out.cpu().numpy()
            assert np.isfinite(got).all()
            assert G.norm_max_err(got, ref) <= TOL
