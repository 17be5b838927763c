"""Projection renderer on the GPU (fomo-projection.cpp:17-193).

Every point adds its emission to the pixel nearest its projection.  The cubes
must match the reference's own renders (tests/golden/projection.npz, the
reference run single-threaded) and the oracle's FP64 sums within 1e-4; the
view quantities (extents, path length, DN pixel area) bit for bit; a batch
mixing projection and nearest-neighbour requests must equal the requests
rendered one at a time.
"""

import math

import numpy as np
import pytest

import fomo_gb300 as fg
import oracle
from fomo_gb300 import synth
from tests import _golden as G

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    with fg.Context(0) as c:
        yield c


@pytest.mark.parametrize("suffix,ek,wk,tk", [("_a", "eps", "fwhm", "table_text"),
                                              ("_b", "eps_band", "fwhm_band", "band_text")])
def test_projection_matches_reference_golden(ctx, suffix, ek, wk, tk):
    d = G.load("projection.npz")
    s = G.snapshot(d)
    t = G.table(d, tk)
    sid = ctx.snapshot(s)
    tid = ctx.table(t)
    nx, ny, nz, L = (int(v) for v in d["res" + suffix])
    for v, (l, b) in enumerate(d["views" + suffix]):
        width = d["meta" + suffix][v][4]
        req = ctx.request(sid, tid, fg.METHOD_PROJECTION, nx, ny, nz, L, float(l), float(b), width)
        cube, _, info = ctx.render(req)
        ref = d["cube" + suffix][v]
        assert G.norm_max_err(cube.ravel(), ref) <= TOL
        oc, _, ov = oracle.projection_render(s, d[ek], d[wk], t.lambda0, l, b, nx, ny, nz, L, width, is_dn=t.is_dn)
        assert G.norm_max_err(cube.ravel(), oc.ravel()) <= TOL
        assert (info.minx, info.maxx, info.miny, info.maxy) == tuple(ov[:4])
        assert info.pathlength == ov[oracle.V_PATHLENGTH] and info.apix == ov[oracle.V_APIX]
    ctx.drop_snapshot(sid)


@pytest.mark.parametrize("l,b", [(0.0, 0.0), (0.7, 0.3), (2.3, -1.1)])
def test_projection_larger_case_against_oracle(ctx, l, b):
    s = synth.loop_snapshot(48, seed=9)
    t = synth.line_table()
    bt = synth.broadband_table(193)
    sid = ctx.snapshot(s)
    tid, bid = ctx.table(t), ctx.table(bt)
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    spec = ctx.request(sid, tid, fg.METHOD_PROJECTION, 96, 80, 128, 64, l, b, width)
    img = ctx.request(sid, bid, fg.METHOD_PROJECTION, 96, 80, 128, 1, l, b, 1e5)
    (cs, ci), infos = ctx.render_batch([spec, img])
    eps, w = oracle.emission(s, t)
    oc, _, _ = oracle.projection_render(s, eps, w, t.lambda0, l, b, 96, 80, 128, 64, width)
    assert G.norm_max_err(cs.ravel(), oc.ravel()) <= TOL
    eps, w = oracle.emission(s, bt, imaging=True)
    oc, _, _ = oracle.projection_render(s, eps, w, bt.lambda0, l, b, 96, 80, 128, 1, 1e5, is_dn=True)
    assert G.norm_max_err(ci.ravel(), oc.ravel()) <= TOL
    assert infos[1].is_dn == 1 and infos[0].observation_type == fg.OBS_SPECTROSCOPIC
    ctx.drop_snapshot(sid)


def test_projection_and_nn_in_one_batch_equal_single_renders(ctx):
    s = synth.loop_snapshot(20, seed=4)
    t = synth.line_table()
    sid = ctx.snapshot(s)
    tid = ctx.table(t)
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    reqs = [ctx.request(sid, tid, m, 24, 20, 40, 16, l, b, width)
            for m in (fg.METHOD_PROJECTION, fg.METHOD_NN) for (l, b) in ((0.2, 0.1), (1.0, -0.5))]
    cubes, _ = ctx.render_batch(reqs)
    for q, c in zip(reqs, cubes):
        single, _, _ = ctx.render(q)
        assert G.norm_max_err(c.ravel(), single.ravel()) <= 1e-6  # atomics: summation order may differ
    # the projection puts all emission on the image: its lambda-integrated total
    # equals the NN render's only in expectation, but both are non-trivial
    assert cubes[0].max() > 0 and cubes[2].max() > 0
    ctx.drop_snapshot(sid)


def test_projection_has_no_neighbour_indices(ctx):
    s = synth.loop_snapshot(8, seed=2)
    t = synth.line_table()
    sid = ctx.snapshot(s)
    tid = ctx.table(t)
    req = ctx.request(sid, tid, fg.METHOD_PROJECTION, 8, 8, 8, 8, 0.1, 0.1, 1e5)
    with pytest.raises(fg.FomoError) as ei:
        ctx.render(req, want_idx=True)
    assert ei.value.code == fg.EINVAL
    ctx.drop_snapshot(sid)
