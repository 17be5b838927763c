"""The nonuniform / Thomson configuration at full size on the GPU.

8,388,608 points: 80 % in a twisted flux rope, 20 % uniform background
(fomo_gb300.synth.flux_rope_snapshot), n log-uniform in 1e8..1e10, T in
5e5..5e6 K.  Six broadband response tables with a DN unit (imaging, arcsec
grid, per-pixel scaling) rendered together at 1024 x 1024 pixels and 1024 LOS
samples; Thomson pB of the same cloud moved to 1.5 solar radii, off the
equator (b = 0.3 rad), where the reference's box is 200 pixels wide
(fomo-thomson.cpp:249-260) and most samples take a distant neighbour.

Sampled image rows are compared with the oracle: cubes within 1e-4
(normalised max error over the rows), and -- at 256 x 256 pixels with the same
1024 samples -- the neighbour index of every sample of the rows bit for bit.
"""

import numpy as np
import pytest

import fomo_gb300 as fg
import oracle
from fomo_gb300 import synth
from tests import _golden as G

pytestmark = pytest.mark.gpu

N_POINTS = 8 * 1024 * 1024
CHANNELS = (94, 131, 171, 193, 211, 335)
TOL = 1e-4
DN6 = "8M-point flux rope, 6 DN channels, 1024x1024 px, 1024 samples (sampled rows)"
THOMSON = "8M-point flux rope at 1.5 Rsun, Thomson pB, b = 0.3, 1024x1024 px (sampled rows)"
WIDE = "512K-point flux rope, 64x64 px, 16 bins, 256 samples, wide boxes (full cubes)"


@pytest.fixture(scope="module")
def ctx():
    with fg.Context(0) as c:
        yield c


@pytest.fixture(scope="module")
def rope():
    return synth.flux_rope_snapshot(N_POINTS, seed=4)


def test_six_dn_channels_full_size_sampled_rows(ctx, rope):
    tabs = [synth.broadband_table(c, peak_logT=5.8 + 0.15 * k) for k, c in enumerate(CHANNELS)]
    sid = ctx.snapshot(rope)
    tids = [ctx.table(t) for t in tabs]
    l, b = 0.6, 0.35
    reqs = [ctx.request(sid, tid, fg.METHOD_NN, 1024, 1024, 1024, 1, l, b, 1e5) for tid in tids]
    cubes, infos = ctx.render_batch(reqs)
    assert all(i.is_dn == 1 for i in infos)
    for k in (0, 3):
        eps, w = oracle.emission(rope, tabs[k], imaging=True)
        for r0 in (200, 700):
            oc, _, ov = oracle.nn_render(rope, eps, w, tabs[k].lambda0, l, b, 1024, 1024, 1024, 1, 1e5, is_dn=True,
                                         rows=(r0, r0 + 1))
            assert infos[k].maxdistance == ov[oracle.V_MAXDIST] and infos[k].apix == ov[oracle.V_APIX]
            assert G.record(DN6, cubes[k][r0:r0 + 1].ravel(), oc.ravel()) <= TOL
    # neighbour indices at 256 x 256 (1024 samples per ray), sampled rows
    q = ctx.request(sid, tids[2], fg.METHOD_NN, 256, 256, 1024, 1, l, b, 1e5)
    cube, idx, info = ctx.render(q, want_idx=True)
    eps, w = oracle.emission(rope, tabs[2], imaging=True)
    for r0 in (40, 128, 230):
        oc, oi, _ = oracle.nn_render(rope, eps, w, tabs[2].lambda0, l, b, 256, 256, 1024, 1, 1e5, is_dn=True,
                                     rows=(r0, r0 + 1), want_idx=True)
        G.record_idx(DN6, idx[r0:r0 + 1], oi)
        np.testing.assert_array_equal(idx[r0:r0 + 1], oi)
    ctx.drop_snapshot(sid)


def test_thomson_off_equator_full_size_sampled_rows(ctx):
    ts = synth.flux_rope_snapshot(N_POINTS, seed=5, center=(1.5 * 695.7, 0.0, 0.0))
    sid = ctx.snapshot(ts)
    l, b = 0.2, 0.3
    q = ctx.request(sid, 0, fg.METHOD_THOMSON, 1024, 1024, 1024, 1, l, b, 1e5)
    cube, _, info = ctx.render(q)
    tot, pol = oracle.thomson_emission(ts)
    for r0 in (600,):  # the oracle's far searches take seconds per row
        oc, _, ov = oracle.thomson_render(ts, tot, pol, l, b, 1024, 1024, 1024, rows=(r0, r0 + 1))
        assert info.maxdistance == ov[oracle.V_MAXDIST]
        assert G.record(THOMSON, cube[r0:r0 + 1].ravel(), oc.ravel()) <= TOL
    q = ctx.request(sid, 0, fg.METHOD_THOMSON, 256, 256, 1024, 1, l, b, 1e5)
    cube, idx, info = ctx.render(q, want_idx=True)
    assert (idx >= 0).mean() > 0.9  # the wide boxes give nearly every sample a neighbour
    for r0 in (20, 131):
        _, oi, _ = oracle.thomson_render(ts, tot, pol, l, b, 256, 256, 1024, rows=(r0, r0 + 1), want_idx=True)
        G.record_idx(THOMSON, idx[r0:r0 + 1], oi)
        np.testing.assert_array_equal(idx[r0:r0 + 1], oi)
    ctx.drop_snapshot(sid)


def test_wide_boxes_dense_cells_full_cube(ctx):
    """A 524,288-point flux rope at 64 x 64 pixels and 256 LOS samples: boxes
    about 1 Mm wide and rope cells of ~90 points, where one lane's ring search
    runs out of budget and whole warps search those samples (march_hard).
    Every sample's neighbour index equal to the oracle's, the cube within 1e-4."""
    s = synth.flux_rope_snapshot(512 * 1024, seed=20)
    t = synth.line_table()
    sid, tid = ctx.snapshot(s), ctx.table(t)
    eps, w = oracle.emission(s, t)
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    for (l, b) in ((0.5, 0.2), (1.2, -0.3)):
        cube, idx, _ = ctx.render(ctx.request(sid, tid, fg.METHOD_NN, 64, 64, 256, 16, l, b, width), want_idx=True)
        oc, oi, _ = oracle.nn_render(s, eps, w, t.lambda0, l, b, 64, 64, 256, 16, width, want_idx=True)
        G.record_idx(WIDE, idx, oi)
        np.testing.assert_array_equal(idx, oi)
        assert G.record(WIDE, cube.ravel(), oc.ravel()) <= TOL
    ctx.drop_snapshot(sid)

