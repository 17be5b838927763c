"""GPU: the headline configurations themselves, against the oracle.

* The batched workload that bench.py times: one 2,097,152-point loop snapshot x
  64 views (l uniform in [0, 90 deg], b uniform in [-20, 20 deg], seeded) x 4
  lines, 256 x 256 px, 64 lambda bins, 512 LOS samples, rendered by one
  fomo_render_batch_graph call and replayed from the same graph with a second
  set of angles.
* The plain single-request configuration: 512 x 512 px, 128 bins, 512 LOS
  samples at l = 0, 30 and 60 deg, b = 0.

Reference behaviour: the view loop and spectral binning of
fomo-nearestneighbour.cpp:145-229, with the Doppler term of :204 exercised by
the b != 0 views.  Neighbour indices are compared bit for bit with the
oracle's on sampled image rows, cubes within 1e-4 normalised max error.
"""

import math

import numpy as np
import pytest

import bench
import fomo_gb300 as fg
import oracle
from fomo_gb300 import synth
from tests import _golden as G

pytestmark = pytest.mark.gpu

TOL = 1e-4  # max|g - o| / max|o| against the FP64 oracle
ROWS = ((1, 3), (127, 129), (253, 255))  # image rows compared: both edges and the middle
BATCHED = "batched 2M-point loop, 64 views x 4 lines, 256x256 px, 64 bins, 512 samples (sampled rows)"
PLAIN = "plain 2M-point loop, 512x512 px, 128 bins, 512 samples, l = 0/30/60 (sampled rows)"


@pytest.fixture(scope="module")
def workload():
    snap, tables, ls, bs = bench.make_workload()
    payload = [oracle.emission(snap, t) for t in tables]
    return snap, tables, ls, bs, payload


def _checked_views(ls, bs):
    """The largest |b|, the smallest and largest l, and one more view."""
    return sorted({int(np.argmax(np.abs(bs))), int(np.argmin(ls)), int(np.argmax(ls)), 17})


def test_batched_workload_graph_replays_match_oracle(workload):
    import torch

    snap, tables, ls, bs, payload = workload
    nl = len(tables)
    rng = np.random.default_rng(7)
    angle_sets = [(ls, bs), (rng.uniform(0.0, math.pi / 2, bench.NVIEWS), rng.uniform(-math.pi / 9, math.pi / 9,
                                                                                         bench.NVIEWS))]
    with fg.Context(0) as ctx:
        sid = ctx.snapshot(snap)
        tids = [ctx.table(t) for t in tables]
        dev = torch.device("cuda", 0)
        outs = [torch.empty((bench.NY, bench.NX, bench.NL), dtype=torch.float32, device=dev)
                for _ in range(bench.NVIEWS * nl)]
        ptrs = [o.data_ptr() for o in outs]
        for lv, bv in angle_sets:  # the second set replays the graph captured by the first
            reqs = [ctx.request(sid, tid, fg.METHOD_NN, bench.NX, bench.NY, bench.NZ, bench.NL, float(lv[v]),
                                float(bv[v]), bench.WIDTH) for v in range(bench.NVIEWS) for tid in tids]
            for o in outs:
                o.fill_(float("nan"))
            ctx.render_batch_device(reqs, ptrs, graph=True)
            ctx.synchronize()
            for v in _checked_views(lv, bv):
                idx = None
                for li in range(nl):
                    q = reqs[v * nl + li]
                    got = outs[v * nl + li].cpu().numpy()
                    # the same request alone (a 1-line launch) gives the same bits
                    single, sidx, info = ctx.render(q, want_idx=(li == 0))
                    np.testing.assert_array_equal(got, single)
                    if li == 0:
                        idx = sidx
                    eps, w = payload[li]
                    for r0, r1 in ROWS:
                        oc, oi, ov = oracle.nn_render(snap, eps, w, tables[li].lambda0, float(lv[v]), float(bv[v]),
                                                      bench.NX, bench.NY, bench.NZ, bench.NL, bench.WIDTH,
                                                      rows=(r0, r1), want_idx=(li == 0))
                        if li == 0:
                            G.record_idx(BATCHED, idx[r0:r1], oi)
                            np.testing.assert_array_equal(idx[r0:r1], oi)
                        assert info.maxdistance == ov[oracle.V_MAXDIST]
                        assert info.pathlength == ov[oracle.V_PATHLENGTH]
                        if np.abs(oc).max() > 0:
                            err = G.record(BATCHED, got[r0:r1].ravel(), oc.ravel())
                            assert err <= TOL, (v, li, r0, err)
                assert (idx >= 0).mean() > 0.3  # the views do see the loop
        ctx.drop_snapshot(sid)


@pytest.fixture(scope="module")
def plain():
    s = synth.loop_snapshot(128, seed=1)
    t = synth.line_table()
    eps, w = oracle.emission(s, t)
    with fg.Context(0) as ctx:
        sid = ctx.snapshot(s)
        tid = ctx.table(t)
        yield ctx, sid, tid, s, t, eps, w


@pytest.mark.parametrize("l_deg", [0.0, 30.0, 60.0])
def test_plain_config_views_sampled_rows(plain, l_deg):
    """2,097,152 points, 512 x 512 px, 128 bins, 512 samples, b = 0: neighbour
    indices of sampled rows bit-exact, their spectra within 1e-4."""
    ctx, sid, tid, s, t, eps, w = plain
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    l = math.radians(l_deg)
    req = ctx.request(sid, tid, fg.METHOD_NN, 512, 512, 512, 128, l, 0.0, width)
    cube, idx, info = ctx.render(req, want_idx=True)
    for r0 in (3, 255, 509):
        oc, oi, ov = oracle.nn_render(s, eps, w, t.lambda0, l, 0.0, 512, 512, 512, 128, width, rows=(r0, r0 + 2),
                                      want_idx=True)
        G.record_idx(PLAIN, idx[r0:r0 + 2], oi)
        np.testing.assert_array_equal(idx[r0:r0 + 2], oi)
        assert info.maxdistance == ov[oracle.V_MAXDIST]
        if np.abs(oc).max() > 0:
            assert G.record(PLAIN, cube[r0:r0 + 2].ravel(), oc.ravel()) <= TOL
    assert (idx >= 0).mean() > 0.5
