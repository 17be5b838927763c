"""GPU parity: the CUDA path, called through the C ABI, against the oracle and
the reference's golden outputs.

Gates (floating point, written here): normalised max error
max|g - o| / max|o| <= 1e-4 against the FP64 oracle and against the
reference's own FP32 cubes; nearest-neighbour indices bit-exact against the
oracle; per-view extents, maxdistance and scales bit-exact (they are FP64
expressions evaluated in the reference's order).
"""

import os

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
    c = fg.Context(0)
    yield c
    c.close()


def _check_view(info, view):
    """Extents / maxdistance / path length / scale identical to the oracle's FP64 values."""
    assert info.minx == view[oracle.V_MINX] and info.maxx == view[oracle.V_MAXX]
    assert info.miny == view[oracle.V_MINY] and info.maxy == view[oracle.V_MAXY]
    assert info.minz == view[oracle.V_MINZ] and info.maxz == view[oracle.V_MAXZ]
    assert info.maxdistance == view[oracle.V_MAXDIST]
    assert info.pathlength == view[oracle.V_PATHLENGTH]
    assert info.scale == view[oracle.V_SCALE]


@pytest.mark.parametrize("name", ["nn_spectro.npz", "nn_medium.npz"])
def test_spectroscopic_golden(ctx, name):
    d = G.load(name)
    s = G.snapshot(d)
    t = G.table(d)
    sid = ctx.snapshot(s)
    tid = ctx.table(t)
    nx, ny, nz, L = (int(v) for v in d["res"])
    for v, (l, b) in enumerate(d["views"]):
        width = d["meta"][v][4]
        req = ctx.request(sid, tid, fg.METHOD_NN, nx, ny, nz, L, l, b, width)
        cube, idx, info = ctx.render(req, want_idx=True)
        ocube, oidx, oview = oracle.nn_render(s, d["eps"], d["fwhm"], t.lambda0, l, b, nx, ny, nz, L, width,
                                              want_idx=True)
        G.record_idx("golden " + name, idx, oidx)
        np.testing.assert_array_equal(idx, oidx)          # neighbours bit-exact
        _check_view(info, oview)
        assert G.record("golden " + name, cube.ravel(), ocube.ravel()) <= TOL      # vs FP64 oracle
        assert G.norm_max_err(cube.ravel(), d["cube"][v]) <= TOL       # vs the reference's own cube
        assert G.l2_rel_err(cube.ravel(), ocube.ravel()) <= TOL
    ctx.drop_snapshot(sid)
    ctx.drop_table(tid)


def test_emission_matches_reference(ctx):
    d = G.load("nn_spectro.npz")
    s = G.snapshot(d)
    path = G.table_file(d)
    try:
        tid = ctx.load_table(path)  # the C++ parser of the CHIANTI text format
    finally:
        os.unlink(path)
    sid = ctx.snapshot(s)
    eps, w = ctx.emission(sid, tid)
    np.testing.assert_array_equal(w, d["fwhm"])  # sqrt and FP64 scale: exact
    rel = np.abs(eps.astype(np.float64) - d["eps"]) / np.maximum(np.abs(d["eps"]), 1e-300)
    assert rel.max() <= 1e-5  # log10f(glibc) vs correctly rounded log10: ~1 ulp
    assert (eps == d["eps"]).mean() > 0.9
    info = ctx.table_info(tid)
    t = G.table(d)
    assert info["lambda0"] == t.lambda0 and info["ion"] == t.ion and info["nt"] == t.nt
    ctx.drop_snapshot(sid)


def test_imaging_dn_golden(ctx):
    d = G.load("nn_imaging.npz")
    s = G.snapshot(d)
    t = G.table(d)
    sid = ctx.snapshot(s)
    tid = ctx.table(t)
    nx, ny, nz, L = (int(v) for v in d["res"])
    for v, (l, b) in enumerate(d["views"]):
        req = ctx.request(sid, tid, fg.METHOD_NN, nx, ny, nz, 1, l, b, d["meta"][v][4])
        cube, idx, info = ctx.render(req, want_idx=True)
        ocube, oidx, oview = oracle.nn_render(s, d["eps"], d["fwhm"], t.lambda0, l, b, nx, ny, nz, 1,
                                              d["meta"][v][4], is_dn=True, want_idx=True)
        G.record_idx("golden nn_imaging.npz", idx, oidx)
        np.testing.assert_array_equal(idx, oidx)
        assert info.is_dn == 1 and info.observation_type == fg.OBS_IMAGING
        assert info.apix == oview[oracle.V_APIX]
        assert G.record("golden nn_imaging.npz", cube.ravel(), ocube.ravel()) <= TOL
        assert G.norm_max_err(cube.ravel(), d["cube"][v]) <= TOL
        gx, gy, _ = fg.render_grid(nx, ny, 1, info, True)
        np.testing.assert_array_equal(gx, d["gx"][v])
        np.testing.assert_array_equal(gy, d["gy"][v])
    ctx.drop_snapshot(sid)


def test_thomson_golden(ctx):
    d = G.load("thomson.npz")
    s = G.snapshot(d)
    sid = ctx.snapshot(s)
    nx, ny, nz, L = (int(v) for v in d["res"])
    for v, (l, b) in enumerate(d["views"]):
        req = ctx.request(sid, 0, fg.METHOD_THOMSON, nx, ny, nz, 1, l, b, 1e5)
        cube, idx, info = ctx.render(req, want_idx=True)
        ocube, oidx, oview = oracle.thomson_render(s, d["tot"], d["pol"], l, b, nx, ny, nz, want_idx=True)
        G.record_idx("golden thomson.npz", idx, oidx)
        np.testing.assert_array_equal(idx, oidx)
        _check_view(info, oview)
        assert G.record("golden thomson.npz", cube.ravel(), ocube.ravel()) <= TOL
        assert G.norm_max_err(cube.ravel(), d["cube"][v]) <= TOL
    ctx.drop_snapshot(sid)


def test_edges_golden(ctx):
    d = G.load("nn_edges.npz")
    s = G.snapshot(d)
    t = G.table(d)
    sid = ctx.snapshot(s)
    tid = ctx.table(t)
    for suffix in ("_a", "_b"):
        nx, ny, nz, L = (int(v) for v in d["res" + suffix])
        for v, (l, b) in enumerate(d["views" + suffix]):
            width = d["meta" + suffix][v][4]
            req = ctx.request(sid, tid, fg.METHOD_NN, nx, ny, nz, L, l, b, width)
            cube, idx, info = ctx.render(req, want_idx=True)
            ocube, oidx, oview = oracle.nn_render(s, d["eps"], d["fwhm"], t.lambda0, l, b, nx, ny, nz, L, width,
                                                  want_idx=True)
            np.testing.assert_array_equal(idx, oidx)
            _check_view(info, oview)
            assert G.norm_max_err(cube.ravel(), d["cube" + suffix][v]) <= TOL
    ctx.drop_snapshot(sid)


LOOP64 = "262K-point loop, 128x128 px, 64 bins, 256 samples, 3 views (full cubes)"


@pytest.mark.parametrize("l,b", [(0.0, 0.0), (0.5236, 0.0), (0.4, -0.3)])
def test_loop_64cubed_reference_scale(ctx, l, b):
    """The CPU-scale loop (64^3 points, 128x128 pixels, 64 bins, 256 samples) with b = 0 and b != 0."""
    s = synth.loop_snapshot(64, seed=1)
    t = synth.line_table()
    eps, w = oracle.emission(s, t)
    sid = ctx.snapshot(s)
    tid = ctx.table(t)
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    req = ctx.request(sid, tid, fg.METHOD_NN, 128, 128, 256, 64, l, b, width)
    cube, idx, info = ctx.render(req, want_idx=True)
    ocube, oidx, oview = oracle.nn_render(s, eps, w, t.lambda0, l, b, 128, 128, 256, 64, width, want_idx=True)
    G.record_idx(LOOP64, idx, oidx)
    np.testing.assert_array_equal(idx, oidx)
    _check_view(info, oview)
    assert G.record(LOOP64, cube.ravel(), ocube.ravel()) <= TOL
    ctx.drop_snapshot(sid)


def test_imaging_with_line_table_is_rejected_like_the_reference(ctx):
    """fomo-CHIANTI.cpp:278 exits when an imaging render uses a table whose ion
    field is not the channel wavelength; here it is an error code, not exit()."""
    s = synth.loop_snapshot(8, seed=2)
    sid = ctx.snapshot(s)
    tid = ctx.table(synth.line_table())
    with pytest.raises(fg.FomoError) as ei:
        ctx.render(ctx.request(sid, tid, fg.METHOD_NN, 8, 8, 8, 1, 0.0, 0.0, 1e5))
    assert ei.value.code == fg.ETABLE
    ctx.drop_snapshot(sid)


def test_batch_equals_single_renders(ctx):
    """Views and lines batched into one launch give the same bits as rendered alone."""
    s = synth.loop_snapshot(24, seed=5)
    tabs = [synth.line_table(peak_logT=p, lambda0=lam) for p, lam in ((5.8, 171.0), (6.0, 193.0), (6.2, 211.0))]
    sid = ctx.snapshot(s)
    tids = [ctx.table(t) for t in tabs]
    reqs = []
    for v, (l, b) in enumerate([(0.1, 0.2), (0.9, -0.1), (1.7, 0.3)]):
        for tid in tids:
            reqs.append(ctx.request(sid, tid, fg.METHOD_NN, 20, 18, 40, 24, l, b, 1.2e5))
    bb = ctx.table(synth.broadband_table(193))
    reqs.append(ctx.request(sid, bb, fg.METHOD_NN, 17, 13, 33, 1, 0.3, 0.4, 1e5))  # imaging in the mix
    cubes, infos = ctx.render_batch(reqs)
    for r, q in enumerate(reqs):
        single, _, _ = ctx.render(q)
        np.testing.assert_array_equal(cubes[r], single)
    ctx.drop_snapshot(sid)
