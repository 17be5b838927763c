"""Pin the oracle (the C restatement) to the reference's own outputs.

The golden fixtures were produced by the reference's unmodified FoMo-C sources
(tests/golden/make_golden.py).  The oracle's FP32-mirror mode must reproduce
them bit for bit on the platform that generated them (same libm); its FP64
mode -- the parity target for the GPU -- must agree within 1e-5 normalised.
"""

import os

import numpy as np
import pytest

import oracle
from tests import _golden as G

CASES_NN = ["nn_spectro.npz", "nn_imaging.npz", "nn_medium.npz"]


def _check_bits(got, ref, d, tol=1e-6):
    if G.same_platform(d):
        np.testing.assert_array_equal(np.asarray(got, np.float32), ref)
    else:  # another libm: allow last-bit differences
        assert G.norm_max_err(got, ref) <= tol


def test_table_parse_matches_reference_text(golden_dir):
    d = G.load("nn_spectro.npz")
    path = G.table_file(d)
    try:
        tb = oracle.table_read(path)
    finally:
        os.unlink(path)
    t = G.table(d)
    assert tb["ion"] == t.ion and tb["unit"] == t.unit
    assert tb["lambda0"] == t.lambda0 and tb["atweight"] == t.atweight
    np.testing.assert_array_equal(tb["logT"], t.logT)
    np.testing.assert_array_equal(tb["logn"], t.logn)
    np.testing.assert_array_equal(tb["G"], t.G)


@pytest.mark.parametrize("name,imaging", [("nn_spectro.npz", False), ("nn_imaging.npz", True),
                                          ("nn_edges.npz", False), ("nn_medium.npz", False)])
def test_emission_matches_reference(name, imaging):
    d = G.load(name)
    s = G.snapshot(d)
    t = G.table(d)
    eps, w = oracle.emission(s, t, imaging=imaging)
    _check_bits(eps, d["eps"], d)
    _check_bits(w, d["fwhm"], d)


def test_thomson_emission_matches_reference():
    d = G.load("thomson.npz")
    s = G.snapshot(d)
    tot, pol = oracle.thomson_emission(s)
    _check_bits(tot, d["tot"], d)
    _check_bits(pol, d["pol"], d)


def _nn_cases(d, suffix=""):
    views = d["views" + suffix]
    nx, ny, nz, L = (int(v) for v in d["res" + suffix])
    return views, nx, ny, nz, L, d["cube" + suffix], d["meta" + suffix]


@pytest.mark.parametrize("name", CASES_NN)
def test_nn_render_mirror_is_bit_exact_and_fp64_close(name):
    d = G.load(name)
    s = G.snapshot(d)
    t = G.table(d)
    views, nx, ny, nz, L, cubes, metas = _nn_cases(d)
    eps, w = d["eps"], d["fwhm"]
    for v, (l, b) in enumerate(views):
        width = metas[v][4]
        mirror, _, _ = oracle.nn_render(s, eps, w, t.lambda0, l, b, nx, ny, nz, L, width, is_dn=t.is_dn, mode=1)
        _check_bits(mirror.ravel(), cubes[v], d)
        fp64, _, _ = oracle.nn_render(s, eps, w, t.lambda0, l, b, nx, ny, nz, L, width, is_dn=t.is_dn, mode=0)
        assert G.norm_max_err(fp64.ravel(), cubes[v]) <= 1e-5


def test_nn_render_edges():
    d = G.load("nn_edges.npz")
    s = G.snapshot(d)
    t = G.table(d)
    for suffix in ("_a", "_b"):
        views, nx, ny, nz, L, cubes, metas = _nn_cases(d, suffix)
        for v, (l, b) in enumerate(views):
            mirror, _, _ = oracle.nn_render(s, d["eps"], d["fwhm"], t.lambda0, l, b, nx, ny, nz, L, metas[v][4],
                                            mode=1)
            _check_bits(mirror.ravel(), cubes[v], d)


def test_thomson_render_mirror_is_bit_exact():
    d = G.load("thomson.npz")
    s = G.snapshot(d)
    views, nx, ny, nz, L, cubes, metas = _nn_cases(d)
    for v, (l, b) in enumerate(views):
        mirror, _, _ = oracle.thomson_render(s, d["tot"], d["pol"], l, b, nx, ny, nz, mode=1)
        _check_bits(mirror.ravel(), cubes[v], d)
        fp64, _, _ = oracle.thomson_render(s, d["tot"], d["pol"], l, b, nx, ny, nz, mode=0)
        assert G.norm_max_err(fp64.ravel(), cubes[v]) <= 1e-5


@pytest.mark.parametrize("suffix,ek,wk,tk", [("_a", "eps", "fwhm", "table_text"),
                                              ("_b", "eps_band", "fwhm_band", "band_text")])
def test_projection_render_mirror_is_bit_exact_and_fp64_close(suffix, ek, wk, tk):
    d = G.load("projection.npz")
    s = G.snapshot(d)
    t = G.table(d, tk)
    views, nx, ny, nz, L, cubes, metas = _nn_cases(d, suffix)
    for v, (l, b) in enumerate(views):
        mirror, pix, _ = oracle.projection_render(s, d[ek], d[wk], t.lambda0, l, b, nx, ny, nz, L, metas[v][4],
                                                  is_dn=t.is_dn, mode=1, want_pix=True)
        _check_bits(mirror.ravel(), cubes[v], d)
        assert pix.min() >= 0 and pix.max() < nx * ny
        fp64, _, _ = oracle.projection_render(s, d[ek], d[wk], t.lambda0, l, b, nx, ny, nz, L, metas[v][4],
                                              is_dn=t.is_dn, mode=0)
        assert G.norm_max_err(fp64.ravel(), cubes[v]) <= 1e-5


@pytest.mark.parametrize("name", ["nn_spectro.npz", "nn_imaging.npz"])
def test_render_grids_match_reference(name):
    d = G.load(name)
    t = G.table(d)
    views, nx, ny, nz, L, cubes, metas = _nn_cases(d)
    s = G.snapshot(d)
    for v, (l, b) in enumerate(views):
        _, _, view = oracle.nn_render(s, d["eps"], d["fwhm"], t.lambda0, l, b, nx, ny, nz, L, metas[v][4],
                                      is_dn=t.is_dn, mode=1)
        gx, gy, gl = oracle.render_grid(nx, ny, L, view, t.lambda0, is_dn=t.is_dn)
        np.testing.assert_array_equal(gx, d["gx"][v])
        np.testing.assert_array_equal(gy, d["gy"][v])
        if L > 1:
            np.testing.assert_array_equal(gl, d["glambda"][v])


@pytest.mark.parametrize("l,b", [(0.0, 0.0), (0.7, 0.5), (2.5, -1.0)])
def test_grid_search_equals_bruteforce(l, b):
    d = G.load("nn_medium.npz")
    s = G.snapshot(d)
    t = G.table(d)
    _, idx_grid, _ = oracle.nn_render(s, d["eps"], d["fwhm"], t.lambda0, l, b, 12, 10, 24, 4, 1e5, want_idx=True)
    _, idx_bf, _ = oracle.nn_render(s, d["eps"], d["fwhm"], t.lambda0, l, b, 12, 10, 24, 4, 1e5, mode=2,
                                    want_idx=True)
    np.testing.assert_array_equal(idx_grid, idx_bf)
    assert (idx_grid >= 0).mean() > 0.5


def test_thomson_grid_search_equals_bruteforce():
    d = G.load("thomson.npz")
    s = G.snapshot(d)
    _, i1, _ = oracle.thomson_render(s, d["tot"], d["pol"], 0.3, 0.4, 10, 9, 12, want_idx=True)
    _, i2, _ = oracle.thomson_render(s, d["tot"], d["pol"], 0.3, 0.4, 10, 9, 12, mode=2, want_idx=True)
    np.testing.assert_array_equal(i1, i2)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference build exists only where the reference tree is")
def test_live_reference_agrees_on_fresh_case(tmp_path):
    """A case not in the fixtures, rendered live by the reference build."""
    from fomo_gb300 import synth
    s = synth.loop_snapshot(10, seed=11)
    t = synth.line_table(peak_logT=6.2, lambda0=211.317)
    p = str(tmp_path / "t.dat")
    synth.write_table(t, p)
    out, _, meta = oracle.ref_render("NearestNeighbour", s, p, 1.3, -0.7, 9, 11, 17, 12, 0.3)
    eps, w = oracle.emission(s, t)
    mirror, _, _ = oracle.nn_render(s, eps, w, t.lambda0, 1.3, -0.7, 9, 11, 17, 12, meta[4], mode=1)
    np.testing.assert_array_equal(mirror.ravel().astype(np.float32), out)
