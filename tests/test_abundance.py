"""Abundance renormalisation (fomo_abundance_ratio; fomo-CHIANTI.cpp:23-62,
264-273) against the oracle's restatement, on CPU: the library parses two
CHIANTI-format abundance files and divides the element's abundance relative
to hydrogen; a file without the element or without hydrogen is an error."""

import pytest

import fomo_gb300 as fg
import oracle


def _write(path, rows, end="-1"):
    with open(path, "w") as f:
        for z, v, sym in rows:
            f.write(f" {z:2d}  {v:6.2f}  {sym}\n")
        f.write(f" {end}\n")
        f.write("comment lines after the terminator are ignored\n")
    return str(path)


def test_ratio_matches_oracle(tmp_path):
    std = _write(tmp_path / "std.abund", [(1, 12.00, "H"), (2, 10.93, "He"), (26, 7.85, "Fe"), (8, 8.69, "O")])
    new = _write(tmp_path / "new.abund", [(1, 12.00, "H"), (26, 7.50, "FE"), (8, 8.83, "o")])
    for ion in ("fe_12", "Fe_9", "o_6"):
        got = fg.abundance_ratio(new, std, ion)
        assert got == pytest.approx(oracle.abundance_ratio(new, std, ion), rel=1e-15)
    assert fg.abundance_ratio(new, std, "fe_12") == pytest.approx(10 ** (7.50 - 7.85), rel=1e-13)
    assert fg.abundance_ratio(std, std, "o_6") == 1.0


def test_missing_element_or_file_is_an_error(tmp_path):
    std = _write(tmp_path / "std.abund", [(1, 12.00, "H"), (26, 7.85, "Fe")])
    noh = _write(tmp_path / "noh.abund", [(26, 7.5, "Fe")])
    with pytest.raises(fg.FomoError) as ei:
        fg.abundance_ratio(std, std, "si_10")
    assert ei.value.code == fg.ETABLE
    with pytest.raises(fg.FomoError):
        fg.abundance_ratio(noh, std, "fe_12")
    with pytest.raises(fg.FomoError):
        fg.abundance_ratio(str(tmp_path / "absent.abund"), std, "fe_12")


@pytest.mark.gpu
def test_render_with_abundance_ratio_matches_oracle(tmp_path):
    """A spectroscopic render with abundratio != 1 (fomo-CHIANTI.cpp:264-273,
    applied to the emissivity at :292-293): neighbour indices bit-exact and the
    cube within 1e-4 of the oracle's, the emissivity within 1e-5, and the cube
    equal to ratio x the render at abundratio 1 up to FP32 rounding."""
    import numpy as np

    from fomo_gb300 import synth
    from tests import _golden as G

    std = _write(tmp_path / "std.abund", [(1, 12.00, "H"), (26, 7.85, "Fe")])
    new = _write(tmp_path / "new.abund", [(1, 12.00, "H"), (26, 7.50, "Fe")])
    ratio = fg.abundance_ratio(new, std, "fe_12")
    assert ratio == pytest.approx(10 ** (7.50 - 7.85), rel=1e-13)
    s = synth.loop_snapshot(16, seed=5)
    t = synth.line_table(lambda0=193.509, ion="fe_12")
    eps, w = oracle.emission(s, t, abundratio=ratio)
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    with fg.Context(0) as ctx:
        sid, tid = ctx.snapshot(s), ctx.table(t)
        e_gpu, w_gpu = ctx.emission(sid, tid, abundratio=ratio)
        assert np.abs(e_gpu.astype(np.float64) - eps).max() <= 1e-5 * np.abs(eps).max()
        np.testing.assert_array_equal(w_gpu, w)
        req = ctx.request(sid, tid, fg.METHOD_NN, 20, 16, 40, 32, 0.4, 0.25, width, abundratio=ratio)
        cube, idx, _ = ctx.render(req, want_idx=True)
        ocube, oidx, _ = oracle.nn_render(s, eps, w, t.lambda0, 0.4, 0.25, 20, 16, 40, 32, width, want_idx=True)
        np.testing.assert_array_equal(idx, oidx)
        assert G.norm_max_err(cube, ocube) <= 1e-4
        one, _, _ = ctx.render(ctx.request(sid, tid, fg.METHOD_NN, 20, 16, 40, 32, 0.4, 0.25, width, abundratio=1.0))
        assert G.norm_max_err(cube, one.astype(np.float64) * ratio) <= 1e-6
