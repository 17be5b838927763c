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
