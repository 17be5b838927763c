"""AMRVAC snapshot ingestion (row f3): the reference's AMRVAC reader
(fomo-c/example/example_mpi_amrvac/read_amrvac_files.cpp) restated, and its
GPU implementation (fomo_snapshot_from_amrvac / fomo_amrvac_points, the C++
read_amrvac_dat_file of include/FoMo-amrvac.h).

CPU: the synthetic data files of tests/golden/amrvac_files.py are the same
bytes as when the golden points were made, and the oracle reads from them the
points the reference's own reader read (tests/golden/amrvac.npz, bit for bit):
3-D and 2-D data with a refined block, version 4 and pre-2017 files, Morton
and x-fastest leaf orders; a version-3 file of the same data reads the same.
GPU: the library's points are the same bits, a snapshot read from the file
renders exactly as one made from those points, and a C++ user program gets
them through read_amrvac_dat_file.
"""

import hashlib
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

import fomo_gb300 as fg
import oracle
from tests import _golden as G

sys.path.insert(0, G.GOLDEN)
import amrvac_files as A  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = ("x", "y", "z", "n", "T", "vx", "vy", "vz")


@pytest.fixture(scope="module")
def golden():
    return G.load("amrvac.npz")


def _expected(d, name):
    return int(d[name + "_ndim"]), [d[f"{name}_{k}"] for k in KEYS]


@pytest.mark.parametrize("name", sorted(A.CASES))
def test_writer_is_deterministic_and_oracle_reads_reference_points(golden, tmp_path, name):
    dat, par, kw = A.write_case(name, str(tmp_path))
    assert hashlib.sha256(open(dat, "rb").read()).hexdigest() == str(golden[name + "_sha256"])
    if par:
        assert hashlib.sha256(open(par, "rb").read()).hexdigest() == str(golden[name + "_par_sha256"])
    nd, want = _expected(golden, name)
    ond, got = oracle.amrvac_read(dat, par, **kw)
    assert ond == nd
    for k, a, b in zip(KEYS, got, want):
        np.testing.assert_array_equal(a, b, err_msg=k)


def test_version3_file_reads_like_version4(golden, tmp_path):
    """Version 3 differs from 4 in the gamma name's match only (the reference's
    dispatch falls through to its pre-2017 reader after the version-3 one; the
    restatement reads a version-3 file with the version-3 reader alone)."""
    dat = str(tmp_path / "v3.dat")
    A.write_new(dat, version=3, ndim=3, pad=b" ")
    nd, want = _expected(golden, "v4_3d")
    ond, got = oracle.amrvac_read(dat, None, "gitlab", 0, **A.UNITS)
    assert ond == nd
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)


def test_cpp_reader_header_compiles(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    if not os.path.exists(fg.LIB_PATH):
        from fomo_gb300 import build
        build.build()
    libdir = os.path.dirname(fg.LIB_PATH)
    exe = str(tmp_path / "amrvac_points")
    r = subprocess.run(["g++", "-std=c++11", "-O1", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "amrvac_points.cpp"), "-L", libdir, "-lfomo_gpu",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


# ---------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(A.CASES))
def test_gpu_points_and_snapshot_match_reference(golden, tmp_path, name):
    dat, par, kw = A.write_case(name, str(tmp_path))
    nd, want = _expected(golden, name)
    with fg.Context(0) as ctx:
        gnd, got = ctx.amrvac_points(dat, par, **kw)
        assert gnd == nd
        for k, a, b in zip(KEYS, got, want):
            np.testing.assert_array_equal(a, b, err_msg=k)
        # the snapshot read from the file renders as the one made from the points
        sid_f = ctx.snapshot_from_amrvac(dat, par, **kw)
        from fomo_gb300 import synth
        pts = synth.Snapshot(*[np.ascontiguousarray(a) for a in want])
        sid_p = ctx.snapshot(pts)
        t = synth.line_table()
        tid = ctx.table(t)
        width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
        for (l, b) in ((0.3, 0.2), (1.1, -0.4)):
            cf, i_f, _ = ctx.render(ctx.request(sid_f, tid, fg.METHOD_NN, 24, 20, 40, 16, l, b, width), want_idx=True)
            cp, i_p, _ = ctx.render(ctx.request(sid_p, tid, fg.METHOD_NN, 24, 20, 40, 16, l, b, width), want_idx=True)
            np.testing.assert_array_equal(i_f, i_p)
            np.testing.assert_array_equal(cf, cp)
            eps, w = oracle.emission(pts, t)
            oc, oi, _ = oracle.nn_render(pts, eps, w, t.lambda0, l, b, 24, 20, 40, 16, width, want_idx=True)
            np.testing.assert_array_equal(i_f, oi)
            if np.abs(oc).max() > 0:
                assert G.norm_max_err(cf, oc) <= 1e-4


@pytest.mark.gpu
def test_gpu_reader_errors(tmp_path):
    dat, par, kw = A.write_case("old_3d_gitlab", str(tmp_path))
    with fg.Context(0) as ctx:
        with pytest.raises(fg.FomoError) as ei:
            ctx.amrvac_points(str(tmp_path / "absent.dat"))
        assert ei.value.code == fg.EIO
        with pytest.raises(fg.FomoError) as ei:
            ctx.amrvac_points(dat, str(tmp_path / "absent.par"), "gitlab", 1, **A.UNITS)
        assert ei.value.code == fg.EIO
        with pytest.raises(fg.FomoError) as ei:
            ctx.amrvac_points(dat, par, "newest", 1, **A.UNITS)
        assert ei.value.code == fg.EINVAL
        bad = str(tmp_path / "truncated.dat")
        A.write_new(bad)
        with open(bad, "r+b") as f:
            f.truncate(os.path.getsize(bad) // 2)
        with pytest.raises(fg.FomoError) as ei:
            ctx.amrvac_points(bad)
        assert ei.value.code == fg.ETABLE


@pytest.mark.gpu
def test_cpp_read_amrvac_dat_file(golden, tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    libdir = os.path.dirname(fg.LIB_PATH)
    exe = str(tmp_path / "amrvac_points")
    r = subprocess.run(["g++", "-std=c++11", "-O1", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "amrvac_points.cpp"), "-L", libdir, "-lfomo_gpu",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for name in ("v4_2d", "old_3d_gitlab"):
        dat, par, kw = A.write_case(name, str(tmp_path))
        out = str(tmp_path / (name + ".bin"))
        r = subprocess.run([exe, dat, par or "", kw["amrvac_version"], str(kw["gamma_eqparposition"]),
                            repr(kw["n_unit"]), repr(kw["Teunit"]), repr(kw["L_unit"]), out],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        nd, want = _expected(golden, name)
        gnd, n = (int(v) for v in r.stdout.split()[-2:])
        assert (gnd, n) == (nd, want[0].size)
        cols = np.fromfile(out, np.float32).reshape(nd + 5, n)
        keys = [k for k in KEYS if nd == 3 or k != "z"]
        for k, col in zip(keys, cols):
            np.testing.assert_array_equal(col, want[KEYS.index(k)], err_msg=k)
