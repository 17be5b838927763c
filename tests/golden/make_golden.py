"""Generate the golden fixtures in this directory from the reference itself.

The reference's own FoMo-C sources (fomo-c/src, unmodified) are compiled in
this container by ``make -C oracle ref`` with header shims for the absent GSL
constants and Boost.Geometry rtree (see oracle/refshim/).  This script drives
them through the public FoMoObject API (oracle/ref_driver.cpp) on small seeded
synthetic cases and stores inputs and outputs as compressed .npz files:

    nn_spectro.npz   NearestNeighbour, spectroscopic, several (l, b) views
    nn_imaging.npz   NearestNeighbour, broadband DN table (imaging, L = 1)
    nn_edges.npz     ragged sizes, nz = 1, empty corners, out-of-table points
    thomson.npz      Thomson (pB) views
    nn_medium.npz    a larger spectroscopic case (24^3 points, 32x32x48, L = 32)
    projection.npz   Projection renders (spectroscopic, and imaging with a DN table)
    writer_*.txt/.dat the reference's own text and binary output files of three
                     small renders (spectroscopic, DN imaging, Thomson), with
                     their inputs in writers.npz
    amrvac.npz       the points the reference's AMRVAC reader (fomo-c/example/
                     example_mpi_amrvac/read_amrvac_files.cpp) reads from the
                     synthetic data files of amrvac_files.py (3-D and 2-D AMR,
                     version 4 and pre-2017 formats, both leaf orders), with the
                     files' SHA-256 (the writer is deterministic)

Run from the repository root:  python tests/golden/make_golden.py [amrvac]
(``amrvac`` regenerates amrvac.npz only.)
The fixtures are committed; the GPU machine has no reference tree and only reads them.
"""

from __future__ import annotations

import os
import platform
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
# one OpenMP thread: the reference's projection renderer accumulates with
# `omp atomic` in thread order; single-threaded its float sums are reproducible
os.environ["OMP_NUM_THREADS"] = "1"

import oracle  # noqa: E402
from fomo_gb300 import synth  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
C = 2.99792458e8


def _snap_dict(s):
    return dict(x=s.x, y=s.y, z=s.z, n=s.n, T=s.T, vx=s.vx, vy=s.vy, vz=s.vz)


def _table_dict(t, prefix="table"):
    return {f"{prefix}_text": np.frombuffer(synth.table_text(t, t.logT.astype(np.float64), t.logn.astype(np.float64),
                                                             t.G.astype(np.float64)).encode(), dtype=np.uint8)}


def _render_cases(method, snap, table, views, nx, ny, nz, L, width, tmp):
    path = ""
    if table is not None:
        path = os.path.join(tmp, "table.dat")
        synth.write_table(table, path)
    cubes, metas, gxs, gys, gls = [], [], [], [], []
    for (l, b) in views:
        out, (gx, gy, gl), meta = oracle.ref_render(method, snap, path, l, b, nx, ny, nz, L, width, want_grid=True)
        cubes.append(out)
        metas.append(meta)
        gxs.append(gx)
        gys.append(gy)
        gls.append(gl if gl is not None else np.zeros(0, np.float32))
    return dict(views=np.array(views, np.float64), cube=np.stack(cubes), meta=np.stack(metas), gx=np.stack(gxs),
                gy=np.stack(gys), glambda=np.stack(gls), res=np.array([nx, ny, nz, L], np.int32),
                width=np.float64(width))


def main():
    if not oracle.ref_available():
        oracle.build(ref=True)
    info = dict(platform=np.array(platform.machine()), generator=np.array("oracle/_ref (reference sources + shims)"))
    with tempfile.TemporaryDirectory() as tmp:
        # 1. spectroscopic NN, several views incl. b != 0 (Doppler shifts)
        s = synth.loop_snapshot(14, seed=1)
        t = synth.line_table()
        tp = os.path.join(tmp, "t.dat")
        synth.write_table(t, tp)
        eps, w = oracle.ref_emission(s, tp)
        d = _render_cases("NearestNeighbour", s, t, [(0.0, 0.0), (0.3, 0.2), (1.0, -0.3), (0.5236, 0.0)], 16, 12,
                          20, 16, 0.6, tmp)
        np.savez_compressed(os.path.join(HERE, "nn_spectro.npz"), eps=eps, fwhm=w, **_snap_dict(s), **_table_dict(t),
                            **d, **info)

        # 2. imaging with a broadband DN table (arcsec grid and apix scaling)
        bt = synth.broadband_table(171)
        bp = os.path.join(tmp, "b.dat")
        synth.write_table(bt, bp)
        eps, w = oracle.ref_emission(s, bp, imaging=True)
        d = _render_cases("NearestNeighbour", s, bt, [(0.4, 0.3), (0.0, 0.0), (2.0, 1.1)], 16, 16, 20, 1, 1e5, tmp)
        np.savez_compressed(os.path.join(HERE, "nn_imaging.npz"), eps=eps, fwhm=w, **_snap_dict(s),
                            **_table_dict(bt), **d, **info)

        # 3. edges: ragged pixel counts, nz = 1, large rotation (empty corners),
        #    points outside the table's T range (G = 0), zero/negative density
        se = synth.loop_snapshot(11, seed=3)
        se.T[::17] = np.float32(5.0e3)     # logT < 4 -> below the table -> G = 0
        se.T[5::23] = np.float32(3.0e8)    # logT > 8 -> above the table -> G = 0
        se.n[7::31] = np.float32(0.0)      # log10(<=0) -> 0 (fomo-operations.cpp:73-77)
        eps, w = oracle.ref_emission(se, tp)
        d1 = _render_cases("NearestNeighbour", se, t, [(0.785, 0.6), (3.0, -1.2)], 7, 5, 13, 9, 0.4, tmp)
        d2 = _render_cases("NearestNeighbour", se, t, [(0.2, 0.1)], 9, 6, 1, 5, 0.5, tmp)
        np.savez_compressed(os.path.join(HERE, "nn_edges.npz"), eps=eps, fwhm=w, **_snap_dict(se), **_table_dict(t),
                            **{k + "_a": v for k, v in d1.items()}, **{k + "_b": v for k, v in d2.items()}, **info)

        # 4. Thomson pB
        ts = synth.thomson_snapshot(12)
        tot, pol = oracle.ref_thomson_emission(ts)
        d = _render_cases("Thomson", ts, None, [(0.0, 0.0), (0.2, 0.3), (0.1, -0.05), (1.2, 1.4)], 12, 10, 16, 1,
                          1e5, tmp)
        np.savez_compressed(os.path.join(HERE, "thomson.npz"), tot=tot, pol=pol, **_snap_dict(ts), **d, **info)

        # 5. medium spectroscopic case
        sm = synth.loop_snapshot(24, seed=2)
        eps, w = oracle.ref_emission(sm, tp)
        d = _render_cases("NearestNeighbour", sm, t, [(0.7, 0.5)], 32, 32, 48, 32, 0.6, tmp)
        np.savez_compressed(os.path.join(HERE, "nn_medium.npz"), eps=eps, fwhm=w, **_snap_dict(sm),
                            **_table_dict(t), **d, **info)

        # 6. on-disk formats: the reference's RenderCube::writegoftcube (text and
        #    binary) of three small renders; table paths are relative so the
        #    file headers do not depend on where this ran
        cwd = os.getcwd()
        os.chdir(tmp)
        try:
            synth.write_table(t, "table.dat")
            synth.write_table(bt, "band.dat")
            ws = synth.loop_snapshot(9, seed=5)
            wt = synth.thomson_snapshot(9)
            oracle.ref_render_and_write("NearestNeighbour", ws, "table.dat", 0.3, 0.2, 8, 6, 10, 8, 0.6, 3, "w_nn.txt")
            oracle.ref_render_and_write("NearestNeighbour", ws, "band.dat", 0.4, -0.3, 7, 5, 10, 1, 1e5, 3,
                                        "w_img.txt")
            oracle.ref_render_and_write("Thomson", wt, "", 0.2, 0.3, 8, 6, 12, 1, 1e5, 3, "w_th.txt")
            for f in ("w_nn", "w_img", "w_th"):
                for ext in (".txt", ".dat"):
                    with open(f + ext, "rb") as src, open(os.path.join(HERE, "writer_" + f[2:] + ext), "wb") as dst:
                        dst.write(src.read())
        finally:
            os.chdir(cwd)
        # 7. projection renders (single-threaded reference: reproducible float sums)
        d1 = _render_cases("Projection", s, t, [(0.3, 0.2), (1.1, -0.4)], 16, 12, 20, 16, 0.6, tmp)
        d2 = _render_cases("Projection", s, bt, [(0.4, 0.3)], 15, 11, 20, 1, 1e5, tmp)
        eps_b, w_b = oracle.ref_emission(s, bp, imaging=True)
        eps_s, w_s = oracle.ref_emission(s, tp)
        np.savez_compressed(os.path.join(HERE, "projection.npz"), eps=eps_s, fwhm=w_s, eps_band=eps_b,
                            fwhm_band=w_b, **_snap_dict(s), **_table_dict(t), **_table_dict(bt, "band"),
                            **{k + "_a": v for k, v in d1.items()}, **{k + "_b": v for k, v in d2.items()}, **info)
        np.savez_compressed(os.path.join(HERE, "writers.npz"), **{"nn_" + k: v for k, v in _snap_dict(ws).items()},
                            **{"th_" + k: v for k, v in _snap_dict(wt).items()}, **_table_dict(t),
                            **_table_dict(bt, "band"), **info)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


def make_amrvac():
    import hashlib

    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import amrvac_files as A

    out = {}
    with tempfile.TemporaryDirectory() as td:
        for name in A.CASES:
            dat, par, kw = A.write_case(name, td)
            nd, arrs = oracle.ref_amrvac_read(dat, par, kw["amrvac_version"], kw["gamma_eqparposition"], kw["n_unit"],
                                              kw["Teunit"], kw["L_unit"])
            out[name + "_sha256"] = np.array(hashlib.sha256(open(dat, "rb").read()).hexdigest())
            if par:
                out[name + "_par_sha256"] = np.array(hashlib.sha256(open(par, "rb").read()).hexdigest())
            out[name + "_ndim"] = np.array(nd)
            for key, a in zip(("x", "y", "z", "n", "T", "vx", "vy", "vz"), arrs):
                out[f"{name}_{key}"] = a
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "amrvac.npz"), **out)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "amrvac":
        make_amrvac()
        sys.exit(0)
    main()
