"""Parity and CPU-baseline report for the five configurations (GPU required).

Prints one JSON line per configuration: the error of the GPU cubes against
the FP64 oracle -- normalised max error max|g - o| / max|o| (the 1e-4 gate),
L2 relative error, and the largest per-element relative error over elements
with |o| >= 1e-6 max|o| -- and the share of LOS samples whose neighbour index
equals the oracle's.  Small configurations are compared in full, large ones
on sampled image rows.  The oracle's own render time on all host cores is
reported as the CPU baseline for the first two configurations.

    python tests/parity_report.py [--quick]
"""

from __future__ import annotations

import json
import math
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import fomo_gb300 as fg  # noqa: E402
import oracle  # noqa: E402
from fomo_gb300 import synth  # noqa: E402


def errors(got, ref):
    g = np.asarray(got, np.float64).ravel()
    o = np.asarray(ref, np.float64).ravel()
    om = np.abs(o).max()
    if om == 0:
        return {"norm_max": float(np.abs(g).max()), "l2_rel": None, "elem_rel_max": None}
    d = np.abs(g - o)
    big = np.abs(o) >= 1e-6 * om
    return {"norm_max": float(d.max() / om), "l2_rel": float(np.linalg.norm(g - o) / np.linalg.norm(o)),
            "elem_rel_max": float((d[big] / np.abs(o[big])).max())}


def merge(acc, e):
    for k, v in e.items():
        if v is not None:
            acc[k] = max(acc.get(k, 0.0), v)
    return acc


def nn_match(got, ref):
    return int(np.count_nonzero(np.asarray(got) == np.asarray(ref))), int(np.asarray(ref).size)


def c1(ctx, cores):
    s = synth.loop_snapshot(64, seed=1)
    t = synth.line_table()
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    sid, tid = ctx.snapshot(s), ctx.table(t)
    eps, w = oracle.emission(s, t)
    acc, same, tot = {}, 0, 0
    for (l, b) in ((0.0, 0.0), (0.4, 0.25)):
        cube, idx, _ = ctx.render(ctx.request(sid, tid, fg.METHOD_NN, 128, 128, 256, 64, l, b, width), want_idx=True)
        oc, oi, _ = oracle.nn_render(s, eps, w, t.lambda0, l, b, 128, 128, 256, 64, width, want_idx=True,
                                     nthreads=cores)
        merge(acc, errors(cube, oc))
        a, n = nn_match(idx, oi)
        same, tot = same + a, tot + n
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        oracle.nn_render(s, eps, w, t.lambda0, 0.0, 0.0, 128, 128, 256, 64, width, nthreads=cores)
        times.append(time.perf_counter() - t0)
    ctx.drop_snapshot(sid)
    return {"config": "C1 262,144 points, 128x128, L=64, nz=256, views (0,0) and (0.4,0.25) rad, full cubes",
            **acc, "nn_equal": same, "nn_samples": tot,
            "cpu_oracle_los_samples_per_s": 128 * 128 * 256 / min(times), "cpu_cores": cores}


def c2(ctx, cores, quick):
    s = synth.loop_snapshot(128, seed=1)
    t = synth.line_table()
    width = 0.6 * fg.SPEED_OF_LIGHT / t.lambda0
    sid, tid = ctx.snapshot(s), ctx.table(t)
    eps, w = oracle.emission(s, t)
    acc, same, tot, cpu_s, cpu_n = {}, 0, 0, 0.0, 0
    rows = (5, 200, 256, 311, 507) if not quick else (256,)
    for deg in (0.0, 30.0, 60.0):
        l = math.radians(deg)
        cube, idx, _ = ctx.render(ctx.request(sid, tid, fg.METHOD_NN, 512, 512, 512, 128, l, 0.0, width),
                                  want_idx=True)
        for r0 in rows:
            t0 = time.perf_counter()
            oc, oi, _ = oracle.nn_render(s, eps, w, t.lambda0, l, 0.0, 512, 512, 512, 128, width, rows=(r0, r0 + 1),
                                         want_idx=True, nthreads=cores)
            cpu_s += time.perf_counter() - t0
            cpu_n += 512 * 512
            merge(acc, errors(cube[r0:r0 + 1], oc))
            a, n = nn_match(idx[r0:r0 + 1], oi)
            same, tot = same + a, tot + n
    ctx.drop_snapshot(sid)
    return {"config": f"C2 2,097,152 points, 512x512, L=128, nz=512, l in (0,30,60) deg, b=0, rows {list(rows)}",
            **acc, "nn_equal": same, "nn_samples": tot, "cpu_oracle_los_samples_per_s": cpu_n / cpu_s,
            "cpu_cores": cores}


def c3(ctx, cores, quick):
    import bench
    snap, tables, ls, bs = bench.make_workload()
    sid = ctx.snapshot(snap)
    tids = [ctx.table(t) for t in tables]
    acc, same, tot = {}, 0, 0
    views = (0, 37) if not quick else (0,)
    for v in views:
        reqs = [ctx.request(sid, tid, fg.METHOD_NN, bench.NX, bench.NY, bench.NZ, bench.NL, float(ls[v]),
                            float(bs[v]), bench.WIDTH) for tid in tids]
        cubes, _ = ctx.render_batch(reqs)
        for t, cube in zip(tables, cubes):
            eps, w = oracle.emission(snap, t)
            for r0 in (60, 128, 190):
                oc, oi, _ = oracle.nn_render(snap, eps, w, t.lambda0, float(ls[v]), float(bs[v]), bench.NX, bench.NY,
                                             bench.NZ, bench.NL, bench.WIDTH, rows=(r0, r0 + 1), want_idx=True,
                                             nthreads=cores)
                merge(acc, errors(cube[r0:r0 + 1], oc))
        _, idx, _ = ctx.render(reqs[0], want_idx=True)
        eps, w = oracle.emission(snap, tables[0])
        for r0 in (60, 128, 190):
            _, oi, _ = oracle.nn_render(snap, eps, w, tables[0].lambda0, float(ls[v]), float(bs[v]), bench.NX,
                                        bench.NY, bench.NZ, bench.NL, bench.WIDTH, rows=(r0, r0 + 1), want_idx=True,
                                        nthreads=cores)
            a, n = nn_match(idx[r0:r0 + 1], oi)
            same, tot = same + a, tot + n
    ctx.drop_snapshot(sid)
    return {"config": f"C3 2,097,152 points, views {list(views)} of 64 x 4 lines, 256x256, L=64, nz=512, "
                      "rows 60/128/190", **acc, "nn_equal": same, "nn_samples": tot}


def c4(ctx, cores, quick):
    rope = synth.flux_rope_snapshot(8 * 1024 * 1024, seed=4)
    chans = (94, 131, 171, 193, 211, 335)
    tabs = [synth.broadband_table(c, peak_logT=5.8 + 0.15 * k) for k, c in enumerate(chans)]
    sid = ctx.snapshot(rope)
    tids = [ctx.table(t) for t in tabs]
    l, b = 0.6, 0.35
    cubes, _ = ctx.render_batch([ctx.request(sid, tid, fg.METHOD_NN, 1024, 1024, 1024, 1, l, b, 1e5) for tid in tids])
    acc = {}
    for k in ((0, 3) if not quick else (0,)):
        eps, w = oracle.emission(rope, tabs[k], imaging=True)
        for r0 in (200, 700):
            oc, _, _ = oracle.nn_render(rope, eps, w, tabs[k].lambda0, l, b, 1024, 1024, 1024, 1, 1e5, is_dn=True,
                                        rows=(r0, r0 + 1), nthreads=cores)
            merge(acc, errors(cubes[k][r0:r0 + 1], oc))
    _, idx, _ = ctx.render(ctx.request(sid, tids[2], fg.METHOD_NN, 256, 256, 1024, 1, l, b, 1e5), want_idx=True)
    eps, w = oracle.emission(rope, tabs[2], imaging=True)
    same, tot = 0, 0
    for r0 in (40, 128, 230):
        _, oi, _ = oracle.nn_render(rope, eps, w, tabs[2].lambda0, l, b, 256, 256, 1024, 1, 1e5, is_dn=True,
                                    rows=(r0, r0 + 1), want_idx=True, nthreads=cores)
        a, n = nn_match(idx[r0:r0 + 1], oi)
        same, tot = same + a, tot + n
    ctx.drop_snapshot(sid)
    out = [{"config": "C4 8,388,608-point flux rope, 6 DN channels, 1024x1024, nz=1024, l=0.6, b=0.35 rad, "
                      "rows 200/700 (cubes), 256x256 rows 40/128/230 (indices)", **acc, "nn_equal": same,
            "nn_samples": tot}]
    ts = synth.flux_rope_snapshot(8 * 1024 * 1024, seed=5, center=(1.5 * 695.7, 0.0, 0.0))
    sid = ctx.snapshot(ts)
    tot_p, pol = oracle.thomson_emission(ts)
    for (l, b) in ((0.2, 0.0), (0.2, 0.3)):
        cube, _, _ = ctx.render(ctx.request(sid, 0, fg.METHOD_THOMSON, 1024, 1024, 1024, 1, l, b, 1e5))
        oc, _, _ = oracle.thomson_render(ts, tot_p, pol, l, b, 1024, 1024, 1024, rows=(600, 601), nthreads=cores)
        out.append({"config": f"C4 Thomson pB, same rope at 1.5 solar radii, 1024x1024, nz=1024, l={l}, b={b} rad, "
                              "row 600", **errors(cube[600:601], oc)})
    ctx.drop_snapshot(sid)
    return out


def main():
    quick = "--quick" in sys.argv
    cores = os.cpu_count() or 1
    with fg.Context(0) as ctx:
        for f in (lambda: c1(ctx, cores), lambda: c2(ctx, cores, quick), lambda: c3(ctx, cores, quick),
                  lambda: c4(ctx, cores, quick)):
            r = f()
            for line in (r if isinstance(r, list) else [r]):
                print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
