"""Benchmark of the GB300 nearest-neighbour render path (one JSON line).

Workload (the batched configuration): one 128^3 = 2,097,152-point jittered
coronal-loop snapshot x 64 views (l uniform in [0, 90 deg], b uniform in
[-20, 20 deg], seeded) x 4 spectral lines (G(T) peaks at logT 5.8/6.0/6.2/6.4,
lambda0 171/193/211/284 A), 256x256 pixels, 64 lambda bins over a common
+-175 km/s window, 512 LOS samples; one persistent launch captured in a CUDA
graph.  A step renders the whole batch.  Synthetic data (the reference has no
benchmark dataset).

value      : line-samples/s of the batched render, inputs resident in HBM, L2
             flushed (256 MiB write) before each timed step, CUDA events.
plain_*    : the plain single-request GPU render (512x512, 128 bins, 512
             samples, l in {0, 30, 60 deg}, b = 0), one request per call --
             the denominator of the batched-vs-plain metric; and the batched
             workload's own 256 requests rendered one per call (identical work).
e2e        : the same batch through the C ABI with pinned host buffers: upload
             the snapshot, build the index, emissivity, render, download every
             cube, per step (median of 9 steps).
roofline   : the march kernel's algorithmic bytes / its event-timed duration
             against the measured HBM copy bandwidth.
cpu_baseline: the oracle (C restatement, OpenMP on all host cores) on a bounded
             sample of rows of the plain configuration.
serving    : Poisson streams of mixed requests (200/s, and 400/s and 800/s above
             the server's one-at-a-time capacity; 8 resident snapshots of 0.5M-8M
             points, random views, pixels, lambda bins and lines) through the
             continuous-batching server: p50/p90/p99 latency and throughput per
             rate, and the same requests alone for comparison (N = 1 only).

--impl reference runs the reference's CPU algorithm (the oracle port; the
reference's own build needs Boost/GSL, absent on the GPU host) on a bounded
sample of the batched workload and prints the same metric.

--profile-case, --c4-case and --far-case are not bench lines: a small
direct-launch batch for ncu captures, the 8M-point flux-rope renders (six DN
channels, Thomson on and off the equator) with per-kernel times, and the
off-equator Thomson render at 512^2 for an ncu capture of the far pass.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LOS samples/s batched vs plain GPU at ≤1e-4 rel err; p50/p99 render latency"
LINES = ((5.8, 171.073, "fe_9"), (6.0, 193.509, "fe_12"), (6.2, 211.317, "fe_14"), (6.4, 284.163, "fe_15"))
WIDTH = 0.6 * 2.99792458e8 / 171.073  # +-0.3 A at 171 A, in m/s (same velocity window for every line)
NVIEWS, NX, NY, NZ, NL = 64, 256, 256, 512, 64


def _rank_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(seed=1):
    from fomo_gb300 import synth
    snap = synth.loop_snapshot(128, seed=seed)
    tables = [synth.line_table(peak_logT=p, lambda0=lam, ion=ion) for p, lam, ion in LINES]
    rng = np.random.default_rng(3)
    ls = rng.uniform(0.0, math.pi / 2, NVIEWS)
    bs = rng.uniform(-math.pi / 9, math.pi / 9, NVIEWS)
    return snap, tables, ls, bs


def kernel_bounds(kernel_ms, counters, ceilings, clocks, samples):
    """Each march kernel of the batch against the ceiling that binds it.

    march_search: instruction issue -- warp instructions per LOS sample (the
    committed ncu figure, profiles/march_ceilings.json) x samples / its time,
    against 4 warp instructions per clock per SM at the sampled SM clock; and
    its point loads (16 B each, counted) against the measured L2 gather rate.
    Emission pass: the same issue figure, and its ex2 evaluations (counted) /
    its time against the measured SFU throughput; it waits on its payload
    gathers, below both.  Deferred / split / hard: their time and share."""
    total = sum(kernel_ms.values()) or 1.0
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    issue_peak = 4.0 * ceilings["sm_count"] * mhz * 1e6  # warp instructions per second
    ipc = None
    try:
        with open(os.path.join(ROOT, "profiles", "march_ceilings.json")) as f:
            ipc = json.load(f)
    except Exception:
        ipc = None
    out = {}
    for name, ms in kernel_ms.items():
        if ms <= 0.0:
            continue
        out[name] = {"ms": ms, "share": ms / total}
    s = out.get("search")
    if s:
        sec = s["ms"] / 1e3
        s["samples_per_s"] = samples / sec
        per = (ipc or {}).get("march_search", {}).get("warp_inst_per_sample")
        if per:
            s["issue"] = {"achieved": per * samples / sec, "peak": issue_peak, "frac": per * samples / sec / issue_peak,
                          "unit": "warp instructions/s", "per_sample": per}
        gb = counters.get("points_loaded", 0) * 16.0 / sec / 1e9
        s["l2_gather"] = {"achieved": gb, "peak": ceilings["l2_gather_gbs"], "frac": gb / ceilings["l2_gather_gbs"],
                          "unit": "GB/s"}
        s["bound"] = "issue"
    e = out.get("emission")
    if e:
        sec = e["ms"] / 1e3
        per = (ipc or {}).get("march_spectral<4,1,shade>", {}).get("warp_inst_per_sample")
        if per:
            e["issue"] = {"achieved": per * samples / sec, "peak": issue_peak, "frac": per * samples / sec / issue_peak,
                          "unit": "warp instructions/s", "per_sample": per}
        if counters.get("ex2"):
            rate = counters["ex2"] / sec
            e["sfu"] = {"achieved": rate, "peak": ceilings["ex2_per_s"], "frac": rate / ceilings["ex2_per_s"],
                        "unit": "ex2/s", "runs": counters.get("runs")}
        e["bound"] = "latency (payload gathers per run)"
    for k in ("deferred", "split", "hard"):
        if k in out:
            out[k]["bound"] = "latency (dependent L2 loads per ring)"
    out["counters"] = {k: v for k, v in counters.items() if v}
    return out


def binding_bound(kernels):
    """The bound that binds the march: its largest kernel against its own ceiling."""
    name = max((k for k in kernels if k != "counters"), key=lambda k: kernels[k]["ms"], default=None)
    if name is None:
        return None
    k = kernels[name]
    lim = k.get("issue") or {}
    return {"kernel": name, "share": k["share"], "bound": k.get("bound"), "frac": lim.get("frac"),
            "unit": lim.get("unit"), "note": "HBM is not the bound: the snapshot stays in L2 (see kernels)"}


def algorithmic_bytes_per_sample(nlines, L, nz):
    # winning point's FP32 position (12 B) + v_los (4 B) + (eps, w) per line (8 B)
    # + the output cube written once per ray, spread over its LOS samples
    return 12 + 4 + 8 * nlines + 4.0 * L * nlines / nz


SERVE_SNAPSHOT_POINTS = (524288, 1048576, 1572864, 2097152, 3145728, 4194304, 6291456, 8388608)
SERVE_CHANNELS = (94, 131, 171, 193, 211, 335)
SERVE_NZ = 256
SERVE_MAX_CUBE = 1 << 22  # floats: larger (pixels, L) draws are redrawn (16 MB host result cap)


def serving_leg(device, n_req=300, rates=(200.0, 400.0, 800.0), seed=11):
    """Mixed request stream through the continuous-batching server.

    Eight resident flux-rope snapshots of 0.5M-8M points; per request a random
    snapshot, view (l in [0, 90 deg], b in [-20, 20 deg]), pixels in {64, 128,
    256, 512, 1024}^2 and L in {1, 16, 64, 128} (L = 1 renders one of six
    broadband DN channels, otherwise one of four spectral lines), nz = 256.
    The requests are first run alone, one at a time, through the same server
    (their latency and throughput), then as Poisson streams (seeded) at each
    rate in `rates`: 200/s is the configured stream, the faster ones are above
    what the server sustains running the requests one at a time.  Latency is
    submit -> result in the caller's host buffer.  Every cube of every stream
    is compared with the same request's cube alone."""
    import fomo_gb300 as fg
    from fomo_gb300 import synth
    rng = np.random.default_rng(seed)
    with fg.Server(device) as srv:
        ctx = srv.ctx
        sids = [ctx.snapshot(synth.flux_rope_snapshot(n, seed=20 + k)) for k, n in enumerate(SERVE_SNAPSHOT_POINTS)]
        line_t = [ctx.table(synth.line_table(peak_logT=p, lambda0=lam, ion=ion)) for p, lam, ion in LINES]
        band_t = [ctx.table(synth.broadband_table(c, peak_logT=5.8 + 0.15 * k)) for k, c in enumerate(SERVE_CHANNELS)]
        reqs = []
        while len(reqs) < n_req:
            npx = int(rng.choice([64, 128, 256, 512, 1024]))
            L = int(rng.choice([1, 16, 64, 128]))
            if npx * npx * L > SERVE_MAX_CUBE:
                continue
            sid = sids[int(rng.integers(len(sids)))]
            tid = band_t[int(rng.integers(len(band_t)))] if L == 1 else line_t[int(rng.integers(len(line_t)))]
            reqs.append(ctx.request(sid, tid, fg.METHOD_NN, npx, npx, SERVE_NZ, L, float(rng.uniform(0, math.pi / 2)),
                                    float(rng.uniform(-math.pi / 9, math.pi / 9)), WIDTH))
        unit_arrivals = np.cumsum(rng.exponential(1.0, n_req))  # Poisson at 1/s, scaled per rate
        # warm-up: every (snapshot, table) pair's emissivity, computed once and kept resident
        pairs = sorted({(q.snapshot, q.table, q.nlambda == 1) for q in reqs})
        for sid, tid, img in pairs:
            q = ctx.request(sid, tid, fg.METHOD_NN, 8, 8, 8, 1 if img else 16, 0.1, 0.1, WIDTH)
            buf = np.empty(8 * 8 * q.nlambda, np.float32)
            srv.wait(srv.submit(q, buf))
        elems = [q.nx * q.ny * q.nlambda for q in reqs]
        samples = float(sum(q.nx * q.ny * q.nz for q in reqs))
        # the requests alone, one at a time
        alone, alone_lat = [], []
        t1 = time.perf_counter()
        for i, q in enumerate(reqs):
            a = np.empty(elems[i], np.float32)
            s = srv.wait(srv.submit(q, a), timeout=900.0)
            alone_lat.append((s.t_done - s.t_submit) * 1e3)
            alone.append(a)
        alone_s = time.perf_counter() - t1
        outs = [np.empty(e, np.float32) for e in elems]
        streams = []
        for rate in rates:
            arrivals = unit_arrivals / rate
            t0 = time.perf_counter()
            tickets = []
            for i, q in enumerate(reqs):
                delay = arrivals[i] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                tickets.append(srv.submit(q, outs[i]))
            st = [srv.wait(t, timeout=900.0) for t in tickets]
            lat = np.array([s.t_done - s.t_submit for s in st]) * 1e3
            span = max(s.t_done for s in st) - min(s.t_submit for s in st)
            worst, equal = 0.0, True
            for a, o in zip(alone, outs):
                equal = equal and np.array_equal(a, o)
                den = float(np.abs(a).max())
                if den > 0:
                    worst = max(worst, float(np.abs(a - o).max()) / den)
            streams.append({"arrival_rate_hz": rate, "p50_ms": float(np.percentile(lat, 50)),
                            "p90_ms": float(np.percentile(lat, 90)), "p99_ms": float(np.percentile(lat, 99)),
                            "mean_ms": float(lat.mean()), "span_s": float(span),
                            "line_samples_per_s": samples / span,
                            "vs_alone_throughput": (samples / span) / (samples / alone_s),
                            "mix_vs_alone_max_norm_err": worst, "mix_bit_equal_alone": bool(equal)})
    head = streams[0]
    return {"requests": n_req, "arrival_rate_hz": head["arrival_rate_hz"], "arrivals": "Poisson, seeded",
            "p50_ms": head["p50_ms"], "p90_ms": head["p90_ms"], "p99_ms": head["p99_ms"], "mean_ms": head["mean_ms"],
            "span_s": head["span_s"], "line_samples_per_s": head["line_samples_per_s"],
            "alone_p50_ms": float(np.percentile(alone_lat, 50)), "alone_p99_ms": float(np.percentile(alone_lat, 99)),
            "alone_line_samples_per_s": samples / alone_s,
            "mix_vs_alone_max_norm_err": max(s["mix_vs_alone_max_norm_err"] for s in streams),
            "mix_bit_equal_alone": all(s["mix_bit_equal_alone"] for s in streams),
            "streams": streams, "snapshots_points": list(SERVE_SNAPSHOT_POINTS), "nz": SERVE_NZ,
            "mix": "pixels {64..1024}^2 x L {1,16,64,128} (cube <= 16 MB), 4 lines / 6 DN channels, random views"}


def cpu_baseline_sample(target_s=10.0):
    """Oracle (C restatement, OpenMP, all host cores) on rows of the plain configuration."""
    import oracle
    from fomo_gb300 import synth
    snap = synth.loop_snapshot(128, seed=1)
    t = synth.line_table()
    cores = os.cpu_count() or 1
    eps, w = oracle.emission(snap, t)
    nx = ny = 512
    nz, L = 512, 128
    width = 0.6 * 2.99792458e8 / t.lambda0
    rows = 1
    t0 = time.perf_counter()
    oracle.nn_render(snap, eps, w, t.lambda0, 0.0, 0.0, nx, ny, nz, L, width, nthreads=cores, rows=(256, 256 + rows))
    dt = time.perf_counter() - t0
    rows = int(max(1, min(ny // 2, target_s / max(dt, 1e-3))))
    t0 = time.perf_counter()
    oracle.nn_render(snap, eps, w, t.lambda0, 0.0, 0.0, nx, ny, nz, L, width, nthreads=cores,
                     rows=(256 - rows // 2, 256 - rows // 2 + rows))
    dt = time.perf_counter() - t0
    samples = rows * nx * nz
    return {"value": samples / dt, "unit": "LOS samples/s", "cores": cores, "kind": "port",
            "sample": f"{rows} image rows x 512 rays x 512 samples of the plain 512x512x128 render "
                      f"(2,097,152 points, l=b=0) by the oracle, {dt:.1f} s"}


def run_reference(args):
    """Reference CPU algorithm (oracle port) on a bounded sample of the batched workload."""
    import oracle
    rank, world, _ = _rank_env()
    if world > 1 and rank != 0:
        return
    snap, tables, ls, bs = make_workload()
    cores = os.cpu_count() or 1
    payload = [oracle.emission(snap, t) for t in tables]
    rows = 2
    times = []
    for step in range(args.warmup + args.steps):
        v = step % NVIEWS
        t0 = time.perf_counter()
        for (eps, w), t in zip(payload, tables):
            oracle.nn_render(snap, eps, w, t.lambda0, ls[v], bs[v], NX, NY, NZ, NL, WIDTH, nthreads=cores,
                             rows=(NY // 2 - rows // 2, NY // 2 - rows // 2 + rows))
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
    line_samples = rows * NX * NZ * len(tables)
    value = line_samples * len(times) / sum(times)
    ms = 1e3 * sum(times) / len(times)
    sample = (f"{rows} central rows x {NX} rays x {NZ} samples x {len(tables)} lines of one view per step "
              f"(oracle, FP64, OpenMP {cores} threads)")
    out = {"metric": METRIC, "value": value, "unit": "line-samples/s", "impl": "reference", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "batched NN render: 2,097,152-point loop x 64 views x 4 lines, 256x256, "
                                  "64 bins, 512 LOS samples", "sample_per_step": sample},
           "cpu_baseline": {"value": value, "unit": "line-samples/s", "cores": cores, "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "line-samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_ours(args):
    import torch

    import fomo_gb300 as fg

    rank, world, local = _rank_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    snap, tables, ls, bs = make_workload(seed=1 + rank)
    ctx = fg.Context(local)
    sid = ctx.snapshot(snap)
    tids = [ctx.table(t) for t in tables]
    reqs = [ctx.request(sid, tid, fg.METHOD_NN, NX, NY, NZ, NL, float(ls[v]), float(bs[v]), WIDTH)
            for v in range(NVIEWS) for tid in tids]
    outs = [torch.empty((NY, NX, NL), dtype=torch.float32, device=dev) for _ in reqs]
    ptrs = [o.data_ptr() for o in outs]
    # a real stream: handle 0 (the legacy default stream) means "the context's stream" to the C ABI
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sh = ctypes_stream(stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    # the autotuner measures its candidates on this batch and keeps the fastest;
    # it writes its choice to a cache file, read back here for the JSON line
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        cache = os.path.join(td, "autotune.txt")
        ctx.autotune(reqs, cache_path=cache)
        with open(cache) as f:
            tuned = [dict(zip(("class", "tile_w", "tile_h", "search_ctas_per_sm_cap", "gather_radius_spacings",
                               "ms_per_batch"), ln.split())) for ln in f if ln.strip()]

    for _ in range(args.warmup):
        ctx.render_batch_device(reqs, ptrs, stream=sh, graph=True)
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    march_ms = []
    with Clocks(local) as clk:
        torch.cuda.synchronize(dev)
        for k in range(args.steps):
            flush.fill_(k & 0xff)
            ev[k][0].record(stream)
            ctx.render_batch_device(reqs, ptrs, stream=sh, graph=True)
            ev[k][1].record(stream)
            try:
                march_ms.append(ctx.last_march_ms())
            except fg.FomoError:
                pass
        torch.cuda.synchronize(dev)
    march_src = "external event nodes inside the replayed graph"
    if not march_ms:
        # timing events inside the graph unavailable: time the same launch issued directly
        march_src = "direct (non-graph) launch of the same batch"
        for _ in range(args.steps):
            flush.fill_(3)
            ctx.render_batch_device(reqs, ptrs, stream=sh, graph=False)
            march_ms.append(ctx.last_march_ms())
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_total = sum(step_ms) / 1e3
    if dist:
        tt = torch.tensor([t_total], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_total = float(tt.item())
        dist.barrier()
    line_samples = float(NVIEWS * len(tables) * NX * NY * NZ)
    value = world * line_samples * args.steps / t_total

    # ---- the batch's kernels one by one: a direct launch of the same batch with
    # events between the march's kernels, then one with the search counters on
    # (they add atomics, so their run is not timed); then the device's ceilings
    ctx.set_profiling(kernel_timing=True, counters=False)
    flush.fill_(7)
    ctx.render_batch_device(reqs, ptrs, stream=sh, graph=False)
    kernel_ms, _ = ctx.profile_read()
    ctx.set_profiling(kernel_timing=False, counters=True)
    ctx.render_batch_device(reqs, ptrs, stream=sh, graph=False)
    _, counters = ctx.profile_read()
    ctx.set_profiling(kernel_timing=False, counters=False)
    ceilings = ctx.measure_ceilings().as_dict()

    # ---- the same 256 requests (64 views x 4 lines), one fomo_render_device call
    # each: batched vs plain on identical work
    torch.cuda.synchronize(dev)
    for q, p in zip(reqs[:8], ptrs[:8]):
        ctx.render_device(q, p, stream=sh)
    torch.cuda.synchronize(dev)
    same_ms = []
    for k in range(2):
        flush.fill_(5 + k)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for q, p in zip(reqs, ptrs):
            ctx.render_device(q, p, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        same_ms.append(e0.elapsed_time(e1))
    plain_same_value = line_samples / (min(same_ms) / 1e3)

    # ---- plain single-request GPU render (denominator)
    from fomo_gb300 import synth
    t171 = ctx.table(synth.line_table())
    preqs = [ctx.request(sid, t171, fg.METHOD_NN, 512, 512, 512, 128, math.radians(a), 0.0, WIDTH)
             for a in (0.0, 30.0, 60.0)]
    pout = torch.empty((512, 512, 128), dtype=torch.float32, device=dev)
    for q in preqs:
        ctx.render_device(q, pout.data_ptr(), stream=sh)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.fill_(1)
    e0.record(stream)
    for q in preqs:
        ctx.render_device(q, pout.data_ptr(), stream=sh)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    plain_s = e0.elapsed_time(e1) / 1e3
    plain_value = 3 * 512 * 512 * 512 / plain_s

    # ---- end to end through the C ABI with pinned host buffers
    hsnap = [torch.from_numpy(a).pin_memory() for a in snap.arrays()]
    hout = [torch.empty((NY, NX, NL), dtype=torch.float32).pin_memory() for _ in range(len(reqs))]
    from fomo_gb300 import Context
    e2e_times = []
    h2d = sum(a.numel() * 4 for a in hsnap) + sum(t.G.nbytes + t.logT.nbytes + t.logn.nbytes for t in tables)
    d2h = sum(o.numel() * 4 for o in hout)
    e2e_steps = 9  # median of 9: host-side copies vary with other jobs on the host
    phases = []
    for k in range(e2e_steps + 1):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        s2 = ctx_snapshot_from_pinned(ctx, hsnap)
        t1 = time.perf_counter()
        tids2 = [ctx.table(t) for t in tables]
        reqs2 = [ctx.request(s2, tid, fg.METHOD_NN, NX, NY, NZ, NL, float(ls[v]), float(bs[v]), WIDTH)
                 for v in range(NVIEWS) for tid in tids2]
        t2 = time.perf_counter()
        cubes, _ = ctx.render_batch(reqs2, outs=[h.numpy() for h in hout])
        t3 = time.perf_counter()
        dt = t3 - t0
        ctx.drop_snapshot(s2)
        for t in tids2:
            ctx.drop_table(t)
        if k > 0:
            e2e_times.append(dt)
            phases.append((t1 - t0, t2 - t1, t3 - t2, time.perf_counter() - t3))
    e2e_med = float(np.median(e2e_times))
    e2e_value = world * line_samples / e2e_med

    # ---- roofline of the march kernel
    avg_march_s = float(np.mean(march_ms)) / 1e3
    bps = algorithmic_bytes_per_sample(len(tables), NL, NZ)
    samples_per_launch = NVIEWS * NX * NY * NZ
    achieved = bps * samples_per_launch / avg_march_s / 1e9
    peak, peak_kind = _peaks()
    traffic = None
    tf = os.path.join(ROOT, "profiles", "march_traffic.json")
    if os.path.exists(tf):
        try:
            with open(tf) as f:
                traffic = json.load(f).get("bytes_per_launch_scaled")
        except Exception:
            traffic = None

    clocks = clk.summary()
    kernels = kernel_bounds(kernel_ms, counters, ceilings, clocks, samples_per_launch)

    serving = None
    if rank == 0 and world == 1 and not args.no_serving:
        ctx.close()  # the server leg builds its own context and snapshots
        ctx = None
        serving = serving_leg(local)

    if rank == 0:
        cpu = cpu_baseline_sample() if not args.no_cpu else None
        out = {
            "metric": METRIC, "value": value, "unit": "line-samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "batched NN render: 2,097,152-point loop x 64 views x 4 lines, 256x256 px, "
                                   "64 lambda bins, 512 LOS samples, one persistent launch in a CUDA graph",
                       "l2": "flushed (256 MiB write) before each timed step; snapshot+payload ~130 MB",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "plain": "512x512 px, 128 bins, 512 samples, l in {0,30,60} deg, b=0, one request per call"},
            "los_samples_per_step": NVIEWS * NX * NY * NZ,
            "plain_value": plain_value, "plain_unit": "LOS samples/s",
            "batched_vs_plain": value / plain_value,
            "plain_same_config_value": plain_same_value, "plain_same_config_unit": "line-samples/s",
            "plain_same_config": "the same 256 requests (64 views x 4 lines), one fomo_render_device call each, "
                                 "L2 flushed before the 256 calls, CUDA events (best of 2)",
            "batched_vs_plain_same_config": value / plain_same_value,
            "march_ms": float(np.mean(march_ms)), "march_timing": march_src,
            "e2e": {"value": e2e_value, "unit": "line-samples/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": len(e2e_times), "stat": "median",
                    "ms_per_step": 1e3 * e2e_med, "ms_min": 1e3 * float(np.min(e2e_times)),
                    "ms_max": 1e3 * float(np.max(e2e_times)), "ms_steps": [1e3 * t for t in e2e_times],
                    "ms_phases": {"snapshot_upload_and_index": [1e3 * p[0] for p in phases],
                                  "tables": [1e3 * p[1] for p in phases],
                                  "render_and_download": [1e3 * p[2] for p in phases],
                                  "release_untimed": [1e3 * p[3] for p in phases]}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs",
                         "bytes_per_sample": bps,
                         "kernel": "march_search (neighbour search, positions to a buffer) + march_split "
                                   "(overflowing segments) + march_far (far samples of wide-box views; an empty "
                                   "list here) + march_deferred (the samples the search leaves) + "
                                   "march_hard (deferred samples over the one-lane budget) + "
                                   "march_spectral<4,1,shade> (emission from the positions), timed together",
                         "binding": binding_bound(kernels)},
            "cpu_baseline": cpu,
            "autotuned": tuned,
            "clocks": clocks,
            "ceilings": ceilings,
            "kernels": kernels,
            # per step: view init, view bounds (per block of cells), view extents (the blocks that can hold an
            # extreme), view finalize, search, overflow split, far pass, deferred march, hard-sample march,
            # emission
            "gpu_launches": 10 * args.steps,
            "serving": serving,
        }
        print(json.dumps(out))
    if ctx is not None:
        ctx.close()
    if dist:
        dist.destroy_process_group()


def ctypes_stream(stream):
    import ctypes
    return ctypes.c_void_p(stream.cuda_stream)


def ctx_snapshot_from_pinned(ctx, hsnap):
    import ctypes

    import fomo_gb300 as fg
    sid = ctypes.c_int()
    ptrs = [ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_float)) for t in hsnap]
    ctx._check(ctx._L.fomo_snapshot_create(ctx.h, hsnap[0].numel(), *ptrs, ctypes.byref(sid)))
    return sid.value


def run_profile_case(args):
    """Small case for ncu: the batched workload cut to 8 views (268 M LOS samples,
    ~130 MB resident), issued directly (no graph), 1 warm-up + 2 launches; then
    (outside any ncu kernel filter of interest) one launch with per-kernel
    events and one with the search counters, printed as JSON.

    --tune-cache PATH: the march configuration of the autotuner's cache file at
    PATH; when PATH does not exist yet, the autotuner first measures its
    candidates on this batch and writes it (run once without ncu, so that a
    capture that follows contains no tuning launches)."""
    import fomo_gb300 as fg
    snap, tables, ls, bs = make_workload()
    tuned = None
    if args.tune_cache and os.path.exists(args.tune_cache):
        os.environ["FOMO_TUNE_CACHE"] = args.tune_cache
        tuned = open(args.tune_cache).read().split()
    with fg.Context(0) as ctx:
        sid = ctx.snapshot(snap)
        tids = [ctx.table(t) for t in tables]
        nv = 8
        reqs = [ctx.request(sid, tid, fg.METHOD_NN, NX, NY, NZ, NL, float(ls[v]), float(bs[v]), WIDTH)
                for v in range(nv) for tid in tids]
        import torch
        dev = torch.device("cuda", 0)
        outs = [torch.empty((NY, NX, NL), dtype=torch.float32, device=dev) for _ in reqs]
        ptrs = [o.data_ptr() for o in outs]
        if args.tune_cache and tuned is None:
            ctx.autotune(reqs, cache_path=args.tune_cache)
            tuned = open(args.tune_cache).read().split()
        for _ in range(3):
            ctx.render_batch_device(reqs, ptrs)
            ms = ctx.last_march_ms()
        ctx.synchronize()
        kernel_ms, counters = None, None
        if not args.no_breakdown:
            ctx.set_profiling(kernel_timing=True, counters=False)
            ctx.render_batch_device(reqs, ptrs)
            kernel_ms, _ = ctx.profile_read()
            ctx.set_profiling(kernel_timing=False, counters=True)
            ctx.render_batch_device(reqs, ptrs)
            _, counters = ctx.profile_read()
            ctx.set_profiling(False, False)
        print(json.dumps({"profile_case": f"{nv} views x {len(tables)} lines, {NX}x{NY}x{NZ}, L={NL}",
                          "march_ms": ms, "los_samples": nv * NX * NY * NZ, "kernel_ms": kernel_ms,
                          "counters": counters, "tuned": tuned}))


def run_rope_cases(args):
    """The 8,388,608-point flux rope (80 % in a twisted rope, 20 % uniform
    background; fomo_gb300.synth.flux_rope_snapshot), rendered directly with
    per-kernel CUDA-event timing after warm-up renders, one JSON line.

    --c4-case: six broadband DN channels at 1024 x 1024 px x 1024 LOS samples
    (l = 0.6, b = 0.35 rad, one batch), then the rope moved to 1.5 solar radii
    rendered in Thomson pB at 1024 x 1024 x 1024, l = 0.2, b = 0 and b = 0.3
    rad (200-pixel boxes away from the equator).
    --far-case: only the off-equator Thomson render, at 512 x 512 x 1024, with
    the march counters on the last render (a small case for an ncu capture of
    march_far: three warm-up renders, then the measured one)."""
    import torch

    import fomo_gb300 as fg
    from fomo_gb300 import synth
    dev = torch.device("cuda", 0)
    out = {}
    n = 8 * 1024 * 1024
    with fg.Context(0) as ctx:
        if args.c4_case:
            s = synth.flux_rope_snapshot(n, seed=4)
            sid = ctx.snapshot(s)
            chans = (94, 131, 171, 193, 211, 335)
            tids = [ctx.table(synth.broadband_table(c, peak_logT=5.8 + 0.15 * k)) for k, c in enumerate(chans)]
            reqs = [ctx.request(sid, t, fg.METHOD_NN, 1024, 1024, 1024, 1, 0.6, 0.35, 1e5) for t in tids]
            outs = [torch.empty((1024, 1024, 1), dtype=torch.float32, device=dev) for _ in reqs]
            ptrs = [o.data_ptr() for o in outs]
            ctx.set_profiling(kernel_timing=True)
            for _ in range(3):
                ctx.render_batch_device(reqs, ptrs)
                ctx.synchronize()
                km, _ = ctx.profile_read()
            out["six_dn_channels_1024"] = {"march_ms": ctx.last_march_ms(), "kernel_ms": km}
            ctx.set_profiling(False, False)
            ctx.drop_snapshot(sid)
        ts = synth.flux_rope_snapshot(n, seed=5, center=(1.5 * 695.7, 0.0, 0.0))
        tsid = ctx.snapshot(ts)
        cases = [(0.0, 1024), (0.3, 1024)] if args.c4_case else [(0.3, 512)]
        for b, px in cases:
            q = ctx.request(tsid, 0, fg.METHOD_THOMSON, px, px, 1024, 1, 0.2, b, 1e5)
            o = torch.empty((px, px, 1), dtype=torch.float32, device=dev)
            for _ in range(3):
                ctx.render_device(q, o.data_ptr())
                ctx.synchronize()
            ctx.set_profiling(kernel_timing=True, counters=args.far_case)
            ctx.render_device(q, o.data_ptr())
            ctx.synchronize()
            km, cn = ctx.profile_read()
            ctx.set_profiling(False, False)
            rec = {"march_ms": ctx.last_march_ms(), "kernel_ms": km}
            if args.far_case:
                rec["counters"] = {k: cn[k] for k in ("deferred", "far_groups", "far")}
            out[f"thomson_{px}_b{b}"] = rec
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving (mixed request stream) leg")
    ap.add_argument("--profile-case", action="store_true", help="small direct-launch case for ncu captures")
    ap.add_argument("--no-breakdown", action="store_true", help="profile case without the timing/counter launches")
    ap.add_argument("--tune-cache", default=None, help="profile case: autotuner cache file (written when absent)")
    ap.add_argument("--c4-case", action="store_true", help="8M-point flux rope: 6 DN channels and Thomson at 1024^2")
    ap.add_argument("--far-case", action="store_true", help="8M-point rope, off-equator Thomson at 512^2 (ncu)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.profile_case:
        run_profile_case(args)
    elif args.c4_case or args.far_case:
        run_rope_cases(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
