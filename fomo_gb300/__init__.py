"""fomo_gb300 -- GB300 implementation of FoMo-C's nearest-neighbour render path.

The product is ``libfomo_gpu.so`` (hand-written sm_103a CUDA kernels plus a C++
runtime) behind the C ABI in ``include/fomo_gpu.h``, and the C++ drop-in
``include/FoMo.h``.  This module is a thin ctypes mirror of that ABI for Python
callers (tests, benchmarks); it holds no compute of its own and raises if the
shared library is missing -- there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfomo_gpu.so")
# the bounds-check build of the same sources (fomo_gb300/build.py): every kernel
# index checked, an index out of range reported as EDEVICE; for tests
LIB_CHECKED_PATH = os.path.join(HERE, "libfomo_gpu_checked.so")

OK = 0
EINVAL, ENOMEM, EADMISSION, EDEVICE, ETIMEOUT, ENOTFOUND, EIO, ETABLE, ECANCELLED, EMETHOD, ENODEVICE = \
    -1, -2, -3, -4, -5, -6, -7, -8, -9, -10, -11
METHOD_NN = 0
METHOD_THOMSON = 1
METHOD_PROJECTION = 2
OBS_SPECTROSCOPIC = 1
OBS_IMAGING = 2
SPEED_OF_LIGHT = 2.99792458e8
# FOMO_KERNEL_* and FOMO_COUNTER_* of include/fomo_gpu.h, in order
KERNELS = ("search", "split", "deferred", "hard", "emission", "fused", "far")
COUNTERS = ("segments", "candidates", "rows", "points_loaded", "not_gathered", "fallbacks", "samples", "scanned",
            "ties", "fb_nocand", "fb_far", "fb_ambiguous", "deferred", "deferred_recs", "hard", "runs", "ex2",
            "far_groups", "far")


class FomoError(RuntimeError):
    def __init__(self, code: int, msg: str, stats=None):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.stats = stats  # Server.wait: the request's timestamps (RequestStats) when it ended with an error


class Request(ctypes.Structure):
    _fields_ = [("snapshot", ctypes.c_int), ("table", ctypes.c_int), ("method", ctypes.c_int),
                ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("nlambda", ctypes.c_int),
                ("l", ctypes.c_double), ("b", ctypes.c_double), ("lambda_width", ctypes.c_double),
                ("abundratio", ctypes.c_double)]


class ViewInfo(ctypes.Structure):
    _fields_ = [("minx", ctypes.c_double), ("maxx", ctypes.c_double), ("miny", ctypes.c_double),
                ("maxy", ctypes.c_double), ("minz", ctypes.c_double), ("maxz", ctypes.c_double),
                ("maxdistance", ctypes.c_double), ("deltaz", ctypes.c_double), ("pathlength", ctypes.c_double),
                ("apix", ctypes.c_double), ("scale", ctypes.c_double), ("lambda_width_A", ctypes.c_double),
                ("lambda0", ctypes.c_double), ("is_dn", ctypes.c_int), ("observation_type", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SnapshotInfo(ctypes.Structure):
    _fields_ = [("npoints", ctypes.c_int64), ("grid_dims", ctypes.c_int * 3), ("cell_edge", ctypes.c_float),
                ("aabb", ctypes.c_float * 6), ("device_bytes", ctypes.c_size_t)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_size_t), ("max_inflight", ctypes.c_int)]


class Ceilings(ctypes.Structure):
    _fields_ = [("l2_read_gbs", ctypes.c_double), ("l2_gather_gbs", ctypes.c_double), ("ex2_per_s", ctypes.c_double),
                ("sm_count", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class RequestStats(ctypes.Structure):
    _fields_ = [("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_start", ctypes.c_double),
                ("t_done", ctypes.c_double), ("status", ctypes.c_int)]


_F = ctypes.POINTER(ctypes.c_float)
_I32 = ctypes.POINTER(ctypes.c_int32)
_lib = None
_lib_checked = None

# (name, argtypes) of every entry point declared in include/fomo_gpu.h
SIGNATURES = {
    "fomo_version": [],
    "fomo_ctx_create": [ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)],
    "fomo_ctx_destroy": [ctypes.c_void_p],
    "fomo_last_error": [ctypes.c_void_p],
    "fomo_ctx_memory": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)],
    "fomo_ctx_synchronize": [ctypes.c_void_p],
    "fomo_host_register": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t],
    "fomo_host_unregister": [ctypes.c_void_p, ctypes.c_void_p],
    "fomo_snapshot_create": [ctypes.c_void_p, ctypes.c_int64] + [_F] * 8 + [ctypes.POINTER(ctypes.c_int)],
    "fomo_snapshot_destroy": [ctypes.c_void_p, ctypes.c_int],
    "fomo_snapshot_create_device": [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 8 + [ctypes.POINTER(ctypes.c_int)],
    "fomo_abundance_ratio": [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                             ctypes.POINTER(ctypes.c_double)],
    "fomo_snapshot_get_info": [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(SnapshotInfo)],
    "fomo_snapshot_from_amrvac": [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                  ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_int)],
    "fomo_amrvac_points": [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                           ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int64,
                           ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int)] + [_F] * 8,
    "fomo_table_create": [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_double, ctypes.c_double, ctypes.c_char_p,
                          ctypes.c_int, ctypes.c_int, _F, _F, _F, ctypes.POINTER(ctypes.c_int)],
    "fomo_table_load": [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)],
    "fomo_table_destroy": [ctypes.c_void_p, ctypes.c_int],
    "fomo_table_get_info": [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.c_char_p, ctypes.c_int,
                            ctypes.c_char_p, ctypes.c_int],
    "fomo_emission": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, _F, _F],
    "fomo_thomson_emission": [ctypes.c_void_p, ctypes.c_int, _F, _F],
    "fomo_render":[ctypes.c_void_p, ctypes.POINTER(Request), _F, _I32, ctypes.POINTER(ViewInfo)],
    "fomo_render_device": [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.POINTER(ViewInfo), ctypes.c_void_p],
    "fomo_render_noalloc": [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_void_p, ctypes.c_void_p],
    "fomo_render_batch": [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_int, ctypes.POINTER(_F),
                          ctypes.POINTER(ViewInfo)],
    "fomo_render_batch_device": [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p],
    "fomo_render_batch_graph": [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_int,
                                ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p],
    "fomo_autotune": [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_int, ctypes.c_char_p],
    "fomo_set_march_config": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int],
    "fomo_last_march_ms": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)],
    "fomo_measure_ceilings": [ctypes.c_void_p, ctypes.POINTER(Ceilings)],
    "fomo_set_profiling": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int],
    "fomo_profile_read": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                          ctypes.POINTER(ctypes.c_uint64), ctypes.c_int],
    "fomo_server_create": [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)],
    "fomo_server_context": [ctypes.c_void_p],
    "fomo_server_submit": [ctypes.c_void_p, ctypes.POINTER(Request), _F, ctypes.POINTER(ctypes.c_uint64)],
    "fomo_server_wait": [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(RequestStats)],
    "fomo_server_cancel": [ctypes.c_void_p, ctypes.c_uint64],
    "fomo_server_destroy": [ctypes.c_void_p],
    "fomo_server_last_error": [ctypes.c_void_p],
}
RESTYPES = {"fomo_version": ctypes.c_char_p, "fomo_last_error": ctypes.c_char_p,
            "fomo_server_last_error": ctypes.c_char_p, "fomo_server_context": ctypes.c_void_p}


def _load(path: str):
    if not os.path.exists(path):
        raise FomoError(ENODEVICE, f"{path} is missing: build it with `python -m fomo_gb300.build`")
    L = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = RESTYPES.get(name, ctypes.c_int)
    return L


def lib(checked: bool = False):
    """Load libfomo_gpu.so (built by fomo_gb300.build); raise if it is missing.
    checked=True loads the bounds-check build instead."""
    global _lib, _lib_checked
    if checked:
        if _lib_checked is None:
            _lib_checked = _load(LIB_CHECKED_PATH)
        return _lib_checked
    if _lib is None:
        _lib = _load(LIB_PATH)
    return _lib


def _fp(a):
    return a.ctypes.data_as(_F)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Context:
    """One libfomo_gpu context (device memory, resident snapshots and tables)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, checked: bool = False):
        """checked=True: a context of the bounds-check build (libfomo_gpu_checked.so)."""
        self._L = lib(checked)
        h = ctypes.c_void_p()
        rc = self._L.fomo_ctx_create(device, hbm_budget, ctypes.byref(h))
        if rc != OK:
            raise FomoError(rc, "fomo_ctx_create failed (no usable CUDA device?)")
        self.h = h

    # -- plumbing
    def _check(self, rc):
        if rc != OK:
            raise FomoError(rc, self._L.fomo_last_error(self.h).decode())

    def close(self):
        if self.h:
            self._L.fomo_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def memory(self):
        u, b = ctypes.c_size_t(), ctypes.c_size_t()
        self._check(self._L.fomo_ctx_memory(self.h, ctypes.byref(u), ctypes.byref(b)))
        return u.value, b.value

    def synchronize(self):
        self._check(self._L.fomo_ctx_synchronize(self.h))

    # -- data
    def snapshot(self, snap) -> int:
        arrs = [_f32(a) for a in snap.arrays()]
        sid = ctypes.c_int()
        self._check(self._L.fomo_snapshot_create(self.h, arrs[0].shape[0], *[_fp(a) for a in arrs],
                                                 ctypes.byref(sid)))
        return sid.value

    def snapshot_device(self, n: int, ptrs) -> int:
        """Snapshot from 8 device arrays (x, y, z, n, T, vx, vy, vz; z may be 0)."""
        sid = ctypes.c_int()
        self._check(self._L.fomo_snapshot_create_device(self.h, n, *[ctypes.c_void_p(p) if p else None for p in ptrs],
                                                        ctypes.byref(sid)))
        return sid.value

    def snapshot_from_amrvac(self, datfile: str, amrvacpar: str | None = None, amrvac_version: str = "gitlab",
                             gamma_eqparposition: int = 0, n_unit: float = 1.0, Teunit: float = 1.0,
                             L_unit: float = 1.0) -> int:
        """A snapshot read from an AMRVAC data file (fomo_snapshot_from_amrvac)."""
        sid = ctypes.c_int()
        self._check(self._L.fomo_snapshot_from_amrvac(self.h, datfile.encode(),
                                                      amrvacpar.encode() if amrvacpar else None,
                                                      amrvac_version.encode(), gamma_eqparposition, n_unit, Teunit,
                                                      L_unit, ctypes.byref(sid)))
        return sid.value

    def amrvac_points(self, datfile: str, amrvacpar: str | None = None, amrvac_version: str = "gitlab",
                      gamma_eqparposition: int = 0, n_unit: float = 1.0, Teunit: float = 1.0, L_unit: float = 1.0):
        """(ndim, [x, y, z, n, T, vx, vy, vz]) of an AMRVAC data file, in the reference's point order."""
        args = (self.h, datfile.encode(), amrvacpar.encode() if amrvacpar else None, amrvac_version.encode(),
                gamma_eqparposition, n_unit, Teunit, L_unit)
        n, nd = ctypes.c_int64(), ctypes.c_int()
        self._check(self._L.fomo_amrvac_points(*args, 0, ctypes.byref(n), ctypes.byref(nd), *([None] * 8)))
        arrs = [np.empty(n.value, np.float32) for _ in range(8)]
        self._check(self._L.fomo_amrvac_points(*args, n.value, ctypes.byref(n), ctypes.byref(nd),
                                               *[_fp(a) for a in arrs]))
        return nd.value, arrs

    def snapshot_info(self, sid: int) -> SnapshotInfo:
        info = SnapshotInfo()
        self._check(self._L.fomo_snapshot_get_info(self.h, sid, ctypes.byref(info)))
        return info

    def drop_snapshot(self, sid: int):
        self._check(self._L.fomo_snapshot_destroy(self.h, sid))

    def table(self, t) -> int:
        tid = ctypes.c_int()
        logT, logn, G = _f32(t.logT), _f32(t.logn), _f32(t.G)
        self._check(self._L.fomo_table_create(self.h, t.ion.encode(), t.lambda0, t.atweight, t.unit.encode(),
                                              t.nt, t.nrho, _fp(logT), _fp(logn), _fp(G), ctypes.byref(tid)))
        return tid.value

    def load_table(self, path: str) -> int:
        tid = ctypes.c_int()
        self._check(self._L.fomo_table_load(self.h, path.encode(), ctypes.byref(tid)))
        return tid.value

    def table_info(self, tid: int):
        lam, atw = ctypes.c_double(), ctypes.c_double()
        nt, nrho, dn = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ion = ctypes.create_string_buffer(256)
        unit = ctypes.create_string_buffer(1024)
        self._check(self._L.fomo_table_get_info(self.h, tid, ctypes.byref(lam), ctypes.byref(atw), ctypes.byref(nt),
                                                ctypes.byref(nrho), ctypes.byref(dn), ion, 256, unit, 1024))
        return dict(lambda0=lam.value, atweight=atw.value, nt=nt.value, nrho=nrho.value, is_dn=bool(dn.value),
                    ion=ion.value.decode(), unit=unit.value.decode())

    def drop_table(self, tid: int):
        self._check(self._L.fomo_table_destroy(self.h, tid))

    def emission(self, sid: int, tid: int, imaging: bool = False, abundratio: float = 1.0, n: int | None = None):
        """Per-point (eps, fwhm) in the snapshot's original point order."""
        if n is None:
            n = self.snapshot_info(sid).npoints
        eps = np.empty(n, np.float32)
        w = np.empty(n, np.float32)
        self._check(self._L.fomo_emission(self.h, sid, tid, int(imaging), abundratio, _fp(eps), _fp(w)))
        return eps, w

    def thomson_emission(self, sid: int, n: int | None = None):
        """Per-point (n*tot, n*pol) Thomson terms in the snapshot's original point order."""
        if n is None:
            n = self.snapshot_info(sid).npoints
        tot = np.empty(n, np.float32)
        pol = np.empty(n, np.float32)
        self._check(self._L.fomo_thomson_emission(self.h, sid, _fp(tot), _fp(pol)))
        return tot, pol

    # -- rendering
    @staticmethod
    def request(snapshot, table=0, method=METHOD_NN, nx=16, ny=16, nz=16, nlambda=16, l=0.0, b=0.0,
                lambda_width=1e5, abundratio=1.0) -> Request:
        return Request(snapshot, table, method, nx, ny, nz, nlambda, l, b, lambda_width, abundratio)

    @staticmethod
    def cube_shape(req: Request):
        L = 1 if req.method == METHOD_THOMSON else req.nlambda
        return (req.ny, req.nx, L)

    def render(self, req: Request, want_idx: bool = False, out=None):
        """Render one view; returns (cube[ny, nx, L] float32, nn_idx or None, ViewInfo)."""
        shape = self.cube_shape(req)
        cube = np.empty(shape, np.float32) if out is None else out
        idx = np.empty((req.ny, req.nx, req.nz), np.int32) if want_idx else None
        info = ViewInfo()
        self._check(self._L.fomo_render(self.h, ctypes.byref(req), _fp(cube),
                                        idx.ctypes.data_as(_I32) if want_idx else None, ctypes.byref(info)))
        return cube, idx, info

    def render_batch(self, reqs, outs=None):
        n = len(reqs)
        arr = (Request * n)(*reqs)
        cubes = [np.empty(self.cube_shape(r), np.float32) for r in reqs] if outs is None else outs
        ptrs = (_F * n)(*[_fp(c) for c in cubes])
        infos = (ViewInfo * n)()
        self._check(self._L.fomo_render_batch(self.h, arr, n, ptrs, infos))
        return cubes, list(infos)

    def render_batch_device(self, reqs, dev_ptrs, stream=None, graph=False):
        n = len(reqs)
        arr = (Request * n)(*reqs)
        ptrs = (ctypes.c_void_p * n)(*dev_ptrs)
        fn = self._L.fomo_render_batch_graph if graph else self._L.fomo_render_batch_device
        self._check(fn(self.h, arr, n, ptrs, stream))

    def render_device(self, req, dev_ptr, stream=None):
        self._check(self._L.fomo_render_device(self.h, ctypes.byref(req), dev_ptr, None, None, stream))

    def autotune(self, reqs, cache_path=None):
        n = len(reqs)
        arr = (Request * n)(*reqs)
        self._check(self._L.fomo_autotune(self.h, arr, n, cache_path.encode() if cache_path else None))

    def set_march_config(self, tile_w=0, tile_h=0, blocks_per_sm=0):
        self._check(self._L.fomo_set_march_config(self.h, tile_w, tile_h, blocks_per_sm))

    def last_march_ms(self) -> float:
        ms = ctypes.c_float()
        self._check(self._L.fomo_last_march_ms(self.h, ctypes.byref(ms)))
        return ms.value

    def set_profiling(self, kernel_timing=True, counters=False):
        """Per-kernel event times and/or search counters of later direct renders."""
        self._check(self._L.fomo_set_profiling(self.h, int(kernel_timing), int(counters)))

    def profile_read(self):
        """({kernel: ms} of the last direct render, {counter: value} since the last read)."""
        ms = (ctypes.c_float * len(KERNELS))()
        cnt = (ctypes.c_uint64 * len(COUNTERS))()
        self._check(self._L.fomo_profile_read(self.h, ms, len(KERNELS), cnt, len(COUNTERS)))
        return dict(zip(KERNELS, list(ms))), dict(zip(COUNTERS, list(cnt)))

    def measure_ceilings(self) -> Ceilings:
        """L2 read and gather bandwidth and SFU ex2 throughput of this device."""
        c = Ceilings()
        self._check(self._L.fomo_measure_ceilings(self.h, ctypes.byref(c)))
        return c

    def register_host(self, arr: np.ndarray):
        self._check(self._L.fomo_host_register(self.h, arr.ctypes.data, arr.nbytes))

    def unregister_host(self, arr: np.ndarray):
        self._check(self._L.fomo_host_unregister(self.h, arr.ctypes.data))


class Server:
    """Continuous-batching render server (fomo_server_* in the C ABI)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, max_inflight: int = 0):
        self._L = lib()
        cfg = ServerConfig(device, hbm_budget, max_inflight)
        h = ctypes.c_void_p()
        rc = self._L.fomo_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != OK:
            raise FomoError(rc, "fomo_server_create failed")
        self.h = h
        self._outs = {}  # ticket -> the caller's result array, alive until wait()
        # the server's own context, for resident snapshots and tables
        self.ctx = Context.__new__(Context)
        self.ctx._L = self._L
        self.ctx.h = ctypes.c_void_p(self._L.fomo_server_context(h))

    def submit(self, req: Request, out: np.ndarray) -> int:
        """Queue a request; the result is written into `out` (float32, C-contiguous,
        at least the cube's size) when it completes.  `out` is kept alive here
        until wait() returns for the ticket."""
        if out.dtype != np.float32 or not out.flags.c_contiguous:
            raise FomoError(EINVAL, "out must be a C-contiguous float32 array")
        L = 1 if req.method == METHOD_THOMSON else req.nlambda
        if out.size < req.nx * req.ny * L:
            raise FomoError(EINVAL, f"out holds {out.size} floats, the cube needs {req.nx * req.ny * L}")
        t = ctypes.c_uint64()
        rc = self._L.fomo_server_submit(self.h, ctypes.byref(req), _fp(out), ctypes.byref(t))
        if rc != OK:
            raise FomoError(rc, self._L.fomo_server_last_error(self.h).decode())
        self._outs[t.value] = out
        return t.value

    def wait(self, ticket: int, timeout: float = 120.0) -> RequestStats:
        st = RequestStats()
        rc = self._L.fomo_server_wait(self.h, ticket, timeout, ctypes.byref(st))
        if rc != OK:
            if rc != ETIMEOUT:
                self._outs.pop(ticket, None)
            raise FomoError(rc, self._L.fomo_server_last_error(self.h).decode(), None if rc == ETIMEOUT else st)
        self._outs.pop(ticket, None)
        return st

    def cancel(self, ticket: int):
        rc = self._L.fomo_server_cancel(self.h, ticket)
        if rc != OK:
            raise FomoError(rc, "cancel failed")

    def close(self):
        if self.h:
            self._L.fomo_server_destroy(self.h)  # finishes or cancels what is in flight
            self.h = None
            self.ctx.h = None
            self._outs.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def abundance_ratio(abund_file: str, standard_file: str, ion: str) -> float:
    """Abundance renormalisation of `ion`'s element: (X/H) in abund_file over (X/H)
    in standard_file (fomo_abundance_ratio in the C ABI)."""
    r = ctypes.c_double()
    rc = lib().fomo_abundance_ratio(None, abund_file.encode(), standard_file.encode(), ion.encode(), ctypes.byref(r))
    if rc != OK:
        raise FomoError(rc, f"abundance files {abund_file!r} / {standard_file!r} do not give {ion!r}")
    return r.value


def render_grid(nx, ny, L, info: ViewInfo, is_dn: bool):
    """The per-element x, y (and lambda) grids of a render cube, regenerated on
    the host from the view extents exactly as the reference stores them
    (fomo-nearestneighbour.cpp:152-153, 209-211, 254-260)."""
    j = np.arange(nx, dtype=np.float64)
    i = np.arange(ny, dtype=np.float64)
    x = (j / (nx - 1) * (info.maxx - info.minx) + info.minx).astype(np.float32)
    y = (i / (ny - 1) * (info.maxy - info.miny) + info.miny).astype(np.float32)
    if is_dn:
        x = ((1.0 / 0.715) * x.astype(np.float64)).astype(np.float32)
        y = ((1.0 / 0.715) * y.astype(np.float64)).astype(np.float32)
    gx = np.broadcast_to(x[None, :, None], (ny, nx, L)).ravel().copy()
    gy = np.broadcast_to(y[:, None, None], (ny, nx, L)).ravel().copy()
    gl = None
    if L > 1:
        il = np.arange(L, dtype=np.float64)
        lw = info.lambda_width_A
        lam = (il / (L - 1) * lw - lw / 2.0 + info.lambda0).astype(np.float32)
        gl = np.broadcast_to(lam[None, None, :], (ny, nx, L)).ravel().copy()
    return gx, gy, gl
