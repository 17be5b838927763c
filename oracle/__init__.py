"""ctypes bindings for the CPU checkers.  TEST INFRASTRUCTURE ONLY.

* ``liboracle.so``        -- the C restatement of FoMo-C's NN render path
                             (oracle/fomo_oracle.c); the oracle.
* ``_ref/libfomo_ref.so`` -- the reference's own FoMo-C sources compiled here
                             with header shims for the absent GSL and Boost
                             (oracle/Makefile target ``ref``); used only in this
                             container to validate the oracle and to generate
                             the golden fixtures in tests/golden/.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
use this package, and only as the checker / baseline, never as the product.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libfomo_ref.so")


def ref_src() -> str:
    """The reference's fomo-c/src directory as the build recipe (oracle/Makefile)
    names it; FOMO_REFERENCE_SRC overrides it.  It exists only where the
    reference tree is mounted (not on the GPU host)."""
    try:
        r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True, check=True)
        return r.stdout.strip()
    except Exception:
        return ""

_F = ctypes.POINTER(ctypes.c_float)
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int32)

# view record layout (fomo_oracle.h)
V_MINX, V_MAXX, V_MINY, V_MAXY, V_MINZ, V_MAXZ, V_MAXDIST, V_DELTAZ, V_PATHLENGTH, V_APIX, V_SCALE, V_LWA = range(12)
V_COUNT = 12


def build(ref: bool = True) -> None:
    """Compile liboracle.so (always) and the reference build (when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref and os.path.isdir(ref_src()):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "-j8"], check=True)


_lib = None
_ref = None


def _fp(a):
    return None if a is None else a.ctypes.data_as(_F)


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _ip(a):
    return None if a is None else a.ctypes.data_as(_I)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = ctypes.CDLL(LIB_PATH)
        L.fo_table_read.restype = ctypes.c_int
        L.fo_emission.restype = ctypes.c_int
        L.fo_nn_render.restype = ctypes.c_int
        L.fo_thomson_render.restype = ctypes.c_int
        L.fo_bruteforce_query.restype = ctypes.c_int32
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        R = ctypes.CDLL(REF_PATH)
        R.ref_render.restype = ctypes.c_int
        R.ref_emission.restype = ctypes.c_int
        R.ref_thomson_emission.restype = ctypes.c_int
        R.ref_render_and_write.restype = ctypes.c_int
        R.ref_last_error.restype = ctypes.c_char_p
        _ref = R
    return _ref


def _c32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


# ---------------------------------------------------------------- oracle API

def table_read(path: str):
    cap = 1 << 20
    logT = np.zeros(cap, np.float32)
    logn = np.zeros(cap, np.float32)
    G = np.zeros(cap, np.float32)
    ion = ctypes.create_string_buffer(256)
    unit = ctypes.create_string_buffer(1024)
    hdr = np.zeros(4)
    nt = ctypes.c_int()
    nrho = ctypes.c_int()
    rc = lib().fo_table_read(path.encode(), ion, 256, unit, 1024, _dp(hdr), ctypes.byref(nt), ctypes.byref(nrho),
                             _fp(logT), _fp(logn), _fp(G), ctypes.c_long(cap))
    if rc != 0:
        raise RuntimeError(f"fo_table_read({path}) failed: {rc}")
    return dict(ion=ion.value.decode(), unit=unit.value.decode(), lambda0=hdr[0], atweight=hdr[1],
                logT=logT[:nt.value].copy(), logn=logn[:nrho.value].copy(),
                G=G[:nt.value * nrho.value].reshape(nrho.value, nt.value).copy())


def emission(snap, table, imaging: bool = False, abundratio: float = 1.0):
    n = snap.npoints
    eps = np.zeros(n, np.float32)
    w = np.zeros(n, np.float32)
    rc = lib().fo_emission(ctypes.c_long(n), _fp(snap.n), _fp(snap.T), table.nt, table.nrho, _fp(_c32(table.logT)),
                           _fp(_c32(table.logn)), _fp(_c32(table.G)), ctypes.c_double(table.lambda0),
                           ctypes.c_double(table.atweight), table.ion.encode(), int(imaging),
                           ctypes.c_double(abundratio), _fp(eps), _fp(w))
    if rc != 0:
        raise RuntimeError(f"fo_emission failed: {rc}")
    return eps, w


def thomson_emission(snap):
    n = snap.npoints
    tot = np.zeros(n, np.float32)
    pol = np.zeros(n, np.float32)
    lib().fo_thomson_emission(ctypes.c_long(n), _fp(snap.x), _fp(snap.y), _fp(snap.z), _fp(snap.n), _fp(tot),
                              _fp(pol))
    return tot, pol


def nn_render(snap, eps, w, lambda0, l, b, nx, ny, nz, L, lambda_width, is_dn=False, mode=0, nthreads=0,
              rows=None, want_idx=False):
    """One view; returns (cube[ny_rows, nx, L] float64, nnidx or None, view record)."""
    r0, r1 = (0, ny) if rows is None else rows
    nray = (r1 - r0) * nx
    cube = np.zeros(nray * L, np.float64)
    idx = np.zeros(nray * nz, np.int32) if want_idx else None
    view = np.zeros(V_COUNT)
    rc = lib().fo_nn_render(ctypes.c_long(snap.npoints), _fp(snap.x), _fp(snap.y), _fp(snap.z), _fp(_c32(eps)),
                            _fp(_c32(w)), _fp(snap.vx), _fp(snap.vy), _fp(snap.vz), ctypes.c_double(lambda0),
                            ctypes.c_double(l), ctypes.c_double(b), nx, ny, nz, L, ctypes.c_double(lambda_width),
                            int(is_dn), int(mode), int(nthreads), r0, r1, _dp(cube), _ip(idx), _dp(view))
    if rc != 0:
        raise RuntimeError(f"fo_nn_render failed: {rc}")
    cube = cube.reshape(r1 - r0, nx, L)
    if idx is not None:
        idx = idx.reshape(r1 - r0, nx, nz)
    return cube, idx, view


def thomson_render(snap, tot, pol, l, b, nx, ny, nz, mode=0, nthreads=0, rows=None, want_idx=False):
    r0, r1 = (0, ny) if rows is None else rows
    nray = (r1 - r0) * nx
    cube = np.zeros(nray, np.float64)
    idx = np.zeros(nray * nz, np.int32) if want_idx else None
    view = np.zeros(V_COUNT)
    rc = lib().fo_thomson_render(ctypes.c_long(snap.npoints), _fp(snap.x), _fp(snap.y), _fp(snap.z),
                                 _fp(_c32(tot)), _fp(_c32(pol)), ctypes.c_double(l), ctypes.c_double(b), nx, ny, nz,
                                 int(mode), int(nthreads), r0, r1, _dp(cube), _ip(idx), _dp(view))
    if rc != 0:
        raise RuntimeError(f"fo_thomson_render failed: {rc}")
    cube = cube.reshape(r1 - r0, nx, 1)
    if idx is not None:
        idx = idx.reshape(r1 - r0, nx, nz)
    return cube, idx, view


def projection_render(snap, eps, w, lambda0, l, b, nx, ny, nz, L, lambda_width, is_dn=False, mode=0,
                      want_pix=False):
    """Projection render (fomo-projection.cpp:17-193); returns (cube[ny, nx, L] float64,
    pixel index per point or None, view record)."""
    cube = np.zeros(nx * ny * L, np.float64)
    pix = np.zeros(snap.npoints, np.int32) if want_pix else None
    view = np.zeros(V_COUNT)
    rc = lib().fo_projection_render(ctypes.c_long(snap.npoints), _fp(snap.x), _fp(snap.y), _fp(snap.z),
                                    _fp(_c32(eps)), _fp(_c32(w)), _fp(snap.vx), _fp(snap.vy), _fp(snap.vz),
                                    ctypes.c_double(lambda0), ctypes.c_double(l), ctypes.c_double(b), nx, ny, nz, L,
                                    ctypes.c_double(lambda_width), int(is_dn), int(mode), _dp(cube), _ip(pix),
                                    _dp(view))
    if rc != 0:
        raise RuntimeError(f"fo_projection_render failed: {rc}")
    return cube.reshape(ny, nx, L), pix, view


def render_grid(nx, ny, L, view, lambda0, is_dn=False):
    n = nx * ny * L
    gx = np.zeros(n, np.float32)
    gy = np.zeros(n, np.float32)
    gl = np.zeros(n, np.float32) if L > 1 else None
    lib().fo_render_grid(nx, ny, L, _dp(np.ascontiguousarray(view, np.float64)), ctypes.c_double(lambda0),
                         int(is_dn), _fp(gx), _fp(gy), _fp(gl))
    return gx, gy, gl


def bruteforce_query(snap, target, lo, hi):
    t = _c32(target)
    a = _c32(lo)
    b = _c32(hi)
    return int(lib().fo_bruteforce_query(ctypes.c_long(snap.npoints), _fp(snap.x), _fp(snap.y), _fp(snap.z),
                                         _fp(t), _fp(a), _fp(b)))


# ------------------------------------------------------- reference build API

def ref_emission(snap, table_path: str, imaging: bool = False):
    n = snap.npoints
    eps = np.zeros(n, np.float32)
    w = np.zeros(n, np.float32)
    lam = ctypes.c_double()
    rc = ref().ref_emission(ctypes.c_long(n), *[_fp(a) for a in snap.arrays()], table_path.encode(), b"/empty",
                            int(imaging), _fp(eps), _fp(w), ctypes.byref(lam))
    if rc != 0:
        raise RuntimeError(ref().ref_last_error().decode())
    return eps, w


def ref_thomson_emission(snap):
    n = snap.npoints
    tot = np.zeros(n, np.float32)
    pol = np.zeros(n, np.float32)
    rc = ref().ref_thomson_emission(ctypes.c_long(n), *[_fp(a) for a in snap.arrays()], _fp(tot), _fp(pol))
    if rc != 0:
        raise RuntimeError(ref().ref_last_error().decode())
    return tot, pol


def ref_render(method: str, snap, table_path: str, l, b, nx, ny, nz, L, lambda_width, want_grid=False):
    """FoMoObject::render(l, b) of the reference; returns (intens, grids, meta)."""
    n = nx * ny * L
    out = np.zeros(n, np.float32)
    gx = np.zeros(n, np.float32) if want_grid else None
    gy = np.zeros(n, np.float32) if want_grid else None
    gl = np.zeros(n, np.float32) if (want_grid and L > 1) else None
    meta = np.zeros(10)
    rc = ref().ref_render(method.encode(), ctypes.c_long(snap.npoints), *[_fp(a) for a in snap.arrays()],
                          (table_path or "").encode(), b"/empty", ctypes.c_double(l), ctypes.c_double(b), nx, ny, nz,
                          L, ctypes.c_double(lambda_width), _fp(out), _fp(gx), _fp(gy), _fp(gl), _dp(meta))
    if rc != 0:
        raise RuntimeError(ref().ref_last_error().decode())
    return out, (gx, gy, gl), meta


def ref_render_and_write(method: str, snap, table_path: str, l, b, nx, ny, nz, L, lambda_width, options: int,
                         out_path: str):
    """FoMoObject::render(l, b) of the reference, then RenderCube::writegoftcube(out_path)
    with the write-option bits `options` (bit 0 binary .dat, bit 1 text .txt)."""
    rc = ref().ref_render_and_write(method.encode(), ctypes.c_long(snap.npoints), *[_fp(a) for a in snap.arrays()],
                                    (table_path or "").encode(), ctypes.c_double(l), ctypes.c_double(b), nx, ny, nz, L,
                                    ctypes.c_double(lambda_width), int(options), out_path.encode())
    if rc != 0:
        raise RuntimeError(ref().ref_last_error().decode())


def abundance_ratio(abund_file: str, standard_file: str, ion: str) -> float:
    """Restatement of abundfromchianti (fomo-CHIANTI.cpp:23-62) applied to both
    files and divided as at fomo-CHIANTI.cpp:264-273: 10^(A_el - A_H) of the
    ion's element ("fe_12" -> "fe", case-insensitive whole-symbol match) in
    abund_file over the same in standard_file."""
    def rel(path):
        name = ion.split("_")[0].lower()
        h = el = 0.0
        toks = open(path).read().split()
        i = 0
        while i + 2 < len(toks) + 0 and int(float(toks[i])) >= 0:
            value, sym = float(toks[i + 1]), toks[i + 2].lower()
            if sym == "h":
                h = value
            if sym == name:
                el = value
            i += 3
        if h == 0.0 or el == 0.0:
            raise ValueError(f"invalid abundance file {path}")
        return 10.0 ** (el - h)
    return rel(abund_file) / rel(standard_file)


def amrvac_read(datfile: str, parfile: str | None = None, amrvac_version: str = "gitlab", gamma_eqparposition: int = 0,
                n_unit: float = 1.0, Teunit: float = 1.0, L_unit: float = 1.0):
    """Restatement of the reference's AMRVAC reader (fo_amrvac_read): (ndim,
    [x, y, z, n, T, vx, vy, vz]) as float32 arrays in the reference's point
    order; z is zero for 2-D data."""
    L = lib()
    L.fo_amrvac_read.restype = ctypes.c_int
    nd, npts = ctypes.c_int(), ctypes.c_long()
    args = [datfile.encode(), parfile.encode() if parfile else None, int(amrvac_version == "gitlab"),
            int(gamma_eqparposition), ctypes.c_double(n_unit), ctypes.c_double(Teunit), ctypes.c_double(L_unit)]
    rc = L.fo_amrvac_read(*args, ctypes.c_long(0), ctypes.byref(nd), ctypes.byref(npts), *([None] * 8))
    if rc not in (0, -3):
        raise RuntimeError(f"fo_amrvac_read({datfile}) failed: {rc}")
    arrs = [np.zeros(npts.value, np.float32) for _ in range(8)]
    rc = L.fo_amrvac_read(*args, ctypes.c_long(npts.value), ctypes.byref(nd), ctypes.byref(npts),
                          *[_fp(a) for a in arrs])
    if rc != 0:
        raise RuntimeError(f"fo_amrvac_read({datfile}) failed: {rc}")
    return nd.value, arrs


def ref_amrvac_read(datfile: str, parfile: str | None, amrvac_version: str, gamma_eqparposition: int,
                    n_unit: float, Teunit: float, L_unit: float, cap: int = 1 << 22):
    """The reference's own AMRVAC reader (read_amrvac_dat_file, compiled from its
    sources into oracle/_ref): (ndim, [x, y, z, n, T, vx, vy, vz])."""
    R = ref()
    R.ref_amrvac_read.restype = ctypes.c_int
    nd, npts = ctypes.c_int(), ctypes.c_long()
    arrs = [np.zeros(cap, np.float32) for _ in range(8)]
    rc = R.ref_amrvac_read(datfile.encode(), (parfile or "").encode(), amrvac_version.encode(),
                           int(gamma_eqparposition), ctypes.c_double(n_unit), ctypes.c_double(Teunit),
                           ctypes.c_double(L_unit), ctypes.c_long(cap), ctypes.byref(nd), ctypes.byref(npts),
                           *[_fp(a) for a in arrs])
    if rc != 0:
        raise RuntimeError(f"ref_amrvac_read failed: {rc} {R.ref_last_error().decode()}")
    return nd.value, [a[:npts.value].copy() for a in arrs]
