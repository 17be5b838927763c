"""Seeded synthetic snapshots and G(T, n) tables for the NN render workloads.

The reference ships no test data for this path (its example input and all
spectral-line G(T) tables are missing from the repository), so every workload
here is synthetic, with the shapes and value distributions of the benchmark
configurations:

* ``loop_snapshot``      -- jittered regular grid with a coronal loop (cylinder
  r < 1 Mm along z), n/T blended by a tanh of width 0.2 Mm, kink velocity
  vx = 10 km/s * sin(2 pi z / 10 Mm).
* ``flux_rope_snapshot`` -- 80 % of the points in a twisted flux rope, 20 %
  uniform background, log-uniform n and T.
* ``line_table``         -- 101 logT (4..8) x 41 logn (8..12) Gaussian-in-logT
  table written in the CHIANTI text format that ``readgoftfromchianti``
  parses (fomo-c/src/fomo-CHIANTI.cpp:143-218).

Coordinates are Mm, n in cm^-3, T in K, v in m/s, all float32 like the
reference's DataCube (fomo-c/src/FoMo.h:20-32).
"""

from __future__ import annotations

import dataclasses
import math
import os

import numpy as np

__all__ = [
    "Snapshot",
    "Table",
    "loop_snapshot",
    "flux_rope_snapshot",
    "thomson_snapshot",
    "line_table",
    "broadband_table",
    "write_table",
    "parse_table_text",
]


@dataclasses.dataclass
class Snapshot:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    n: np.ndarray
    T: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    vz: np.ndarray

    @property
    def npoints(self) -> int:
        return int(self.x.shape[0])

    def arrays(self):
        return (self.x, self.y, self.z, self.n, self.T, self.vx, self.vy, self.vz)

    def nbytes(self) -> int:
        return sum(a.nbytes for a in self.arrays())


@dataclasses.dataclass
class Table:
    """A G(T, n) table as the reference holds it after parsing.

    ``logT`` (nt) and ``logn`` (nrho) are the axes, ``G`` is (nrho, nt) with T
    fastest, all float32 (parsed as double then stored as float, as
    fomo-CHIANTI.cpp:176-188 does).
    """

    ion: str
    lambda0: float
    atweight: float
    minlevel: float
    maxlevel: float
    unit: str
    version: str
    logT: np.ndarray
    logn: np.ndarray
    G: np.ndarray

    @property
    def nt(self) -> int:
        return int(self.logT.shape[0])

    @property
    def nrho(self) -> int:
        return int(self.logn.shape[0])

    @property
    def is_dn(self) -> bool:
        return "DN" in self.unit


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def loop_snapshot(n_side: int, seed: int = 1, half_width: float = 5.0,
                  jitter: float = 0.1, center=(0.0, 0.0, 0.0)) -> Snapshot:
    """Coronal loop on an n_side^3 jittered grid over [-hw, hw]^3 Mm.

    Inside the loop (r < 1 Mm) n = 1e9 cm^-3, T = 1e6 K; outside n = 1e8,
    T = 2e6; blend f = (1 - tanh((r - 1)/0.2))/2.  vx = 1e4 sin(2 pi z/10).
    Jitter is uniform in +-jitter cells per coordinate.
    """
    rng = np.random.default_rng(seed)
    cell = 2.0 * half_width / (n_side - 1)
    ax = -half_width + cell * np.arange(n_side, dtype=np.float64)
    zz, yy, xx = np.meshgrid(ax, ax, ax, indexing="ij")
    x = xx.ravel() + rng.uniform(-jitter, jitter, xx.size) * cell
    y = yy.ravel() + rng.uniform(-jitter, jitter, xx.size) * cell
    z = zz.ravel() + rng.uniform(-jitter, jitter, xx.size) * cell
    r = np.sqrt(x * x + y * y)
    f = 0.5 * (1.0 - np.tanh((r - 1.0) / 0.2))
    n = f * 1e9 + (1.0 - f) * 1e8
    T = f * 1e6 + (1.0 - f) * 2e6
    vx = 1e4 * np.sin(2.0 * np.pi * z / 10.0)
    zeros = np.zeros_like(x)
    return Snapshot(_f32(x + center[0]), _f32(y + center[1]), _f32(z + center[2]), _f32(n), _f32(T),
                    _f32(vx), _f32(zeros), _f32(zeros))


def flux_rope_snapshot(npoints: int, seed: int = 4, half_width: float = 10.0,
                       rope_radius: float = 1.5, twist_length: float = 20.0,
                       rope_fraction: float = 0.8, center=(0.0, 0.0, 0.0)) -> Snapshot:
    """Nonuniform cloud: a twisted flux rope along z plus uniform background.

    A fraction ``rope_fraction`` of the points fill a cylinder of radius
    ``rope_radius`` (uniform in area) along z, with the azimuth advanced by
    2 pi z / twist_length; the rest fill the cube [-hw, hw]^3 uniformly.  n is
    log-uniform in 1e8..1e10, T log-uniform in 5e5..5e6 K, and the velocity is
    the rope's twist flow (10 km/s azimuthal inside the rope).
    """
    rng = np.random.default_rng(seed)
    n_rope = int(round(npoints * rope_fraction))
    n_bg = npoints - n_rope
    rad = rope_radius * np.sqrt(rng.uniform(0.0, 1.0, n_rope))
    zr = rng.uniform(-half_width, half_width, n_rope)
    phi = rng.uniform(0.0, 2.0 * np.pi, n_rope) + 2.0 * np.pi * zr / twist_length
    xr = rad * np.cos(phi)
    yr = rad * np.sin(phi)
    xb = rng.uniform(-half_width, half_width, n_bg)
    yb = rng.uniform(-half_width, half_width, n_bg)
    zb = rng.uniform(-half_width, half_width, n_bg)
    x = np.concatenate([xr, xb])
    y = np.concatenate([yr, yb])
    z = np.concatenate([zr, zb])
    perm = rng.permutation(npoints)
    x, y, z = x[perm], y[perm], z[perm]
    n = 10.0 ** rng.uniform(8.0, 10.0, npoints)
    T = 10.0 ** rng.uniform(math.log10(5e5), math.log10(5e6), npoints)
    rr = np.sqrt(x * x + y * y)
    inside = rr < rope_radius
    vphi = np.where(inside, 1e4, 0.0)
    safe = np.maximum(rr, 1e-6)
    vx = -vphi * y / safe
    vy = vphi * x / safe
    vz = np.zeros_like(x)
    return Snapshot(_f32(x + center[0]), _f32(y + center[1]), _f32(z + center[2]), _f32(n), _f32(T),
                    _f32(vx), _f32(vy), _f32(vz))


def thomson_snapshot(n_side: int, seed: int = 7, center_rsun: float = 1.5) -> Snapshot:
    """The loop cloud moved out to r ~ center_rsun solar radii (along +x).

    The reference's Thomson coefficients are NaN inside the Sun (r < 695.7 Mm,
    fomo-c/src/fomo-thomson.cpp:39-45), so Thomson clouds must sit at r > R_sun.
    """
    rsun = 695.7
    return loop_snapshot(n_side, seed=seed, center=(center_rsun * rsun, 0.0, 0.0))


def _table_G(logT, logn, peak_logT=6.0, sigma=0.15, amplitude=1e-24, n_slope=0.05):
    lt = logT[None, :]
    ln = logn[:, None]
    return amplitude * np.exp(-((lt - peak_logT) ** 2) / (2.0 * sigma * sigma)) * (1.0 + n_slope * (ln - 10.0))


def _as_parsed_f32(values: np.ndarray) -> np.ndarray:
    # The text is written with repr() (round-trips the double exactly); the
    # reference parses it as double and stores it as float.
    return _f32(np.asarray(values, dtype=np.float64))


def line_table(peak_logT: float = 6.0, lambda0: float = 171.073, ion: str = "fe_9",
               atweight: float = 55.845, sigma: float = 0.15, amplitude: float = 1e-24,
               nt: int = 101, nrho: int = 41) -> Table:
    """Spectral-line table: G = A exp(-(logT - peak)^2 / (2 sigma^2)) (1 + 0.05 (logn - 10))."""
    logT = np.linspace(4.0, 8.0, nt)
    logn = np.linspace(8.0, 12.0, nrho)
    G = _table_G(logT, logn, peak_logT, sigma, amplitude)
    return Table(ion=ion, lambda0=float(lambda0), atweight=float(atweight), minlevel=1.0, maxlevel=2.0,
                 unit="erg cm^3 s^-1 sr^-1", version="synthetic-1", logT=_as_parsed_f32(logT),
                 logn=_as_parsed_f32(logn), G=_as_parsed_f32(G))


def broadband_table(channel: int = 171, peak_logT: float = 5.9, sigma: float = 0.2,
                    amplitude: float = 1e-27, nt: int = 101, nrho: int = 41) -> Table:
    """Broadband (imaging) response table.

    The ion field is the integer channel wavelength so that the reference's
    imaging check ``atoi(ion) == int(lambda0 + 0.5)`` passes
    (fomo-CHIANTI.cpp:278), and the unit contains "DN" so the arcsec / per-pixel
    scaling runs (fomo-nearestneighbour.cpp:254-265).
    """
    logT = np.linspace(4.0, 8.0, nt)
    logn = np.linspace(8.0, 12.0, nrho)
    G = _table_G(logT, logn, peak_logT, sigma, amplitude, n_slope=0.0)
    return Table(ion=str(int(channel)), lambda0=float(channel), atweight=0.0, minlevel=float(channel) - 1.0,
                 maxlevel=float(channel) + 1.0, unit="cm^5 DN s^{-1} sr^{-1}", version="synthetic-1",
                 logT=_as_parsed_f32(logT), logn=_as_parsed_f32(logn), G=_as_parsed_f32(G))


def _fmt(v: float) -> str:
    return repr(float(v))


def table_text(t: Table, logT_text=None, logn_text=None, G_text=None) -> str:
    logT = t.logT if logT_text is None else logT_text
    logn = t.logn if logn_text is None else logn_text
    G = t.G if G_text is None else G_text
    lines = [t.ion, _fmt(t.lambda0), _fmt(t.atweight), f"{_fmt(t.minlevel)} {_fmt(t.maxlevel)}", t.unit,
             t.version, f"{t.nrho} {t.nt}", " ".join(_fmt(v) for v in logT)]
    for r in range(t.nrho):
        lines.append(_fmt(logn[r]) + " " + " ".join(_fmt(v) for v in G[r]))
    return "\n".join(lines) + "\n"


def write_table(t: Table, path: str) -> str:
    """Write ``t`` in the CHIANTI text format (float32 values, written exactly)."""
    with open(path, "w") as f:
        f.write(table_text(t, t.logT.astype(np.float64), t.logn.astype(np.float64), t.G.astype(np.float64)))
    return path


def parse_table_text(text: str) -> Table:
    """Parse the CHIANTI text format like fomo-CHIANTI.cpp:143-218 (test helper)."""
    lines = text.split("\n")
    toks0 = " ".join(lines[:4]).split()
    ion, lambda0, atweight, minlevel, maxlevel = toks0[0], float(toks0[1]), float(toks0[2]), float(toks0[3]), float(toks0[4])
    # header occupies the first tokens up to maxlevel; the rest of that line is skipped
    idx = 0
    seen = 0
    for i, ln in enumerate(lines):
        seen += len(ln.split())
        if seen >= 5:
            idx = i
            break
    unit = lines[idx + 1]
    version = lines[idx + 2]
    rest = " ".join(lines[idx + 3:]).split()
    nrho, nt = int(rest[0]), int(rest[1])
    vals = [float(v) for v in rest[2:]]
    logT = np.array(vals[:nt])
    body = np.array(vals[nt:]).reshape(-1, nt + 1)
    return Table(ion=ion, lambda0=lambda0, atweight=atweight, minlevel=minlevel, maxlevel=maxlevel, unit=unit,
                 version=version, logT=_f32(logT), logn=_f32(body[:, 0]), G=_f32(body[:, 1:]))


def ensure_dir(path: str) -> str:
    os.makedirs(path, exist_ok=True)
    return path
