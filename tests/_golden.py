"""Helpers to load the golden fixtures (tests/golden/*.npz) and the error metrics."""

from __future__ import annotations

import os
import platform
import tempfile

import numpy as np

from fomo_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name: str):
    return dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))


def snapshot(d) -> synth.Snapshot:
    return synth.Snapshot(*(np.ascontiguousarray(d[k]) for k in ("x", "y", "z", "n", "T", "vx", "vy", "vz")))


def table(d, key="table_text") -> synth.Table:
    return synth.parse_table_text(bytes(d[key]).decode())


def table_file(d, key="table_text") -> str:
    fd, path = tempfile.mkstemp(suffix=".dat")
    with os.fdopen(fd, "wb") as f:
        f.write(bytes(d[key]))
    return path


def same_platform(d) -> bool:
    return str(d["platform"]) == platform.machine()


def norm_max_err(got, ref) -> float:
    """max|g - o| / max|o| -- the gate metric (<= 1e-4)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.abs(ref).max()
    if den == 0:
        return float(np.abs(got).max())
    return float(np.abs(got - ref).max() / den)


def l2_rel_err(got, ref) -> float:
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(got - ref) / den) if den else float(np.linalg.norm(got))


def sig_rel_err(got, ref, floor=1e-6) -> float:
    """Max relative error over elements with |o| >= floor * max|o| (reported)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    m = np.abs(ref) >= floor * np.abs(ref).max()
    if not m.any():
        return 0.0
    return float((np.abs(got[m] - ref[m]) / np.abs(ref[m])).max())
