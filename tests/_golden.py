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
    top = np.abs(ref).max()
    if top == 0:
        return float(np.abs(got).max())
    m = np.abs(ref) >= floor * top
    if not m.any():
        return 0.0
    return float((np.abs(got[m] - ref[m]) / np.abs(ref[m])).max())


# Per-configuration parity record, printed at the end of the pytest run
# (tests/conftest.py): the largest errors seen against the FP64 oracle and the
# neighbour indices compared, so the figures quoted for each configuration come
# from the asserting tests themselves.
REPORT: dict = {}


def _entry(case: str) -> dict:
    return REPORT.setdefault(case, dict(norm_max=0.0, l2=0.0, sig=0.0, cubes=0, nn_equal=0, nn_total=0))


def record(case: str, got, ref) -> float:
    """norm_max_err(got, ref), also kept (with the L2 and significant-element
    relative errors) as the running maximum of `case`."""
    e = _entry(case)
    err = norm_max_err(got, ref)
    e["norm_max"] = max(e["norm_max"], err)
    e["l2"] = max(e["l2"], l2_rel_err(got, ref))
    e["sig"] = max(e["sig"], sig_rel_err(got, ref))
    e["cubes"] += 1
    return err


def record_idx(case: str, idx, oidx) -> None:
    """Count equal neighbour indices of `case` (the caller asserts equality)."""
    idx = np.asarray(idx)
    oidx = np.asarray(oidx)
    e = _entry(case)
    if idx.shape == oidx.shape:
        e["nn_equal"] += int((idx == oidx).sum())
    e["nn_total"] += int(oidx.size)
