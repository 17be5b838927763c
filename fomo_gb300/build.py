"""Build libfomo_gpu.so in-tree: hand-written CUDA for sm_103a plus the C++ runtime.

    python -m fomo_gb300.build            # build (incremental)
    python -m fomo_gb300.build --clean

Every translation unit is compiled by nvcc with
``-gencode arch=compute_103a,code=sm_103a`` in parallel, then linked with the
static CUDA runtime into ``fomo_gb300/libfomo_gpu.so``.  The same sources are
compiled a second time, at the same time, with ``-DFOMO_BOUNDS_CHECK=1`` into
``fomo_gb300/libfomo_gpu_checked.so``: the bounds-check build, in which every
gather and scatter index of the kernels is checked (an index out of range is
recorded in a device error word and reported as FOMO_EDEVICE instead of being
accessed).  It serves the tests, as the substitute for a memory checker.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfomo_gpu.so")
BUILD_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(HERE, "libfomo_gpu_checked.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfomo_gpu")
    return cand


def _flags(checked: bool = False):
    f = ["-std=c++17", "-O3", ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-O3", "-I" + CSRC,
         "-I" + os.path.join(ROOT, "include")]
    if checked:
        f.append("-DFOMO_BOUNDS_CHECK=1")
    return f


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers_mtime() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src: str, verbose: bool, checked: bool = False) -> str:
    obj = os.path.join(BUILD_CHECKED if checked else BUILD, os.path.basename(src) + ".o")
    hm = _headers_mtime()
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hm, os.path.getmtime(__file__)):
        return obj
    cmd = [_nvcc()] + _flags(checked)
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"] if verbose else []
    else:
        cmd += ["-x", "c++"]
    cmd += ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        with open(obj + ".log", "w") as f:
            f.write(r.stderr)
    return obj


def _link(objs, lib: str) -> None:
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(lib) or os.path.getmtime(lib) < newest:
        tmp = lib + ".tmp"
        cmd = [_nvcc(), ARCH, "-shared", "-cudart=static", "-o", tmp] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)


def build(verbose: bool = False, jobs: int | None = None, checked: bool = True) -> str:
    """Build libfomo_gpu.so and (unless checked=False) libfomo_gpu_checked.so;
    every translation unit of both compiles in parallel.  Returns the regular
    library's path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    tasks = [(s, False) for s in srcs]
    if checked:
        os.makedirs(BUILD_CHECKED, exist_ok=True)
        tasks += [(s, True) for s in srcs]
    # the largest translation units first, so that they do not finish last
    tasks.sort(key=lambda t: -os.path.getsize(t[0]))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 8, len(tasks))) as ex:
        objs = list(ex.map(lambda t: (t[1], _compile(t[0], verbose and not t[1], t[1])), tasks))
    _link(sorted(o for c, o in objs if not c), LIB)
    if checked:
        _link(sorted(o for c, o in objs if c), LIB_CHECKED)
    return LIB


def clean() -> None:
    shutil.rmtree(BUILD, ignore_errors=True)
    shutil.rmtree(BUILD_CHECKED, ignore_errors=True)
    for lib in (LIB, LIB_CHECKED):
        if os.path.exists(lib):
            os.remove(lib)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    else:
        print(build(verbose="-v" in sys.argv))
