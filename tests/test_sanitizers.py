"""CPU: the host code under the compilers' sanitizers (memory and race
checking on the GPU itself is left to the bounds-check build).

* the oracle (oracle/fomo_oracle.c), driven through every entry point by
  tests/cpp/oracle_driver.c, built with AddressSanitizer and
  UndefinedBehaviorSanitizer (any report is fatal);
* the C++ cube writers and reader (fomo_io.cpp, with the cube classes of
  fomo_object.cpp) in the round-trip program, built with ASan + UBSan and,
  separately, ThreadSanitizer (the text body is formatted and parsed by
  several threads): they must run clean and write the same bytes as the
  library's own build.

The reference has no sanitizer runs; its NN loop has a data race on its
progress counter (fomo-nearestneighbour.cpp:228).
"""

import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

import fomo_gb300 as fg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fomo_gb300", "csrc")
GOLD = os.path.join(ROOT, "tests", "golden")
ASAN = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-g", "-O1"]
TSAN = ["-fsanitize=thread", "-fno-omit-frame-pointer", "-g", "-O1"]


def _supported(flags, tmp):
    src = os.path.join(tmp, "probe.c")
    with open(src, "w") as f:
        f.write("int main(void) { return 0; }\n")
    r = subprocess.run(["gcc", *flags, src, "-o", os.path.join(tmp, "probe")], capture_output=True)
    return r.returncode == 0 and subprocess.run([os.path.join(tmp, "probe")], capture_output=True).returncode == 0


@pytest.fixture(scope="module")
def sanbin(tmp_path_factory):
    if shutil.which("gcc") is None or shutil.which("g++") is None:
        pytest.skip("gcc / g++ not available")
    tmp = str(tmp_path_factory.mktemp("san"))
    if not _supported(ASAN, tmp):
        pytest.skip("the compiler's address / undefined-behaviour sanitizers are not available here")
    return tmp


def _env():
    env = dict(os.environ)
    env["ASAN_OPTIONS"] = "detect_leaks=1:abort_on_error=0:halt_on_error=1"
    env["UBSAN_OPTIONS"] = "print_stacktrace=1:halt_on_error=1"
    env["TSAN_OPTIONS"] = "halt_on_error=1:second_deadlock_stack=1"
    env["OMP_NUM_THREADS"] = "2"
    return env


def test_oracle_under_address_and_undefined_sanitizers(sanbin, tmp_path):
    exe = os.path.join(sanbin, "oracle_driver")
    r = subprocess.run(["gcc", "-std=c11", *ASAN, "-ffp-contract=off", "-fopenmp", "-I", os.path.join(ROOT, "oracle"),
                        os.path.join(ROOT, "oracle", "fomo_oracle.c"),
                        os.path.join(ROOT, "tests", "cpp", "oracle_driver.c"), "-lm", "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    env = _env()
    env["ASAN_OPTIONS"] = "detect_leaks=0:halt_on_error=1"  # libgomp keeps its thread pool to exit
    r = subprocess.run([exe, str(tmp_path / "table.dat")], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
    assert "runtime error" not in r.stderr and "Sanitizer" not in r.stderr, r.stderr


def _roundtrip(sanbin, flags, tag):
    if not os.path.exists(fg.LIB_PATH):
        from fomo_gb300 import build
        build.build()
    exe = os.path.join(sanbin, "roundtrip_" + tag)
    libdir = os.path.dirname(fg.LIB_PATH)
    # the cube classes and the I/O compiled into the program with the
    # sanitizer; the C ABI the object layer calls comes from the library
    r = subprocess.run(["g++", "-std=c++17", *flags, "-I", os.path.join(ROOT, "include"), "-I", CSRC,
                        os.path.join(ROOT, "tests", "cpp", "roundtrip_cube.cpp"), os.path.join(CSRC, "fomo_io.cpp"),
                        os.path.join(CSRC, "fomo_object.cpp"), "-L", libdir, "-lfomo_gpu", "-Wl,-rpath," + libdir,
                        "-pthread", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _cases(tmp_path):
    """The reference's own cube files, and a cube of 300,000 random rows (ten
    blocks of lines for the threads)."""
    rng = np.random.default_rng(9)
    ng = 300_000
    cols = np.stack([rng.uniform(-5, 5, ng), rng.uniform(-5, 5, ng), rng.uniform(170, 172, ng),
                     rng.lognormal(0, 6, ng)]).astype(np.float32)
    big = str(tmp_path / "big.dat")
    with open(big, "wb") as f:
        f.write(b"FoMo-vtest#")
        f.write(struct.pack("<iii", 3, ng, 1))
        for s in ["Mm", "Mm", "A", "erg", "table.dat", "/empty"]:
            f.write(struct.pack("<q", len(s)) + s.encode())
        f.write(cols.tobytes())
    return [os.path.join(GOLD, f"writer_{c}.dat") for c in ("nn", "img", "th")] + [big]


@pytest.mark.parametrize("kind", ["asan_ubsan", "tsan"])
def test_cube_io_under_sanitizers(sanbin, tmp_path, kind):
    flags = ASAN if kind == "asan_ubsan" else TSAN
    if kind == "tsan" and not _supported(TSAN, sanbin):
        pytest.skip("the thread sanitizer is not available here")
    san = _roundtrip(sanbin, flags, kind)
    plain = _roundtrip(sanbin, ["-O1"], "plain_" + kind)
    env = _env()
    for k, src in enumerate(_cases(tmp_path)):
        outs = {}
        for tag, exe in (("san", san), ("plain", plain)):
            d = tmp_path / f"{tag}{k}"
            d.mkdir()
            # .dat -> .dat + .txt + .gz, then the .txt read back -> .dat
            r = subprocess.run([exe, src, str(d / "c.txt"), str(0b0111)], capture_output=True, text=True, env=env,
                               timeout=600)
            assert r.returncode == 0, (tag, src, r.stderr[-3000:])
            r = subprocess.run([exe, str(d / "c.txt"), str(d / "back.txt"), "1"], capture_output=True, text=True,
                               env=env, timeout=600)
            assert r.returncode == 0, (tag, src, r.stderr[-3000:])
            assert "Sanitizer" not in r.stderr and "runtime error" not in r.stderr, r.stderr[-3000:]
            outs[tag] = [open(str(d / f), "rb").read() for f in ("c.dat", "c.txt", "c.txt.gz", "back.dat")]
        assert outs["san"] == outs["plain"], src
