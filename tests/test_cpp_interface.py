"""The C++ object interface (include/FoMo.h) as a FoMo-C user sees it.

CPU: the reader and writers reproduce the reference's own output files
byte for byte (tests/golden/writer_*, written by the reference's
RenderCube::writegoftcube, fomo-io.cpp:26-150), the gzip option produces
readable .gz files, and a user program in the style of the reference's
example (fomo-c/example/example.cpp) compiles, links and -- without a GPU --
fails loudly instead of falling back to a CPU path.

GPU: that program renders the golden cases through FoMoObject::render and its
files match the reference's: same header, same image grid (bit for bit), the
intensities within the render tolerance.
"""

import gzip
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

import fomo_gb300 as fg
from tests import _golden as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
TOL = 1e-4  # normalised max error of a rendered cube


def read_cube(path):
    """Parse a FoMo cube file (.txt or .dat, optionally .gz) into a dict."""
    raw = open(path, "rb").read()
    if path.endswith(".gz"):
        raw = gzip.decompress(raw)
    stem = path[:-3] if path.endswith(".gz") else path
    if stem.endswith(".dat"):
        end = raw.index(b"#")
        version = raw[:end].decode()
        off = end + 1
        dim, ng, nvars = struct.unpack_from("<iii", raw, off)
        off += 12

        def string():
            nonlocal off
            (n,) = struct.unpack_from("<q", raw, off)
            off += 8
            s = raw[off:off + n].decode()
            off += n
            return s

        units = [string() for _ in range(dim + nvars)]
        chianti, abund = string(), string()
        cols = np.frombuffer(raw, np.float32, (dim + nvars) * ng, off).reshape(dim + nvars, ng)
        return dict(version=version, dim=dim, ng=ng, nvars=nvars, units=units, chianti=chianti, abund=abund,
                    data=cols.T.copy(), body=raw[end:])
    lines = raw.decode().split("\n")
    dim, ng, nvars = int(lines[1]), int(lines[2]), int(lines[3])
    units = lines[4].split("\t")[:dim + nvars]
    rows = [list(map(float, ln.split())) for ln in lines[7:7 + ng]]
    return dict(version=lines[0], dim=dim, ng=ng, nvars=nvars, units=units, chianti=lines[5], abund=lines[6],
                data=np.array(rows, np.float64).reshape(ng, dim + nvars), body="\n".join(lines[1:]).encode())


@pytest.fixture(scope="module")
def programs(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    if not os.path.exists(fg.LIB_PATH):
        from fomo_gb300 import build
        build.build()
    out = tmp_path_factory.mktemp("cpp")
    libdir = os.path.dirname(fg.LIB_PATH)
    progs = {}
    for name in ("example_render", "roundtrip_cube", "resolution_units"):
        exe = str(out / name)
        cmd = ["g++", "-std=c++11", "-O1", "-I", os.path.join(ROOT, "include"),
               os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-L", libdir, "-lfomo_gpu",
               "-Wl,-rpath," + libdir, "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        progs[name] = exe
    return progs


# ---------------------------------------------------------------- CPU

@pytest.mark.parametrize("case", ["nn", "img", "th"])
def test_writers_reproduce_the_reference_files(programs, tmp_path, case):
    src = os.path.join(GOLD, f"writer_{case}.dat")
    out = str(tmp_path / "copy.txt")
    r = subprocess.run([programs["roundtrip_cube"], src, out, "3"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for ext in (".dat", ".txt"):
        ours, ref = read_cube(str(tmp_path / ("copy" + ext))), read_cube(os.path.join(GOLD, f"writer_{case}{ext}"))
        assert ours["version"].startswith("FoMo-v") and ref["version"].startswith("FoMo-v")
        assert ours["body"] == ref["body"], ext  # everything after the version string


def test_reader_accepts_the_reference_text_format(programs, tmp_path):
    src = os.path.join(GOLD, "writer_nn.txt")
    out = str(tmp_path / "fromtext.dat")
    r = subprocess.run([programs["roundtrip_cube"], src, out, "1"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ours, ref = read_cube(out), read_cube(os.path.join(GOLD, "writer_nn.dat"))
    assert (ours["dim"], ours["ng"], ours["nvars"]) == (ref["dim"], ref["ng"], ref["nvars"])
    assert ours["units"] == ref["units"] and ours["chianti"] == ref["chianti"]
    np.testing.assert_allclose(ours["data"], ref["data"], rtol=1e-7, atol=0)


def test_gzip_option_and_delete_option(programs, tmp_path):
    src = os.path.join(GOLD, "writer_img.dat")
    out = str(tmp_path / "z.txt")
    r = subprocess.run([programs["roundtrip_cube"], src, out, str(0b0111)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for ext in (".dat", ".txt"):
        plain = open(str(tmp_path / ("z" + ext)), "rb").read()
        assert gzip.decompress(open(str(tmp_path / ("z" + ext + ".gz")), "rb").read()) == plain
    out2 = str(tmp_path / "d.txt")
    r = subprocess.run([programs["roundtrip_cube"], src, out2, str(0b1111)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert not os.path.exists(str(tmp_path / "d.dat")) and not os.path.exists(str(tmp_path / "d.txt"))
    assert read_cube(str(tmp_path / "d.dat.gz"))["body"] == read_cube(src)["body"]


def test_gzip_output_is_compressed_and_exact(programs, tmp_path):
    """The .gz files are DEFLATE streams (several 1 MB chunks compressed at
    once, Huffman codes made per chunk, stored blocks where the data do not
    compress) that any gzip reader turns back into the plain file's bytes; the
    text of a cube compresses as zlib's default level does, within 10 %."""
    import zlib
    rng = np.random.default_rng(13)
    ng = 120_000  # about 5 MB of text: several chunks
    cols = np.stack([rng.uniform(-5, 5, ng).astype(np.float32), rng.uniform(-5, 5, ng).astype(np.float32),
                     rng.uniform(170, 172, ng).astype(np.float32),
                     rng.integers(0, 2 ** 32, ng, dtype=np.uint64).astype(np.uint32).view(np.float32)])
    src = str(tmp_path / "in.dat")
    _write_dat(src, cols, 3, ["Mm", "Mm", "A", "erg"])
    out = str(tmp_path / "z.txt")
    r = subprocess.run([programs["roundtrip_cube"], src, out, str(0b0111)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for ext in (".txt", ".dat"):
        plain = open(str(tmp_path / ("z" + ext)), "rb").read()
        packed = open(str(tmp_path / ("z" + ext + ".gz")), "rb").read()
        assert gzip.decompress(packed) == plain, ext
        assert len(packed) <= 1.1 * len(zlib.compress(plain, 6)) + 64, (ext, len(packed), len(plain))
    assert len(open(str(tmp_path / "z.txt.gz"), "rb").read()) < 0.6 * os.path.getsize(str(tmp_path / "z.txt"))


def test_gzip_of_skewed_and_repetitive_bytes(programs, tmp_path):
    """Byte counts in a Fibonacci progression (a Huffman tree 24 deep, which
    the 15-bit limit of DEFLATE must flatten), long runs (matches of the
    longest length, 258, at distance 1) and the cube text around them: every
    .gz must read back to the plain bytes."""
    rng = np.random.default_rng(17)
    fib = [1, 1]
    while len(fib) < 26:
        fib.append(fib[-1] + fib[-2])
    skewed = np.repeat(np.arange(26, dtype=np.uint8) * 9 + 7, fib)
    rng.shuffle(skewed)
    runs = np.concatenate([np.full(300_000, 0x41, np.uint8), np.full(70_001, 0x00, np.uint8),
                           np.tile(np.arange(7, dtype=np.uint8), 40_000)])
    raw = np.concatenate([skewed, runs])
    raw = raw[: raw.size // 4 * 4]
    col = raw.view(np.float32)
    ng = col.size // 2
    cols = np.stack([col[:ng], col[ng:2 * ng]])
    src = str(tmp_path / "in.dat")
    _write_dat(src, cols, 1, ["Mm", "erg"])
    out = str(tmp_path / "z.txt")
    r = subprocess.run([programs["roundtrip_cube"], src, out, str(0b0111)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for ext in (".txt", ".dat"):
        plain = open(str(tmp_path / ("z" + ext)), "rb").read()
        assert gzip.decompress(open(str(tmp_path / ("z" + ext + ".gz")), "rb").read()) == plain, ext
    assert os.path.getsize(str(tmp_path / "z.dat.gz")) < 0.7 * os.path.getsize(str(tmp_path / "z.dat"))


@pytest.mark.parametrize("ng", [131061, 131062, 131063, 262124])
def test_gzip_at_chunk_boundaries(programs, tmp_path, ng):
    """The .dat of a 1-column cube is 80 header bytes + 8 per point: these
    sizes put its end just before, on and just past the 1 MB chunk boundary
    of the compressor (a last chunk of 8 bytes), and on two chunks exactly."""
    rng = np.random.default_rng(ng)
    cols = np.stack([np.round(rng.uniform(-5, 5, ng), 2).astype(np.float32),
                     rng.integers(0, 2 ** 32, ng, dtype=np.uint64).astype(np.uint32).view(np.float32)])
    src = str(tmp_path / "in.dat")
    _write_dat(src, cols, 1, ["Mm", "erg"])
    out = str(tmp_path / "z.dat")
    r = subprocess.run([programs["roundtrip_cube"], src, out, str(0b0101)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    plain = open(out, "rb").read()
    assert len(plain) == 80 + 8 * ng
    assert gzip.decompress(open(out + ".gz", "rb").read()) == plain


def _write_dat(path, cols, dim, units):
    """A .dat cube (the binary format above) from FP32 columns [dim + nvars][ng]."""
    with open(path, "wb") as f:
        f.write(b"FoMo-vtest#")
        f.write(struct.pack("<iii", dim, cols.shape[1], cols.shape[0] - dim))
        for s in units + ["table.dat", "/empty"]:
            f.write(struct.pack("<q", len(s)) + s.encode())
        f.write(np.ascontiguousarray(cols, np.float32).tobytes())


def test_text_writer_formats_every_float_like_the_stream(programs, tmp_path):
    """The text body is formatted by several threads in blocks of lines; every
    value must still read as the reference's stream writes it at precision 8,
    which is the C library's "%.8g" of the float widened to double.  Checked on
    557,179 lines (18 blocks of 2^15 lines: more than one wave of threads) of
    random bit patterns of every class (subnormals, normals over the whole
    exponent range, zeros, infinities, NaNs of either sign) and random values,
    with the line number as one column so that a block out of order shows."""
    import ctypes
    rng = np.random.default_rng(11)
    ng = 17 * 32768 + 123
    bits = rng.integers(0, 2 ** 32, ng, dtype=np.uint64).astype(np.uint32)
    special = np.array([0, 0x80000000, 0x7F800000, 0xFF800000, 0x7FC00000, 0xFFC00000, 0x7F800001, 1, 0x807FFFFF,
                        0x00800000, 0x7F7FFFFF, 0xFF7FFFFF, 0x3F800000, 0x4B189680], np.uint32)
    bits[:special.size] = special
    cols = np.stack([bits.view(np.float32),
                     (rng.standard_normal(ng) * 10.0 ** rng.integers(-12, 12, ng)).astype(np.float32),
                     np.arange(ng, dtype=np.float32),
                     rng.uniform(170.0, 172.0, ng).astype(np.float32)])
    src = str(tmp_path / "in.dat")
    _write_dat(src, cols, 3, ["Mm", "Mm", "A", "erg"])
    out = str(tmp_path / "out.txt")
    r = subprocess.run([programs["roundtrip_cube"], src, out, "2"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = open(out, "rb").read().decode().split("\n")
    assert lines[:7] == ["FoMo-" + lines[0][5:], "3", str(ng), "1", "Mm\tMm\tA\terg\t", "table.dat", "/empty"]
    assert len(lines) == 7 + ng + 1 and lines[-1] == ""
    libc = ctypes.CDLL(None)
    buf = ctypes.create_string_buffer(64)

    def printf_g8(v):
        libc.snprintf(buf, 64, b"%.8g", ctypes.c_double(float(v)))
        return buf.value.decode()

    with np.errstate(invalid="ignore"):  # the signalling NaNs are quieted, as the C++ widening does
        vals = cols.T.astype(np.float64)
    for c in range(4):
        got = [ln.split(" ")[c] for ln in lines[7:7 + ng]]
        col = vals[:, c]
        nan = np.isnan(col)
        # Python's "%.8g" rounds exactly as the C library does for finite and
        # infinite values; NaNs (whose sign the C library prints) go through it
        want = ["%.8g" % v for v in col]
        for k in np.flatnonzero(nan):
            want[k] = printf_g8(col[k])
        bad = [k for k in range(ng) if got[k] != want[k]]
        assert not bad, (c, [(k, got[k], want[k]) for k in bad[:5]])
    assert all(ln.endswith(" ") for ln in lines[7:7 + ng])
    # the C library agrees with Python's formatting on a sample of the finite values
    for v in vals[:4000, 0][np.isfinite(vals[:4000, 0])]:
        assert printf_g8(v) == "%.8g" % v


def test_text_reader_reads_what_the_stream_reads(programs, tmp_path):
    """readgoftcube parses a text body by several threads with std::from_chars;
    every value must be the float the reference's stream read (strtof in the
    "C" locale) gives.  The same file with its first value written "+v" (a
    form only the stream takes) is read value by value through the stream: the
    two reads must agree bit for bit, and with the C library's strtof on a
    sample.  Text the stream rejects (nan, a missing value) is an error."""
    import ctypes
    rng = np.random.default_rng(5)
    ng = 9 * 32768 + 77
    bits = rng.integers(0, 2 ** 32, ng, dtype=np.uint64).astype(np.uint32)
    bits[(bits & 0x7F800000) == 0x7F800000] &= 0xBF7FFFFF  # finite only: the stream reads no inf or nan
    bits[0] &= 0x7FFFFFFF  # the first value positive, so that "+v" is a number
    cols = np.stack([bits.view(np.float32),
                     (rng.standard_normal(ng) * 10.0 ** rng.integers(-30, 30, ng)).astype(np.float32),
                     np.arange(ng, dtype=np.float32)])
    src = str(tmp_path / "in.dat")
    _write_dat(src, cols, 2, ["Mm", "Mm", "erg"])
    txt = str(tmp_path / "in.txt")
    r = subprocess.run([programs["roundtrip_cube"], src, txt, "2"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = open(txt, "rb").read()
    lines = raw.split(b"\n")
    plus = str(tmp_path / "plus.txt")
    lines_p = list(lines)
    lines_p[7] = b"+" + lines_p[7]
    open(plus, "wb").write(b"\n".join(lines_p))
    got = {}
    for name, path in (("fast", txt), ("stream", plus)):
        out = str(tmp_path / (name + ".dat"))
        r = subprocess.run([programs["roundtrip_cube"], path, out, "1"], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        got[name] = read_cube(out)["data"]
    assert got["fast"].shape == (ng, 3)
    assert np.array_equal(got["fast"].view(np.uint32), got["stream"].view(np.uint32))
    assert np.array_equal(got["fast"][:, 2], np.arange(ng, dtype=np.float32))  # every value in its place
    libc = ctypes.CDLL(None)
    libc.strtof.restype = ctypes.c_float
    libc.strtof.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
    for j in rng.choice(ng, 3000, replace=False):
        toks = lines[7 + j].split()
        for c in range(2):
            want = np.float32(libc.strtof(toks[c], None))
            assert got["fast"][j, c].view(np.uint32) == want.view(np.uint32), (j, c, toks[c])
    # what the stream cannot read is an error, as in the reference
    for k, bad in enumerate((lines[:7] + [b"nan 1 2 "] + lines[8:], lines[:-3] + [b""])):
        path = str(tmp_path / f"bad{k}.txt")
        open(path, "wb").write(b"\n".join(bad))
        r = subprocess.run([programs["roundtrip_cube"], path, str(tmp_path / "bad.dat"), "1"],
                           capture_output=True, text=True)
        assert r.returncode == 2 and "truncated cube file" in r.stderr, (k, r.stderr)


def _write_data(path, snap):
    cols = np.stack([snap.x, snap.y, snap.z, snap.n, snap.T, snap.vx, snap.vy, snap.vz], axis=1)
    with open(path, "w") as f:
        for row in cols:
            f.write(" ".join("%.9g" % v for v in row) + "\n")


def test_example_program_fails_loudly_without_a_gpu(programs, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from fomo_gb300 import synth
    data = str(tmp_path / "points.txt")
    _write_data(data, synth.loop_snapshot(4))
    synth.write_table(synth.line_table(), str(tmp_path / "table.dat"))
    r = subprocess.run([programs["example_render"], data, "table.dat", "NearestNeighbour", "0.1", "0.2", "8", "6",
                        "10", "8", "0.6", str(tmp_path / "out.txt")], capture_output=True, text=True,
                       cwd=str(tmp_path))
    assert r.returncode == 2
    assert "no usable CUDA device" in r.stderr
    assert not os.path.exists(str(tmp_path / "out.txt"))


def test_reference_example_program_compiles_unchanged(tmp_path):
    """The drop-in criterion: the reference's own user program
    (fomo-c/example/example.cpp), unmodified, compiles against include/FoMo.h
    and links against libfomo_gpu.so.  Read where the reference tree is
    mounted (the build recipe names it); skipped elsewhere."""
    import oracle
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = os.path.join(os.path.dirname(oracle.ref_src()), "example", "example.cpp")
    if not os.path.isfile(src):
        pytest.skip("the reference tree is not mounted here")
    if not os.path.exists(fg.LIB_PATH):
        from fomo_gb300 import build
        build.build()
    libdir = os.path.dirname(fg.LIB_PATH)
    exe = str(tmp_path / "example")
    r = subprocess.run(["g++", "-std=c++11", "-O1", "-I", os.path.join(ROOT, "include"), src, "-L", libdir,
                        "-lfomo_gpu", "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.getsize(exe) > 0


def test_angstrom_width_is_converted_with_the_rendering_lambda0(programs, tmp_path):
    """setresolution with a width below 1 (Angstrom) stores width * c / lambda0
    of the rendering, whose lambda0 only setchiantifile sets: before it, the
    default 193.509 A applies (fomo-rendercube.cpp:74-79, fomo-object.cpp:110-116)."""
    from fomo_gb300 import synth
    t = synth.line_table(lambda0=171.073)
    synth.write_table(t, str(tmp_path / "table.dat"))
    r = subprocess.run([programs["resolution_units"], str(tmp_path / "table.dat")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    w_after, w_before, w_ms = (float(v) for v in r.stdout.split("\n")[-4:-1])  # after the unit warnings
    assert w_after == 0.6 * fg.SPEED_OF_LIGHT / 171.073
    assert w_before == 0.6 * fg.SPEED_OF_LIGHT / 193.509
    assert w_ms == 150000.0
    assert r.stdout.count("converted to") == 2  # the reference's warning, once per conversion


def test_unknown_method_is_an_exception(programs, tmp_path):
    from fomo_gb300 import synth
    data = str(tmp_path / "points.txt")
    _write_data(data, synth.loop_snapshot(3))
    synth.write_table(synth.line_table(), str(tmp_path / "table.dat"))
    r = subprocess.run([programs["example_render"], data, "table.dat", "NoSuchMethod", "0", "0", "8", "6", "10", "8",
                        "0.6", str(tmp_path / "out.txt")], capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 2 and "unknown rendering method" in r.stderr


# ---------------------------------------------------------------- GPU

CASES = {
    # name: (method, table key, l, b, nx, ny, nz, L, width)
    "nn": ("NearestNeighbourGPU", "table", 0.3, 0.2, 8, 6, 10, 8, 0.6),
    "img": ("NearestNeighbour", "band", 0.4, -0.3, 7, 5, 10, 1, 1e5),
    "th": ("ThomsonGPU", None, 0.2, 0.3, 8, 6, 12, 1, 1e5),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_example_program_matches_the_reference_files(programs, tmp_path, case):
    method, tkey, l, b, nx, ny, nz, L, width = CASES[case]
    z = G.load("writers.npz")
    pre = "th_" if case == "th" else "nn_"
    snap = G.snapshot({k[len(pre):]: v for k, v in z.items() if k.startswith(pre)})
    data = str(tmp_path / "points.txt")
    _write_data(data, snap)
    table = ""
    if tkey:
        table = "table.dat" if tkey == "table" else "band.dat"
        with open(str(tmp_path / table), "wb") as f:
            f.write(bytes(z[f"{tkey}_text"]))
    out = str(tmp_path / "out.txt")
    r = subprocess.run([programs["example_render"], data, table, method, repr(l), repr(b), str(nx), str(ny), str(nz),
                        str(L), repr(width), out, "3"], capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert f"points {nx * ny * L}" in r.stdout
    assert f"method {method}" in r.stdout
    for ext in (".dat", ".txt"):
        ours = read_cube(str(tmp_path / ("out" + ext)))
        ref = read_cube(os.path.join(GOLD, f"writer_{case}{ext}"))
        for k in ("dim", "ng", "nvars", "units", "chianti", "abund"):
            assert ours[k] == ref[k], (ext, k)
        d = ours["dim"]
        if ext == ".dat":
            assert np.array_equal(ours["data"][:, :d], ref["data"][:, :d])  # the image grid, bit for bit
        else:
            np.testing.assert_allclose(ours["data"][:, :d], ref["data"][:, :d], rtol=1e-7)
        assert G.norm_max_err(ours["data"][:, d:], ref["data"][:, d:]) <= TOL, ext
    # render() itself wrote the view with the default write options (text only)
    # three characters, zero-filled on the left as iostream pads: 17 -> "017", -5 -> "0-5"
    deg = lambda a: ("%d" % int(round(a * 180.0 / np.pi))).rjust(3, "0")  # noqa: E731
    view = tmp_path / ("view-l%sb%s.txt" % (deg(l), deg(b)))
    assert view.exists(), sorted(os.listdir(str(tmp_path)))
    assert not (tmp_path / (view.name[:-4] + ".dat")).exists()


@pytest.mark.gpu
def test_example_program_with_an_abundance_file(programs, tmp_path):
    """FoMoObject::setabundfile on a spectroscopic render: the element's
    abundance in the file over that in the standard file the tables were made
    with (FOMO_STANDARD_ABUND) scales the emissivity (fomo-CHIANTI.cpp:264-273).
    The written cube matches the oracle's render at that ratio; without a
    standard file the render fails with an error, as the reference's does."""
    import oracle
    from fomo_gb300 import synth
    snap = synth.loop_snapshot(8, seed=2)
    data = str(tmp_path / "points.txt")
    _write_data(data, snap)
    t = synth.line_table(lambda0=193.509, ion="fe_12")
    synth.write_table(t, str(tmp_path / "table.dat"))
    rows = {"std.abund": [(1, 12.00, "H"), (26, 7.85, "Fe")], "new.abund": [(1, 12.00, "H"), (26, 8.10, "Fe")]}
    for name, rr in rows.items():
        with open(str(tmp_path / name), "w") as f:
            f.write("".join(f" {z:2d}  {v:6.2f}  {sym}\n" for z, v, sym in rr) + " -1\n")
    l, b, nx, ny, nz, L, width = 0.35, -0.2, 9, 7, 16, 12, 0.6
    args = [programs["example_render"], data, "table.dat", "NearestNeighbourGPU", repr(l), repr(b), str(nx), str(ny),
            str(nz), str(L), repr(width), str(tmp_path / "out.txt"), "1", "new.abund"]
    env = dict(os.environ, FOMO_STANDARD_ABUND=str(tmp_path / "std.abund"))
    r = subprocess.run(args, capture_output=True, text=True, cwd=str(tmp_path), env=env)
    assert r.returncode == 0, r.stderr
    ours = read_cube(str(tmp_path / "out.dat"))
    ratio = oracle.abundance_ratio(str(tmp_path / "new.abund"), str(tmp_path / "std.abund"), "fe_12")
    eps, w = oracle.emission(snap, t, abundratio=ratio)
    ocube, _, _ = oracle.nn_render(snap, eps, w, t.lambda0, l, b, nx, ny, nz, L, width * fg.SPEED_OF_LIGHT / t.lambda0)
    assert G.norm_max_err(ours["data"][:, ours["dim"]:].ravel(), ocube.ravel()) <= TOL
    assert ours["abund"] == "new.abund"
    env.pop("FOMO_STANDARD_ABUND")
    r = subprocess.run(args, capture_output=True, text=True, cwd=str(tmp_path), env=env)
    assert r.returncode == 2 and "abundance" in r.stderr
