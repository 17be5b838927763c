"""C ABI checks that need no GPU: the library loads, exports every entry point
include/fomo_gpu.h declares, and reports the absence of a device cleanly."""

import os
import re

import pytest

import fomo_gb300 as fg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "fomo_gpu.h")).read()
    return sorted(set(re.findall(r"\b(fomo_[a-z_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(fg.LIB_PATH):
        from fomo_gb300 import build
        build.build()
    return fg.lib()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(fg.SIGNATURES), set(names) ^ set(fg.SIGNATURES)


def test_version_string(lib):
    assert b"sm_103a" in lib.fomo_version()


def test_no_device_is_an_error_not_a_fallback(lib):
    import ctypes
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert lib.fomo_ctx_create(0, 0, ctypes.byref(h)) == fg.ENODEVICE
    with pytest.raises(fg.FomoError):
        fg.Context(0)


def _prototypes():
    text = open(os.path.join(ROOT, "include", "fomo_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for name, args in re.findall(r"\b(fomo_[a-z_]+)\s*\(([^;{}]*?)\)\s*;", text, flags=re.S):
        args = " ".join(args.split())
        out[name] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_python_signatures_take_the_declared_number_of_arguments():
    protos = _prototypes()
    assert set(protos) == set(fg.SIGNATURES), set(protos) ^ set(fg.SIGNATURES)
    for name, n in protos.items():
        assert len(fg.SIGNATURES[name]) == n, (name, n, len(fg.SIGNATURES[name]))


def test_struct_layouts_match_the_header(tmp_path):
    import ctypes
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    structs = {"fomo_request": fg.Request, "fomo_view_info": fg.ViewInfo, "fomo_snapshot_info": fg.SnapshotInfo,
               "fomo_server_config": fg.ServerConfig, "fomo_request_stats": fg.RequestStats,
               "fomo_ceilings": fg.Ceilings}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "fomo_gpu.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    for ln in filter(None, got):
        cname, field, val = ln.split()
        cls = structs[cname]
        want = ctypes.sizeof(cls) if field == "sizeof" else getattr(cls, field).offset
        assert int(val) == want, (cname, field, int(val), want)
