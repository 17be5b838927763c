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
