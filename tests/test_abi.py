"""The C ABI library builds, loads and exports every symbol include/fclg.h
declares (no GPU needed: nothing here launches work)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(fclg_\w+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def lib():
    import build as fclg_build
    fclg_build.build()
    from fclg.api import load_library
    return load_library()


def test_exports_every_declared_symbol(lib):
    declared = _declared()
    assert len(declared) >= 10
    for name in sorted(declared):
        assert hasattr(lib, name), name


def test_binding_lists_every_symbol(lib):
    from fclg.api import EXPORTS
    assert set(EXPORTS) == _declared()


def test_metadata_calls(lib):
    assert lib.fclg_version() >= 100
    assert lib.fclg_built_arch() == 1030


def test_create_without_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.fclg_create(ctypes.byref(h), 0)
    assert rc == -4 and not h.value
    assert lib.fclg_last_error(None) == b"null context"


def test_layouts_match_header():
    from fclg.layout import PAIR_DTYPE, RESULT_DTYPE, SHAPE_DTYPE
    hdr = open(os.path.join(ROOT, "include", "fclg.h")).read()
    assert "fclg_shape { /* 32 bytes */" in hdr and SHAPE_DTYPE.itemsize == 32
    assert "fclg_pair { /* 64 bytes */" in hdr and PAIR_DTYPE.itemsize == 64
    assert "fclg_result { /* 48 bytes */" in hdr and RESULT_DTYPE.itemsize == 48
