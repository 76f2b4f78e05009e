"""The C ABI library loads and exports every symbol include/fbgpu.h
declares (no GPU needed: nothing here launches work)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "fbgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fb_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from fbgpu import build
    build.build()
    return C.CDLL(build.LIB)


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_python_mirror_binds_every_symbol():
    import fbgpu
    assert set(_declared()) <= set(fbgpu._SIGS)


def test_version_string(lib):
    lib.fb_version.restype = C.c_char_p
    assert b"sm_103a" in lib.fb_version()


def test_null_context_is_rejected(lib):
    lib.fb_neighbors.argtypes = [C.c_void_p]
    assert lib.fb_neighbors(None) == 1  # FB_ERR_ARG
    lib.fb_last_error.restype = C.c_char_p
    lib.fb_last_error.argtypes = [C.c_void_p]
    assert lib.fb_last_error(None) == b"null context"


def test_library_is_built_for_sm_103a():
    from fbgpu import build
    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)
