"""libmgx.so builds for sm_103a, loads without a GPU and exports every entry point of include/mgx.h."""
import ctypes as C
import os
import re

import pytest

from magex_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "mgx.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mgx_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build_library()
    return _lib.load()


def test_header_declares_entry_points():
    names = _declared()
    assert "mgx_llg_step" in names and "mgx_model_create" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(_declared()) == set(_lib.SIGNATURES), set(_declared()) ^ set(_lib.SIGNATURES)


def test_version_and_errors_without_gpu(lib):
    assert lib.mgx_version() == 1
    h = C.c_void_p()
    # invalid descriptors are rejected on the host before any device call
    assert lib.mgx_model_create(None, None, C.byref(h)) == _lib.MGX_ERR_INVALID
    assert "null" in _lib.last_error()
    d = _lib.LatticeDesc()
    d.ns = 0
    assert lib.mgx_model_create(C.byref(d), None, C.byref(h)) == _lib.MGX_ERR_INVALID
    assert "ns" in _lib.last_error()
    with pytest.raises(ValueError):
        _lib.check(_lib.MGX_ERR_INVALID, "probe")
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.MGX_ERR_UNSUPPORTED, "probe")


def test_struct_layouts_match_header():
    # sizes of the C structs as laid out by the x86-64 / aarch64 LP64 ABIs
    assert C.sizeof(_lib.LLGParams) == 56
    assert C.sizeof(_lib.SiteDesc) == 24
    assert C.sizeof(_lib.LatticeDesc) == 4 + 12 + 12 + 4 + 3 * 8 + 4 + 4 + 4 * 8 + 24


def test_build_is_sm103a_only():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
