"""The C-ABI library builds, loads and exports every entry point include/glasma_gb300.h declares.
CPU only: no call here touches a GPU."""
import ctypes
import os
import re

import pytest

from soerenpragya3dglasma_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(glasma_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols("glasma_gb300.h")
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(lib, s), s


def test_binding_table_matches_header():
    syms = set(declared_symbols("glasma_gb300.h"))
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert syms == bound


def test_null_handle_is_an_error_not_a_crash(lib):
    assert lib.glasma_step(None, 0.1, 1, 0) == 1
    assert b"null" in lib.glasma_last_error()
    assert lib.glasma_bulk(None, None) == 1
    assert lib.glasma_destroy(None) == 0
    assert lib.glasma_field_doubles(None, 0) == -1
    assert lib.glasma_status_string(5) == b"numerical guard fired"


def test_create_rejects_bad_shapes(lib):
    h = ctypes.c_void_p()
    assert lib.glasma_create(1, 4, 4, 1.0, 1.0, 1.0, 0, 0, ctypes.byref(h)) == 2
    assert lib.glasma_create(4, 4, 4, -1.0, 1.0, 1.0, 0, 0, ctypes.byref(h)) == 2
    assert lib.glasma_create(4, 4, 4, 1.0, 1.0, 1.0, 7, 0, ctypes.byref(h)) == 1
    assert lib.glasma_create(4, 4, 4, 1.0, 1.0, 1.0, 0, 0, None) == 1


def test_gauss_noalloc_rejects_shapes_before_touching_a_device(lib):
    """The allocation-free Gauss entry point checks its sizes first and reports through
    glasma_last_error() like every other entry point (no device call is made for these)."""
    p = ctypes.c_void_p(16)
    assert lib.glasma_gauss_noalloc(p, p, p, p, 4, 4, 993, 1.0, 1.0, 1.0, 1.0, p, None, None) == 2
    assert b"exceeds the maximum" in lib.glasma_last_error()
    assert lib.glasma_gauss_noalloc(p, p, p, p, 1 << 20, 1 << 20, 900, 1.0, 1.0, 1.0, 1.0, p, None, None) == 2
    assert b"too large" in lib.glasma_last_error()
    assert lib.glasma_gauss_noalloc(p, p, p, p, 1, 4, 4, 1.0, 1.0, 1.0, 1.0, p, None, None) == 2
