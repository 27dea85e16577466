"""The C-ABI library loads and exports every entry point declared in include/vivsim_gb300.h.

Runs without a GPU: loading the library makes no CUDA call.
"""

import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "vivsim_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(vs_[a-z_0-9]+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from vivsim_gb300 import _build, _lib
    if not os.path.exists(_build.lib_path()):
        _build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "vs_step" in names and "vs_ib_mdf" in names and len(names) >= 35


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_matches_header(lib):
    from vivsim_gb300 import _lib
    assert set(_lib.exported_symbols()) <= set(declared_functions())


def test_status_strings(lib):
    assert lib.vs_status_string(0) == b"ok"
    assert lib.vs_version() >= 100


def test_invalid_arguments_return_status_without_gpu(lib):
    # argument validation happens before any CUDA call
    import ctypes as C
    rc = lib.vs_streaming(7, 0, None, None, 4, 4, 1, None)
    assert rc == 1
    assert b"distinct" in lib.vs_last_error() or b"q must" in lib.vs_last_error()
    rc = lib.vs_collision(9, 5, 0, C.c_void_p(8), C.c_void_p(8), 1.0, C.c_void_p(8), 4, None)
    assert rc == 1 and b"dtype" in lib.vs_last_error()
