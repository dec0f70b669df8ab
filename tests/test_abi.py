"""libilm.so loads on a machine without a GPU and exports every symbol that
include/ilm.h declares; the ctypes binding covers the same set."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "ilm.h")).read()
    return sorted(set(re.findall(r"ILM_API\s+(?:const\s+char\s*\*|int)\s+(ilm_\w+)\s*\(", txt)))


def test_header_parses():
    syms = header_symbols()
    assert "ilm_regularize" in syms and "ilm_solve_dirichlet" in syms
    assert len(syms) >= 30


def test_library_exports_header_symbols(lib_built):
    import ctypes
    from immersedlayers import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_matches_header(lib_built):
    from immersedlayers import _lib
    assert set(header_symbols()) == set(_lib.exported_symbols())


def test_status_strings_without_gpu(lib_built):
    from immersedlayers import _lib
    lib = _lib.load()
    assert lib.ilm_version() >= 10000
    assert lib.ilm_status_string(0) == b"ok"
    assert b"converge" in lib.ilm_status_string(4)


def test_invalid_arguments_rejected_on_host(lib_built):
    """Argument validation happens on the host before any device work."""
    import ctypes as C
    from immersedlayers import _lib
    lib = _lib.load()
    g = C.c_void_p()
    assert lib.ilm_grid_create(2, 2, 0.1, 1, 1, C.byref(g)) == 1
    assert b"4x4" in lib.ilm_last_error()
    assert lib.ilm_grid_create(64, 64, -1.0, 32, 32, C.byref(g)) == 1
    assert lib.ilm_regularize(None, 0, None, None, None) == 1
