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


@pytest.mark.gpu
def test_device_buffer_helpers(cuda):
    """ilm_alloc / ilm_copy_h2d / ilm_copy_d2h / ilm_free round trip, and a
    regularization through buffers the library allocated."""
    import ctypes as C
    import numpy as np
    import torch
    import immersedlayers as il
    from immersedlayers import _lib as L
    lib = L.load()
    rng = np.random.default_rng(9)
    host = rng.standard_normal(1000)
    p = C.c_void_p()
    assert lib.ilm_alloc(host.nbytes, C.byref(p)) == 0 and p.value
    assert lib.ilm_copy_h2d(p, host.ctypes.data_as(C.c_void_p), host.nbytes, None) == 0
    back = np.zeros_like(host)
    assert lib.ilm_copy_d2h(back.ctypes.data_as(C.c_void_p), p, host.nbytes, None) == 0
    assert np.array_equal(back, host)
    assert lib.ilm_free(p) == 0
    # regularize f from a library buffer into a library buffer; compare with the torch path
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), 0.04)
    c = il.SurfaceScalarCache(il.circle(1.0, ds=0.056), g, dtype=torch.float64)
    N = len(c)
    f = rng.standard_normal(N)
    ref = il.NodesPrimal.zeros(g, torch.float64)
    il.regularize_(ref, il.ScalarData(torch.tensor(f, device="cuda")), c)
    fd, od = C.c_void_p(), C.c_void_p()
    n_out = ref.data.numel()
    assert lib.ilm_alloc(f.nbytes, C.byref(fd)) == 0 and lib.ilm_alloc(n_out * 8, C.byref(od)) == 0
    assert lib.ilm_copy_h2d(fd, f.ctypes.data_as(C.c_void_p), f.nbytes, None) == 0
    assert lib.ilm_regularize(c._h, L.NODES_PRIMAL, fd, od, None) == 0
    out = np.zeros(n_out)
    assert lib.ilm_copy_d2h(out.ctypes.data_as(C.c_void_p), od, n_out * 8, None) == 0
    assert np.array_equal(out, ref.data.cpu().numpy().ravel())
    assert lib.ilm_free(fd) == 0 and lib.ilm_free(od) == 0
