"""The allocation-free inner product, called through the C ABI.

ilm_dot_grid_noalloc serves callers that cannot allocate device memory when
they need an inner product (for example host code running during a CUDA-graph
stream capture, or a service whose memory pool owns the whole device).  It
must give the same value as the regular, cache-based ilm_dot_grid.  It is
called twice in a row on different data, because every call reuses the same
fixed scratch array, and it must reject grids larger than that array."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _kinds(il):
    return [il.NodesPrimal, il.NodesDual, il.EdgesPrimal, il.EdgeGradientPrimal]


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_noalloc_dot_matches_cache_dot_twice(cuda, dtype):
    import torch
    import immersedlayers as il
    from immersedlayers import _lib as L
    lib = L.load()
    dt = torch.float64 if dtype == "f64" else torch.float32
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), 0.04)
    cache = il.SurfaceScalarCache(il.circle(1.0, ds=0.056), g, dtype=dt)
    gen = torch.Generator(device="cuda").manual_seed(7)
    for cls in _kinds(il):
        for call in range(2):
            a = cls.zeros(g, dt)
            b = cls.zeros(g, dt)
            a.data.copy_(torch.randn(a.data.shape, generator=gen, device="cuda", dtype=dt))
            b.data.copy_(torch.randn(b.data.shape, generator=gen, device="cuda", dtype=dt))
            ref = il.dot(a, b, cache)
            r = C.c_double(float("nan"))
            st = lib.ilm_dot_grid_noalloc(g.nx, g.ny, g.h, L.GRID_SCALING, a.kind, L.F64 if dt == torch.float64
                                          else L.F32, C.c_void_p(a.data.data_ptr()), C.c_void_p(b.data.data_ptr()),
                                          C.byref(r), None)
            assert st == 0, lib.ilm_last_error()
            assert abs(r.value - ref) <= 1e-12 * max(1.0, abs(ref)), (cls.__name__, call, r.value, ref)


def test_noalloc_rejects_oversized_grid(cuda):
    import torch
    from immersedlayers import _lib as L
    lib = L.load()
    a = torch.zeros(16, dtype=torch.float64, device="cuda")
    r = C.c_double()
    st = lib.ilm_dot_grid_noalloc(20000, 64, 0.01, L.GRID_SCALING, L.NODES_PRIMAL, L.F64,
                                  C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()), C.byref(r), None)
    assert st == 7 and b"exceeds the fixed scratch" in lib.ilm_last_error()
