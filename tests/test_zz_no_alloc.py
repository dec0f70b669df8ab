"""The allocation-free inner product, called through the C ABI.

ilm_dot_grid_noalloc serves callers that cannot allocate device memory when
they need an inner product: a service whose memory pool owns the whole device,
or a loop that must not call cudaMalloc / cudaFree.  It must give the same
value as the regular, cache-based ilm_dot_grid.  It is called twice in a row
on different data, because every call reuses the same fixed scratch array; it
is checked at the array's row limit (ny = 16384) and on a grid much wider than
that (nx is not limited), and it must reject taller grids."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def _kinds(il):
    return [il.NodesPrimal, il.NodesDual, il.EdgesPrimal, il.EdgeGradientPrimal]


def _noalloc(lib, L, g, a, b, dt, stream=None):
    import torch
    r = C.c_double(float("nan"))
    st = lib.ilm_dot_grid_noalloc(g.nx, g.ny, g.h, L.GRID_SCALING, a.kind, L.F64 if dt == torch.float64 else L.F32,
                                  C.c_void_p(a.data.data_ptr()), C.c_void_p(b.data.data_ptr()), C.byref(r),
                                  None if stream is None else C.c_void_p(stream.cuda_stream))
    assert st == 0, lib.ilm_last_error()
    return r.value


def _random_pair(cls, g, dt, gen):
    import torch
    a = cls.zeros(g, dt)
    b = cls.zeros(g, dt)
    a.data.copy_(torch.randn(a.data.shape, generator=gen, device="cuda", dtype=dt))
    b.data.copy_(torch.randn(b.data.shape, generator=gen, device="cuda", dtype=dt))
    return a, b


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
    stream = torch.cuda.Stream()
    for cls in _kinds(il):
        for call in range(2):
            a, b = _random_pair(cls, g, dt, gen)
            ref = il.dot(a, b, cache)
            torch.cuda.synchronize()
            r = _noalloc(lib, L, g, a, b, dt, stream if call else None)
            assert abs(r - ref) <= 1e-12 * max(1.0, abs(ref)), (cls.__name__, call, r, ref)


def test_noalloc_dot_at_the_row_limit(cuda):
    """ny = 16384 dual nodes fills the scratch array exactly."""
    import torch
    import immersedlayers as il
    from immersedlayers import _lib as L
    lib = L.load()
    g = il.PhysicalGrid(h=0.01, nx=8, ny=16384)
    cache = il.SurfaceScalarCache(None, g, dtype=torch.float64)
    gen = torch.Generator(device="cuda").manual_seed(11)
    for cls in (il.NodesDual, il.EdgesPrimal):
        for _ in range(2):
            a, b = _random_pair(cls, g, torch.float64, gen)
            ref = il.dot(a, b, cache)
            r = _noalloc(lib, L, g, a, b, torch.float64)
            assert abs(r - ref) <= 1e-12 * max(1.0, abs(ref)), (cls.__name__, r, ref)


def test_noalloc_dot_on_a_grid_wider_than_the_row_limit(cuda):
    """nx = 20000 dual nodes (wider than any cache grid) is accepted: rows of
    any length are reduced by a loop.  Nodes{Dual}: ghosts excluded, h^2
    weights."""
    import torch
    from immersedlayers import _lib as L
    lib = L.load()
    nx, ny, h = 20000, 8, 0.01
    gen = torch.Generator(device="cuda").manual_seed(13)
    a = torch.randn(ny, nx, generator=gen, device="cuda", dtype=torch.float64)
    b = torch.randn(ny, nx, generator=gen, device="cuda", dtype=torch.float64)
    ref = float((a[1:-1, 1:-1] * b[1:-1, 1:-1]).sum()) * h * h
    for _ in range(2):
        r = C.c_double(float("nan"))
        st = lib.ilm_dot_grid_noalloc(nx, ny, h, L.GRID_SCALING, L.NODES_DUAL, L.F64, C.c_void_p(a.data_ptr()),
                                      C.c_void_p(b.data_ptr()), C.byref(r), None)
        assert st == 0, lib.ilm_last_error()
        assert abs(r.value - ref) <= 1e-12 * max(1.0, abs(ref)), (r.value, ref)


def test_noalloc_rejects_oversized_grid(cuda):
    import torch
    from immersedlayers import _lib as L
    lib = L.load()
    a = torch.zeros(16, dtype=torch.float64, device="cuda")
    r = C.c_double()
    st = lib.ilm_dot_grid_noalloc(64, 16385, 0.01, L.GRID_SCALING, L.NODES_PRIMAL, L.F64,
                                  C.c_void_p(a.data_ptr()), C.c_void_p(a.data_ptr()), C.byref(r), None)
    assert st == 7 and b"exceeds the fixed scratch" in lib.ilm_last_error()
