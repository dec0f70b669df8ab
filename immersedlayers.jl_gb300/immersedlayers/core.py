"""Host-side mirror of ImmersedLayers.jl's cache and operator API.

Julia's mutating `op!(out, in, cache)` methods become `op_(out, in, cache)`
here (a trailing underscore marks the in-place form, as `!` does in Julia);
dispatch on the CartesianGrids data types (Nodes{Primal}, Edges{Primal}, ...)
is reproduced by the small data classes below.  Every operator forwards to the
CUDA kernels in libilm.so through its C ABI; grid and surface data live in
device memory as torch tensors (torch is used only for allocation).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib as L
from .bodies import Body, BodyList, as_bodylist

Primal = "Primal"
Dual = "Dual"

GridScaling = "GridScaling"
IndexScaling = "IndexScaling"

_DT = {torch.float64: L.F64, torch.float32: L.F32}


def _stream_ptr(stream=None):
    if stream is None:
        return None
    return C.c_void_p(stream.cuda_stream)


def _ptr(t):
    return C.c_void_p(t.data_ptr())


# ---------------------------------------------------------------------------
# grid
# ---------------------------------------------------------------------------
class PhysicalGrid:
    """CartesianGrids PhysicalGrid: nx x ny dual nodes (ghosts included),
    1-based origin index (i0x, i0y), spacing h.  Primal node i sits at
    x = (i - i0x) h, dual node i at x = (i - i0x - 1/2) h."""

    def __init__(self, xlim=None, ylim=None, h=None, *, nx=None, ny=None, i0=None):
        if nx is None:
            def one(lim):
                nl = int(math.ceil(-lim[0] / h - 1e-12))
                nr = int(math.ceil(lim[1] / h - 1e-12))
                return nl + nr + 2 * 2 + 2, nl + 3
            nx, i0x = one(xlim)
            ny, i0y = one(ylim)
        else:
            ny = nx if ny is None else ny
            i0x, i0y = (nx // 2, ny // 2) if i0 is None else i0
        self.nx, self.ny, self.h = int(nx), int(ny), float(h)
        self.i0 = (int(i0x), int(i0y))
        h_ = C.c_void_p()
        L.call("ilm_grid_create", self.nx, self.ny, self.h, self.i0[0], self.i0[1], C.byref(h_))
        self._h = h_

    @classmethod
    def from_cells(cls, n, h, ny=None):
        """Grid of n x ny dual nodes centred on the origin."""
        return cls(h=h, nx=n, ny=ny)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                L.load().ilm_grid_destroy(self._h)
        except Exception:
            pass

    def __repr__(self):
        return f"PhysicalGrid(({self.nx}, {self.ny}), {self.i0}, {self.h})"

    @property
    def size(self):
        return (self.nx, self.ny)

    def cellsize(self):
        return self.h

    def shape(self, dual_x, dual_y):
        return (self.nx if dual_x else self.nx - 1, self.ny if dual_y else self.ny - 1)

    def coordinates(self, dual_x, dual_y):
        n1, n2 = self.shape(dual_x, dual_y)
        x = (np.arange(1, n1 + 1) - self.i0[0] - 0.5 * dual_x) * self.h
        y = (np.arange(1, n2 + 1) - self.i0[1] - 0.5 * dual_y) * self.h
        return x, y

    def limits(self):
        return (((1 - self.i0[0]) * self.h, (self.nx - 1 - self.i0[0]) * self.h),
                ((1 - self.i0[1]) * self.h, (self.ny - 1 - self.i0[1]) * self.h))


# ---------------------------------------------------------------------------
# grid data (CartesianGrids Nodes / Edges / EdgeGradient)
# ---------------------------------------------------------------------------
_COMPONENTS = {
    L.NODES_PRIMAL: [(0, 0)],
    L.NODES_DUAL: [(1, 1)],
    L.EDGES_PRIMAL: [(1, 0), (0, 1)],
    L.EDGES_DUAL: [(0, 1), (1, 0)],
    L.EDGEGRAD_PRIMAL: [(0, 0), (1, 1), (1, 1), (0, 0)],
}


class GridData:
    """Flat device buffer of one CartesianGrids grid type, column-major with x
    fastest (the reference's memory layout)."""

    kind = None
    names = ()

    def __init__(self, grid: PhysicalGrid, data: torch.Tensor):
        self.grid = grid
        self.data = data
        self._offs = [0]
        for dx, dy in _COMPONENTS[self.kind]:
            n1, n2 = grid.shape(dx, dy)
            self._offs.append(self._offs[-1] + n1 * n2)
        assert data.numel() == self._offs[-1], (data.numel(), self._offs[-1])

    @classmethod
    def zeros(cls, grid, dtype=torch.float64, device="cuda"):
        n = sum(grid.shape(dx, dy)[0] * grid.shape(dx, dy)[1] for dx, dy in _COMPONENTS[cls.kind])
        return cls(grid, torch.zeros(n, dtype=dtype, device=device))

    def similar(self):
        return type(self)(self.grid, torch.zeros_like(self.data))

    def component(self, i):
        """2-D view (n2, n1) of component i, indexed [j, i] (x fastest)."""
        dx, dy = _COMPONENTS[self.kind][i]
        n1, n2 = self.grid.shape(dx, dy)
        return self.data[self._offs[i]:self._offs[i + 1]].view(n2, n1)

    def __getattr__(self, name):
        if name in type(self).names:
            return self.component(type(self).names.index(name))
        raise AttributeError(name)

    def fill_(self, v):
        self.data.fill_(v)
        return self

    def numpy_components(self):
        """Components as float64 numpy arrays of shape (n1, n2) indexed [i, j]."""
        out = [self.component(i).detach().cpu().double().numpy().T.copy() for i in range(len(_COMPONENTS[self.kind]))]
        return out[0] if len(out) == 1 else tuple(out)

    def set_numpy(self, arrs):
        if not isinstance(arrs, (tuple, list)):
            arrs = (arrs,)
        for i, a in enumerate(arrs):
            self.component(i).copy_(torch.as_tensor(np.ascontiguousarray(np.asarray(a).T), dtype=self.data.dtype))
        return self


class NodesPrimal(GridData):
    kind = L.NODES_PRIMAL


class NodesDual(GridData):
    kind = L.NODES_DUAL


class EdgesPrimal(GridData):
    kind = L.EDGES_PRIMAL
    names = ("u", "v")


class EdgesDual(GridData):
    kind = L.EDGES_DUAL
    names = ("u", "v")


class EdgeGradientPrimal(GridData):
    kind = L.EDGEGRAD_PRIMAL
    names = ("dudx", "dudy", "dvdx", "dvdy")


def Nodes(cell, grid, dtype=torch.float64):
    return (NodesPrimal if cell == Primal else NodesDual).zeros(grid, dtype)


def Edges(cell, grid, dtype=torch.float64):
    return (EdgesPrimal if cell == Primal else EdgesDual).zeros(grid, dtype)


def EdgeGradient(cell, grid, dtype=torch.float64):
    assert cell == Primal
    return EdgeGradientPrimal.zeros(grid, dtype)


# ---------------------------------------------------------------------------
# point data (ScalarData / VectorData / TensorData)
# ---------------------------------------------------------------------------
class PointData:
    ncomp = 1
    kind = L.SCALAR_DATA
    names = ()

    def __init__(self, data: torch.Tensor):
        self.data = data
        self.npts = data.numel() // self.ncomp

    @classmethod
    def zeros(cls, n, dtype=torch.float64, device="cuda"):
        return cls(torch.zeros(n * cls.ncomp, dtype=dtype, device=device))

    def similar(self):
        return type(self)(torch.zeros_like(self.data))

    def __getattr__(self, name):
        if name in type(self).names:
            i = type(self).names.index(name)
            return self.data[i * self.npts:(i + 1) * self.npts]
        raise AttributeError(name)

    def numpy(self):
        return self.data.detach().cpu().double().numpy().copy()


class ScalarData(PointData):
    pass


class VectorData(PointData):
    ncomp = 2
    kind = L.VECTOR_DATA
    names = ("u", "v")


class TensorData(PointData):
    ncomp = 4
    kind = L.TENSOR_DATA
    names = ("dudx", "dudy", "dvdx", "dvdy")


# ---------------------------------------------------------------------------
# cache (src/cache.jl:164-261)
# ---------------------------------------------------------------------------
class BasicILMCache:
    """SurfaceScalarCache / SurfaceVectorCache: the points, normals and areas of
    the immersed surface(s), the DDF transfer windows and the inverse-Laplacian
    plans, held on the device by libilm."""

    def __init__(self, bodies, grid: PhysicalGrid, kind, ddftype="Yang3", scaling=GridScaling,
                 dtype=torch.float64):
        bl = as_bodylist(bodies) if bodies is not None else BodyList()
        self.bl = bl
        self.g = grid
        self.kind = kind
        self.ddftype = ddftype
        self.scaling = scaling
        self.dtype = dtype
        x, y = bl.x, bl.y
        nx, ny, ds = bl.nx, bl.ny, bl.ds
        self.N = int(len(x))
        self._host = dict(x=x, y=y, nx=nx, ny=ny, ds=ds)
        arr = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, nx, ny, ds)]
        ptrs = [a.ctypes.data_as(C.POINTER(C.c_double)) for a in arr]
        h = C.c_void_p()
        L.call("ilm_cache_create", grid._h, kind, self.N, *ptrs, L.DDF[ddftype],
               L.GRID_SCALING if scaling == GridScaling else L.INDEX_SCALING, _DT[dtype], C.byref(h))
        self._h = h
        dev = torch.device("cuda")
        self.pts = VectorData(torch.tensor(np.concatenate([x, y]), dtype=dtype, device=dev))
        self.nrm = VectorData(torch.tensor(np.concatenate([nx, ny]), dtype=dtype, device=dev))
        self.ds = ScalarData(torch.tensor(ds, dtype=dtype, device=dev))

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                L.load().ilm_cache_destroy(self._h)
        except Exception:
            pass

    def __len__(self):
        return self.N

    def __repr__(self):
        kind = "scalar" if self.kind == L.CACHE_SCALAR else "vector"
        return (f"Surface cache with scaling of type {self.scaling}\n  {self.N} point data, {kind} grid data on "
                f"{self.g!r}")

    def cellsize(self):
        return self.g.h

    # allocators (src/cache.jl:399-775)
    def _grid_type(self):
        return NodesPrimal if self.kind == L.CACHE_SCALAR else EdgesPrimal

    def _surf_type(self):
        return ScalarData if self.kind == L.CACHE_SCALAR else VectorData

    def update_points_(self, x, y, nx, ny, ds, stream=None):
        """Moving bodies: new point positions, normals and areas (device
        float64 tensors of the same length), re-binned on the device without
        rebuilding the cache (the cache rebuild of update_system,
        src/system.jl:26-49)."""
        t = [torch.as_tensor(a, dtype=torch.float64, device="cuda").contiguous() for a in (x, y, nx, ny, ds)]
        if any(a.numel() != self.N for a in t):
            raise ValueError(f"update_points_: {self.N} points expected")
        L.call("ilm_cache_update_points", self._h, *[_ptr(a) for a in t], _stream_ptr(stream))
        self._dev_points = t  # keep the inputs alive until the stream has used them
        self.pts.data.copy_(torch.cat([t[0], t[1]]).to(self.dtype))
        self.nrm.data.copy_(torch.cat([t[2], t[3]]).to(self.dtype))
        self.ds.data.copy_(t[4].to(self.dtype))
        return self


def SurfaceScalarCache(bodies, grid, ddftype="Yang3", scaling=GridScaling, dtype=torch.float64):
    return BasicILMCache(bodies, grid, L.CACHE_SCALAR, ddftype, scaling, dtype)


def SurfaceVectorCache(bodies, grid, ddftype="Yang3", scaling=GridScaling, dtype=torch.float64):
    return BasicILMCache(bodies, grid, L.CACHE_VECTOR, ddftype, scaling, dtype)


def points(cache):
    return cache.pts


def normals(cache):
    return cache.nrm


def areas(cache):
    return cache.ds


def zeros_grid(cache):
    return cache._grid_type().zeros(cache.g, cache.dtype)


def ones_grid(cache):
    return zeros_grid(cache).fill_(1.0)


def zeros_gridcurl(cache):
    return NodesDual.zeros(cache.g, cache.dtype)


def zeros_gridgrad(cache):
    t = EdgesPrimal if cache.kind == L.CACHE_SCALAR else EdgeGradientPrimal
    return t.zeros(cache.g, cache.dtype)


def zeros_griddiv(cache):
    return None if cache.kind == L.CACHE_SCALAR else NodesPrimal.zeros(cache.g, cache.dtype)


def zeros_surface(cache):
    return cache._surf_type().zeros(cache.N, cache.dtype)


def ones_surface(cache):
    s = zeros_surface(cache)
    s.data.fill_(1.0)
    return s


def zeros_surfacescalar(cache):
    return ScalarData.zeros(cache.N, cache.dtype)


def _coords(cache, g, axis):
    for i, (dx, dy) in enumerate(_COMPONENTS[g.kind]):
        x, y = cache.g.coordinates(dx, dy)
        c = x[None, :] if axis == 0 else y[:, None]
        g.component(i).copy_(torch.as_tensor(np.ascontiguousarray(np.broadcast_to(c, (len(y), len(x))))))
    return g


def x_grid(cache):
    return _coords(cache, zeros_grid(cache), 0)


def y_grid(cache):
    return _coords(cache, zeros_grid(cache), 1)


def x_gridcurl(cache):
    """x coordinates of the curl grid data (Nodes{Dual})."""
    return _coords(cache, zeros_gridcurl(cache), 0)


def y_gridcurl(cache):
    return _coords(cache, zeros_gridcurl(cache), 1)


def x_gridgrad(cache):
    """x coordinates of the gradient grid data (Edges{Primal} for scalar
    caches, EdgeGradient{Primal} for vector caches; src/cache.jl:684-689)."""
    return _coords(cache, zeros_gridgrad(cache), 0)


def y_gridgrad(cache):
    return _coords(cache, zeros_gridgrad(cache), 1)


def x_griddiv(cache):
    """x coordinates of the divergence grid data (Nodes{Primal}, vector caches)."""
    return _coords(cache, NodesPrimal.zeros(cache.g, cache.dtype), 0)


def y_griddiv(cache):
    return _coords(cache, NodesPrimal.zeros(cache.g, cache.dtype), 1)


# ---------------------------------------------------------------------------
# operators (src/surface_operators.jl, src/grid_operators.jl)
# ---------------------------------------------------------------------------
def _check(cache, *objs):
    for o in objs:
        if o is None:
            continue
        if o.data.dtype != cache.dtype or not o.data.is_cuda or not o.data.is_contiguous():
            raise TypeError("operand must be a contiguous CUDA tensor of the cache dtype")
        if isinstance(o, GridData) and o.grid.size != cache.g.size:
            raise ValueError("grid data do not match the cache grid")
        if isinstance(o, PointData) and o.npts != cache.N:
            raise ValueError(f"point data of {o.npts} points; cache has {cache.N}")


def regularize_(out: GridData, f: PointData, cache, stream=None):
    """regularize!(s, f, cache): Nodes{Primal|Dual} <- ScalarData,
    Edges{Primal} <- VectorData (src/surface_operators.jl:13-46)."""
    _check(cache, out, f)
    L.call("ilm_regularize", cache._h, out.kind, _ptr(f.data), _ptr(out.data), _stream_ptr(stream))
    return out


def interpolate_(f: PointData, s: GridData, cache, stream=None):
    """interpolate!(f, s, cache) (src/surface_operators.jl:56-88)."""
    _check(cache, f, s)
    L.call("ilm_interpolate", cache._h, s.kind, _ptr(s.data), _ptr(f.data), _stream_ptr(stream))
    return f


def regularize_normal_(out, f, cache, stream=None):
    _check(cache, out, f)
    L.call("ilm_regularize_normal", cache._h, _ptr(f.data), _ptr(out.data), _stream_ptr(stream))
    return out


def regularize_normal_symm_(out, f, cache, stream=None):
    _check(cache, out, f)
    L.call("ilm_regularize_normal_symm", cache._h, _ptr(f.data), _ptr(out.data), _stream_ptr(stream))
    return out


def regularize_normal_cross_(out, f, cache, stream=None):
    _check(cache, out, f)
    L.call("ilm_regularize_normal_cross", cache._h, out.kind, _ptr(f.data), _ptr(out.data), _stream_ptr(stream))
    return out


def regularize_normal_dot_(out, f, cache, stream=None):
    _check(cache, out, f)
    L.call("ilm_regularize_normal_dot", cache._h, out.kind, _ptr(f.data), _ptr(out.data), _stream_ptr(stream))
    return out


def normal_interpolate_(out, q, cache, stream=None):
    _check(cache, out, q)
    L.call("ilm_normal_interpolate", cache._h, _ptr(q.data), _ptr(out.data), _stream_ptr(stream))
    return out


def normal_interpolate_symm_(out, q, cache, stream=None):
    _check(cache, out, q)
    L.call("ilm_normal_interpolate_symm", cache._h, _ptr(q.data), _ptr(out.data), _stream_ptr(stream))
    return out


def normal_cross_interpolate_(out, q, cache, stream=None):
    _check(cache, out, q)
    L.call("ilm_normal_cross_interpolate", cache._h, q.kind, _ptr(q.data), _ptr(out.data), _stream_ptr(stream))
    return out


def normal_dot_interpolate_(out, q, cache, stream=None):
    _check(cache, out, q)
    L.call("ilm_normal_dot_interpolate", cache._h, q.kind, _ptr(q.data), _ptr(out.data), _stream_ptr(stream))
    return out


def surface_divergence_(out, f, cache, stream=None):
    _check(cache, out, f)
    L.call("ilm_surface_divergence", cache._h, _ptr(f.data), _ptr(out.data), _stream_ptr(stream))
    return out


def surface_divergence_symm_(out, f, cache, stream=None):
    _check(cache, out, f)
    L.call("ilm_surface_divergence_symm", cache._h, _ptr(f.data), _ptr(out.data), _stream_ptr(stream))
    return out


def surface_grad_(out, w, cache, stream=None):
    _check(cache, out, w)
    L.call("ilm_surface_grad", cache._h, _ptr(w.data), _ptr(out.data), _stream_ptr(stream))
    return out


def surface_grad_symm_(out, w, cache, stream=None):
    _check(cache, out, w)
    L.call("ilm_surface_grad_symm", cache._h, _ptr(w.data), _ptr(out.data), _stream_ptr(stream))
    return out


def surface_curl_(out, inp, cache, stream=None):
    """surface_curl!: Nodes{Dual} <- point data (C_s^T) or point data <- Nodes{Dual} (C_s)."""
    _check(cache, out, inp)
    if isinstance(out, GridData):
        L.call("ilm_surface_curl", cache._h, 0, inp.kind, _ptr(inp.data), _ptr(out.data), _stream_ptr(stream))
    else:
        L.call("ilm_surface_curl", cache._h, 1, out.kind, _ptr(inp.data), _ptr(out.data), _stream_ptr(stream))
    return out


def surface_curl_cross_(out, inp, cache, stream=None):
    _check(cache, out, inp)
    direction = 0 if isinstance(out, GridData) else 1
    L.call("ilm_surface_curl_cross", cache._h, direction, _ptr(inp.data), _ptr(out.data), _stream_ptr(stream))
    return out


def surface_divergence_cross_(out, f, cache, stream=None):
    _check(cache, out, f)
    L.call("ilm_surface_divergence_cross", cache._h, _ptr(f.data), _ptr(out.data), _stream_ptr(stream))
    return out


def surface_grad_cross_(out, w, cache, stream=None):
    _check(cache, out, w)
    L.call("ilm_surface_grad_cross", cache._h, _ptr(w.data), _ptr(out.data), _stream_ptr(stream))
    return out


def divergence_(out, q, cache, stream=None):
    _check(cache, out, q)
    L.call("ilm_divergence", cache._h, q.kind, _ptr(q.data), _ptr(out.data), _stream_ptr(stream))
    return out


def grad_(out, p, cache, stream=None):
    _check(cache, out, p)
    L.call("ilm_grad", cache._h, p.kind, _ptr(p.data), _ptr(out.data), _stream_ptr(stream))
    return out


def curl_(out, inp, cache, stream=None):
    _check(cache, out, inp)
    L.call("ilm_curl", cache._h, inp.kind, _ptr(inp.data), _ptr(out.data), _stream_ptr(stream))
    return out


class ConvectiveDerivativeCache:
    """ConvectiveDerivativeCache (src/grid_operators.jl:193-208).  The device
    forms the convective derivative in one fused stencil pass, so this extra
    cache holds no temporaries; it keeps the reference's call signatures."""

    def __init__(self, cache_or_data=None):
        self.base = cache_or_data


class RotConvectiveDerivativeCache(ConvectiveDerivativeCache):
    """RotConvectiveDerivativeCache (src/grid_operators.jl:376-392), for w_cross_v_."""


def convective_derivative_(out, v, *args, stream=None):
    """convective_derivative!(out, v, q, base_cache[, extra_cache]) -- v . grad q
    for q on Nodes{Primal}, Nodes{Dual} or Edges{Primal} -- and
    convective_derivative!(out, u, base_cache[, extra_cache]) -- u . grad u
    (src/grid_operators.jl:258-315); scaled by 1/h under GridScaling."""
    if isinstance(args[0], BasicILMCache):
        q, cache = v, args[0]
    else:
        q, cache = args[0], args[1]
    _check(cache, out, v, q)
    if not isinstance(v, EdgesPrimal):
        raise TypeError("convective_derivative_: the velocity must be Edges{Primal}")
    if type(out) is not type(q) or q.kind not in (L.NODES_PRIMAL, L.NODES_DUAL, L.EDGES_PRIMAL):
        raise TypeError("convective_derivative_: out and q must be Nodes{Primal}, Nodes{Dual} or Edges{Primal} alike")
    L.call("ilm_convective_derivative", cache._h, q.kind, _ptr(v.data), _ptr(q.data), _ptr(out.data),
           _stream_ptr(stream))
    return out


def convective_derivative(v, q_or_cache, cache=None):
    """convective_derivative(v, q, base_cache) / convective_derivative(u, base_cache)."""
    if cache is None:
        q, cache = v, q_or_cache
    else:
        q = q_or_cache
    return convective_derivative_(q.similar(), v, q, cache)


def w_cross_v_(out, w, v, base_cache, extra_cache=None, stream=None):
    """w_cross_v!(out::Edges{Primal}, w::Nodes{Dual}, v::Edges{Primal})
    (src/grid_operators.jl:401-434)."""
    _check(base_cache, out, w, v)
    if not (isinstance(out, EdgesPrimal) and isinstance(w, NodesDual) and isinstance(v, EdgesPrimal)):
        raise TypeError("w_cross_v_: out and v Edges{Primal}, w Nodes{Dual}")
    L.call("ilm_w_cross_v", base_cache._h, _ptr(w.data), _ptr(v.data), _ptr(out.data), _stream_ptr(stream))
    return out


def w_cross_v(w, v, base_cache):
    return w_cross_v_(v.similar(), w, v, base_cache)


def laplacian_(out, s, cache, stream=None):
    _check(cache, out, s)
    L.call("ilm_laplacian", cache._h, s.kind, _ptr(s.data), _ptr(out.data), _stream_ptr(stream))
    return out


def inverse_laplacian_(out, rhs=None, cache=None, stream=None):
    """inverse_laplacian!(w, cache) (in place) or inverse_laplacian!(sol, rhs, cache)."""
    if cache is None:  # in-place form inverse_laplacian_(w, cache)
        rhs, cache = out, rhs
    _check(cache, out, rhs)
    L.call("ilm_inverse_laplacian", cache._h, rhs.kind, _ptr(rhs.data), _ptr(out.data), _stream_ptr(stream))
    return out


def mask(cache, kind=None):
    """mask(cache): 1 inside the surface(s), 0 outside, on the basic grid type."""
    out = zeros_grid(cache) if kind is None else kind.zeros(cache.g, cache.dtype)
    L.call("ilm_mask", cache._h, out.kind, 0, _ptr(out.data), None)
    return out


def complementary_mask(cache, kind=None):
    out = zeros_grid(cache) if kind is None else kind.zeros(cache.g, cache.dtype)
    L.call("ilm_mask", cache._h, out.kind, 1, _ptr(out.data), None)
    return out


def _shape_cache(w: GridData, surface, grid):
    """The temporary cache of mask!(w, surface, grid) (src/surface_operators.jl:
    804-806): scalar for Nodes, vector for Edges and EdgeGradient."""
    vec = isinstance(w, (EdgesPrimal, EdgeGradientPrimal))
    return (SurfaceVectorCache if vec else SurfaceScalarCache)(surface, grid, dtype=w.data.dtype)


def mask_(w: GridData, cache, grid=None):
    """mask!(w, cache): multiply w by the mask interpolated to w's grid type;
    mask!(w, surface, grid): the same for the surface(s) of a body."""
    if grid is not None:
        cache = _shape_cache(w, cache, grid)
    m = type(w).zeros(cache.g, cache.dtype)
    L.call("ilm_mask", cache._h, w.kind, 0, _ptr(m.data), None)
    w.data.mul_(m.data)
    return w


def complementary_mask_(w: GridData, cache, grid=None):
    if grid is not None:
        cache = _shape_cache(w, cache, grid)
    m = type(w).zeros(cache.g, cache.dtype)
    L.call("ilm_mask", cache._h, w.kind, 1, _ptr(m.data), None)
    w.data.mul_(m.data)
    return w


def dot(a, b, cache):
    """Weighted inner product of grid data (cell volume) or point data (ds)."""
    r = C.c_double()
    if isinstance(a, GridData):
        _check(cache, a, b)
        L.call("ilm_dot_grid", cache._h, a.kind, _ptr(a.data), _ptr(b.data), C.byref(r), None)
    else:
        _check(cache, a, b)
        L.call("ilm_dot_surface", cache._h, a.ncomp, _ptr(a.data), _ptr(b.data), C.byref(r), None)
    return r.value


def norm(a, cache):
    return math.sqrt(dot(a, a, cache))


def integrate(a, cache):
    if isinstance(a, GridData):
        o = type(a)(a.grid, torch.ones_like(a.data))
        return dot(a, o, cache)
    o = type(a)(torch.ones_like(a.data))
    return dot(a, o, cache)


# ---------------------------------------------------------------------------
# Schur complements (src/matrix_operators.jl)
# ---------------------------------------------------------------------------
def _schur(cache, which, scale):
    scalar_data = cache.kind == L.CACHE_SCALAR or which == "CLinvCT_scalar"
    n = cache.N * (1 if scalar_data else 2)
    A = torch.empty((n, n), dtype=torch.float64, device="cuda")
    L.call("ilm_schur_build", cache._h, L.SCHUR[which], float(scale), _ptr(A), None)
    # device buffer is column-major (A[k + N l]) -> transpose the row-major view
    return A.t()


def create_RTLinvR(cache, scale=1.0):
    return _schur(cache, "RTLinvR", scale)


def create_CLinvCT(cache, scale=1.0):
    return _schur(cache, "CLinvCT", scale)


def create_GLinvD(cache, scale=1.0):
    return _schur(cache, "GLinvD", scale)


def create_nRTRn(cache, scale=1.0):
    return _schur(cache, "nRTRn", scale)


def create_CLinvCT_scalar(cache, scale=1.0):
    """-C_s L^-1 C_s^T on the ScalarData of a vector cache (src/matrix_operators.jl:71-93)."""
    return _schur(cache, "CLinvCT_scalar", scale)


def create_CL2invCT(cache, scale=1.0):
    """-C_s L^-2 C_s^T on VectorData (vector cache, src/matrix_operators.jl:102-125)."""
    return _schur(cache, "CL2invCT", scale)


def create_GLinvD_symm(cache, scale=1.0):
    """-G_s L^-1 D_s with the symmetric-tensor operators (vector cache, src/matrix_operators.jl:165-185)."""
    return _schur(cache, "GLinvD_symm", scale)


def create_GLinvD_cross(cache, scale=1.0):
    """-G^x_s L^-1 D^x_s (scalar cache, src/matrix_operators.jl:195-215; the
    reference's version raises, its surface_divergence_cross! refers to an
    undefined variable)."""
    return _schur(cache, "GLinvD_cross", scale)


class SurfaceFilter:
    """The surface filter C = E~ R of create_surface_filter
    (src/matrix_operators.jl:254-268) as an operator: ``C @ s`` filters the
    surface data once, ``(C ** k) @ s`` k times (the C^6 s of
    test/literate/problems.jl:107,297).  E~ = W^-1 E with W = diag(E R 1)
    (the filtered interpolation of CartesianGrids' Regularize(filter=true));
    no matrix is formed, each power is one regularize, one interpolation and
    one row scaling on the device."""

    def __init__(self, cache, power=1):
        self.cache = cache
        self.power = int(power)

    def __pow__(self, k):
        return SurfaceFilter(self.cache, self.power * int(k))

    def apply_(self, out: PointData, s: PointData, stream=None):
        c = self.cache
        _check(c, out, s)
        if not isinstance(s, c._surf_type()) or type(out) is not type(s):
            raise TypeError(f"surface filter acts on {c._surf_type().__name__}")
        L.call("ilm_surface_filter", c._h, self.power, _ptr(s.data), _ptr(out.data), _stream_ptr(stream))
        return out

    def __matmul__(self, s: PointData):
        return self.apply_(s.similar(), s)

    __mul__ = __matmul__


def create_surface_filter(cache):
    return SurfaceFilter(cache)
