"""Helmholtz decomposition of grid vector fields with surface jumps
(src/helmholtz.jl) on a vector cache.

vecfield_helmholtz_ is one device call (ilm_vecfield_helmholtz: two
regularizations of the surface jump, two LGF convolutions, the curl and the
gradient); the other functions mirror the reference's building blocks on top
of the device operators."""
from __future__ import annotations

import torch

from . import _lib as L
from .core import (EdgesPrimal, NodesDual, NodesPrimal, PointData, _check, _ptr, _stream_ptr, curl_, grad_,
                   inverse_laplacian_, regularize_normal_cross_, regularize_normal_dot_, x_griddiv, x_gridcurl,
                   y_griddiv, y_gridcurl, zeros_grid, zeros_gridcurl, zeros_surface)


def _vector_cache(c):
    if c.kind != L.CACHE_VECTOR:
        raise TypeError("the Helmholtz caches need a vector cache (src/helmholtz.jl:34)")


class ScalarPotentialCache:
    """ScalarPotentialCache (src/helmholtz.jl:34-40)."""

    def __init__(self, base_cache):
        _vector_cache(base_cache)
        self.dv = zeros_surface(base_cache)
        self.ftemp = NodesPrimal.zeros(base_cache.g, base_cache.dtype)
        self.divv_temp = NodesPrimal.zeros(base_cache.g, base_cache.dtype)


class VectorPotentialCache:
    """VectorPotentialCache (src/helmholtz.jl:49-55)."""

    def __init__(self, base_cache):
        self.dv = zeros_surface(base_cache)
        self.stemp = zeros_gridcurl(base_cache)
        self.curlv_temp = zeros_gridcurl(base_cache)


class VectorFieldCache:
    """VectorFieldCache (src/helmholtz.jl:64-72)."""

    def __init__(self, base_cache):
        _vector_cache(base_cache)
        self.psitemp = zeros_gridcurl(base_cache)
        self.vpsi = zeros_grid(base_cache)
        self.phitemp = NodesPrimal.zeros(base_cache.g, base_cache.dtype)
        self.vphi = zeros_grid(base_cache)
        self.wcache = VectorPotentialCache(base_cache)
        self.dcache = ScalarPotentialCache(base_cache)


def _has_points(dv):
    return dv is not None and dv.data.numel() > 0


def vectorpotential_from_curlv_(psi, curlv, base_cache):
    """L psi = -curlv (src/helmholtz.jl:117-120)."""
    inverse_laplacian_(psi, curlv, base_cache)
    psi.data.neg_()
    return psi


def vectorpotential_from_masked_curlv_(psi, curlv, dv, base_cache, wcache):
    """L psi = -(curlv + R_n n x [v]) (src/helmholtz.jl:85-106)."""
    st = wcache.stemp
    st.data.zero_()
    if _has_points(dv):
        regularize_normal_cross_(st, dv, base_cache)
    st.data.add_(curlv.data)
    return vectorpotential_from_curlv_(psi, st, base_cache)


def vecfield_from_vectorpotential_(v, psi, base_cache):
    """v = curl psi (src/helmholtz.jl:130-134)."""
    return curl_(v, psi, base_cache)


def masked_curlv_from_curlv_masked_(masked_curlv, curlv, dv, base_cache, wcache=None):
    """masked curl = curl of masked v - R_n n x [v] (src/helmholtz.jl:145-159)."""
    if _has_points(dv):
        regularize_normal_cross_(masked_curlv, dv, base_cache)
        masked_curlv.data.neg_().add_(curlv.data)
    else:
        masked_curlv.data.copy_(curlv.data)
    return masked_curlv


def curlv_masked_from_masked_curlv_(curlv, masked_curlv, dv, base_cache, wcache=None):
    """curl of masked v = masked curl + R_n n x [v] (src/helmholtz.jl:170-184)."""
    if _has_points(dv):
        regularize_normal_cross_(curlv, dv, base_cache)
        curlv.data.add_(masked_curlv.data)
    else:
        curlv.data.copy_(masked_curlv.data)
    return curlv


def scalarpotential_from_divv_(phi, divv, base_cache):
    """L phi = divv (src/helmholtz.jl:227-231)."""
    return inverse_laplacian_(phi, divv, base_cache)


def scalarpotential_from_masked_divv_(phi, divv, dv, base_cache, dcache):
    """L phi = divv + R_c n . [v] (src/helmholtz.jl:196-215)."""
    ft = dcache.ftemp
    ft.data.zero_()
    if _has_points(dv):
        regularize_normal_dot_(ft, dv, base_cache)
    ft.data.add_(divv.data)
    return scalarpotential_from_divv_(phi, ft, base_cache)


def vecfield_from_scalarpotential_(v, phi, base_cache):
    """v = grad phi (src/helmholtz.jl:241-245)."""
    return grad_(v, phi, base_cache)


def masked_divv_from_divv_masked_(masked_divv, divv, dv, base_cache, dcache=None):
    """masked divergence = div of masked v - R_c n . [v] (src/helmholtz.jl:256-271)."""
    if _has_points(dv):
        regularize_normal_dot_(masked_divv, dv, base_cache)
        masked_divv.data.neg_().add_(divv.data)
    else:
        masked_divv.data.copy_(divv.data)
    return masked_divv


def divv_masked_from_masked_divv_(divv, masked_divv, dv, base_cache, dcache=None):
    """div of masked v = masked divergence + R_c n . [v] (src/helmholtz.jl:283-297)."""
    if _has_points(dv):
        regularize_normal_dot_(divv, dv, base_cache)
        divv.data.add_(masked_divv.data)
    else:
        divv.data.copy_(masked_divv.data)
    return divv


def vecfield_helmholtz_(v, curlv, divv, dv, vp, base_cache, veccache=None, stream=None):
    """vecfield_helmholtz!(v, curlv, divv, dv, vp, base_cache, veccache)
    (src/helmholtz.jl:327-347): v = curl psi + grad phi + vp; vp is
    Edges{Primal}, a uniform (Vx, Vy) tuple or None.  One device call."""
    _vector_cache(base_cache)
    _check(base_cache, v, curlv, divv, dv if _has_points(dv) else None)
    if not (isinstance(v, EdgesPrimal) and isinstance(curlv, NodesDual) and isinstance(divv, NodesPrimal)):
        raise TypeError("vecfield_helmholtz_: v Edges{Primal}, curlv Nodes{Dual}, divv Nodes{Primal}")
    import ctypes as C
    vp_ptr, uni = None, None
    if isinstance(vp, tuple):
        uni = (C.c_double * 2)(float(vp[0]), float(vp[1]))
    elif vp is not None:
        _check(base_cache, vp)
        vp_ptr = _ptr(vp.data)
    L.call("ilm_vecfield_helmholtz", base_cache._h, _ptr(curlv.data), _ptr(divv.data),
           _ptr(dv.data) if _has_points(dv) else None, vp_ptr,
           C.cast(uni, C.POINTER(C.c_double)) if uni is not None else None, _ptr(v.data), _stream_ptr(stream))
    return v


def vectorpotential_uniformvecfield_(psi, Vx, Vy, base_cache):
    """psi = Vx y - Vy x on the curl grid (src/helmholtz.jl:354-361)."""
    psi.data.copy_(Vx * y_gridcurl(base_cache).data - Vy * x_gridcurl(base_cache).data)
    return psi


def scalarpotential_uniformvecfield_(phi, Vx, Vy, base_cache):
    """phi = Vx x + Vy y on the divergence grid (src/helmholtz.jl:368-375)."""
    phi.data.copy_(Vx * x_griddiv(base_cache).data + Vy * y_griddiv(base_cache).data)
    return phi


def vecfield_uniformvecfield_(v, Vx, Vy, base_cache=None):
    """v.u = Vx, v.v = Vy (src/helmholtz.jl:382-386)."""
    v.component(0).fill_(Vx)
    v.component(1).fill_(Vy)
    return v
