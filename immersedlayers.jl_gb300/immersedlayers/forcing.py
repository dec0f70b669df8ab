"""Forcing regions on the device: area, line and point forcing models, their
region caches and apply_forcing! (src/forcing.jl).

A forcing model bundles a shape and a model function
``fcn(str, state, t, fcache, phys_params)`` that fills the strength ``str``
(device data, in place).  apply_forcing! clears the output, then adds every
region's contribution: area forcing ``str .* mask`` (ilm_grid_mul_add), line
and point forcing ``R str`` (ilm_regularize_add: the accumulating DDF
scatter, which visits only the tiles that hold points).

Not covered: the motion transforms of src/forcing.jl (shapes are placed in
the inertial frame) and the spatial-field helper of area forcing (the model
function can build any device field itself).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib as L
from .bodies import Body, BodyList, as_bodylist
from .core import (GridScaling, ScalarData, SurfaceScalarCache, SurfaceVectorCache, VectorData, _ptr,
                   _stream_ptr, mask)


class AreaForcingModel:
    """AreaForcingModel(shape, fcn) / AreaForcingModel(fcn) (whole domain),
    src/forcing.jl:15-79."""

    def __init__(self, shape_or_fcn, fcn=None, ddftype=None):
        if fcn is None:
            self.shape, self.fcn = None, shape_or_fcn
        else:
            self.shape, self.fcn = shape_or_fcn, fcn
        self.ddftype = ddftype


class LineForcingModel:
    """LineForcingModel(shape, fcn): forcing on a curve (src/forcing.jl:81-96)."""

    def __init__(self, shape, fcn, ddftype=None):
        self.shape, self.fcn, self.ddftype = shape, fcn, ddftype


class PointForcingModel:
    """PointForcingModel(pts, fcn): forcing at points (x, y arrays or a
    VectorData of [x; y]) (src/forcing.jl:98-112)."""

    def __init__(self, pts, fcn, ddftype=None):
        self.pts, self.fcn, self.ddftype = pts, fcn, ddftype


class AreaRegionCache:
    """The mask of the shape (or 1 everywhere) on the base cache's grid data
    type, and a strength field of that type (src/forcing.jl:174-180)."""

    def __init__(self, shape, base, ddftype=None):
        self.cache = base
        proto = base._grid_type().zeros(base.g, base.dtype)
        self.str = proto
        if shape is None:
            self.mask = base._grid_type().zeros(base.g, base.dtype)
            self.mask.data.fill_(1.0)
        else:  # the Heaviside function of the shape on the base cache's grid data type
            sc = SurfaceScalarCache(as_bodylist(shape), base.g, ddftype=ddftype or base.ddftype,
                                    scaling=base.scaling, dtype=base.dtype)
            self.mask = mask(sc, kind=type(proto))
            self.shape_cache = sc


class LineRegionCache:
    """A surface cache on the line shape and its strength (src/forcing.jl:182-186)."""

    def __init__(self, shape, base, ddftype=None):
        mk = SurfaceScalarCache if base.kind == L.CACHE_SCALAR else SurfaceVectorCache
        self.cache = mk(as_bodylist(shape), base.g, ddftype=ddftype or base.ddftype, scaling=base.scaling,
                        dtype=base.dtype)
        self.s = as_bodylist(shape).bodies[0].arcs if isinstance(as_bodylist(shape), BodyList) else None
        self.str = self.cache._surf_type().zeros(len(self.cache), base.dtype)


class PointRegionCache:
    """A point collection: Regularize(X, h) with unit weights, i.e. the DDF
    scaled by 1/h^2 (ScalarPointCollectionCache / VectorPointCollectionCache,
    src/cache.jl:277-291), and its strength (src/forcing.jl:188-191)."""

    def __init__(self, pts, base, ddftype=None):
        if isinstance(pts, (ScalarData, VectorData)) or torch.is_tensor(pts):
            data = pts.data if hasattr(pts, "data") else pts
            xy = data.detach().double().cpu().numpy()
            n = xy.size // 2
            x, y = xy[:n], xy[n:]
        else:
            x, y = (np.asarray(a, dtype=np.float64) for a in pts)
        n = x.size
        body = Body(x, y, np.ones(n), np.zeros(n), np.ones(n), name="points")
        mk = SurfaceScalarCache if base.kind == L.CACHE_SCALAR else SurfaceVectorCache
        self.cache = mk(body, base.g, ddftype=ddftype or base.ddftype, scaling=GridScaling, dtype=base.dtype)
        self.str = self.cache._surf_type().zeros(n, base.dtype)


class ForcingModelAndRegion:
    """A forcing model with its region cache on the base cache
    (src/forcing.jl:235-305)."""

    def __init__(self, model, base):
        self.model = model
        self.fcn = model.fcn
        if isinstance(model, AreaForcingModel):
            self.region_cache = AreaRegionCache(model.shape, base, model.ddftype)
        elif isinstance(model, LineForcingModel):
            self.region_cache = LineRegionCache(model.shape, base, model.ddftype)
        elif isinstance(model, PointForcingModel):
            self.region_cache = PointRegionCache(model.pts, base, model.ddftype)
        else:
            raise TypeError(f"unknown forcing model {type(model).__name__}")


def forcing_regions(models, base):
    """ForcingModelAndRegion(models, base_cache) for a list of models."""
    if not isinstance(models, (list, tuple)):
        models = [models]
    return [ForcingModelAndRegion(m, base) for m in models]


def apply_forcing_(out, y, x, t, fr, sys=None, phys_params=None, stream=None):
    """apply_forcing!(out, y, x, t, fr, sys) (src/forcing.jl:407-420): out is
    cleared, then every region's contribution is added."""
    if sys is not None and phys_params is None:
        phys_params = sys.phys_params
    if not isinstance(fr, (list, tuple)):
        fr = [fr]
    out.data.zero_()
    for f in fr:
        rc = f.region_cache
        rc.str.data.zero_()
        f.fcn(rc.str, y, t, rc, phys_params)
        if isinstance(rc, AreaRegionCache):
            L.call("ilm_grid_mul_add", out.data.numel(), 0 if out.data.dtype == torch.float64 else 1,
                   _ptr(rc.str.data), _ptr(rc.mask.data), _ptr(out.data), _stream_ptr(stream))
        else:
            L.call("ilm_regularize_add", rc.cache._h, out.kind, _ptr(rc.str.data), _ptr(out.data),
                   _stream_ptr(stream))
    return out
