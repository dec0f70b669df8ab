"""Shared test geometries: the reference's own unit-test set-ups."""
import math

import numpy as np

import ilm_oracle as O
from immersedlayers import bodies as B


def surface_ops_case():
    """test/surface_ops.jl:4-13: h = 0.04 on [-2,2]^2, circle R = 1, ds = 1.4 h."""
    h = 0.04
    g = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    b = B.circle(1.0, ds=1.4 * h)
    return g, b


def tools_case():
    """test/tools.jl:5-17: h = 0.02 on [-5.98,5.98]^2, circle R = 1, ds = 1.5 h."""
    h = 0.02
    g = O.Grid.physical((-5.98, 5.98), (-5.98, 5.98), h)
    b = B.circle(1.0, ds=1.5 * h)
    return g, b


def dirichlet_config1():
    """Plain Dirichlet Poisson: [-2,2]^2, h = 0.02, circle r = 0.5 with 157
    points, f_b = cos(theta) + 0.1 N(0,1) (numpy default_rng(1))."""
    h = 0.02
    g = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    b = B.circle(0.5, n=157)
    th = np.arctan2(b.y, b.x)
    rng = np.random.default_rng(1)
    fb = np.cos(th) + 0.1 * rng.standard_normal(len(b))
    return g, b, fb


def heat_case(h=0.02, r=0.4, ds_factor=1.4):
    """Small heat-conduction set-up: [-1.28,1.28]^2 with spacing h, a circle
    of radius r at ds = 1.4 h (the reference example at a smaller size)."""
    g = O.Grid.physical((-1.28, 1.28), (-1.28, 1.28), h)
    b = B.circle(r, ds=ds_factor * h)
    return g, b


def oracle_cache(g, b, kind="scalar", ddf="Yang3"):
    return O.SurfaceCache(b.x, b.y, b.nx, b.ny, b.ds, g, kind=kind, ddftype=ddf)


def angles(n):
    return 2 * math.pi * np.arange(n) / n
