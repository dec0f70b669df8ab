"""CPU FP64 oracle for the immersed-layer hot path -- TEST INFRASTRUCTURE ONLY.

This module restates, in NumPy/SciPy FP64, the algorithms that ImmersedLayers.jl
(v0.5.6) runs on its hot path, so that the CUDA product path can be checked
against it.  It is imported only by ``tests/``, by ``__graft_entry__.smoke()``
and by the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``; the
product path never routes through it.

The reference's arithmetic lives in three un-vendored Julia packages
(CartesianGrids.jl 0.1.29/0.2, RigidBodyTools.jl 0.5.6, ConstrainedSystems.jl
0.3.8, pinned in Project.toml:20-30).  Their published algorithms are restated
here from first principles:

* staggered-grid conventions (array extents, node positions, ghost layers) are
  inferred from the printed cache/grid objects in examples/caches.ipynb
  (PhysicalGrid((-2,2),(-2,2),0.01) -> size (406,406), I0=(203,203),
  Nodes{Primal} 405x405 with x from -2.02 to 2.02, Nodes{Dual} 406x406);
* discrete delta functions from their papers (Yang et al. 2009 smoothed
  3-point "Yang3"; Roma, Peskin & Berger 1999; Monaghan M4'; hat; M3);
* the lattice Green's function of the 5-point Laplacian from its integral
  representation (normalised G(0,0)=0, so G(1,0)=1/4, G(1,1)=1/pi);
* the composite layer operators, Schur-complement builders and block-LU solves
  follow src/surface_operators.jl, src/matrix_operators.jl,
  test/literate/problems.jl and test/literate/neumann.jl line by line.

Parity is pinned against the reference's own known-answer tests
(test/tools.jl:107-120, test/surface_ops.jl:63-77,127-146,180-256) and the
notebook outputs; absolute grid offsets, the LGF constant and the IF-HERK
tableau are "parity unpinned" (the reference's Julia path cannot run here).

Grid data are numpy arrays of shape (n1, n2) indexed [i, j] with i along x
(the reference's column-major, first-index-x layout).  Vector grid data are
tuples of component arrays.  Point data are flat arrays like the reference's
ScalarData (N), VectorData ([u; v], 2N) and TensorData
([dudx; dudy; dvdx; dvdy], 4N).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass

import numpy as np
import scipy.fft as sfft
import scipy.sparse as sp

EULER_GAMMA = 0.57721566490153286060651209

# ---------------------------------------------------------------------------
# Discrete delta functions (1-D kernels in index units, sum_j phi(r-j) = 1)
# ---------------------------------------------------------------------------


def ddf_yang3(r):
    """Smoothed 3-point kernel of Yang, Zhang, Li & Yang (JCP 228, 2009),
    the reference default (src/ImmersedLayers.jl:83, DEFAULT_DDF = Yang3)."""
    r = np.abs(np.asarray(r, dtype=np.float64))
    out = np.zeros_like(r)
    s3 = math.sqrt(3.0)
    m1 = r <= 1.0
    r1 = r[m1]
    out[m1] = (17.0 / 48.0 + s3 * math.pi / 108.0 + r1 / 4.0 - r1 * r1 / 4.0
               + (1.0 - 2.0 * r1) / 16.0 * np.sqrt(np.maximum(-12.0 * r1 * r1 + 12.0 * r1 + 1.0, 0.0))
               - s3 / 12.0 * np.arcsin(s3 / 2.0 * (2.0 * r1 - 1.0)))
    m2 = (r > 1.0) & (r < 2.0)
    r2 = r[m2]
    out[m2] = (55.0 / 48.0 - s3 * math.pi / 108.0 - 13.0 * r2 / 12.0 + r2 * r2 / 4.0
               + (2.0 * r2 - 3.0) / 48.0 * np.sqrt(np.maximum(-12.0 * r2 * r2 + 36.0 * r2 - 23.0, 0.0))
               + s3 / 36.0 * np.arcsin(s3 / 2.0 * (2.0 * r2 - 3.0)))
    return out


def ddf_roma(r):
    """3-point kernel of Roma, Peskin & Berger (JCP 153, 1999)."""
    r = np.abs(np.asarray(r, dtype=np.float64))
    out = np.zeros_like(r)
    m1 = r <= 0.5
    out[m1] = (1.0 + np.sqrt(1.0 - 3.0 * r[m1] ** 2)) / 3.0
    m2 = (r > 0.5) & (r < 1.5)
    out[m2] = (5.0 - 3.0 * r[m2] - np.sqrt(np.maximum(1.0 - 3.0 * (1.0 - r[m2]) ** 2, 0.0))) / 6.0
    return out


def ddf_m4prime(r):
    """Monaghan's M4' kernel (cubic, interpolating, 4-point support)."""
    r = np.abs(np.asarray(r, dtype=np.float64))
    out = np.zeros_like(r)
    m1 = r <= 1.0
    out[m1] = 1.0 - 2.5 * r[m1] ** 2 + 1.5 * r[m1] ** 3
    m2 = (r > 1.0) & (r < 2.0)
    out[m2] = 0.5 * (2.0 - r[m2]) ** 2 * (1.0 - r[m2])
    return out


def ddf_witchhat(r):
    """Linear hat kernel (2-point support)."""
    r = np.abs(np.asarray(r, dtype=np.float64))
    return np.where(r < 1.0, 1.0 - r, 0.0)


def ddf_m3(r):
    """Quadratic B-spline M3 kernel (3-point support)."""
    r = np.abs(np.asarray(r, dtype=np.float64))
    out = np.zeros_like(r)
    m1 = r <= 0.5
    out[m1] = 0.75 - r[m1] ** 2
    m2 = (r > 0.5) & (r < 1.5)
    out[m2] = 0.5 * (1.5 - r[m2]) ** 2
    return out


# name -> (kernel, half-support radius in cells)
DDFS = {
    "Yang3": (ddf_yang3, 2.0),
    "Roma": (ddf_roma, 1.5),
    "M4prime": (ddf_m4prime, 2.0),
    "Witchhat": (ddf_witchhat, 1.0),
    "M3": (ddf_m3, 1.5),
}

# ---------------------------------------------------------------------------
# Grid
# ---------------------------------------------------------------------------

# Position classes: (dual_x, dual_y); 1 = half-cell offset ("dual" direction)
NODES_PRIMAL = (0, 0)
NODES_DUAL = (1, 1)
EDGES_PRIMAL_U = (1, 0)   # Edges{Primal}.u  (also Edges{Dual}.v)
EDGES_PRIMAL_V = (0, 1)   # Edges{Primal}.v  (also Edges{Dual}.u)


@dataclass
class Grid:
    """PhysicalGrid restatement: NX x NY dual nodes (ghosts included), origin
    index I0 (1-based, as printed by the reference), spacing h.

    Node positions (1-based index i): primal x = (i - I0) h, i = 1..NX-1;
    dual x = (i - I0 - 1/2) h, i = 1..NX.
    """
    nx: int
    ny: int
    h: float
    i0x: int
    i0y: int

    @classmethod
    def physical(cls, xlim, ylim, h):
        """Grid covering xlim x ylim with two cells of padding on each side
        (the (406,406)/(203,203) sizing printed in examples/caches.ipynb)."""
        def one(lim):
            nl = int(math.ceil(-lim[0] / h - 1e-12))
            nr = int(math.ceil(lim[1] / h - 1e-12))
            n = nl + nr + 2 * 2 + 2
            i0 = nl + 2 + 1
            return n, i0
        nx, i0x = one(xlim)
        ny, i0y = one(ylim)
        return cls(nx, ny, float(h), i0x, i0y)

    @classmethod
    def centered(cls, n, h, ny=None):
        """n x ny dual-node grid with the origin at its centre (used for the
        grids given by cell count)."""
        ny = n if ny is None else ny
        return cls(n, ny, float(h), n // 2, ny // 2)

    def shape(self, cls_):
        dx, dy = cls_
        return (self.nx if dx else self.nx - 1, self.ny if dy else self.ny - 1)

    def coords(self, cls_):
        dx, dy = cls_
        n1, n2 = self.shape(cls_)
        x = (np.arange(1, n1 + 1) - self.i0x - 0.5 * dx) * self.h
        y = (np.arange(1, n2 + 1) - self.i0y - 0.5 * dy) * self.h
        return x, y

    def limits(self):
        return ((1 - self.i0x) * self.h, (self.nx - 1 - self.i0x) * self.h), \
               ((1 - self.i0y) * self.h, (self.ny - 1 - self.i0y) * self.h)


def zeros(g: Grid, kind):
    """kind: 'nodes_primal' | 'nodes_dual' | 'edges_primal' | 'edgegrad_primal'."""
    if kind == "nodes_primal":
        return np.zeros(g.shape(NODES_PRIMAL))
    if kind == "nodes_dual":
        return np.zeros(g.shape(NODES_DUAL))
    if kind == "edges_primal":
        return (np.zeros(g.shape(EDGES_PRIMAL_U)), np.zeros(g.shape(EDGES_PRIMAL_V)))
    if kind == "edgegrad_primal":
        return (np.zeros(g.shape(NODES_PRIMAL)), np.zeros(g.shape(NODES_DUAL)),
                np.zeros(g.shape(NODES_DUAL)), np.zeros(g.shape(NODES_PRIMAL)))
    raise ValueError(kind)


# ---------------------------------------------------------------------------
# Weighted inner products (src/tools.jl:101-236 on top of CartesianGrids' dot)
# ---------------------------------------------------------------------------

def _axis_weights(n, dual):
    """Dual direction: ghosts at both ends excluded; primal: trapezoid."""
    w = np.ones(n)
    if dual:
        w[0] = 0.0
        w[-1] = 0.0
    else:
        w[0] = 0.5
        w[-1] = 0.5
    return w


def grid_dot_array(a, b, cls_, h):
    wx = _axis_weights(a.shape[0], cls_[0])
    wy = _axis_weights(a.shape[1], cls_[1])
    return float(np.einsum("ij,ij,i,j->", a, b, wx, wy)) * h * h


# ---------------------------------------------------------------------------
# Lattice Green's function of the 5-point Laplacian
# ---------------------------------------------------------------------------

def _lgf_nodes(levels=40, npts=24):
    """Composite Gauss-Legendre nodes on [0, pi], dyadically graded towards 0."""
    xg, wg = np.polynomial.legendre.leggauss(npts)
    edges = [math.pi * 2.0 ** (-k) for k in range(levels, -1, -1)]
    edges = [0.0] + edges
    a_list, w_list = [], []
    for a, b in zip(edges[:-1], edges[1:]):
        a_list.append(0.5 * (b - a) * xg + 0.5 * (b + a))
        w_list.append(0.5 * (b - a) * wg)
    return np.concatenate(a_list), np.concatenate(w_list)


def lgf_values(m, n):
    """G(m, n) = (1/2pi) int_0^pi (1 - cos(p a) e^{-q s(a)}) / sinh s(a) da,
    cosh s = 2 - cos a, p = min(|m|,|n|), q = max(|m|,|n|).  This is the
    lattice Green's function of the 5-point Laplacian (L G = delta) with
    G(0,0) = 0.  Vectorised over m, n."""
    m = np.abs(np.asarray(m, dtype=np.int64))
    n = np.abs(np.asarray(n, dtype=np.int64))
    p = np.minimum(m, n).astype(np.float64).ravel()
    q = np.maximum(m, n).astype(np.float64).ravel()
    a, w = _lgf_nodes()
    u = 2.0 * np.sin(0.5 * a) ** 2             # cosh s - 1
    sh = np.sqrt(u * (u + 2.0))                # sinh s
    s = np.log1p(u + sh)                       # s
    wt = w / sh
    out = np.empty(p.shape)
    chunk = 4096
    for c0 in range(0, p.size, chunk):
        pc = p[c0:c0 + chunk, None]
        qc = q[c0:c0 + chunk, None]
        e = np.exp(-qc * s[None, :])
        num = -np.expm1(-qc * s[None, :]) + 2.0 * e * np.sin(0.5 * pc * a[None, :]) ** 2
        out[c0:c0 + chunk] = (num * wt[None, :]).sum(axis=1)
    return (out / (2.0 * math.pi)).reshape(m.shape)


_LGF_TABLE_CACHE = {}


def lgf_table(M):
    """G(m, n) for 0 <= m, n <= M as an (M+1, M+1) array (symmetric)."""
    if M in _LGF_TABLE_CACHE:
        return _LGF_TABLE_CACHE[M]
    for MM, tab in _LGF_TABLE_CACHE.items():
        if MM >= M:
            return tab[:M + 1, :M + 1]
    ii, jj = np.triu_indices(M + 1)
    vals = lgf_values(ii, jj)
    tab = np.zeros((M + 1, M + 1))
    tab[ii, jj] = vals
    tab[jj, ii] = vals
    _LGF_TABLE_CACHE[M] = tab
    return tab


def good_fft_size(n):
    """Smallest 2^a 3^b >= n with a >= 2."""
    best = None
    p3 = 1
    while p3 < 4 * n:
        p2 = 4
        while p2 * p3 < n:
            p2 *= 2
        cand = p2 * p3
        if best is None or cand < best:
            best = cand
        p3 *= 3
    return best


class InverseLaplacian:
    """Unbounded-domain inverse of factor*L (5-point) on an n1 x n2 array:
    linear convolution with G/factor via a zero-padded circulant embedding
    (grid_operators.jl:153-179, plan_laplacian(...; with_inverse=true))."""

    def __init__(self, n1, n2, factor):
        self.n1, self.n2, self.factor = n1, n2, factor
        self.P1 = good_fft_size(2 * n1 - 1)
        self.P2 = good_fft_size(2 * n2 - 1)
        M = max(self.P1, self.P2) // 2
        tab = lgf_table(M)
        i1 = np.arange(self.P1)
        i1 = np.minimum(i1, self.P1 - i1)
        i2 = np.arange(self.P2)
        i2 = np.minimum(i2, self.P2 - i2)
        kern = tab[i1[:, None], i2[None, :]]
        self.spec = sfft.rfft2(kern).real  # real and even

    def __call__(self, w):
        W = sfft.rfft2(w, s=(self.P1, self.P2), workers=os.cpu_count())
        out = sfft.irfft2(W * self.spec, s=(self.P1, self.P2), workers=os.cpu_count())
        return out[:self.n1, :self.n2] / self.factor


# ---------------------------------------------------------------------------
# Staggered stencils (CartesianGrids divergence!/grad!/curl!/laplacian!)
# ---------------------------------------------------------------------------

def divergence_edges(q):
    """Edges{Primal} -> Nodes{Primal}: w = u[i+1]-u[i] + v[j+1]-v[j] (all nodes)."""
    u, v = q
    return (u[1:, :] - u[:-1, :]) + (v[:, 1:] - v[:, :-1])


def grad_nodes(w, g: Grid):
    """Nodes{Primal} -> Edges{Primal}; boundary (ghost-adjacent) faces zero."""
    u = np.zeros(g.shape(EDGES_PRIMAL_U))
    v = np.zeros(g.shape(EDGES_PRIMAL_V))
    u[1:-1, :] = w[1:, :] - w[:-1, :]
    v[:, 1:-1] = w[:, 1:] - w[:, :-1]
    return (u, v)


def curl_nodes_dual(s, g: Grid):
    """Nodes{Dual} -> Edges{Primal}: u = s[j+1]-s[j], v = s[i]-s[i+1]."""
    u = s[:, 1:] - s[:, :-1]
    v = s[:-1, :] - s[1:, :]
    return (u, v)


def curl_edges(q, g: Grid):
    """Edges{Primal} -> Nodes{Dual} (interior dual nodes; ghosts zero)."""
    u, v = q
    w = np.zeros(g.shape(NODES_DUAL))
    w[1:-1, 1:-1] = (v[1:, 1:-1] - v[:-1, 1:-1]) - (u[1:-1, 1:] - u[1:-1, :-1])
    return w


def grad_edges(q, g: Grid):
    """Edges{Primal} -> EdgeGradient{Primal} (dudx, dudy, dvdx, dvdy)."""
    u, v = q
    dudx = u[1:, :] - u[:-1, :]
    dvdy = v[:, 1:] - v[:, :-1]
    dudy = np.zeros(g.shape(NODES_DUAL))
    dvdx = np.zeros(g.shape(NODES_DUAL))
    dudy[1:-1, 1:-1] = u[1:-1, 1:] - u[1:-1, :-1]
    dvdx[1:-1, 1:-1] = v[1:, 1:-1] - v[:-1, 1:-1]
    return (dudx, dudy, dvdx, dvdy)


def divergence_edgegrad(t, g: Grid):
    """EdgeGradient{Primal} -> Edges{Primal} (negative adjoint of grad_edges)."""
    dudx, dudy, dvdx, dvdy = t
    u = np.zeros(g.shape(EDGES_PRIMAL_U))
    v = np.zeros(g.shape(EDGES_PRIMAL_V))
    u[1:-1, :] = (dudx[1:, :] - dudx[:-1, :]) + (dudy[1:-1, 1:] - dudy[1:-1, :-1])
    v[:, 1:-1] = (dvdx[1:, 1:-1] - dvdx[:-1, 1:-1]) + (dvdy[:, 1:] - dvdy[:, :-1])
    return (u, v)


def laplacian_nodes(w, factor=1.0):
    """5-point Laplacian on the interior of a node array, times factor."""
    out = np.zeros_like(w)
    out[1:-1, 1:-1] = (w[2:, 1:-1] + w[:-2, 1:-1] + w[1:-1, 2:] + w[1:-1, :-2]
                       - 4.0 * w[1:-1, 1:-1])
    return out * factor


def grid_interpolate_primal_to_dual(p, g: Grid):
    out = np.zeros(g.shape(NODES_DUAL))
    out[1:-1, 1:-1] = 0.25 * (p[:-1, :-1] + p[1:, :-1] + p[:-1, 1:] + p[1:, 1:])
    return out


def grid_interpolate_primal_to_edges(p, g: Grid):
    u = np.zeros(g.shape(EDGES_PRIMAL_U))
    v = np.zeros(g.shape(EDGES_PRIMAL_V))
    u[1:-1, :] = 0.5 * (p[:-1, :] + p[1:, :])
    v[:, 1:-1] = 0.5 * (p[:, :-1] + p[:, 1:])
    return (u, v)


# ---------------------------------------------------------------------------
# Cache (src/cache.jl:164-261, 305-324)
# ---------------------------------------------------------------------------

GRID_SCALING = "GridScaling"
INDEX_SCALING = "IndexScaling"


class SurfaceCache:
    """BasicILMCache restatement for scalar ('scalar') or vector ('vector')
    grid data.  Holds the DDF interpolation matrices Phi_c (cells x points)
    for the four position classes and the inverse Laplacian."""

    def __init__(self, X, Y, nrmx, nrmy, ds, g: Grid, kind="scalar",
                 ddftype="Yang3", scaling=GRID_SCALING):
        self.X = np.asarray(X, dtype=np.float64)
        self.Y = np.asarray(Y, dtype=np.float64)
        self.nx = np.asarray(nrmx, dtype=np.float64)
        self.ny = np.asarray(nrmy, dtype=np.float64)
        self.ds = np.asarray(ds, dtype=np.float64)
        self.N = self.X.size
        self.g = g
        self.kind = kind
        self.ddftype = ddftype
        self.scaling = scaling
        self.h = g.h
        self._phi = {}
        self._linv = {}

    # -- DDF matrices -------------------------------------------------------
    def phi(self, cls_):
        if cls_ in self._phi:
            return self._phi[cls_]
        kern, rad = DDFS[self.ddftype]
        xg, yg = self.g.coords(cls_)
        n1, n2 = len(xg), len(yg)
        h = self.h
        rows, cols, vals = [], [], []
        span = int(math.ceil(rad)) + 1
        for k in range(self.N):
            ix = int(math.floor((self.X[k] - xg[0]) / h))
            iy = int(math.floor((self.Y[k] - yg[0]) / h))
            ii = np.arange(ix - span, ix + span + 1)
            jj = np.arange(iy - span, iy + span + 1)
            ii = ii[(ii >= 0) & (ii < n1)]
            jj = jj[(jj >= 0) & (jj < n2)]
            wx = kern((xg[ii] - self.X[k]) / h)
            wy = kern((yg[jj] - self.Y[k]) / h)
            W = np.outer(wx, wy)
            nz = W != 0.0
            I, J = np.meshgrid(ii, jj, indexing="ij")
            rows.append((I + n1 * J)[nz])
            cols.append(np.full(int(nz.sum()), k))
            vals.append(W[nz])
        rows = np.concatenate(rows) if rows else np.zeros(0, int)
        cols = np.concatenate(cols) if cols else np.zeros(0, int)
        vals = np.concatenate(vals) if vals else np.zeros(0)
        M = sp.csr_matrix((vals, (rows, cols)), shape=(n1 * n2, self.N))
        self._phi[cls_] = M
        return M

    def _wscale(self):
        if self.scaling == GRID_SCALING:
            return self.ds / (self.h * self.h)
        return np.ones(self.N)

    def reg_cls(self, f, cls_):
        """R_c f onto position class cls_ (fill 0 + mul!)."""
        n1, n2 = self.g.shape(cls_)
        return (self.phi(cls_) @ (self._wscale() * f)).reshape((n1, n2), order="F")

    def interp_cls(self, s, cls_):
        """E_c s from position class cls_."""
        return self.phi(cls_).T @ np.asarray(s).ravel(order="F")

    # -- derivative scaling (grid_operators.jl:8-9) -------------------------
    def dscale(self):
        return 1.0 / self.h if self.scaling == GRID_SCALING else 1.0

    def lfactor(self):
        return 1.0 / self.h ** 2 if self.scaling == GRID_SCALING else 1.0

    def inverse_laplacian(self, w):
        """inverse_laplacian! on Nodes (array) or Edges (tuple), per component."""
        if isinstance(w, tuple):
            return tuple(self.inverse_laplacian(c) for c in w)
        key = w.shape
        if key not in self._linv:
            self._linv[key] = InverseLaplacian(w.shape[0], w.shape[1], self.lfactor())
        return self._linv[key](w)

    def laplacian(self, w):
        if isinstance(w, tuple):
            return tuple(self.laplacian(c) for c in w)
        return laplacian_nodes(w, self.lfactor())


# ---- basic transfers (surface_operators.jl:13-88) --------------------------

def regularize_scalar(c: SurfaceCache, f, target="nodes_primal"):
    cls_ = NODES_PRIMAL if target == "nodes_primal" else NODES_DUAL
    return c.reg_cls(f, cls_)


def interpolate_scalar(c: SurfaceCache, s, source="nodes_primal"):
    cls_ = NODES_PRIMAL if source == "nodes_primal" else NODES_DUAL
    return c.interp_cls(s, cls_)


def regularize_vector(c: SurfaceCache, vb):
    """VectorData -> Edges{Primal}."""
    N = c.N
    return (c.reg_cls(vb[:N], EDGES_PRIMAL_U), c.reg_cls(vb[N:], EDGES_PRIMAL_V))


def interpolate_vector(c: SurfaceCache, q):
    return np.concatenate([c.interp_cls(q[0], EDGES_PRIMAL_U), c.interp_cls(q[1], EDGES_PRIMAL_V)])


def regularize_tensor(c: SurfaceCache, t):
    """TensorData -> EdgeGradient{Primal}."""
    N = c.N
    return (c.reg_cls(t[:N], NODES_PRIMAL), c.reg_cls(t[N:2 * N], NODES_DUAL),
            c.reg_cls(t[2 * N:3 * N], NODES_DUAL), c.reg_cls(t[3 * N:], NODES_PRIMAL))


def interpolate_tensor(c: SurfaceCache, q):
    return np.concatenate([c.interp_cls(q[0], NODES_PRIMAL), c.interp_cls(q[1], NODES_DUAL),
                           c.interp_cls(q[2], NODES_DUAL), c.interp_cls(q[3], NODES_PRIMAL)])


# ---- normal products (surface_operators.jl:98-343) ---------------------------

def regularize_normal(c: SurfaceCache, f):
    """Scalar f -> Edges{Primal}: R_f (n o f)."""
    return regularize_vector(c, np.concatenate([c.nx * f, c.ny * f]))


def normal_interpolate(c: SurfaceCache, q):
    """Edges{Primal} -> scalar: n . R_f^T q."""
    v = interpolate_vector(c, q)
    return c.nx * v[:c.N] + c.ny * v[c.N:]


def regularize_normal_cross(c: SurfaceCache, f):
    """Scalar f -> Edges{Primal}: R_f (n x f e_z) = R_f (n_y f, -n_x f)."""
    return regularize_vector(c, np.concatenate([c.ny * f, -c.nx * f]))


def normal_cross_interpolate(c: SurfaceCache, q):
    """Edges{Primal} -> scalar: e_z . (n x R_f^T q) = n_x v_y - n_y v_x."""
    v = interpolate_vector(c, q)
    return c.nx * v[c.N:] - c.ny * v[:c.N]


def regularize_normal_dot(c: SurfaceCache, vs):
    """VectorData -> Nodes{Primal}: R_c (n . v)."""
    return c.reg_cls(c.nx * vs[:c.N] + c.ny * vs[c.N:], NODES_PRIMAL)


def normal_dot_interpolate(c: SurfaceCache, p):
    """Nodes{Primal} -> VectorData: n (R_c^T p)."""
    s = c.interp_cls(p, NODES_PRIMAL)
    return np.concatenate([c.nx * s, c.ny * s])


def _tensor_nv(c, v):
    """pointwise_tensorproduct!(n, v) in TensorData slots (dudx, dudy, dvdx,
    dvdy) = (n_x v_x, n_y v_x, n_x v_y, n_y v_y): the slot d(c)/d(k) holds n_k
    times component c, so that the tensor divergence of n o 1 (u: d/dx dudx +
    d/dy dudy) is the scalar double layer on each edge component -- the
    vector-cache mask of src/surface_operators.jl:872-877 then integrates to
    the enclosed area, as test/surface_ops.jl:221-231 requires."""
    N = c.N
    vx, vy = v[:N], v[N:]
    return np.concatenate([c.nx * vx, c.ny * vx, c.nx * vy, c.ny * vy])


def _tensor_dot_n(c, t):
    """pointwise_dot!(n, tau), the adjoint of _tensor_nv:
    (n_x dudx + n_y dudy, n_x dvdx + n_y dvdy)."""
    N = c.N
    t11, t12, t21, t22 = t[:N], t[N:2 * N], t[2 * N:3 * N], t[3 * N:]
    return np.concatenate([c.nx * t11 + c.ny * t12, c.nx * t21 + c.ny * t22])


def regularize_normal_dot_tensor(c: SurfaceCache, taus):
    """regularize_normal_dot!(v::Edges{Primal}, taus::TensorData)
    (src/surface_operators.jl:205-215): R_f (n . tau)."""
    return regularize_vector(c, _tensor_dot_n(c, taus))


def normal_dot_interpolate_tensor(c: SurfaceCache, q):
    """normal_dot_interpolate!(taus::TensorData, v::Edges{Primal})
    (src/surface_operators.jl:332-343): n o R_f^T v."""
    return _tensor_nv(c, interpolate_vector(c, q))


def regularize_normal_tensor(c: SurfaceCache, v):
    """VectorData -> EdgeGradient: R_t (n o v)."""
    return regularize_tensor(c, _tensor_nv(c, v))


def regularize_normal_symm(c: SurfaceCache, v):
    """R_t (n o v + v o n - (n.v) I)   (surface_operators.jl:125-133)."""
    N = c.N
    t = _tensor_nv(c, v)
    tt = np.concatenate([t[:N], t[2 * N:3 * N], t[N:2 * N], t[3 * N:]])
    t = t + tt
    nv = c.nx * v[:N] + c.ny * v[N:]
    t[:N] -= nv
    t[3 * N:] -= nv
    return regularize_tensor(c, t)


def normal_interpolate_tensor(c: SurfaceCache, A):
    """EdgeGradient -> VectorData: n . R_t^T A."""
    return _tensor_dot_n(c, interpolate_tensor(c, A))


def normal_interpolate_symm(c: SurfaceCache, A):
    """n . R_t^T (A + A^T - tr(A) I)   (surface_operators.jl:274-283)."""
    dudx, dudy, dvdx, dvdy = A
    tr = dudx + dvdy
    B = (dudx + dudx - tr, dudy + dvdx, dvdx + dudy, dvdy + dvdy - tr)
    return _tensor_dot_n(c, interpolate_tensor(c, B))


# ---- composite layer operators (surface_operators.jl:357-725) ---------------

def surface_divergence(c: SurfaceCache, f):
    """theta = D R_f (n o f) / h  (scalar cache)."""
    return divergence_edges(regularize_normal(c, f)) * c.dscale()


def surface_grad(c: SurfaceCache, w):
    """vn = n . R_f^T G w / h."""
    return normal_interpolate(c, grad_nodes(w, c.g)) * c.dscale()


def surface_curl_T(c: SurfaceCache, f):
    """w = C^T R_f (n o f) / h: scalar f -> Nodes{Dual} (scalar cache)."""
    return curl_edges(regularize_normal(c, f), c.g) * c.dscale()


def surface_curl(c: SurfaceCache, s):
    """vn = n . R_f^T C s / h: Nodes{Dual} -> scalar (scalar cache)."""
    return normal_interpolate(c, curl_nodes_dual(s, c.g)) * c.dscale()


def surface_curl_cross_T(c: SurfaceCache, f):
    """w = C^T R_f (n x f e_z) / h."""
    return curl_edges(regularize_normal_cross(c, f), c.g) * c.dscale()


def surface_curl_cross(c: SurfaceCache, s):
    """gamma = e_z . (n x R_f^T C s) / h."""
    return normal_cross_interpolate(c, curl_nodes_dual(s, c.g)) * c.dscale()


def surface_divergence_cross(c: SurfaceCache, f):
    """theta = D R_f (n x f e_z) / h."""
    return divergence_edges(regularize_normal_cross(c, f)) * c.dscale()


def surface_grad_cross(c: SurfaceCache, w):
    """gamma = e_z . (n x R_f^T G w) / h."""
    return normal_cross_interpolate(c, grad_nodes(w, c.g)) * c.dscale()


# vector-cache composite operators
def surface_curl_T_vector(c: SurfaceCache, v):
    """w = C^T R_f v / h: VectorData -> Nodes{Dual}."""
    return curl_edges(regularize_vector(c, v), c.g) * c.dscale()


def surface_curl_vector(c: SurfaceCache, s):
    """v = R_f^T C s / h: Nodes{Dual} -> VectorData."""
    return interpolate_vector(c, curl_nodes_dual(s, c.g)) * c.dscale()


def surface_curl_T_vector_scalar(c: SurfaceCache, f):
    """Vector cache, scalar input: C^T R_f (n o f) / h with R_f = cache.R."""
    return surface_curl_T_vector(c, np.concatenate([c.nx * f, c.ny * f]))


def surface_curl_vector_scalar(c: SurfaceCache, s):
    """Vector cache, scalar output: n . R_f^T C s / h."""
    v = surface_curl_vector(c, s)
    return c.nx * v[:c.N] + c.ny * v[c.N:]


def surface_divergence_vector(c: SurfaceCache, dv):
    """Edges{Primal} = D R_t (n o dv) / h."""
    return tuple(x * c.dscale() for x in divergence_edgegrad(regularize_normal_tensor(c, dv), c.g))


def surface_divergence_symm(c: SurfaceCache, dv):
    return tuple(x * c.dscale() for x in divergence_edgegrad(regularize_normal_symm(c, dv), c.g))


def surface_grad_vector(c: SurfaceCache, q):
    return normal_interpolate_tensor(c, grad_edges(q, c.g)) * c.dscale()


def surface_grad_symm(c: SurfaceCache, q):
    return normal_interpolate_symm(c, grad_edges(q, c.g)) * c.dscale()


# ---- masks (surface_operators.jl:737-923) ----------------------------------

def mask(c: SurfaceCache):
    """H = -L^{-1} D_s 1 on Nodes{Primal} (scalar cache)."""
    return -c.inverse_laplacian(surface_divergence(c, np.ones(c.N)))


# ---- Schur-complement builders (matrix_operators.jl:9-244) ------------------

def create_RTLinvR(c: SurfaceCache, scale=1.0):
    A = np.empty((c.N, c.N))
    e = np.zeros(c.N)
    for col in range(c.N):
        e[:] = 0.0
        e[col] = 1.0
        w = c.inverse_laplacian(regularize_scalar(c, e))
        A[:, col] = -scale * interpolate_scalar(c, w)
    return A


def create_CLinvCT(c: SurfaceCache, scale=1.0):
    A = np.empty((c.N, c.N))
    e = np.zeros(c.N)
    for col in range(c.N):
        e[:] = 0.0
        e[col] = 1.0
        w = c.inverse_laplacian(surface_curl_T(c, e))
        A[:, col] = -scale * surface_curl(c, w)
    return A


def create_GLinvD(c: SurfaceCache, scale=1.0):
    A = np.empty((c.N, c.N))
    e = np.zeros(c.N)
    for col in range(c.N):
        e[:] = 0.0
        e[col] = 1.0
        w = c.inverse_laplacian(surface_divergence(c, e))
        A[:, col] = -scale * surface_grad(c, w)
    return A


def create_nRTRn(c: SurfaceCache, scale=1.0):
    A = np.empty((c.N, c.N))
    e = np.zeros(c.N)
    for col in range(c.N):
        e[:] = 0.0
        e[col] = 1.0
        A[:, col] = scale * normal_interpolate(c, regularize_normal(c, e))
    return A


def create_GLinvD_vector(c: SurfaceCache, scale=1.0):
    n = 2 * c.N
    A = np.empty((n, n))
    e = np.zeros(n)
    for col in range(n):
        e[:] = 0.0
        e[col] = 1.0
        w = c.inverse_laplacian(surface_divergence_vector(c, e))
        A[:, col] = -scale * surface_grad_vector(c, w)
    return A


# ---------------------------------------------------------------------------
# Matrix-free Schur operators (what the GPU CG applies)
# ---------------------------------------------------------------------------

def schur_dirichlet_apply(c: SurfaceCache, s):
    """S s = E L^{-1} R s  (= -create_RTLinvR(c) @ s)."""
    return interpolate_scalar(c, c.inverse_laplacian(regularize_scalar(c, s)))


def schur_neumann_apply(c: SurfaceCache, s):
    """S s = -C_s L^{-1} C_s^T s  (= create_CLinvCT(c) @ s)."""
    return -surface_curl(c, c.inverse_laplacian(surface_curl_T(c, s)))


# ---------------------------------------------------------------------------
# Problem solves (test/literate/problems.jl:259-298, neumann.jl:101-142)
# ---------------------------------------------------------------------------

def solve_dirichlet(c: SurfaceCache, fplus, fminus, S=None):
    """Block-LU Dirichlet Poisson solve with dense Schur complement, as the
    reference's DirichletPoissonProblem `solve` (without the C^6 filter).
    Returns (f on Nodes{Primal}, s jump strength)."""
    if S is None:
        S = create_RTLinvR(c)
    jump = fplus - fminus
    avg = 0.5 * (fplus + fminus)
    fstar = c.inverse_laplacian(surface_divergence(c, jump))
    s = avg - interpolate_scalar(c, fstar)
    s = -np.linalg.solve(S, s)
    f = c.inverse_laplacian(regularize_scalar(c, s)) + fstar
    return f, s


def solve_neumann(c: SurfaceCache, vplus, vminus, S=None):
    """Neumann Poisson solve (neumann.jl:101-142): returns (f, df, s, ds)."""
    if S is None:
        S = create_CLinvCT(c)
    dvn = vplus - vminus
    vn = 0.5 * (vplus + vminus)
    fstar = c.inverse_laplacian(regularize_scalar(c, dvn))
    df = vn - surface_grad(c, fstar)
    df = -np.linalg.solve(S, df)
    f = c.inverse_laplacian(surface_divergence(c, df)) + fstar
    sstar = surface_curl_T(c, df)
    ds = np.linalg.solve(S, surface_grad_cross(c, fstar))
    s = -(surface_curl_cross_T(c, ds) - sstar)
    s = c.inverse_laplacian(s)
    return f, df, s, ds


# ---------------------------------------------------------------------------
# Heat conduction with a Dirichlet surface: IF-HERK time marching
# (test/literate/heatconduction.jl:66-189, src/timemarching.jl:254-277)
# ---------------------------------------------------------------------------
# Liska & Colonius (2016) IF-HERK, scheme "A": c = (0, 1/3, 1),
# a21 = 1/3, a31 = -1, a32 = 2, b = (0, 3/4, 1/4).
IFHERK_A = dict(c=(0.0, 1.0 / 3.0, 1.0), a21=1.0 / 3.0, a31=-1.0, a32=2.0, b=(0.0, 0.75, 0.25))


def heat_kernel_1d(a, tol=1e-17, rmax=32):
    """1-D factor of the lattice heat kernel exp(a L5): e^{-2a} I_m(2a)."""
    from scipy.special import ive
    if a == 0.0:
        return np.array([1.0])
    m = np.arange(0, rmax + 1)
    k = ive(m, 2.0 * a)            # e^{-2a} I_m(2a)
    R = int(np.nonzero(k > tol)[0].max()) if np.any(k > tol) else 0
    k = k[:R + 1]
    return np.concatenate([k[:0:-1], k])


def apply_if(w, a):
    """exp(a L5) w on an unbounded lattice (zero outside the array)."""
    from scipy.ndimage import convolve1d
    k = heat_kernel_1d(a)
    if k.size == 1:
        return w.copy()
    t = convolve1d(w, k, axis=0, mode="constant")
    return convolve1d(t, k, axis=1, mode="constant")


def heat_schur(c: SurfaceCache, a):
    """S_a = E exp(a L) R (dense, by columns): the stage Schur complement."""
    N = c.N
    S = np.empty((N, N))
    e = np.zeros(N)
    for col in range(N):
        e[:] = 0.0
        e[col] = 1.0
        S[:, col] = interpolate_scalar(c, apply_if(regularize_scalar(c, e), a))
    return S


def heat_march(c: SurfaceCache, T0, tb_plus, tb_minus, kappa, dt, nsteps, scheme=IFHERK_A):
    """Advance dT/dt = kappa L T + R sigma - kappa D_s[T] with E T = avg(T_b)
    by IF-HERK (the DirichletHeatConduction problem of the reference).
    Returns (T, sigma of the last stage)."""
    h = c.h
    cc, a21, a31, a32, b = scheme["c"], scheme["a21"], scheme["a31"], scheme["a32"], scheme["b"]
    af = kappa * dt / h ** 2     # IF argument of a full step (grid units)
    jump = tb_plus - tb_minus
    avg = 0.5 * (tb_plus + tb_minus)
    r1 = -kappa * surface_divergence(c, jump)
    Sm = {t: heat_schur(c, af * t) for t in (cc[1], cc[2] - cc[1], 0.0)}
    T = T0.copy()
    sig = np.zeros(c.N)

    def F(s):
        return r1 + regularize_scalar(c, s)

    for _ in range(nsteps):
        # stage 2
        yh = apply_if(T + dt * a21 * r1, af * cc[1])
        s1 = np.linalg.lstsq(Sm[cc[1]], (avg - interpolate_scalar(c, yh)) / (dt * a21), rcond=None)[0]
        # stage 3
        U = apply_if(T + dt * a31 * F(s1), af * cc[1])
        yh = apply_if(U + dt * a32 * r1, af * (cc[2] - cc[1]))
        s2 = np.linalg.lstsq(Sm[cc[2] - cc[1]], (avg - interpolate_scalar(c, yh)) / (dt * a32), rcond=None)[0]
        # final update
        V = apply_if(T + dt * b[0] * F(s1), af * cc[1])
        yh = apply_if(V + dt * b[1] * F(s2), af * (cc[2] - cc[1])) + dt * b[2] * r1
        s3 = np.linalg.lstsq(Sm[0.0], (avg - interpolate_scalar(c, yh)) / (dt * b[2]), rcond=None)[0]
        T = yh + dt * b[2] * regularize_scalar(c, s3)
        sig = s3
    return T, sig


# ---------------------------------------------------------------------------
# Stokes flow (test/literate/stokes.jl:52-166; src/matrix_operators.jl:64-128,
# 247-262) on a vector cache
# ---------------------------------------------------------------------------
EDGES_PRIMAL_V = (0, 1)


def create_CL2invCT_vector(c: SurfaceCache, scale=1.0):
    """-C_s L^-2 C_s^T on VectorData (src/matrix_operators.jl:102-128)."""
    n = 2 * c.N
    A = np.empty((n, n))
    e = np.zeros(n)
    for col in range(n):
        e[:] = 0.0
        e[col] = 1.0
        w = c.inverse_laplacian(c.inverse_laplacian(surface_curl_T_vector(c, e)))
        A[:, col] = -scale * surface_curl_vector(c, w)
    return A


def create_CLinvCT_scalar_vector(c: SurfaceCache, scale=1.0):
    """-C_s L^-1 C_s^T on ScalarData of a vector cache (src/matrix_operators.jl:71-93)."""
    A = np.empty((c.N, c.N))
    e = np.zeros(c.N)
    for col in range(c.N):
        e[:] = 0.0
        e[col] = 1.0
        w = c.inverse_laplacian(surface_curl_T_vector_scalar(c, e))
        A[:, col] = -scale * surface_curl_vector_scalar(c, w)
    return A


def _filter_rows(ER):
    d = ER.sum(axis=1, keepdims=True)
    return np.where(d != 0.0, ER / np.where(d != 0.0, d, 1.0), 0.0)


def surface_filter_scalar(c: SurfaceCache):
    """Surface filter C = E~ R on ScalarData through Nodes{Primal}
    (create_surface_filter, src/matrix_operators.jl:254-268): the rows of
    E R normalised to sum to one (E~ = W^-1 E, W = diag(E R 1), as in
    surface_filter_vector).  Returns the N x N matrix."""
    P = c.phi(NODES_PRIMAL)
    return _filter_rows((P.T @ (P @ sp.diags(c._wscale()))).toarray())


def surface_filter(c: SurfaceCache, s, power=1, vector=False):
    """C^power s (test/literate/problems.jl:107,297 apply C^6)."""
    F = surface_filter_vector(c) if vector else surface_filter_scalar(c)
    out = np.asarray(s, dtype=np.float64)
    for _ in range(power):
        out = F @ out
    return out


def surface_filter_vector(c: SurfaceCache):
    """Surface filter E~ R on VectorData (src/matrix_operators.jl:247-262).
    The filtered interpolation E~ of CartesianGrids' Regularize(filter=true)
    is un-vendored; restated from Goza, Liska, Morley & Colonius (2016), the
    method it implements: E~ = W^-1 E with W = diag(E R 1), i.e. the rows of
    E R normalised so that constant surface data are reproduced.  Returns the
    2N x 2N block-diagonal matrix (u and v components on their own edges)."""
    n = c.N
    F = np.zeros((2 * n, 2 * n))
    for k, cls_ in enumerate((EDGES_PRIMAL_U, EDGES_PRIMAL_V)):
        P = c.phi(cls_)
        ER = (P.T @ (P @ sp.diags(c._wscale()))).toarray()
        F[k * n:(k + 1) * n, k * n:(k + 1) * n] = _filter_rows(ER)
    return F


def solve_stokes(c: SurfaceCache, vplus, vminus, S=None, Ss=None, filt=None):
    """Stokes flow with no-slip surfaces by the reference's block-LU
    (test/literate/stokes.jl:101-166).  vplus / vminus: VectorData (2N) of
    the exterior / interior surface velocities.  Returns (v: Edges{Primal}
    tuple, s: Nodes{Dual} streamfunction, sigma: VectorData traction)."""
    if S is None:
        S = create_CL2invCT_vector(c)
    if Ss is None:
        Ss = create_CLinvCT_scalar_vector(c)
    if filt is None:
        filt = surface_filter_vector(c)
    n = c.N
    dv = vplus - vminus
    vb = 0.5 * (vplus + vminus)
    # psi*
    sstar = -curl_edges(surface_divergence_symm(c, dv), c.g) * c.dscale()
    sstar = c.inverse_laplacian(c.inverse_laplacian(sstar))
    # normal-velocity jump: potential part
    dvn = c.nx * dv[:n] + c.ny * dv[n:]
    phi = c.inverse_laplacian(regularize_scalar(c, dvn))
    vphi = tuple(x * c.dscale() for x in grad_nodes(phi, c.g))
    vprime = vb - interpolate_vector(c, vphi)
    # surface velocity of psi*
    v = tuple(x * c.dscale() for x in curl_nodes_dual(sstar, c.g))
    vprime = vprime - interpolate_vector(c, v)
    sigma = np.linalg.solve(S, vprime)
    # correction streamfunction
    s = -surface_curl_T_vector(c, sigma)
    s = c.inverse_laplacian(c.inverse_laplacian(s)) + sstar
    v = tuple(a * c.dscale() + b for a, b in zip(curl_nodes_dual(s, c.g), vphi))
    # streamfunction equivalent of the scalar potential
    dsc = np.linalg.solve(Ss, surface_grad_cross(c, phi))
    s = s + c.inverse_laplacian(-surface_curl_cross_T(c, dsc))
    sigma = filt @ (filt @ sigma)
    return v, s, sigma


# ---------------------------------------------------------------------------
# Grid averaging, convective derivatives and w x v (src/grid_operators.jl:186-434)
# ---------------------------------------------------------------------------
# CartesianGrids' grid_interpolate! (un-vendored) restated as staggered-grid
# averaging: along a direction where the target sits on the primal lattice
# and the source on the dual one, every target value is the mean of its two
# neighbours; from primal to dual, only the non-ghost dual positions
# (1..n-2) have two neighbours and the two ghost layers stay zero (the same
# boundary rule as grad! / curl! onto dual positions above).  Edges{Dual}.u
# sits where Edges{Primal}.v sits and Edges{Dual}.v where Edges{Primal}.u
# sits.  The results carry no known-answer test in the reference ("parity
# unpinned"): the tests check them against this restatement and against
# exact answers for linear fields.

def _avg_d2p(a, axis):
    """Dual -> primal along `axis`: (a[k] + a[k+1]) / 2 at every primal k."""
    a = np.asarray(a)
    if axis == 0:
        return 0.5 * (a[:-1, :] + a[1:, :])
    return 0.5 * (a[:, :-1] + a[:, 1:])


def _avg_p2d(a, axis):
    """Primal -> dual along `axis`: (a[k-1] + a[k]) / 2 at dual k = 1..n-2
    (n = primal length + 1); the ghost ends are zero."""
    a = np.asarray(a)
    if axis == 0:
        out = np.zeros((a.shape[0] + 1, a.shape[1]))
        out[1:-1, :] = 0.5 * (a[:-1, :] + a[1:, :])
    else:
        out = np.zeros((a.shape[0], a.shape[1] + 1))
        out[:, 1:-1] = 0.5 * (a[:, :-1] + a[:, 1:])
    return out


def grad_nodes_dual(w):
    """grad!(Edges{Dual}, Nodes{Dual}): u = w[i+1]-w[i] (at Edges{Primal}.v
    positions), v = w[j+1]-w[j] (at Edges{Primal}.u positions), every value."""
    return (w[1:, :] - w[:-1, :], w[:, 1:] - w[:, :-1])


def convective_derivative_nodes_primal(u, p, g: Grid, scale=1.0):
    """u . grad p for p on Nodes{Primal}, u on Edges{Primal}
    (_unscaled_convective_derivative!, src/grid_operators.jl:318-327):
    grad p onto the edges, times u, averaged back onto the nodes (the two
    components summed), times the derivative scale (:8-9)."""
    gx, gy = grad_nodes(p, g)
    return (_avg_d2p(u[0] * gx, 0) + _avg_d2p(u[1] * gy, 1)) * scale


def convective_derivative_nodes_dual(u, w, g: Grid, scale=1.0):
    """u . grad w for w on Nodes{Dual}, u on Edges{Primal} (:330-342): u is
    averaged onto the Edges{Dual} positions (four-point means), times the
    Edges{Dual} gradient of w, averaged onto the non-ghost dual nodes."""
    gu, gv = grad_nodes_dual(w)
    ud_u = _avg_p2d(_avg_d2p(u[0], 0), 1)      # Edges{Dual}.u (primal x, dual y)
    ud_v = _avg_p2d(_avg_d2p(u[1], 1), 0)      # Edges{Dual}.v (dual x, primal y)
    tu, tv = ud_u * gu, ud_v * gv
    out = np.zeros(w.shape)
    out[1:-1, 1:-1] = (0.5 * (tu[:-1, :] + tu[1:, :]))[:, 1:-1] + (0.5 * (tv[:, :-1] + tv[:, 1:]))[1:-1, :]
    return out * scale


def convective_derivative_edges(v, u, g: Grid, scale=1.0):
    """v . grad u for Edges{Primal} v and u (:344-371; u . grad u with
    v = u): v averaged onto the EdgeGradient positions (u-component onto
    dudx/dudy, v-component onto dvdx/dvdy), transposed (dudy <-> dvdx),
    times grad u, averaged back onto the edges."""
    vu, vv = v
    a_dudx = _avg_d2p(vu, 0)                   # Nodes{Primal}
    a_dudy = _avg_p2d(vu, 1)                   # Nodes{Dual}
    a_dvdx = _avg_p2d(vv, 0)                   # Nodes{Dual}
    a_dvdy = _avg_d2p(vv, 1)                   # Nodes{Primal}
    dudx, dudy, dvdx, dvdy = grad_edges(u, g)
    t_dudx, t_dudy = a_dudx * dudx, a_dvdx * dudy     # transposed: dudy slot holds the dvdx average
    t_dvdx, t_dvdy = a_dudy * dvdx, a_dvdy * dvdy
    ou = _avg_p2d(t_dudx, 0) + _avg_d2p(t_dudy, 1)
    ov = _avg_d2p(t_dvdx, 0) + _avg_p2d(t_dvdy, 1)
    ou[0, :] = 0.0
    ou[-1, :] = 0.0
    ov[:, 0] = 0.0
    ov[:, -1] = 0.0
    return (ou * scale, ov * scale)


def w_cross_v(w, u):
    """w x v for vorticity w (Nodes{Dual}) and velocity u (Edges{Primal})
    (_unscaled_w_cross_v!, src/grid_operators.jl:419-434):
    (w x v).u = mean_y( -mean_x(v) w ),  (w x v).v = mean_x( mean_y(u) w )."""
    vd = _avg_p2d(u[1], 0)                     # v onto dual nodes
    ud = _avg_p2d(u[0], 1)                     # u onto dual nodes
    return (_avg_d2p(-vd * w, 1), _avg_d2p(ud * w, 0))


# ---------------------------------------------------------------------------
# Helmholtz decomposition (src/helmholtz.jl)
# ---------------------------------------------------------------------------

def regularize_normal_cross_vector(c: SurfaceCache, vs):
    """regularize_normal_cross!(w::Nodes{Dual}, vs::VectorData)
    (src/surface_operators.jl:167-178): R_n (n x v) = R_n (n_x v_y - n_y v_x)."""
    return c.reg_cls(c.nx * vs[c.N:] - c.ny * vs[:c.N], NODES_DUAL)


def vectorpotential_from_masked_curlv(c: SurfaceCache, curlv, dv):
    """L psi = -(curlv + R_n n x [v]) (src/helmholtz.jl:85-100,117-120)."""
    rhs = curlv + (regularize_normal_cross_vector(c, dv) if c.N else 0.0)
    return -c.inverse_laplacian(rhs)


def scalarpotential_from_masked_divv(c: SurfaceCache, divv, dv):
    """L phi = divv + R_c n . [v] (src/helmholtz.jl:196-207,227-231)."""
    rhs = divv + (regularize_normal_dot(c, dv) if c.N else 0.0)
    return c.inverse_laplacian(rhs)


def vecfield_helmholtz(c: SurfaceCache, curlv, divv, dv, vp=None):
    """v = curl psi + grad phi + v_p (src/helmholtz.jl:327-344); curl and
    grad carry the derivative scale of the cache; vp: Edges tuple, a
    uniform (Vx, Vy) pair, or None."""
    psi = vectorpotential_from_masked_curlv(c, curlv, dv)
    phi = scalarpotential_from_masked_divv(c, divv, dv)
    vpsi = tuple(a * c.dscale() for a in curl_nodes_dual(psi, c.g))
    vphi = tuple(a * c.dscale() for a in grad_nodes(phi, c.g))
    v = (vpsi[0] + vphi[0], vpsi[1] + vphi[1])
    if vp is not None:
        v = (v[0] + vp[0], v[1] + vp[1])
    return v


# ---------------------------------------------------------------------------
# Schur complements of vector caches and the remaining kinds, by columns
# (src/matrix_operators.jl:9-244), as the reference builds them
# ---------------------------------------------------------------------------

def _columns(n, apply, scale):
    A = np.empty((n, n))
    e = np.zeros(n)
    for col in range(n):
        e[:] = 0.0
        e[col] = 1.0
        A[:, col] = scale * apply(e)
    return A


def create_RTLinvR_vector(c: SurfaceCache, scale=1.0):
    return _columns(2 * c.N, lambda e: interpolate_vector(c, c.inverse_laplacian(regularize_vector(c, e))), -scale)


def create_CLinvCT_vector(c: SurfaceCache, scale=1.0):
    return _columns(2 * c.N, lambda e: surface_curl_vector(c, c.inverse_laplacian(surface_curl_T_vector(c, e))),
                    -scale)


def create_nRTRn_vector(c: SurfaceCache, scale=1.0):
    return _columns(2 * c.N, lambda e: normal_interpolate_tensor(c, regularize_normal_tensor(c, e)), scale)


def create_GLinvD_symm(c: SurfaceCache, scale=1.0):
    """create_GLinvD_symm (src/matrix_operators.jl:165-185), vector caches."""
    return _columns(2 * c.N, lambda e: surface_grad_symm(c, c.inverse_laplacian(surface_divergence_symm(c, e))),
                    -scale)


def create_GLinvD_cross(c: SurfaceCache, scale=1.0):
    """-G^x_s L^-1 D^x_s (src/matrix_operators.jl:195-215, the operator its
    documentation states; the reference's own call raises)."""
    return _columns(c.N, lambda e: surface_grad_cross(c, c.inverse_laplacian(surface_divergence_cross(c, e))),
                    -scale)


def mask_vector(c: SurfaceCache, kind="edges_primal"):
    """Vector-cache mask (src/surface_operators.jl:872-877, :907-923): H on
    Edges{Primal} = -L^{-1} D_s 1 with the all-ones VectorData, other grid
    types from its u component (Nodes{Dual}: mean over y onto the non-ghost
    rows; Nodes{Primal}: mean over x)."""
    H = tuple(-x for x in c.inverse_laplacian(surface_divergence_vector(c, np.ones(2 * c.N))))
    if kind == "edges_primal":
        return H
    nd, npr = _avg_p2d(H[0], 1), _avg_d2p(H[0], 0)
    if kind == "nodes_dual":
        return nd
    if kind == "nodes_primal":
        return npr
    return (npr, nd, nd, npr)
