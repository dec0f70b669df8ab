"""Closed surface shapes for immersion (the RigidBodyTools.jl subset the hot
path uses: Circle, Ellipse, Rectangle/Square, Polygon, BodyList).

Every shape is a closed polygon of vertices ordered counter-clockwise.  The
immersed points are the panel midpoints, the areas are the panel lengths and the
normals are the outward panel normals -- the midpoint rule that
ImmersedLayers.jl's `points`, `areas` and `normals` use (src/tools.jl:16-38,
`normalmid`/`dlengthmid`).  For a circle of radius a with N points this puts the
points exactly on the circle at angles 2 pi k/N, with areas 2 a tan(pi/N), which
reproduces the reference's printed circumference dot(1,1,ds) = 6.283288300933757
for Circle(1.0, 0.014) (examples/caches.ipynb, 448 points).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Body:
    """One closed surface: points (x, y), outward normals (nx, ny), areas ds."""
    x: np.ndarray
    y: np.ndarray
    nx: np.ndarray
    ny: np.ndarray
    ds: np.ndarray
    name: str = "body"

    def __len__(self):
        return int(self.x.size)

    @property
    def arcs(self):
        """Arc-length coordinate of each point (src/tools.jl:46, `arcs`)."""
        return np.concatenate([[0.0], np.cumsum(0.5 * (self.ds[:-1] + self.ds[1:]))])


def from_vertices(vx, vy, name="polygon") -> Body:
    """Midpoint-rule surface from counter-clockwise closed-polygon vertices."""
    vx = np.asarray(vx, dtype=np.float64)
    vy = np.asarray(vy, dtype=np.float64)
    wx = np.roll(vx, -1)
    wy = np.roll(vy, -1)
    dx = wx - vx
    dy = wy - vy
    ln = np.hypot(dx, dy)
    return Body(0.5 * (vx + wx), 0.5 * (vy + wy), dy / ln, -dx / ln, ln, name)


def _npts_circle(a, ds):
    return 4 * int(round(math.pi * a / (2.0 * ds)))


def circle(a, ds=None, n=None, center=(0.0, 0.0)) -> Body:
    """Circle of radius a with n points (or n chosen from spacing ds as
    4 round(pi a / 2 ds), which gives the reference's 448 points for
    Circle(1.0, 0.014) and 224 for Circle(0.5, 0.014))."""
    if n is None:
        n = _npts_circle(a, ds)
    th = 2.0 * math.pi * np.arange(n) / n
    rv = a / math.cos(math.pi / n)
    tv = th - math.pi / n
    b = from_vertices(center[0] + rv * np.cos(tv), center[1] + rv * np.sin(tv), "circle")
    return b


def _equal_arc_vertices(fx, fy, n, nfine=20000):
    """n vertices equally spaced in arc length along the closed curve
    t in [0, 2 pi) -> (fx(t), fy(t))."""
    t = np.linspace(0.0, 2.0 * math.pi, nfine + 1)
    x, y = fx(t), fy(t)
    seg = np.hypot(np.diff(x), np.diff(y))
    s = np.concatenate([[0.0], np.cumsum(seg)])
    target = np.arange(n) * s[-1] / n
    tv = np.interp(target, s, t)
    return fx(tv), fy(tv), s[-1]


def ellipse(a, b, ds=None, n=None, center=(0.0, 0.0), angle=0.0) -> Body:
    """Ellipse with semi-axes a (along the rotated x axis) and b."""
    ca, sa = math.cos(angle), math.sin(angle)

    def fx(t):
        return center[0] + ca * a * np.cos(t) - sa * b * np.sin(t)

    def fy(t):
        return center[1] + sa * a * np.cos(t) + ca * b * np.sin(t)

    if n is None:
        # Ramanujan's perimeter
        h = ((a - b) / (a + b)) ** 2
        per = math.pi * (a + b) * (1 + 3 * h / (10 + math.sqrt(4 - 3 * h)))
        n = max(8, int(round(per / ds)))
    vx, vy, _ = _equal_arc_vertices(fx, fy, n)
    return from_vertices(vx, vy, "ellipse")


def star(r0, amps, phases, n, center=(0.0, 0.0)) -> Body:
    """Star-shaped body r(th) = r0 (1 + sum_k a_k cos(k th + phi_k)),
    k = 2..(len(amps)+1), with n points equally spaced in arc length."""
    ks = np.arange(2, 2 + len(amps))

    def r(t):
        t = np.asarray(t)
        return r0 * (1.0 + np.sum(np.asarray(amps)[:, None] * np.cos(ks[:, None] * t[None, :]
                                                                        + np.asarray(phases)[:, None]), axis=0))

    vx, vy, _ = _equal_arc_vertices(lambda t: center[0] + r(t) * np.cos(t),
                                    lambda t: center[1] + r(t) * np.sin(t), n)
    return from_vertices(vx, vy, "star")


def polygon(corners, ds, name="polygon") -> Body:
    """Closed polygon through counter-clockwise corners, each side split into
    round(length/ds) equal panels."""
    corners = np.asarray(corners, dtype=np.float64)
    vx, vy = [], []
    m = corners.shape[0]
    for i in range(m):
        p, q = corners[i], corners[(i + 1) % m]
        ln = float(np.hypot(*(q - p)))
        k = max(1, int(round(ln / ds)))
        t = np.arange(k) / k
        vx.append(p[0] + t * (q[0] - p[0]))
        vy.append(p[1] + t * (q[1] - p[1]))
    return from_vertices(np.concatenate(vx), np.concatenate(vy), name)


def rectangle(a, b, ds, center=(0.0, 0.0), angle=0.0) -> Body:
    """Rectangle with half-lengths a (x) and b (y)."""
    c = np.array([[-a, -b], [a, -b], [a, b], [-a, b]])
    ca, sa = math.cos(angle), math.sin(angle)
    rot = c @ np.array([[ca, sa], [-sa, ca]])
    return polygon(rot + np.asarray(center), ds, "rectangle")


def square(a, ds, center=(0.0, 0.0)) -> Body:
    return rectangle(a, a, ds, center)


def hexagon(side, ds, center=(0.0, 0.0), angle=0.0) -> Body:
    th = angle + np.arange(6) * math.pi / 3.0
    c = np.stack([center[0] + side * np.cos(th), center[1] + side * np.sin(th)], axis=1)
    return polygon(c, ds, "hexagon")


@dataclass
class BodyList:
    """Concatenation of bodies; `firstindices` partitions surface vectors by
    body (src/cache.jl:390-391)."""
    bodies: list = field(default_factory=list)

    def append(self, b: Body):
        self.bodies.append(b)
        return self

    def _cat(self, attr):
        if not self.bodies:
            return np.zeros(0)
        return np.concatenate([getattr(b, attr) for b in self.bodies])

    @property
    def x(self):
        return self._cat("x")

    @property
    def y(self):
        return self._cat("y")

    @property
    def nx(self):
        return self._cat("nx")

    @property
    def ny(self):
        return self._cat("ny")

    @property
    def ds(self):
        return self._cat("ds")

    def __len__(self):
        return sum(len(b) for b in self.bodies)

    def firstindices(self):
        out = [0]
        for b in self.bodies:
            out.append(out[-1] + len(b))
        return np.asarray(out, dtype=np.int64)


def as_bodylist(b) -> BodyList:
    if isinstance(b, BodyList):
        return b
    return BodyList([b])
