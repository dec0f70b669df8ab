"""Seeded synthetic workloads with the shapes and value distributions of the
benchmark configurations (no external data set exists for this path).

* plain Dirichlet: [-2,2]^2, h = 0.02, circle r = 0.5 with 157 points,
  f_b = cos(theta) + 0.1 N(0,1) (numpy default_rng(1));
* batched: 256 problems, n ~ U{128,192,256,384,512} dual nodes per side,
  h = 4/n, 1-3 bodies (circles r ~ U(0.2,0.6); ellipses a ~ U(0.2,0.6),
  a/b ~ U(1,4), angle ~ U(0,pi)) at ds = 1.4 h, non-overlapping; surface data
  sum_{k=1..8} (a_k cos + b_k sin)(2 pi k s / l) with a_k, b_k ~ N(0, 1/k^2);
  even problems Dirichlet, odd problems Neumann; rng seed 3 + i.
"""
from __future__ import annotations

import math

import numpy as np

from . import bodies as B

BATCH_SIZES = (128, 192, 256, 384, 512)


def fourier_surface_data(bl, rng, nmodes=8):
    """Per body: sum of nmodes arc-length Fourier modes, N(0, 1/k^2) coefficients."""
    out = []
    for b in bl.bodies:
        s = b.arcs
        ell = float(b.ds.sum())
        f = np.zeros(len(b))
        for k in range(1, nmodes + 1):
            a, c = rng.normal(0.0, 1.0 / k, size=2)
            f += a * np.cos(2 * math.pi * k * s / ell) + c * np.sin(2 * math.pi * k * s / ell)
        out.append(f)
    return np.concatenate(out)


def random_bodies(rng, h, nbody, lim=1.25, margin_cells=6):
    """1-3 non-overlapping circles/ellipses inside [-lim, lim]^2."""
    placed = []
    bl = B.BodyList()
    tries = 0
    while len(placed) < nbody and tries < 2000:
        tries += 1
        if rng.random() < 0.5:
            r = rng.uniform(0.2, 0.6)
            a = b = r
            ang = 0.0
        else:
            a = rng.uniform(0.2, 0.6)
            b = a / rng.uniform(1.0, 4.0)
            ang = rng.uniform(0.0, math.pi)
        R = max(a, b)
        c = rng.uniform(-lim + R, lim - R, size=2)
        if any(np.hypot(*(c - q)) < R + Rq + margin_cells * h for q, Rq in placed):
            continue
        placed.append((c, R))
        if a == b:
            bl.append(B.circle(a, ds=1.4 * h, center=tuple(c)))
        else:
            bl.append(B.ellipse(a, b, ds=1.4 * h, center=tuple(c), angle=ang))
    return bl


def batch_problem(i, sizes=BATCH_SIZES):
    """Problem i of the batched configuration: (n, h, bodylist, kind, fplus)."""
    rng = np.random.default_rng(3 + i)
    n = int(sizes[rng.integers(len(sizes))])
    h = 4.0 / n
    nbody = int(rng.integers(1, 4))
    bl = random_bodies(rng, h, nbody)
    f = fourier_surface_data(bl, rng)
    kind = 0 if i % 2 == 0 else 1
    return n, h, bl, kind, f


def batch_specs(nprob=256, sizes=BATCH_SIZES):
    from .batch import BatchProblemSpec
    specs = []
    for i in range(nprob):
        n, h, bl, kind, f = batch_problem(i, sizes)
        specs.append(BatchProblemSpec(n, h, bl, kind, f))
    return specs


def dirichlet_plain():
    """Plain Dirichlet configuration: grid limits, h, body, surface data."""
    h = 0.02
    b = B.circle(0.5, n=157)
    th = np.arctan2(b.y, b.x)
    fb = np.cos(th) + 0.1 * np.random.default_rng(1).standard_normal(len(b))
    return (-2.0, 2.0), (-2.0, 2.0), h, b, fb


def _split_counts(perims, total, multiple_last=6):
    """Points per body in proportion to perimeter, summing to `total`, the
    last body's count a multiple of `multiple_last` (a hexagon's six sides)."""
    P = float(sum(perims))
    n_last = int(round(total * perims[-1] / P / multiple_last)) * multiple_last
    rest = total - n_last
    Q = float(sum(perims[:-1]))
    counts = [int(round(rest * p / Q)) for p in perims[:-1]]
    counts[-1] += rest - sum(counts)
    return counts + [n_last]


def operators_at_scale(npts=4096, seed=2, ds_factor=None):
    """Operators-at-scale / heat configuration: 1024 x 1024 dual nodes with
    h = 0.005 centred on the origin; a circle r = 0.3, an ellipse 0.4 x 0.1
    rotated by U(0, pi) and a regular hexagon of side 0.25 at non-overlapping
    centres (rejection sampling, margin >= 4h, numpy default_rng(seed)),
    `npts` points split by perimeter (ds ~ 0.25 h at 4096 points).  Heat
    data: kappa = 1, dt = 0.5 h^2, 1000 steps, T0 = exp(-r^2 / (2 0.2^2)),
    surface temperature 1 on both sides of every surface.  With `ds_factor`
    the same bodies get points ds_factor * h apart instead of `npts` in total.
    Returns dict(n, h, bodies, kappa, dt, nsteps, T0(x, y))."""
    n, h = 1024, 0.005
    rng = np.random.default_rng(seed)
    ang = float(rng.uniform(0.0, math.pi))
    a_e, b_e = 0.4, 0.1
    he = ((a_e - b_e) / (a_e + b_e)) ** 2
    per = [2 * math.pi * 0.3, math.pi * (a_e + b_e) * (1 + 3 * he / (10 + math.sqrt(4 - 3 * he))), 6 * 0.25]
    radii = [0.3, 0.4, 0.25]
    centres = []
    lim = 1.6
    while len(centres) < 3:
        c = rng.uniform(-lim + radii[len(centres)], lim - radii[len(centres)], size=2)
        if all(np.hypot(*(c - q)) >= radii[len(centres)] + rq + 4 * h for q, rq in zip(centres, radii)):
            centres.append(c)
    if ds_factor is not None:
        npts = 6 * int(round(sum(per) / (ds_factor * h) / 6))
    counts = _split_counts(per, npts)
    bl = B.BodyList()
    bl.append(B.circle(0.3, n=counts[0], center=tuple(centres[0])))
    bl.append(B.ellipse(a_e, b_e, n=counts[1], center=tuple(centres[1]), angle=ang))
    bl.append(B.hexagon(0.25, ds=per[2] / counts[2], center=tuple(centres[2])))
    assert len(bl) == npts, len(bl)

    def T0(x, y):
        return np.exp(-(x[:, None] ** 2 + y[None, :] ** 2) / (2 * 0.2 ** 2))

    return dict(n=n, h=h, bodies=bl, kappa=1.0, dt=0.5 * h * h, nsteps=1000, T0=T0)


def learned_problem(i, n=512):
    """Learned-preconditioner configuration, problem i: n x n dual nodes with
    h = 4/n, one star-shaped body r(theta) = 0.5 (1 + sum_{k=2..6} a_k
    cos(k theta + phi_k)), a_k ~ U(0, 0.08), phi_k ~ U(0, 2 pi), with
    N_p ~ U{256..1024} points equally spaced in arc length (numpy
    default_rng(i); training seeds 10^6 + j, held-out 2 10^6 + j).
    Returns (n, h, BodyList)."""
    rng = np.random.default_rng(int(i))
    amps = rng.uniform(0.0, 0.08, 5)
    phases = rng.uniform(0.0, 2 * math.pi, 5)
    npts = int(rng.integers(256, 1025))
    bl = B.BodyList()
    bl.append(B.star(0.5, amps, phases, npts))
    return n, 4.0 / n, bl


LEARNED_TRAIN_SEED = 1_000_000
LEARNED_TEST_SEED = 2_000_000


def stokes_scale(npts=8192, seed=5, nrhs=16, ds_factor=None, n=2048):
    """Stokes configuration: n x n dual nodes with h = 0.002 (n = 2048)
    centred on the origin; 2 circles r ~ U(0.1, 0.3) and 2 plates (rectangles
    of half-lengths 0.25 x h) at non-overlapping seeded centres (margin 4h),
    `npts` points split by perimeter (ds ~ 0.35 h at 8192), or points
    ds_factor * h apart; `nrhs` rigid-body surface velocity sets with
    translation and rotation rates ~ N(0, 1) per body (numpy
    default_rng(seed)).  Returns dict(n, h, bodies, vplus (nrhs x 2N))."""
    h = 0.002
    rng = np.random.default_rng(seed)
    radii = [float(rng.uniform(0.1, 0.3)), float(rng.uniform(0.1, 0.3))]
    reach = radii + [0.25, 0.25]
    centres = []
    lim = 1.5
    while len(centres) < 4:
        R = reach[len(centres)]
        c = rng.uniform(-lim + R, lim - R, size=2)
        if all(np.hypot(*(c - q)) >= R + rq + 4 * h for q, rq in zip(centres, reach)):
            centres.append(c)
    angles = rng.uniform(0.0, math.pi, 2)
    per = [2 * math.pi * radii[0], 2 * math.pi * radii[1], 4 * (0.25 + h), 4 * (0.25 + h)]
    if ds_factor is not None:
        npts = int(round(sum(per) / (ds_factor * h)))
    P = sum(per)
    counts = [max(16, int(round(npts * p / P))) for p in per]
    bl = B.BodyList()
    bl.append(B.circle(radii[0], n=counts[0], center=tuple(centres[0])))
    bl.append(B.circle(radii[1], n=counts[1], center=tuple(centres[1])))
    for k in (2, 3):
        bl.append(B.rectangle(0.25, h, ds=per[k] / counts[k], center=tuple(centres[k]), angle=float(angles[k - 2])))
    N = len(bl)
    fi = bl.firstindices()
    V = np.zeros((nrhs, 2 * N))
    for r in range(nrhs):
        for b in range(4):
            s = slice(fi[b], fi[b + 1])
            ux, uy, om = rng.standard_normal(3)
            cx, cy = centres[b]
            V[r, s] = ux - om * (bl.y[s] - cy)
            V[r, N + fi[b]:N + fi[b + 1]] = uy + om * (bl.x[s] - cx)
    return dict(n=n, h=h, bodies=bl, vplus=V)
