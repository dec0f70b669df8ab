"""Timing of the reference's CPU algorithm for the batched Poisson workload --
TEST / MEASUREMENT INFRASTRUCTURE ONLY (the cpu_baseline and --impl reference
legs of bench.py).

Per problem the reference (test/literate/problems.jl:243-298 and
test/literate/neumann.jl:79-127) builds its Schur complement with one
operator application per surface point (create_RTLinvR / create_CLinvCT,
src/matrix_operators.jl:9-61: regularize!, FFT inverse Laplacian, interpolate!
per column) and then solves with a dense LU plus two grid inverse Laplacians.
This module times that algorithm, restated in NumPy/SciPy FP64 with
scipy.fft on all host cores (FFTW's role in the reference), on a bounded
sample: for every sampled problem `k_cols` Schur columns are timed and scaled
by npts / k_cols; the rest of the solve is timed in full.
"""
from __future__ import annotations

import os
import time

import numpy as np

import ilm_oracle as O


def _problem_cost(spec, k_cols):
    g = O.Grid(spec.nx, spec.ny, spec.h, *spec.i0)
    bl = spec.bl
    t0 = time.perf_counter()
    c = O.SurfaceCache(bl.x, bl.y, bl.nx, bl.ny, bl.ds, g)
    for cls_ in (O.NODES_PRIMAL, O.NODES_DUAL, O.EDGES_PRIMAL_U, O.EDGES_PRIMAL_V):
        c.phi(cls_)
    t_setup = time.perf_counter() - t0
    # the per-grid-size LGF table and spectrum are built once per size and
    # excluded, as for the device path
    c.inverse_laplacian(np.zeros(g.shape(O.NODES_PRIMAL)))
    c.inverse_laplacian(np.zeros(g.shape(O.NODES_DUAL)))
    N = c.N
    k = min(k_cols, N)
    e = np.zeros(N)
    t0 = time.perf_counter()
    cols = np.empty((N, k))
    for col in range(k):
        e[:] = 0.0
        e[col] = 1.0
        if spec.kind == 0:
            w = c.inverse_laplacian(O.regularize_scalar(c, e))
            cols[:, col] = -O.interpolate_scalar(c, w)
        else:
            w = c.inverse_laplacian(O.surface_curl_T(c, e))
            cols[:, col] = -O.surface_curl(c, w)
    t_cols = (time.perf_counter() - t0) * N / k
    # the rest of the solve, with a stand-in dense S of the right size for the LU
    S = np.eye(N) + 1e-3 * np.random.default_rng(0).standard_normal((N, N))
    t0 = time.perf_counter()
    if spec.kind == 0:
        fstar = c.inverse_laplacian(O.surface_divergence(c, spec.fplus - spec.fminus))
        s = 0.5 * (spec.fplus + spec.fminus) - O.interpolate_scalar(c, fstar)
        s = -np.linalg.solve(S, s)
        c.inverse_laplacian(O.regularize_scalar(c, s))
    else:
        fstar = c.inverse_laplacian(O.regularize_scalar(c, spec.fplus - spec.fminus))
        df = 0.5 * (spec.fplus + spec.fminus) - O.surface_grad(c, fstar)
        df = -np.linalg.solve(S, df)
        c.inverse_laplacian(O.surface_divergence(c, df))
    t_solve = time.perf_counter() - t0
    return dict(npts=N, n=spec.nx, kind=spec.kind, setup=t_setup, schur=t_cols, solve=t_solve,
                total=t_setup + t_cols + t_solve)


def sample_indices(specs, per_size=1):
    """Sample `per_size` problems of each grid size, first in batch order."""
    seen = {}
    out = []
    for i, s in enumerate(specs):
        if seen.get(s.nx, 0) < per_size:
            seen[s.nx] = seen.get(s.nx, 0) + 1
            out.append(i)
    return out


def estimate_batch_time(specs, per_size=2, k_cols=32):
    """Estimated seconds for the reference algorithm on the whole batch.

    Each problem is charged the measured cost of a sampled problem of the same
    grid size, with its Schur-column part scaled by the ratio of point counts.
    """
    idx = sample_indices(specs, per_size)
    t0 = time.perf_counter()
    costs = [(_problem_cost(specs[i], k_cols), i) for i in idx]
    wall = time.perf_counter() - t0
    by_n = {}
    for cst, i in costs:
        by_n.setdefault(specs[i].nx, []).append(cst)
    total = 0.0
    for s in specs:
        cs = by_n[s.nx]
        per_col = np.mean([c["schur"] / c["npts"] for c in cs])
        rest = np.mean([c["setup"] + c["solve"] for c in cs])
        total += per_col * s.npts + rest
    return dict(batch_seconds=total, sample=[i for _, i in costs], sample_wall=wall,
                k_cols=k_cols, cores=os.cpu_count(), details=[c for c, _ in costs])
