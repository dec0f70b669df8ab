"""Problem / system framework: the `@ilmproblem`, `construct_system`,
`prob_cache` and `solve` layer of ImmersedLayers.jl (src/problem.jl:58-139,
src/system.jl:18-82), with the Dirichlet and Neumann Poisson problems of the
reference's literate tests (test/literate/problems.jl:43-298,
test/literate/neumann.jl:70-142) solved on the device by libilm.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib as L
from .bodies import as_bodylist
from .core import (GridScaling, NodesPrimal, PointData, ScalarData, SurfaceScalarCache, SurfaceVectorCache,
                   VectorData, _ptr, _stream_ptr, zeros_grid, zeros_surface)


@dataclass
class ILMProblem:
    """Problem specification (the constructor `@ilmproblem` generates)."""
    g: object
    bodies: object
    scaling: str = GridScaling
    ddftype: str = "Yang3"
    dtype: torch.dtype = torch.float64
    bc: dict = field(default_factory=dict)
    phys_params: dict = field(default_factory=dict)
    forcing: object = None
    timestep_func: object = None
    motions: object = None
    datatype = "scalar"


class DirichletPoissonProblem(ILMProblem):
    datatype = "scalar"


class NeumannPoissonProblem(ILMProblem):
    datatype = "scalar"


class StokesFlowProblem(ILMProblem):
    """`@ilmproblem StokesFlow vector` (test/literate/stokes.jl:52)."""
    datatype = "vector"


@dataclass
class ILMSystem:
    """`ILMSystem`: base cache + problem extra cache (src/ImmersedLayers.jl:100-110)."""
    base_cache: object
    extra_cache: object
    bc: dict
    phys_params: dict
    forcing: object
    motions: object
    timestep_func: object
    last_info: dict = field(default_factory=dict)


def prob_cache(prob, base_cache):
    """Extension point (src/problem.jl:129-139); the built-in problems need no
    extra cache: their Schur complements live inside the libilm cache."""
    return None


def construct_system(prob: ILMProblem) -> ILMSystem:
    mk = SurfaceScalarCache if prob.datatype == "scalar" else SurfaceVectorCache
    base = mk(prob.bodies, prob.g, ddftype=prob.ddftype, scaling=prob.scaling, dtype=prob.dtype)
    return ILMSystem(base, prob_cache(prob, base), prob.bc, prob.phys_params, prob.forcing, prob.motions,
                     prob.timestep_func)


def update_system_(sys: ILMSystem, bodies, stream=None) -> ILMSystem:
    """update_system!(sys, u, sysold, t) / update_system(sysold, bodies)
    (src/system.jl:26-49): the system for a new configuration of its bodies.
    The reference regenerates the problem and rebuilds every cache; here the
    base cache re-bins the new points on the device (same point count)."""
    bl = as_bodylist(bodies)
    sys.base_cache.update_points_(bl.x, bl.y, bl.nx, bl.ny, bl.ds, stream=stream)
    sys.base_cache.bl = bl
    return sys


def _as_point(v, like: PointData):
    if isinstance(v, PointData):
        return v.data
    t = torch.as_tensor(np.asarray(v) if not torch.is_tensor(v) else v, dtype=like.data.dtype)
    return t.to(like.data.device).reshape(-1)


def prescribed_surface_jump_(dfb: PointData, sys: ILMSystem):
    """dfb = bc["exterior"] - bc["interior"] (src/bc.jl:14-34)."""
    if sys.base_cache.N == 0:
        dfb.data.zero_()
        return dfb
    ext = _as_point(sys.bc["exterior"](sys.base_cache, sys.phys_params), dfb)
    itr = _as_point(sys.bc["interior"](sys.base_cache, sys.phys_params), dfb)
    dfb.data.copy_(ext - itr)
    return dfb


def prescribed_surface_average_(fb: PointData, sys: ILMSystem):
    """fb = (bc["exterior"] + bc["interior"]) / 2 (src/bc.jl:36-56)."""
    if sys.base_cache.N == 0:
        fb.data.zero_()
        return fb
    ext = _as_point(sys.bc["exterior"](sys.base_cache, sys.phys_params), fb)
    itr = _as_point(sys.bc["interior"](sys.base_cache, sys.phys_params), fb)
    fb.data.copy_(0.5 * (ext + itr))
    return fb


def _sides(sys):
    c = sys.base_cache
    plus = zeros_surface(c)
    minus = zeros_surface(c)
    if c.N:
        plus.data.copy_(_as_point(sys.bc["exterior"](c, sys.phys_params), plus))
        minus.data.copy_(_as_point(sys.bc["interior"](c, sys.phys_params), minus))
    return plus, minus


def solve_dirichlet(cache, fplus: PointData, fminus: PointData, tol=1e-8, maxiter=5000, stream=None):
    """Device Dirichlet solve; returns (f::Nodes{Primal}, s::ScalarData, info)."""
    f = zeros_grid(cache)
    s = zeros_surface(cache)
    info = L.SolveInfo()
    L.call("ilm_solve_dirichlet", cache._h, _ptr(fplus.data), _ptr(fminus.data), _ptr(f.data), _ptr(s.data),
           float(tol), int(maxiter), C.byref(info), _stream_ptr(stream))
    return f, s, dict(iterations=info.iterations, converged=bool(info.converged), rel_residual=info.rel_residual)


def solve_neumann(cache, vplus: PointData, vminus: PointData, tol=1e-8, maxiter=5000, stream=None):
    """Device Neumann solve; returns (f::Nodes{Primal}, df::ScalarData, info)."""
    f = zeros_grid(cache)
    df = zeros_surface(cache)
    info = L.SolveInfo()
    L.call("ilm_solve_neumann", cache._h, _ptr(vplus.data), _ptr(vminus.data), _ptr(f.data), _ptr(df.data),
           float(tol), int(maxiter), C.byref(info), _stream_ptr(stream))
    return f, df, dict(iterations=info.iterations, converged=bool(info.converged), rel_residual=info.rel_residual)


def _refined(name, cache, plus, minus, tol, maxiter, max_refine, stream):
    N = plus.data.numel()
    f = NodesPrimal.zeros(cache.g, torch.float64)
    s = ScalarData(torch.zeros(N, dtype=torch.float64, device=plus.data.device))
    p64 = plus.data.to(torch.float64).contiguous()
    m64 = minus.data.to(torch.float64).contiguous()
    info = L.SolveInfo()
    L.call(name, cache._h, _ptr(p64), _ptr(m64), _ptr(f.data), _ptr(s.data), float(tol), int(maxiter),
           int(max_refine), C.byref(info), _stream_ptr(stream))
    return f, s, dict(iterations=info.iterations, converged=bool(info.converged), rel_residual=info.rel_residual)


def solve_dirichlet_refined(cache, fplus: PointData, fminus: PointData, tol=1e-12, maxiter=20000, max_refine=8,
                            stream=None):
    """Dirichlet solve with FP64 iterative refinement (FP64 outputs for any
    cache dtype): the cache's own solve, then FP64 Schur residuals and CG
    corrections until ||b - S s|| / ||b|| <= tol; f assembled in FP64.
    Returns (f::Nodes{Primal} FP64, s::ScalarData FP64, info)."""
    return _refined("ilm_solve_dirichlet_refined", cache, fplus, fminus, tol, maxiter, max_refine, stream)


def solve_neumann_refined(cache, vplus: PointData, vminus: PointData, tol=1e-12, maxiter=20000, max_refine=8,
                          stream=None):
    """Neumann solve (f and [phi]) with FP64 iterative refinement; see
    solve_dirichlet_refined."""
    return _refined("ilm_solve_neumann_refined", cache, vplus, vminus, tol, maxiter, max_refine, stream)


def solve_neumann_full(cache, vplus: PointData, vminus: PointData, tol=1e-8, maxiter=5000, stream=None):
    """The literate NeumannPoissonProblem solve (test/literate/neumann.jl:101-142)
    on the device: returns (f::Nodes{Primal}, df::ScalarData,
    s::Nodes{Dual} streamfunction, ds::ScalarData, info)."""
    from .core import zeros_gridcurl
    f = zeros_grid(cache)
    df = zeros_surface(cache)
    s = zeros_gridcurl(cache)
    ds = zeros_surface(cache)
    info = L.SolveInfo()
    L.call("ilm_solve_neumann_full", cache._h, _ptr(vplus.data), _ptr(vminus.data), _ptr(f.data), _ptr(df.data),
           _ptr(s.data), _ptr(ds.data), float(tol), int(maxiter), C.byref(info), _stream_ptr(stream))
    return f, df, s, ds, dict(iterations=info.iterations, converged=bool(info.converged),
                              rel_residual=info.rel_residual)


def solve_stokes(cache, vplus: PointData, vminus: PointData, tol=1e-8, maxiter=5000, stream=None):
    """Device Stokes solve (vector cache); returns (v::Edges{Primal},
    s::Nodes{Dual}, sigma::VectorData, info)."""
    from .core import zeros_gridcurl
    v = zeros_grid(cache)
    s = zeros_gridcurl(cache)
    sigma = zeros_surface(cache)
    info = L.SolveInfo()
    L.call("ilm_solve_stokes", cache._h, _ptr(vplus.data), _ptr(vminus.data), _ptr(v.data), _ptr(s.data),
           _ptr(sigma.data), float(tol), int(maxiter), C.byref(info), _stream_ptr(stream))
    return v, s, sigma, dict(iterations=info.iterations, converged=bool(info.converged),
                             rel_residual=info.rel_residual)


def solve_stokes_multi(cache, vplus: torch.Tensor, vminus: torch.Tensor = None, tol=1e-8, maxiter=5000,
                       precond=True, stream=None):
    """Stokes solves for several velocity right-hand sides at once
    (stokes.jl:138,156 with one S for every surface velocity).  vplus /
    vminus: (nrhs, 2N) tensors of VectorData rows in the cache dtype
    (vminus None: zeros).  Both Schur systems are solved by block CG over
    the right-hand sides; `precond` preconditions S with the inverse of the
    gauge-shifted point-point Schur complement -E L^-1 E^T per velocity
    component.  Returns (v: nrhs Edges{Primal}, s: nrhs Nodes{Dual},
    sigma: nrhs VectorData, infos: one dict per right-hand side)."""
    from .core import zeros_gridcurl
    if vplus.dim() != 2 or vplus.shape[1] != 2 * len(cache):
        raise ValueError(f"vplus must be (nrhs, {2 * len(cache)})")
    nrhs = vplus.shape[0]
    if not 1 <= nrhs <= L.STOKES_MAX_RHS:
        raise ValueError(f"nrhs must be in 1..{L.STOKES_MAX_RHS}")
    vplus = vplus.contiguous()
    vminus = torch.zeros_like(vplus) if vminus is None else vminus.contiguous()
    vs = [zeros_grid(cache) for _ in range(nrhs)]
    ss = [zeros_gridcurl(cache) for _ in range(nrhs)]
    v_all = torch.empty((nrhs,) + tuple(vs[0].data.shape), dtype=vs[0].data.dtype, device=vs[0].data.device)
    s_all = torch.empty((nrhs,) + tuple(ss[0].data.shape), dtype=ss[0].data.dtype, device=ss[0].data.device)
    sig_all = torch.empty_like(vplus)
    infos = (L.SolveInfo * nrhs)()
    L.call("ilm_solve_stokes_multi", cache._h, nrhs, _ptr(vplus), _ptr(vminus), _ptr(v_all), _ptr(s_all),
           _ptr(sig_all), float(tol), int(maxiter), 1 if precond else 0, infos, _stream_ptr(stream))
    sig = []
    for r in range(nrhs):
        vs[r].data.copy_(v_all[r])
        ss[r].data.copy_(s_all[r])
        sig.append(VectorData(sig_all[r].clone()))
    return vs, ss, sig, [dict(iterations=i.iterations, converged=bool(i.converged), rel_residual=i.rel_residual)
                         for i in infos]


def solve_stokes_multi_refined(cache, vplus: torch.Tensor, vminus: torch.Tensor = None, tol=1e-10, maxiter=2000,
                               max_refine=8, stream=None):
    """Stokes solves for several right-hand sides with FP64 iterative
    refinement (FP64 outputs for any cache dtype): FP64 pre-step, residuals
    and fields on an FP64 cache of the same points, corrections by block CG
    with the cache's own operator.  vplus / vminus: (nrhs, 2N) tensors
    (converted to FP64).  Returns (v: nrhs Edges{Primal} FP64, s: nrhs
    Nodes{Dual} FP64, sigma: nrhs VectorData FP64, infos)."""
    from .core import EdgesPrimal, NodesDual
    if vplus.dim() != 2 or vplus.shape[1] != 2 * len(cache):
        raise ValueError(f"vplus must be (nrhs, {2 * len(cache)})")
    nrhs = vplus.shape[0]
    if not 1 <= nrhs <= L.STOKES_MAX_RHS:
        raise ValueError(f"nrhs must be in 1..{L.STOKES_MAX_RHS}")
    p64 = vplus.to(torch.float64).contiguous()
    m64 = torch.zeros_like(p64) if vminus is None else vminus.to(torch.float64).contiguous()
    vs = [EdgesPrimal.zeros(cache.g, torch.float64) for _ in range(nrhs)]
    ss = [NodesDual.zeros(cache.g, torch.float64) for _ in range(nrhs)]
    v_all = torch.empty((nrhs,) + tuple(vs[0].data.shape), dtype=torch.float64, device=p64.device)
    s_all = torch.empty((nrhs,) + tuple(ss[0].data.shape), dtype=torch.float64, device=p64.device)
    sig_all = torch.empty_like(p64)
    infos = (L.SolveInfo * nrhs)()
    L.call("ilm_solve_stokes_multi_refined", cache._h, nrhs, _ptr(p64), _ptr(m64), _ptr(v_all), _ptr(s_all),
           _ptr(sig_all), float(tol), int(maxiter), int(max_refine), infos, _stream_ptr(stream))
    sig = []
    for r in range(nrhs):
        vs[r].data.copy_(v_all[r])
        ss[r].data.copy_(s_all[r])
        sig.append(VectorData(sig_all[r].clone()))
    return vs, ss, sig, [dict(iterations=i.iterations, converged=bool(i.converged), rel_residual=i.rel_residual)
                         for i in infos]


def solve(prob: ILMProblem, sys: ILMSystem, tol=1e-8, maxiter=5000, filter_power=0):
    """`solve(prob, sys)` for the built-in problems (bc from `prob.bc`):
    Dirichlet (f, s), Neumann (f, df, s, ds) as test/literate/neumann.jl:140,
    Stokes (v, s, sigma).
    filter_power=k returns the Dirichlet surface data filtered k times,
    C^k s with C = create_surface_filter(base_cache) (the literate
    DirichletPoissonProblem returns C^6 s, test/literate/problems.jl:297)."""
    plus, minus = _sides(sys)
    if isinstance(prob, DirichletPoissonProblem):
        f, s, info = solve_dirichlet(sys.base_cache, plus, minus, tol, maxiter)
        if filter_power:
            from .core import SurfaceFilter
            SurfaceFilter(sys.base_cache, filter_power).apply_(s, s)
    elif isinstance(prob, NeumannPoissonProblem):
        f, df, s, ds, info = solve_neumann_full(sys.base_cache, plus, minus, tol, maxiter)
        sys.last_info = info
        return f, df, s, ds
    elif isinstance(prob, StokesFlowProblem):
        v, s, sigma, info = solve_stokes(sys.base_cache, plus, minus, tol, maxiter)
        sys.last_info = info
        return v, s, sigma
    else:
        raise NotImplementedError(type(prob).__name__)
    sys.last_info = info
    return f, s
