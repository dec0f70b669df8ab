"""Time marching of constrained problems: the `init_sol` / `timestep` /
`init(u0, tspan, sys)` / `step!(integrator, dt)` layer of ImmersedLayers.jl
(src/timemarching.jl:143-277) for the Dirichlet heat-conduction problem of
test/literate/heatconduction.jl:66-189.

The reference hands its ODE pieces (heatconduction_ode_rhs!,
heatconduction_bc_rhs!, heatconduction_constraint_force!,
heatconduction_bc_op!) to ConstrainedSystems' LiskaIFHERK.  Here the same
system -- dT/dt = kappa L T - kappa D_s[T_b+ - T_b-] - R sigma with
E T = (T_b+ + T_b-)/2 -- is advanced by libilm's device integrator
(ilm_heat_*): IF-HERK scheme A with the exact lattice integrating factor,
sparse stage Schur complements and warm-started device CG.  A step issues
no host<->device copies of the state.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L
from .core import GridScaling, PointData, _ptr, _stream_ptr, zeros_grid, zeros_surface
from .problems import ILMProblem, ILMSystem


class DirichletHeatConductionProblem(ILMProblem):
    """`@ilmproblem DirichletHeatConduction scalar`: phys_params holds
    "diffusivity" (and "Fourier" for `timestep_fourier`); bc holds the
    "exterior" / "interior" surface temperatures as
    f(t, x, cache, phys_params, motions) (or f(cache, phys_params))."""
    datatype = "scalar"


@dataclass
class ConstrainedSolution:
    """Solution vector with a state (grid temperature) and a constraint
    (surface Lagrange multipliers) part."""
    state: object
    constraint: object


def state(u: ConstrainedSolution):
    return u.state


def constraint(u: ConstrainedSolution):
    return u.constraint


def init_sol(sys: ILMSystem, s=None) -> ConstrainedSolution:
    """Zeroed solution prototype (src/timemarching.jl:148-163); with `s`, the
    state starts as a copy of that grid field."""
    T = zeros_grid(sys.base_cache)
    if s is not None:
        T.data.copy_(s.data if hasattr(s, "data") else torch.as_tensor(s, dtype=T.data.dtype).reshape(-1))
    return ConstrainedSolution(T, zeros_surface(sys.base_cache))


def timestep_fourier(u, sys: ILMSystem) -> float:
    """dt = Fo h^2 / kappa (test/literate/heatconduction.jl:178-185)."""
    kappa = sys.phys_params["diffusivity"]
    return sys.phys_params["Fourier"] * sys.base_cache.g.h ** 2 / kappa


def timestep(u, sys: ILMSystem) -> float:
    return sys.timestep_func(u, sys)


def _bc_values(sys: ILMSystem, side: str, t: float):
    fn = sys.bc[side]
    c = sys.base_cache
    try:
        v = fn(t, None, c, sys.phys_params, sys.motions)
    except TypeError:
        v = fn(c, sys.phys_params)
    if isinstance(v, PointData):
        v = v.data
    if torch.is_tensor(v):
        v = v.detach().cpu().numpy()
    return np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (c.N,)))


class HeatIntegrator:
    """Integrator returned by `init`: `u` (state + constraint), `t`, `dt`,
    `step_(dt_advance)`; the surface temperatures are sampled at creation
    (stationary data, as in the reference example)."""

    def __init__(self, u0: ConstrainedSolution, tspan, sys: ILMSystem, dt=None, tol=1e-10, maxiter=2000,
                 stream=None):
        c = sys.base_cache
        if c.scaling != GridScaling:
            raise ValueError("heat conduction requires a GridScaling cache")
        self.sys = sys
        self.u = ConstrainedSolution(zeros_grid(c), zeros_surface(c))
        self.u.state.data.copy_(u0.state.data)
        self.t = float(tspan[0])
        self.tspan = (float(tspan[0]), float(tspan[1]))
        self.dt = float(dt if dt is not None else timestep(u0, sys))
        self.stream = stream
        tp = _bc_values(sys, "exterior", self.t)
        tm = _bc_values(sys, "interior", self.t)
        h = C.c_void_p()
        L.call("ilm_heat_create", c._h, float(sys.phys_params["diffusivity"]), self.dt,
               tp.ctypes.data_as(C.POINTER(C.c_double)), tm.ctypes.data_as(C.POINTER(C.c_double)), float(tol),
               int(maxiter), C.byref(h))
        self._h = h

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                L.load().ilm_heat_destroy(self._h)
        except Exception:
            pass

    def advance(self, nsteps: int):
        """Take `nsteps` steps of size dt."""
        L.call("ilm_heat_advance", self._h, _ptr(self.u.state.data), _ptr(self.u.constraint.data), int(nsteps),
               _stream_ptr(self.stream))
        self.t += nsteps * self.dt
        return self

    def step_(self, dt_advance=None):
        """`step!(integrator[, dt])`: one step, or as many whole steps as fit
        in `dt_advance` (at least one)."""
        n = 1 if dt_advance is None else max(1, int(round(dt_advance / self.dt)))
        return self.advance(n)

    def info(self):
        it = (C.c_int * 3)()
        rr = (C.c_double * 3)()
        nnz = (C.c_size_t * 4)()
        L.call("ilm_heat_info", self._h, it, rr, nnz)
        return dict(iterations=list(it), rel_residual=list(rr), nnz=list(nnz))


def init(u0: ConstrainedSolution, tspan, sys: ILMSystem, **kw) -> HeatIntegrator:
    """`init(u0, tspan, sys)` (src/timemarching.jl:254-259)."""
    return HeatIntegrator(u0, tspan, sys, **kw)


def step_(integrator: HeatIntegrator, dt_advance=None) -> HeatIntegrator:
    return integrator.step_(dt_advance)


def temperature(integrator_or_u):
    u = integrator_or_u.u if isinstance(integrator_or_u, HeatIntegrator) else integrator_or_u
    return u.state
