"""Moving bodies: a cache whose points are replaced on the device
(ilm_cache_update_points, the update_system / update_system! path of
src/system.jl:26-49) gives the transfers and solves of a cache built from
scratch at the new positions."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _moved(bl, dx, dy, theta):
    """A rigid motion of a body list: rotation by theta about the origin,
    then a translation."""
    c, s = math.cos(theta), math.sin(theta)
    x = c * bl.x - s * bl.y + dx
    y = s * bl.x + c * bl.y + dy
    nx = c * bl.nx - s * bl.ny
    ny = s * bl.nx + c * bl.ny
    return x, y, nx, ny, bl.ds.copy()


@pytest.mark.parametrize("dtype,ddf", [("f64", "Yang3"), ("f32", "Yang3"), ("f64", "Roma")])
def test_update_points_matches_fresh_cache(cuda, dtype, ddf):
    import torch
    import immersedlayers as il
    from immersedlayers import bodies as B
    dt = torch.float64 if dtype == "f64" else torch.float32
    h = 0.02
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    bl = B.BodyList()
    bl.append(B.ellipse(0.5, 0.2, ds=1.4 * h))
    bl.append(B.circle(0.3, ds=1.4 * h))
    moving = il.SurfaceScalarCache(bl, g, ddftype=ddf, dtype=dt)
    rng = np.random.default_rng(11)
    f = il.ScalarData(torch.tensor(rng.standard_normal(len(bl)), dtype=dt, device="cuda"))
    for step in range(3):
        x, y, nx, ny, ds = _moved(bl, 0.07 * (step + 1), -0.05 * step, 0.3 * (step + 1))
        moving.update_points_(x, y, nx, ny, ds)
        fresh = il.SurfaceScalarCache(B.Body(x, y, nx, ny, ds), g, ddftype=ddf, dtype=dt)
        for make, op in [(il.zeros_grid, il.regularize_)]:
            a = op(make(moving), f, moving)
            b = op(make(fresh), f, fresh)
            torch.cuda.synchronize()
            err = ((a.data - b.data).abs().max() / b.data.abs().max()).item()
            assert err < (1e-13 if dt == torch.float64 else 1e-6), (step, err)
        # gather and the double layer (normals) on the new geometry
        w = il.zeros_grid(fresh)
        w.data.normal_()
        ga = il.interpolate_(il.zeros_surface(moving), w, moving)
        gb = il.interpolate_(il.zeros_surface(fresh), w, fresh)
        assert ((ga.data - gb.data).abs().max() / gb.data.abs().max()).item() < (1e-13 if dt == torch.float64 else 1e-6)
        da = il.surface_divergence_(il.zeros_grid(moving), f, moving)
        db = il.surface_divergence_(il.zeros_grid(fresh), f, fresh)
        assert ((da.data - db.data).abs().max() / db.data.abs().max()).item() < (1e-12 if dt == torch.float64 else 1e-5)


def test_update_system_solve(cuda):
    """A Dirichlet solve after update_system_ (cached Schur complement
    invalidated and rebuilt) equals the solve on a fresh system."""
    import torch
    import immersedlayers as il
    from immersedlayers import bodies as B
    h = 0.04
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    bl = B.BodyList()
    bl.append(B.circle(0.6, ds=1.4 * h))
    c = il.SurfaceScalarCache(bl, g)
    fp = il.ScalarData(torch.tensor(np.cos(np.arctan2(bl.y, bl.x)), device="cuda"))
    fm = il.ScalarData.zeros(len(bl))
    il.solve_dirichlet(c, fp, fm, tol=1e-10)       # builds and caches S for the first position
    x, y, nx, ny, ds = _moved(bl, 0.3, 0.1, 0.0)
    sysd = il.construct_system(il.DirichletPoissonProblem(g, bl))
    il.update_system_(sysd, B.Body(x, y, nx, ny, ds))
    c.update_points_(x, y, nx, ny, ds)
    f1, s1, info1 = il.solve_dirichlet(c, fp, fm, tol=1e-10)
    fresh = il.SurfaceScalarCache(B.Body(x, y, nx, ny, ds), g)
    f2, s2, info2 = il.solve_dirichlet(fresh, fp, fm, tol=1e-10)
    assert info1["converged"] and info2["converged"]
    err = ((f1.data - f2.data).abs().max() / f2.data.abs().max()).item()
    assert err < 1e-9, err
    f3, s3, info3 = il.solve_dirichlet(sysd.base_cache, fp, fm, tol=1e-10)
    assert ((f3.data - f2.data).abs().max() / f2.data.abs().max()).item() < 1e-9
