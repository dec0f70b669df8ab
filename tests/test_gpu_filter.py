"""Surface filter C = E~ R (create_surface_filter,
src/matrix_operators.jl:254-268) and its powers (C^6 s,
test/literate/problems.jl:107,297) on the device against the oracle's
dense filter matrices, for scalar and vector caches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import ilm_oracle as O
from geometry import oracle_cache


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max()


def _bodies(h):
    from immersedlayers import bodies as B
    bl = B.BodyList()
    bl.append(B.circle(0.5, ds=1.4 * h))
    bl.append(B.rectangle(0.4, 0.2, ds=1.4 * h, center=(0.3, 1.0)))
    return bl


@pytest.mark.parametrize("dtype,ddf", [("f64", "Yang3"), ("f32", "Yang3"), ("f64", "Roma")])
def test_scalar_filter_matches_oracle(cuda, dtype, ddf):
    import torch
    import immersedlayers as il
    dt = torch.float64 if dtype == "f64" else torch.float32
    h = 0.04
    og = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    bl = _bodies(h)
    c = il.SurfaceScalarCache(bl, g, ddftype=ddf, dtype=dt)
    oc = oracle_cache(og, bl, kind="scalar", ddf=ddf)
    rng = np.random.default_rng(3)
    s_h = np.cos(3 * np.arctan2(bl.y, bl.x)) + 0.3 * rng.standard_normal(len(bl))
    s = il.ScalarData(torch.tensor(s_h, dtype=dt, device="cuda"))
    C = il.create_surface_filter(c)
    tol = 1e-12 if dtype == "f64" else 2e-5
    for k in (1, 2, 6):
        got = ((C ** k) @ s).data.double().cpu().numpy()
        ref = O.surface_filter(oc, s_h, power=k)
        assert rel(got, ref) < tol, (k, rel(got, ref))
    # constants pass unchanged; the filter smooths (smaller spread than s)
    one = il.ones_surface(c)
    assert (C @ one).data.sub(1).abs().max().item() < (1e-13 if dtype == "f64" else 1e-6)
    f6 = ((C ** 6) @ s).data.double().cpu().numpy()
    assert np.std(np.diff(f6)) < np.std(np.diff(s_h))
    # in place, and power 0 copies
    t = il.ScalarData(s.data.clone())
    (C ** 6).apply_(t, t)
    assert torch.equal(t.data, (C ** 6 @ s).data)
    assert torch.equal((C ** 0 @ s).data, s.data)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_vector_filter_matches_oracle(cuda, dtype):
    import torch
    import immersedlayers as il
    dt = torch.float64 if dtype == "f64" else torch.float32
    h = 0.04
    og = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    bl = _bodies(h)
    c = il.SurfaceVectorCache(bl, g, dtype=dt)
    oc = oracle_cache(og, bl, kind="vector")
    rng = np.random.default_rng(4)
    v_h = rng.standard_normal(2 * len(bl))
    v = il.VectorData(torch.tensor(v_h, dtype=dt, device="cuda"))
    got = ((il.create_surface_filter(c) ** 2) @ v).data.double().cpu().numpy()
    ref = O.surface_filter(oc, v_h, power=2, vector=True)
    assert rel(got, ref) < (1e-12 if dtype == "f64" else 2e-5), rel(got, ref)


def test_filter_follows_moving_points(cuda):
    """After ilm_cache_update_points the filter uses the new points (its
    row weights W are formed again): equal to a fresh cache's filter."""
    import torch
    import immersedlayers as il
    from immersedlayers import bodies as B
    h = 0.04
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    b0 = B.circle(0.5, ds=1.4 * h)
    c = il.SurfaceScalarCache(b0, g)
    s = il.ScalarData(torch.linspace(-1, 1, len(b0), dtype=torch.float64, device="cuda"))
    C = il.create_surface_filter(c)
    _ = C @ s
    b1 = B.circle(0.5, ds=1.4 * h, center=(0.31, -0.17))
    c.update_points_(b1.x, b1.y, b1.nx, b1.ny, b1.ds)
    fresh = il.SurfaceScalarCache(b1, g)
    got = (C @ s).data
    ref = (il.create_surface_filter(fresh) @ s).data
    assert (got - ref).abs().max().item() < 1e-13


def test_dirichlet_solve_filtered(cuda):
    """solve(prob, sys, filter_power=6): the literate Dirichlet problem's
    returned surface data C^6 s (test/literate/problems.jl:297)."""
    import torch
    import immersedlayers as il
    from geometry import dirichlet_config1
    og, b, fb = dirichlet_config1()
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)
    c = il.SurfaceScalarCache(b, g)
    p = il.ScalarData(torch.tensor(fb, dtype=torch.float64, device="cuda"))
    m = il.ScalarData(torch.zeros_like(p.data))
    f, s, info = il.solve_dirichlet(c, p, m, tol=1e-11, maxiter=20000)
    oc = oracle_cache(og, b, kind="scalar")
    fr, sr = O.solve_dirichlet(oc, fb, np.zeros_like(fb))
    s6 = ((il.create_surface_filter(c) ** 6) @ s).data.cpu().numpy()
    assert rel(s6, O.surface_filter(oc, sr, power=6)) < 1e-7
