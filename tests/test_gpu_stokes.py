"""Stokes flow (test/literate/stokes.jl:101-166) on the device against the
oracle's dense block-LU solve: velocity, streamfunction, filtered traction,
and the no-slip condition."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import ilm_oracle as O
from geometry import oracle_cache


def rel(a, b):
    a = np.concatenate([np.ravel(x) for x in a]) if isinstance(a, tuple) else np.ravel(a)
    b = np.concatenate([np.ravel(x) for x in b]) if isinstance(b, tuple) else np.ravel(b)
    return np.abs(a - b).max() / np.abs(b).max()


def _case(two_bodies=False):
    from immersedlayers import bodies as B
    h = 0.04
    og = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    bl = B.BodyList()
    bl.append(B.rectangle(0.5, 0.25, ds=1.4 * h))          # the reference example's body
    if two_bodies:
        bl.append(B.circle(0.3, ds=1.4 * h, center=(0.2, 1.1)))
    return og, bl


@pytest.mark.parametrize("two_bodies", [False, True])
def test_stokes_matches_oracle(cuda, two_bodies):
    import torch
    import immersedlayers as il
    og, bl = _case(two_bodies)
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)
    c = il.SurfaceVectorCache(bl, g, dtype=torch.float64)
    N = len(bl)
    vp_h = np.concatenate([np.ones(N), np.zeros(N)])      # translate right at unit speed
    if two_bodies:
        vp_h[N - len(bl.bodies[1]):N] = 0.0
        vp_h[2 * N - len(bl.bodies[1]):] = 0.5                # second body moves up
    vp = il.VectorData(torch.tensor(vp_h, device="cuda"))
    vm = il.VectorData.zeros(N)
    v, s, sigma, info = il.solve_stokes(c, vp, vm, tol=1e-11, maxiter=20000)
    assert info["converged"], info
    oc = oracle_cache(og, bl, kind="vector")
    v_ref, s_ref, sig_ref = O.solve_stokes(oc, vp_h, np.zeros(2 * N))
    assert rel(v.numpy_components(), v_ref) < 1e-7
    assert rel(s.numpy_components(), s_ref) < 1e-7
    assert rel(sigma.numpy(), sig_ref) < 1e-4     # sigma inherits cond(S) ~ 1e6
    # no slip: E v equals the average surface velocity
    vi = O.interpolate_vector(oc, v.numpy_components())
    assert np.abs(vi - 0.5 * vp_h).max() < 1e-8


def test_stokes_fp32(cuda):
    import torch
    import immersedlayers as il
    og, bl = _case()
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)
    c = il.SurfaceVectorCache(bl, g, dtype=torch.float32)
    N = len(bl)
    vp_h = np.concatenate([np.ones(N), np.zeros(N)])
    vp = il.VectorData(torch.tensor(vp_h, dtype=torch.float32, device="cuda"))
    vm = il.VectorData.zeros(N, torch.float32)
    v, s, sigma, info = il.solve_stokes(c, vp, vm, tol=1e-5, maxiter=5000)
    assert info["converged"], info
    oc = oracle_cache(og, bl, kind="vector")
    v_ref, s_ref, sig_ref = O.solve_stokes(oc, vp_h, np.zeros(2 * N))
    # FP32 grid work and CG vectors, CG to 1e-5
    assert rel(v.numpy_components(), v_ref) < 1e-3
    assert rel(s.numpy_components(), s_ref) < 1e-3
    assert rel(sigma.numpy(), sig_ref) < 5e-2


def test_stokes_problem_api(cuda):
    import torch
    import immersedlayers as il
    og, bl = _case()
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)

    def vsplus(c, p):
        out = il.zeros_surface(c)
        out.data[:len(c)] = 1.0
        return out

    prob = il.StokesFlowProblem(g, bl, bc={"exterior": vsplus, "interior": lambda c, p: il.zeros_surface(c)})
    sys = il.construct_system(prob)
    v, s, sigma = il.solve(prob, sys, tol=1e-10)
    assert sys.last_info["converged"]
    # drag of the translating rectangle is negative along x, no net y force
    ds = np.asarray(bl.ds)
    N = len(bl)
    fx, fy = sigma.numpy()[:N] @ ds, sigma.numpy()[N:] @ ds
    assert fx < 0 and abs(fy) < 1e-6 * abs(fx)
