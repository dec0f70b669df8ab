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


def _rigid_rhs(bl, nrhs, seed):
    """Rigid-body surface velocities (translation + rotation ~ N(0, 1) per
    body) for `nrhs` right-hand sides."""
    rng = np.random.default_rng(seed)
    N = len(bl)
    fi = bl.firstindices()
    V = np.zeros((nrhs, 2 * N))
    for r in range(nrhs):
        for b in range(len(fi) - 1):
            s = slice(fi[b], fi[b + 1])
            ux, uy, om = rng.standard_normal(3)
            cx, cy = bl.x[s].mean(), bl.y[s].mean()
            V[r, s] = ux - om * (bl.y[s] - cy)
            V[r, N + fi[b]:N + fi[b + 1]] = uy + om * (bl.x[s] - cx)
    return V


def test_stokes_multi_rhs_matches_oracle(cuda):
    """Block CG over five right-hand sides (preconditioned and plain): every
    right-hand side's v, s and sigma against the oracle's dense block-LU
    solve at the single-solve tolerances; the preconditioner cuts the block
    iterations."""
    import torch
    import immersedlayers as il
    og, bl = _case(two_bodies=True)
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)
    c = il.SurfaceVectorCache(bl, g, dtype=torch.float64)
    N = len(bl)
    V = _rigid_rhs(bl, 5, 3)
    oc = oracle_cache(og, bl, kind="vector")
    S = O.create_CL2invCT_vector(oc)
    Ss = O.create_CLinvCT_scalar_vector(oc)
    filt = O.surface_filter_vector(oc)
    its = {}
    for pc in (True, False):
        vs, ss, sig, infos = il.solve_stokes_multi(c, torch.tensor(V, device="cuda"), tol=1e-11, maxiter=20000,
                                                   precond=pc)
        assert all(i["converged"] for i in infos), infos
        its[pc] = infos[0]["iterations"]
        for r in range(V.shape[0]):
            v_ref, s_ref, sig_ref = O.solve_stokes(oc, V[r], np.zeros(2 * N), S=S, Ss=Ss, filt=filt)
            assert rel(vs[r].numpy_components(), v_ref) < 1e-7, (pc, r)
            assert rel(ss[r].numpy_components(), s_ref) < 1e-7, (pc, r)
            assert rel(sig[r].numpy(), sig_ref) < 1e-4, (pc, r)
            vi = O.interpolate_vector(oc, vs[r].numpy_components())
            assert np.abs(vi - 0.5 * V[r]).max() < 1e-8 * max(1.0, np.abs(V[r]).max()), (pc, r)
    assert its[True] < its[False], its


def test_stokes_multi_equals_single(cuda):
    """One right-hand side through ilm_solve_stokes_multi equals ilm_solve_stokes."""
    import torch
    import immersedlayers as il
    og, bl = _case()
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)
    c = il.SurfaceVectorCache(bl, g, dtype=torch.float64)
    V = _rigid_rhs(bl, 1, 4)
    N = len(bl)
    v1, s1, sig1, i1 = il.solve_stokes(c, il.VectorData(torch.tensor(V[0], device="cuda")), il.VectorData.zeros(N),
                                       tol=1e-10, maxiter=5000)
    vs, ss, sig, infos = il.solve_stokes_multi(c, torch.tensor(V, device="cuda"), tol=1e-10, maxiter=5000)
    assert i1["converged"] and infos[0]["converged"]
    assert torch.equal(v1.data, vs[0].data) and torch.equal(sig1.data, sig[0].data)
    assert i1["iterations"] == infos[0]["iterations"]


def test_stokes_multi_rejects_bad_arguments(cuda):
    import torch
    import immersedlayers as il
    from immersedlayers._lib import ILMError
    og, bl = _case()
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)
    c = il.SurfaceVectorCache(bl, g, dtype=torch.float64)
    N = len(bl)
    with pytest.raises(ValueError):
        il.solve_stokes_multi(c, torch.zeros(33, 2 * N, dtype=torch.float64, device="cuda"))
    with pytest.raises(ValueError):
        il.solve_stokes_multi(c, torch.zeros(2, N, dtype=torch.float64, device="cuda"))
    sc = il.SurfaceScalarCache(bl, g, dtype=torch.float64)
    with pytest.raises(ILMError, match="vector cache"):
        il.solve_stokes_multi(sc, torch.zeros(1, 2 * N, dtype=torch.float64, device="cuda"))


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_stokes_multi_refined_matches_oracle(cuda, dtype):
    """FP64 refinement of the Stokes solves from an FP32 (or FP64) cache:
    FP64 outputs, Schur residuals <= 1e-10, and every right-hand side's v, s
    and sigma against the oracle's dense block-LU solve at the FP64 bars."""
    import torch
    import immersedlayers as il
    og, bl = _case(two_bodies=True)
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)
    c = il.SurfaceVectorCache(bl, g, dtype=torch.float32 if dtype == "f32" else torch.float64)
    N = len(bl)
    V = _rigid_rhs(bl, 3, 5)
    vs, ss, sig, infos = il.solve_stokes_multi_refined(c, torch.tensor(V, device="cuda"), tol=1e-10)
    assert all(i["converged"] and i["rel_residual"] <= 1e-10 for i in infos), infos
    assert vs[0].data.dtype == torch.float64 and sig[0].data.dtype == torch.float64
    oc = oracle_cache(og, bl, kind="vector")
    S = O.create_CL2invCT_vector(oc)
    Ss = O.create_CLinvCT_scalar_vector(oc)
    filt = O.surface_filter_vector(oc)
    for r in range(V.shape[0]):
        v_ref, s_ref, sig_ref = O.solve_stokes(oc, V[r], np.zeros(2 * N), S=S, Ss=Ss, filt=filt)
        assert rel(vs[r].numpy_components(), v_ref) < 1e-7, r
        assert rel(ss[r].numpy_components(), s_ref) < 1e-7, r
        assert rel(sig[r].numpy(), sig_ref) < 1e-4, r
