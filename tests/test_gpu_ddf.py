"""Every DDF of the reference's cache set-up (src/cache.jl:305-313: Yang3,
Roma, M4prime, Witchhat, M3) under both weight scalings (GridScaling:
R = ds/h^2 phi phi, E = phi phi; IndexScaling: R = E^T, `issymmetric=true`,
cache.jl:309-310) on the device against the oracle, on the reference's unit
test geometry (h = 0.04 on [-2,2]^2, circle R = 1, ds = 1.4 h).

Tolerances (relative to the max magnitude): FP64 1e-12 for transfers and
composite layer operators, 1e-11 for FFT-based operators and Schur entries,
1e-10 for solves; FP32 2e-6 for transfers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import ilm_oracle as O
from geometry import oracle_cache, surface_ops_case

DDFS = ["Yang3", "Roma", "M4prime", "Witchhat", "M3"]
SCALINGS = ["GridScaling", "IndexScaling"]


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def relt(a, b):
    if isinstance(b, tuple):
        return max(rel(x, y) for x, y in zip(a, b))
    return rel(a, b)


def caches(ddf, scaling, dtype, kind="scalar"):
    import torch
    import immersedlayers as il
    og, b = surface_ops_case()
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)
    mk = il.SurfaceScalarCache if kind == "scalar" else il.SurfaceVectorCache
    c = mk(b, g, ddftype=ddf, scaling=scaling, dtype=dtype)
    oc = O.SurfaceCache(b.x, b.y, b.nx, b.ny, b.ds, og, kind=kind, ddftype=ddf, scaling=scaling)
    return il, g, b, c, oc


@pytest.mark.parametrize("scaling", SCALINGS)
@pytest.mark.parametrize("ddf", DDFS)
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_transfers_every_ddf_and_scaling(cuda, ddf, scaling, dtype):
    """regularize! / interpolate! on Nodes{Primal}, Nodes{Dual} and
    Edges{Primal} (src/surface_operators.jl:13-88)."""
    import torch
    dt = torch.float64 if dtype == "f64" else torch.float32
    tol = 1e-12 if dt == torch.float64 else 2e-6
    il, g, b, c, oc = caches(ddf, scaling, dt)
    N = len(b)
    rng = np.random.default_rng(5)
    f = rng.standard_normal(N)
    fd = il.ScalarData(torch.tensor(f, dtype=dt, device="cuda"))
    for cls, kind in [(il.NodesPrimal, O.NODES_PRIMAL), (il.NodesDual, O.NODES_DUAL)]:
        out = cls.zeros(g, dt)
        out.fill_(3.0)
        il.regularize_(out, fd, c)
        assert rel(out.numpy_components(), oc.reg_cls(f, kind)) < tol, (cls.__name__,)
        fo = il.ScalarData.zeros(N, dt)
        il.interpolate_(fo, out, c)
        assert rel(fo.numpy(), oc.interp_cls(out.numpy_components(), kind)) < tol, (cls.__name__,)
    v = rng.standard_normal(2 * N)
    q = il.EdgesPrimal.zeros(g, dt)
    il.regularize_(q, il.VectorData(torch.tensor(v, dtype=dt, device="cuda")), c)
    assert relt(q.numpy_components(), O.regularize_vector(oc, v)) < tol
    vo = il.VectorData.zeros(N, dt)
    il.interpolate_(vo, q, c)
    assert rel(vo.numpy(), O.interpolate_vector(oc, q.numpy_components())) < tol


@pytest.mark.parametrize("scaling", SCALINGS)
@pytest.mark.parametrize("ddf", DDFS)
def test_layer_operators_every_ddf_and_scaling(cuda, ddf, scaling):
    """surface_divergence! / surface_grad! (the double layer and its
    adjoint, with the scaling's derivative factor, src/surface_operators.jl:
    357-420) and the inverse Laplacian of the double layer (the mask, which
    the reference defines for GridScaling caches only)."""
    import torch
    il, g, b, c, oc = caches(ddf, scaling, torch.float64)
    N = len(b)
    f = np.cos(2 * np.arctan2(b.y, b.x))
    w = il.NodesPrimal.zeros(g, torch.float64)
    il.surface_divergence_(w, il.ScalarData(torch.tensor(f, dtype=torch.float64, device="cuda")), c)
    assert rel(w.numpy_components(), O.surface_divergence(oc, f)) < 1e-12
    fo = il.ScalarData.zeros(N, torch.float64)
    il.surface_grad_(fo, w, c)
    assert rel(fo.numpy(), O.surface_grad(oc, w.numpy_components())) < 1e-12
    if scaling == "GridScaling":
        m = il.mask(c)
        assert rel(m.numpy_components(), O.mask(oc)) < 1e-11
    else:   # mask(cache::BasicILMCache{N,GridScaling}) only (src/surface_operators.jl:737)
        from immersedlayers._lib import ILMError
        with pytest.raises(ILMError, match="GridScaling"):
            il.mask(c)


@pytest.mark.parametrize("scaling", SCALINGS)
@pytest.mark.parametrize("ddf", DDFS)
def test_schur_and_dirichlet_solve_every_ddf_and_scaling(cuda, ddf, scaling):
    """create_RTLinvR (src/matrix_operators.jl:9-27) from the device's LGF
    point-pair sums against the oracle's column-by-column build, and the
    refined Dirichlet solve (FP64 Schur residual <= 1e-13; cond(S) ~ 1e3
    leaves s to ~1e-11) against the oracle's dense-LU solve."""
    import torch
    il, g, b, c, oc = caches(ddf, scaling, torch.float64)
    N = len(b)
    S_ref = O.create_RTLinvR(oc)
    S_dev = il.create_RTLinvR(c).cpu().numpy()
    assert rel(S_dev, S_ref) < 1e-11
    fb = np.cos(np.arctan2(b.y, b.x)) + 0.3 * np.sin(3 * np.arctan2(b.y, b.x))
    fp = il.ScalarData(torch.tensor(fb, dtype=torch.float64, device="cuda"))
    fm = il.ScalarData.zeros(N, torch.float64)
    f, s, info = il.solve_dirichlet_refined(c, fp, fm, tol=1e-13)
    assert info["converged"], info
    fr, sr = O.solve_dirichlet(oc, fb, np.zeros_like(fb), S_ref)
    assert rel(f.numpy_components(), fr) < 1e-10
    assert rel(s.numpy(), sr) < 1e-10
