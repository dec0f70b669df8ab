"""Dirichlet and Neumann Poisson solves on the device against the oracle's
dense-LU solves (test/literate/problems.jl:259-298, neumann.jl:101-142)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import ilm_oracle as O
from geometry import dirichlet_config1, oracle_cache


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max()


def relt(a, b):
    if isinstance(b, tuple):
        return max(rel(x, y) for x, y in zip(a, b))
    return rel(a, b)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_dirichlet_config1(cuda, dtype):
    import torch
    import immersedlayers as il
    dt = torch.float64 if dtype == "f64" else torch.float32
    og, b, fb = dirichlet_config1()
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)
    c = il.SurfaceScalarCache(b, g, dtype=dt)
    fp = il.ScalarData(torch.tensor(fb, dtype=dt, device="cuda"))
    fm = il.ScalarData.zeros(len(b), dt)
    f, s, info = il.solve_dirichlet(c, fp, fm, tol=1e-10)
    assert info["converged"] and info["rel_residual"] <= 1e-10
    oc = oracle_cache(og, b)
    S = O.create_RTLinvR(oc)
    f_ref, s_ref = O.solve_dirichlet(oc, fb, np.zeros_like(fb), S)
    # s inherits the conditioning of S (cond ~ 4e4 here): at a 1e-10
    # residual it is determined to ~1e-9 (FP64); FP32 grid work leaves f and
    # s within 1e-5 (measured 4.9e-6 and 1.0e-6)
    if dt == torch.float64:
        assert rel(f.numpy_components(), f_ref) < 1e-9
        assert rel(s.numpy(), s_ref) < 1e-8
    else:
        assert rel(f.numpy_components(), f_ref) < 1e-5
        assert rel(s.numpy(), s_ref) < 1e-5
    # residual of the device s in the oracle's FP64 operator
    rhs = O.interpolate_scalar(oc, oc.inverse_laplacian(O.surface_divergence(oc, fb))) - 0.5 * fb
    r = np.linalg.norm(S @ s.numpy() - rhs) / np.linalg.norm(rhs)
    assert r < (1e-9 if dt == torch.float64 else 1e-5)


def test_neumann_circle(cuda):
    import torch
    import immersedlayers as il
    from immersedlayers import bodies as B
    h = 0.04
    og = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    b = B.circle(1.0, ds=1.4 * h)
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    c = il.SurfaceScalarCache(b, g)
    vplus = b.nx.copy()   # neumann.jl:157-168: v_n+ = n_x, v_n- = 0
    vp = il.ScalarData(torch.tensor(vplus, device="cuda"))
    vm = il.ScalarData.zeros(len(b))
    f, df, info = il.solve_neumann(c, vp, vm, tol=1e-10, maxiter=20000)
    assert info["converged"], info
    oc = oracle_cache(og, b)
    f_ref, df_ref, _, _ = O.solve_neumann(oc, vplus, np.zeros_like(vplus))
    # the field is insensitive to the (near-)null space of S; compare it
    assert rel(f.numpy_components(), f_ref) < 1e-6


def test_neumann_streamfunction_circle(cuda):
    """The whole literate Neumann solve (test/literate/neumann.jl:101-142):
    potential, [phi], streamfunction and [psi] against the oracle's
    block-LU solve on the reference example (v_n+ = n_x, v_n- = 0); S is
    well conditioned here (cond ~1.3e3), so ds and s are determined."""
    import torch
    import immersedlayers as il
    from immersedlayers import bodies as B
    h = 0.04
    og = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    b = B.circle(1.0, ds=1.4 * h)
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    c = il.SurfaceScalarCache(b, g)
    vplus = b.nx.copy()
    vp = il.ScalarData(torch.tensor(vplus, device="cuda"))
    vm = il.ScalarData.zeros(len(b))
    f, df, s, ds, info = il.solve_neumann_full(c, vp, vm, tol=1e-11, maxiter=20000)
    assert info["converged"], info
    f_ref, df_ref, s_ref, ds_ref = O.solve_neumann(oracle_cache(og, b), vplus, np.zeros_like(vplus))
    assert rel(f.numpy_components(), f_ref) < 1e-6
    assert rel(s.numpy_components(), s_ref) < 1e-6
    assert rel(ds.numpy(), ds_ref) < 1e-6
    assert rel(df.numpy(), df_ref) < 1e-5
    # the problem API returns the same four fields
    prob = il.NeumannPoissonProblem(g, b, bc={"exterior": lambda c_, pp: c_.nrm.data[:len(b)],
                                              "interior": lambda c_, pp: 0.0 * c_.nrm.data[:len(b)]})
    sys_ = il.construct_system(prob)
    f2, df2, s2, ds2 = il.solve(prob, sys_, tol=1e-11, maxiter=20000)
    assert rel(s2.numpy_components(), s_ref) < 1e-6


def test_schur_builds_vector_cache_and_remaining_kinds(cuda):
    """Every Schur kind of src/matrix_operators.jl:9-244 on the device against
    the oracle's column-by-column builds: the vector-cache kinds (VectorData
    2N x 2N, and the ScalarData CLinvCT_scalar) and GLinvD_cross on a scalar
    cache."""
    import torch
    import immersedlayers as il
    from immersedlayers import bodies as B
    h = 0.04
    og = O.Grid.physical((-1.0, 1.0), (-1.0, 1.0), h)
    b = B.circle(0.4, ds=1.4 * h)
    g = il.PhysicalGrid((-1.0, 1.0), (-1.0, 1.0), h)
    vc = il.SurfaceVectorCache(b, g)
    ovc = oracle_cache(og, b, "vector")
    cases = [(il.create_RTLinvR, O.create_RTLinvR_vector), (il.create_CLinvCT, O.create_CLinvCT_vector),
             (il.create_GLinvD, O.create_GLinvD_vector), (il.create_nRTRn, O.create_nRTRn_vector),
             (il.create_CLinvCT_scalar, O.create_CLinvCT_scalar_vector), (il.create_CL2invCT, O.create_CL2invCT_vector),
             (il.create_GLinvD_symm, O.create_GLinvD_symm)]
    for fn, ref in cases:
        A = fn(vc, scale=0.5).cpu().numpy()
        R = ref(ovc, scale=0.5)
        assert A.shape == R.shape, fn.__name__
        assert rel(A, R) < 1e-10, (fn.__name__, rel(A, R))
    sc = il.SurfaceScalarCache(b, g)
    A = il.create_GLinvD_cross(sc).cpu().numpy()
    assert rel(A, O.create_GLinvD_cross(oracle_cache(og, b))) < 1e-10
    with pytest.raises(il._lib.ILMError):
        il.create_CL2invCT(sc)


def test_vector_cache_masks(cuda):
    """Masks of a vector cache (src/surface_operators.jl:872-877, :907-923)
    against the oracle on every grid type, and the enclosed area."""
    import torch
    import immersedlayers as il
    from immersedlayers import bodies as B
    h = 0.04
    og = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    b = B.circle(1.0, ds=1.4 * h)
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    vc = il.SurfaceVectorCache(b, g)
    ovc = oracle_cache(og, b, "vector")
    for kind, okind in [(il.EdgesPrimal, "edges_primal"), (il.NodesDual, "nodes_dual"),
                        (il.NodesPrimal, "nodes_primal"), (il.EdgeGradientPrimal, "edgegrad")]:
        m = il.mask(vc, kind).numpy_components()
        ref = O.mask_vector(ovc, okind)
        assert relt(m, ref) < 1e-10, kind.__name__
        cm = il.complementary_mask(vc, kind).numpy_components()
        if kind is il.EdgesPrimal:
            assert relt(cm, tuple(1.0 - x for x in ref)) < 1e-10
    mu = il.mask(vc).numpy_components()[0]
    area = mu.sum() * h * h
    assert abs(area - np.pi) < 1e-2 * np.pi, area


def test_tensor_normal_dot_transfers(cuda):
    """regularize_normal_dot!(v::Edges, taus::TensorData) and
    normal_dot_interpolate!(taus::TensorData, v::Edges)
    (src/surface_operators.jl:205-215, :332-343) on a vector cache against
    the oracle (TensorData slots dudx, dudy, dvdx, dvdy = n_x s_x, n_y s_x,
    n_x s_y, n_y s_y)."""
    import torch
    import immersedlayers as il
    from immersedlayers import bodies as B
    h = 0.04
    og = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    b = B.circle(1.0, ds=1.4 * h)
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    vc = il.SurfaceVectorCache(b, g)
    ovc = oracle_cache(og, b, "vector")
    N = len(b)
    rng = np.random.default_rng(21)
    t_h = rng.standard_normal(4 * N)
    tau = il.TensorData(torch.tensor(t_h, device="cuda"))
    q = il.regularize_normal_dot_(il.EdgesPrimal.zeros(g), tau, vc)
    assert relt(q.numpy_components(), O.regularize_normal_dot_tensor(ovc, t_h)) < 1e-12
    e = il.EdgesPrimal.zeros(g)
    e_h = (rng.standard_normal(e.numpy_components()[0].shape), rng.standard_normal(e.numpy_components()[1].shape))
    e.set_numpy(e_h)
    out = il.TensorData.zeros(N)
    il.normal_dot_interpolate_(out, e, vc)
    assert rel(out.numpy(), O.normal_dot_interpolate_tensor(ovc, e_h)) < 1e-12


def test_shape_masks_area(cuda):
    """mask!(w, surface, grid) (test/surface_ops.jl:235-252): Rectangle(0.5,
    0.25) on Nodes{Primal}, Nodes{Dual}, Edges{Primal} and EdgeGradient,
    each component integrating to 0.5 within 1e-3."""
    import immersedlayers as il
    from immersedlayers import bodies as B
    h = 0.04
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    r = B.rectangle(0.5, 0.25, ds=1.4 * h)
    for kind in (il.NodesPrimal, il.NodesDual, il.EdgesPrimal, il.EdgeGradientPrimal):
        w = kind.zeros(g).fill_(1.0)
        il.mask_(w, r, g)
        comps = w.numpy_components()
        for comp in (comps if isinstance(comps, tuple) else (comps,)):
            assert abs(comp.sum() * h * h - 0.5) < 1e-3, kind.__name__
