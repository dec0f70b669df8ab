"""The CPU oracle against the reference's own known-answer tests
(test/tools.jl, test/surface_ops.jl) and published LGF values."""
import math

import numpy as np
import pytest

import ilm_oracle as O
from geometry import angles, oracle_cache, surface_ops_case, tools_case


def test_ddf_partition_of_unity():
    r = np.linspace(-0.5, 0.5, 41)
    for name, (k, _) in O.DDFS.items():
        s = sum(k(r - j) for j in range(-4, 5))
        assert np.abs(s - 1.0).max() < 1e-14, name


def test_lgf_known_values():
    # exact values of the square-lattice Green's function (G(0,0) = 0)
    m = np.array([1, 1, 2, 2, 2, 3, 5, 20])
    n = np.array([0, 1, 0, 1, 2, 0, 5, 20])
    G = O.lgf_values(m, n)
    exact = [0.25, 1 / math.pi, 1 - 2 / math.pi, -0.25 + 2 / math.pi, 4 / (3 * math.pi), 17 / 4 - 12 / math.pi,
             sum(1 / (2 * k - 1) for k in range(1, 6)) / math.pi, sum(1 / (2 * k - 1) for k in range(1, 21)) / math.pi]
    assert np.abs(G - np.array(exact)).max() < 1e-14


def test_lgf_far_field():
    for m, n in [(300, 0), (200, 150)]:
        r = math.hypot(m, n)
        th = math.atan2(n, m)
        asym = (math.log(r) + O.EULER_GAMMA + 1.5 * math.log(2)) / (2 * math.pi) - math.cos(4 * th) / (24 * math.pi * r * r)
        assert abs(O.lgf_values(np.array([m]), np.array([n]))[0] - asym) < 1e-10


def test_lgf_inverts_laplacian():
    rng = np.random.default_rng(0)
    w = np.zeros((40, 36))
    w[12:28, 10:26] = rng.standard_normal((16, 16))
    il = O.InverseLaplacian(40, 36, 1.0)
    u = il(w)
    lap = O.laplacian_nodes(u)
    assert np.abs(lap[1:-1, 1:-1] - w[1:-1, 1:-1]).max() < 1e-11


def test_grid_sizing_matches_reference_print():
    # examples/caches.ipynb: PhysicalGrid((-2,2),(-2,2),0.01) -> (406,406), (203,203), xlim +-2.02
    g = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), 0.01)
    assert (g.nx, g.ny, g.i0x, g.i0y) == (406, 406, 203, 203)
    x, _ = g.coords(O.NODES_PRIMAL)
    assert g.shape(O.NODES_PRIMAL) == (405, 405)
    assert abs(x[0] + 2.02) < 1e-12 and abs(x[-1] - 2.02) < 1e-12


def test_tools_inner_products_and_adjointness():
    g, b = tools_case()
    c = oracle_cache(g, b)
    h = g.h
    os_ = np.ones(len(b))
    oc = np.ones(g.shape(O.NODES_DUAL))
    # test/tools.jl:36-48
    lim = g.limits()
    assert math.sqrt(O.grid_dot_array(oc, oc, O.NODES_DUAL, h)) == pytest.approx(
        math.sqrt((lim[0][1] - lim[0][0]) * (lim[1][1] - lim[1][0])), abs=1e-12)
    assert abs(np.dot(os_, os_ * b.ds) - 2 * math.pi) < 1e-3
    assert abs(np.sum((b.nx ** 2 + b.ny ** 2) * b.ds) - 2 * math.pi) < 1e-3
    # test/tools.jl:107,112
    assert abs(O.grid_dot_array(oc, c.reg_cls(os_, O.NODES_DUAL), O.NODES_DUAL, h) - np.dot(os_, os_ * b.ds)) < 1e-14
    rng = np.random.default_rng(0)
    u = rng.standard_normal(g.shape(O.NODES_DUAL))
    phi = rng.standard_normal(len(b))
    lhs = O.grid_dot_array(u, c.reg_cls(phi, O.NODES_DUAL), O.NODES_DUAL, h)
    rhs = np.dot(c.interp_cls(u, O.NODES_DUAL), phi * b.ds)
    assert abs(lhs - rhs) < 1e-13
    # test/tools.jl:119-120 (Edges{Dual}.u lives on the (primal x, dual y) class)
    rf = c.reg_cls(os_, O.EDGES_PRIMAL_V)
    val = O.grid_dot_array(np.ones_like(rf), rf, O.EDGES_PRIMAL_V, h)
    assert abs(val - b.ds.sum()) < 1e-12
    assert abs(val - 2 * math.pi) < 1e-3


def test_circle_circumference_matches_notebook():
    # examples/caches.ipynb: dot(os,os,cache) = 6.283288300933757 for Circle(1.0, 0.014)
    from immersedlayers import bodies as B
    b = B.circle(1.0, ds=0.014)
    assert len(b) == 448
    assert abs(b.ds.sum() - 6.283288300933757) < 1e-9


def test_surface_ops_known_answers():
    g, b = surface_ops_case()
    c = oracle_cache(g, b)
    h = g.h
    N = len(b)
    f = np.sin(angles(N) - math.pi / 4)
    f2 = O.normal_interpolate(c, O.regularize_normal(c, f))
    assert f2.max() == pytest.approx(11, abs=1.0)          # test/surface_ops.jl:66
    assert f2.min() == pytest.approx(-11, abs=1.0)         # :67
    A = O.create_CLinvCT(c, scale=h)
    assert np.abs(np.linalg.eigvals(A)).max() == pytest.approx(0.2, abs=0.1)    # :71
    A = O.create_GLinvD(c, scale=h)
    assert np.abs(np.linalg.eigvals(A)).max() == pytest.approx(0.45, abs=0.1)   # :74
    A = O.create_nRTRn(c)
    assert np.linalg.svd(A, compute_uv=False).max() == pytest.approx(11, abs=1.0)  # :77


def test_vector_surface_ops_known_answers():
    g, b = surface_ops_case()
    c = oracle_cache(g, b, kind="vector")
    N = len(b)
    f = np.sin(angles(N) - math.pi / 4)
    vs = np.zeros(2 * N)
    vs[:N] = f
    vs = O.normal_interpolate_tensor(c, O.regularize_normal_tensor(c, vs))   # :131-132
    vs[:N] = f
    vs = O.normal_interpolate_symm(c, O.regularize_normal_symm(c, vs))      # :135-137
    assert vs[:N].min() == pytest.approx(-22.5, abs=1.0)
    assert vs[:N].max() == pytest.approx(22.5, abs=1.0)
    A = O.create_GLinvD_vector(c, scale=g.h)
    assert np.abs(np.linalg.eigvals(A)).max() == pytest.approx(0.45, abs=0.1)   # :146


def test_masks_area():
    g, b = surface_ops_case()
    c = oracle_cache(g, b)
    m = O.mask(c)
    assert abs(O.grid_dot_array(np.ones_like(m), m, O.NODES_PRIMAL, g.h) - math.pi) < 2e-3   # :186
    md = O.grid_interpolate_primal_to_dual(m, g)
    assert abs(O.grid_dot_array(np.ones_like(md), md, O.NODES_DUAL, g.h) - math.pi) < 1e-3  # :198


def test_dirichlet_exterior_analytic():
    # f+ = x on a circle of radius R: exterior solution x R^2 / r^2
    from immersedlayers import bodies as B
    h = 0.02
    g = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    b = B.circle(0.5, ds=1.4 * h)
    c = oracle_cache(g, b)
    f, s = O.solve_dirichlet(c, b.x.copy(), np.zeros(len(b)))
    x, y = g.coords(O.NODES_PRIMAL)
    X, Y = np.meshgrid(x, y, indexing="ij")
    r = np.hypot(X, Y)
    m = (r > 0.7) & (r < 1.5)
    assert np.abs(f[m] - X[m] * 0.25 / r[m] ** 2).max() < 5e-3


def test_oracle_stokes_no_slip_and_symmetry():
    """Stokes oracle (test/literate/stokes.jl:101-166): W S symmetric and
    negative definite, the velocity satisfies no-slip exactly, and the
    translating rectangle's traction has no net lift."""
    from immersedlayers import bodies as B
    h = 0.04
    g = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    b = B.rectangle(0.5, 0.25, ds=1.4 * h)
    c = O.SurfaceCache(b.x, b.y, b.nx, b.ny, b.ds, g, kind="vector")
    S = O.create_CL2invCT_vector(c)
    W = np.diag(np.concatenate([c.ds, c.ds]))
    WS = W @ S
    assert np.abs(WS - WS.T).max() < 1e-12 * np.abs(WS).max()
    assert np.linalg.eigvalsh(0.5 * (WS + WS.T)).max() < 0
    vp = np.concatenate([np.ones(c.N), np.zeros(c.N)])
    v, s, sig = O.solve_stokes(c, vp, np.zeros(2 * c.N), S=S)
    assert np.abs(O.interpolate_vector(c, v) - 0.5 * vp).max() < 1e-12
    assert abs(sig[c.N:] @ c.ds) < 1e-10 * abs(sig[:c.N] @ c.ds)
    F = O.surface_filter_vector(c)
    assert np.allclose(F @ np.ones(2 * c.N), 1.0)


def test_oracle_surface_filter_properties():
    """The oracle's surface filter (create_surface_filter,
    src/matrix_operators.jl:254-268): rows sum to one (constants pass), the
    entries are those of E R up to the row scaling, and C^6 smooths."""
    g, b = surface_ops_case()
    c = O.SurfaceCache(b.x, b.y, b.nx, b.ny, b.ds, g)
    F = O.surface_filter_scalar(c)
    np.testing.assert_allclose(F.sum(axis=1), 1.0, rtol=0, atol=1e-13)
    P = c.phi(O.NODES_PRIMAL)
    ER = np.asarray((P.T @ P).toarray()) * c._wscale()[None, :]
    np.testing.assert_allclose(F * ER.sum(axis=1, keepdims=True), ER, rtol=1e-12, atol=1e-15)
    th = np.arctan2(b.y, b.x)
    s = np.cos(th) + 0.3 * np.sin(40 * th)
    s6 = O.surface_filter(c, s, power=6)
    # the low mode survives, the high mode is damped
    lo, hi = np.cos(th), np.sin(40 * th)
    assert abs(np.dot(s6, lo) / np.dot(lo, lo) - 1.0) < 0.01
    assert abs(np.dot(s6, hi) / np.dot(hi, hi)) < 0.3 * 0.05


def test_oracle_convective_derivatives_exact_on_linear_fields():
    """The oracle's convective derivatives (src/grid_operators.jl:318-371) and
    w x v (:419-434) reproduce the exact answers of uniform and linear
    fields away from the ghost layers."""
    g, _ = surface_ops_case()
    h = g.h
    xu, yu = g.coords(O.EDGES_PRIMAL_U)
    xv, yv = g.coords(O.EDGES_PRIMAL_V)
    xp, yp = g.coords(O.NODES_PRIMAL)
    xd, yd = g.coords(O.NODES_DUAL)
    a, b, c, d = 0.7, -1.3, 2.0, 0.5
    unif = (np.full(g.shape(O.EDGES_PRIMAL_U), a), np.full(g.shape(O.EDGES_PRIMAL_V), b))
    p = c * xp[:, None] + d * yp[None, :]
    r = O.convective_derivative_nodes_primal(unif, p, g, 1.0 / h)
    np.testing.assert_allclose(r[2:-2, 2:-2], a * c + b * d, atol=1e-11)
    w = c * xd[:, None] + d * yd[None, :]
    r = O.convective_derivative_nodes_dual(unif, w, g, 1.0 / h)
    np.testing.assert_allclose(r[2:-2, 2:-2], a * c + b * d, atol=1e-11)
    assert np.all(r[0, :] == 0) and np.all(r[:, -1] == 0)
    # u = (x, y): u . grad u = (x, y)
    u = (np.broadcast_to(xu[:, None], g.shape(O.EDGES_PRIMAL_U)).copy(),
         np.broadcast_to(yv[None, :], g.shape(O.EDGES_PRIMAL_V)).copy())
    ru, rv = O.convective_derivative_edges(u, u, g, 1.0 / h)
    np.testing.assert_allclose(ru[2:-2, 2:-2], np.broadcast_to(xu[:, None], ru.shape)[2:-2, 2:-2], atol=1e-11)
    np.testing.assert_allclose(rv[2:-2, 2:-2], np.broadcast_to(yv[None, :], rv.shape)[2:-2, 2:-2], atol=1e-11)
    # uniform w and v: w x v = (-w b, w a)
    wu = np.full(g.shape(O.NODES_DUAL), 1.5)
    ou, ov = O.w_cross_v(wu, unif)
    np.testing.assert_allclose(ou[1:-1, :], -1.5 * b, atol=1e-13)
    np.testing.assert_allclose(ov[:, 1:-1], 1.5 * a, atol=1e-13)


def test_vector_cache_masks_area():
    """test/surface_ops.jl:214-231: the masks of a vector cache on
    Nodes{Primal}, Nodes{Dual}, Edges{Primal} and EdgeGradient{Primal}
    integrate to pi (1e-3) for the unit circle.  This pins the TensorData
    layout of the normal products (dudy = n_y v_x): the transposed layout
    gives pi/2 on the edges."""
    g, b = surface_ops_case()
    c = oracle_cache(g, b, "vector")
    for kind in ("nodes_primal", "nodes_dual", "edges_primal", "edgegrad"):
        H = O.mask_vector(c, kind)
        for comp in (H if isinstance(H, tuple) else (H,)):
            assert abs(comp.sum() * g.h * g.h - math.pi) < 1e-3, kind


def test_shape_masks_area():
    """test/surface_ops.jl:235-252: masks of Rectangle(0.5, 0.25) (half
    lengths) built from a scalar cache (Nodes) or a vector cache (Edges,
    EdgeGradient) integrate to 0.5 within 1e-3."""
    from immersedlayers import bodies as B
    g, _ = surface_ops_case()
    r = B.rectangle(0.5, 0.25, ds=1.4 * g.h)
    m = O.mask(oracle_cache(g, r))
    assert abs(m.sum() * g.h ** 2 - 0.5) < 1e-3
    assert abs(O.grid_interpolate_primal_to_dual(m, g).sum() * g.h ** 2 - 0.5) < 1e-3
    vc = oracle_cache(g, r, "vector")
    for kind in ("edges_primal", "edgegrad"):
        for comp in O.mask_vector(vc, kind):
            assert abs(comp.sum() * g.h ** 2 - 0.5) < 1e-3, kind


def test_helmholtz_known_answer():
    """test/surface_ops.jl:312-341: for random masked curl w, masked
    divergence d and surface jump dv, the field v = vecfield_helmholtz(w, d,
    dv) has masked curl w and masked divergence d at the interior nodes
    (1e-8)."""
    g, b = surface_ops_case()
    c = oracle_cache(g, b, "vector")
    rng = np.random.default_rng(0)
    w = rng.standard_normal(g.shape(O.NODES_DUAL))
    d = rng.standard_normal(g.shape(O.NODES_PRIMAL))
    dv = rng.standard_normal(2 * c.N)
    v = O.vecfield_helmholtz(c, w, d, dv, (0.0, 0.0))
    mw = O.curl_edges(v, g) * c.dscale() - O.regularize_normal_cross_vector(c, dv)
    md = O.divergence_edges(v) * c.dscale() - O.regularize_normal_dot(c, dv)
    assert np.abs(mw[1:-1, 1:-1] - w[1:-1, 1:-1]).max() < 1e-8
    assert np.abs(md[1:-1, 1:-1] - d[1:-1, 1:-1]).max() < 1e-8
