"""Convective derivatives and w x v (src/grid_operators.jl:186-434) and the
Helmholtz decomposition (src/helmholtz.jl) on the device against the oracle.

These rows have no known-answer test in the reference (CartesianGrids'
grid_interpolate! is un-vendored): the checks are parity with the oracle's
restatement and the exact answers of linear fields.  Tolerances: FP64 1e-12,
FP32 2e-6 relative to the largest magnitude; fields that pass through the
LGF convolution: FP64 1e-11, FP32 1e-4 (the Helmholtz velocity is a
difference quotient of the potentials, which loses the ratio of the
potential to its one-cell change in FP32 digits)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import ilm_oracle as O
from geometry import oracle_cache, surface_ops_case


def rel(a, b):
    if isinstance(b, tuple):
        return max(rel(x, y) for x, y in zip(a, b))
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module", params=["f64", "f32"])
def S(request, cuda):
    import torch
    import immersedlayers as il
    dt = torch.float64 if request.param == "f64" else torch.float32
    og, b = surface_ops_case()
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)
    return dict(il=il, torch=torch, dt=dt, g=g, og=og, b=b,
                sc=il.SurfaceScalarCache(b, g, dtype=dt), vc=il.SurfaceVectorCache(b, g, dtype=dt),
                tol=1e-12 if dt == torch.float64 else 2e-6, itol=1e-11 if dt == torch.float64 else 1e-4)


def _rand(S, cls, seed):
    rng = np.random.default_rng(seed)
    f = cls.zeros(S["g"], S["dt"])
    comps = f.numpy_components()
    comps = comps if isinstance(comps, tuple) else (comps,)
    arrs = tuple(rng.standard_normal(c.shape) for c in comps)
    f.set_numpy(arrs)
    return f, (arrs if len(arrs) > 1 else arrs[0])


def test_convective_derivative_nodes(S):
    il, og = S["il"], S["og"]
    v, vh = _rand(S, il.EdgesPrimal, 1)
    p, ph = _rand(S, il.NodesPrimal, 2)
    w, wh = _rand(S, il.NodesDual, 3)
    sc = 1.0 / og.h
    out = il.convective_derivative_(il.NodesPrimal.zeros(S["g"], S["dt"]), v, p, S["sc"], il.ConvectiveDerivativeCache(S["sc"]))
    assert rel(out.numpy_components(), O.convective_derivative_nodes_primal(vh, ph, og, sc)) < S["tol"]
    out = il.convective_derivative(v, w, S["sc"])
    assert rel(out.numpy_components(), O.convective_derivative_nodes_dual(vh, wh, og, sc)) < S["tol"]


def test_convective_derivative_edges(S):
    il, og = S["il"], S["og"]
    v, vh = _rand(S, il.EdgesPrimal, 4)
    u, uh = _rand(S, il.EdgesPrimal, 5)
    sc = 1.0 / og.h
    out = il.convective_derivative(u, S["vc"])            # u . grad u
    assert rel(out.numpy_components(), O.convective_derivative_edges(uh, uh, og, sc)) < S["tol"]
    out = il.EdgesPrimal.zeros(S["g"], S["dt"])
    il.convective_derivative_(out, v, u, S["vc"], il.ConvectiveDerivativeCache(S["vc"]))   # v . grad u
    assert rel(out.numpy_components(), O.convective_derivative_edges(vh, uh, og, sc)) < S["tol"]


def test_w_cross_v(S):
    il, og = S["il"], S["og"]
    v, vh = _rand(S, il.EdgesPrimal, 6)
    w, wh = _rand(S, il.NodesDual, 7)
    out = il.EdgesPrimal.zeros(S["g"], S["dt"])
    il.w_cross_v_(out, w, v, S["vc"], il.RotConvectiveDerivativeCache(S["vc"]))
    assert rel(out.numpy_components(), O.w_cross_v(wh, vh)) < S["tol"]
    assert rel(il.w_cross_v(w, v, S["vc"]).numpy_components(), O.w_cross_v(wh, vh)) < S["tol"]


@pytest.mark.parametrize("nx,ny", [(37, 23), (70, 9), (5, 6), (33, 34)])
def test_convective_ragged_grids(S, nx, ny):
    """Rectangular grids whose sizes are not multiples of the kernels' tiles
    (32 columns by 32 rows, four consecutive rows per thread): every output
    of the convective kernels, the gradient, the divergence, the curl both
    ways, the Laplacian and the vector gradient and divergence, ghost layers
    included, against the oracle."""
    il, torch = S["il"], S["torch"]
    h = 0.1
    g = il.PhysicalGrid(h=h, nx=nx, ny=ny)
    og = O.Grid(nx, ny, h, g.i0[0], g.i0[1])
    S2 = dict(S, g=g)
    sc = il.SurfaceScalarCache(None, g, dtype=S["dt"])
    vc = il.SurfaceVectorCache(None, g, dtype=S["dt"])
    v, vh = _rand(S2, il.EdgesPrimal, 11)
    u, uh = _rand(S2, il.EdgesPrimal, 12)
    p, ph = _rand(S2, il.NodesPrimal, 13)
    w, wh = _rand(S2, il.NodesDual, 14)
    s = 1.0 / h
    out = il.convective_derivative(v, p, sc)
    assert rel(out.numpy_components(), O.convective_derivative_nodes_primal(vh, ph, og, s)) < S["tol"]
    out = il.convective_derivative(v, w, sc)
    assert rel(out.numpy_components(), O.convective_derivative_nodes_dual(vh, wh, og, s)) < S["tol"]
    out = il.EdgesPrimal.zeros(g, S["dt"])
    il.convective_derivative_(out, v, u, vc, il.ConvectiveDerivativeCache(vc))
    assert rel(out.numpy_components(), O.convective_derivative_edges(vh, uh, og, s)) < S["tol"]
    assert rel(il.w_cross_v(w, v, vc).numpy_components(), O.w_cross_v(wh, vh)) < S["tol"]
    q = il.EdgesPrimal.zeros(g, S["dt"])
    il.grad_(q, p, sc)
    assert rel(q.numpy_components(), tuple(x * s for x in O.grad_nodes(ph, og))) < S["tol"]
    d = il.NodesPrimal.zeros(g, S["dt"])
    il.divergence_(d, v, sc)
    assert rel(d.numpy_components(), O.divergence_edges(vh) * s) < S["tol"]
    il.curl_(q, w, sc)                                   # Nodes{Dual} -> Edges{Primal}
    assert rel(q.numpy_components(), tuple(x * s for x in O.curl_nodes_dual(wh, og))) < S["tol"]
    wd = il.NodesDual.zeros(g, S["dt"])
    il.curl_(wd, v, sc)                                  # Edges{Primal} -> Nodes{Dual}
    assert rel(wd.numpy_components(), O.curl_edges(vh, og) * s) < S["tol"]
    lap = il.NodesPrimal.zeros(g, S["dt"])
    il.laplacian_(lap, p, sc)
    assert rel(lap.numpy_components(), O.laplacian_nodes(ph, s * s)) < S["tol"]
    t = il.EdgeGradientPrimal.zeros(g, S["dt"])
    il.grad_(t, v, vc)                                   # Edges{Primal} -> EdgeGradient{Primal}
    assert rel(t.numpy_components(), tuple(x * s for x in O.grad_edges(vh, og))) < S["tol"]
    th = t.numpy_components()
    q2 = il.EdgesPrimal.zeros(g, S["dt"])
    il.divergence_(q2, t, vc)                            # EdgeGradient{Primal} -> Edges{Primal}
    assert rel(q2.numpy_components(), tuple(x * s for x in O.divergence_edgegrad(th, og))) < S["tol"]


def test_convective_derivative_linear_fields_exact(S):
    """Uniform velocity (a, b) and linear p = c x + d y: v . grad p = a c + b d
    away from the ghost layers (GridScaling: differences / h)."""
    il, og = S["il"], S["og"]
    a, b, c, d = 0.7, -1.3, 2.0, 0.5
    v = il.vecfield_uniformvecfield_(il.EdgesPrimal.zeros(S["g"], S["dt"]), a, b)
    p = il.x_grid(S["sc"])
    p.data.mul_(c).add_(d * il.y_grid(S["sc"]).data)
    out = il.convective_derivative(v, p, S["sc"]).numpy_components()
    assert np.abs(out[2:-2, 2:-2] - (a * c + b * d)).max() < (1e-10 if S["dt"].itemsize == 8 else 2e-4)
    # u . grad u of a uniform field is zero; of u = (y, 0): (0, 0) as well
    u = il.vecfield_uniformvecfield_(il.EdgesPrimal.zeros(S["g"], S["dt"]), a, b)
    assert np.abs(np.concatenate([x.ravel() for x in il.convective_derivative(u, S["vc"]).numpy_components()])).max() < 1e-5


def test_convective_derivative_rejects_aliasing(S):
    il = S["il"]
    v, _ = _rand(S, il.EdgesPrimal, 8)
    with pytest.raises(il._lib.ILMError):
        il.convective_derivative_(v, v, S["vc"])


def test_vecfield_helmholtz_matches_oracle(S):
    import torch
    il, og, b = S["il"], S["og"], S["b"]
    vc = S["vc"]
    ovc = oracle_cache(og, b, "vector")
    N = len(b)
    rng = np.random.default_rng(9)
    xd, yd = og.coords(O.NODES_DUAL)
    xp, yp = og.coords(O.NODES_PRIMAL)
    cv = np.exp(-((xd[:, None] - 0.3) ** 2 + (yd[None, :] + 0.2) ** 2) / 0.1)
    dvv = np.exp(-((xp[:, None] + 0.4) ** 2 + (yp[None, :] - 0.1) ** 2) / 0.2)
    dv = rng.standard_normal(2 * N)
    curlv = il.NodesDual.zeros(S["g"], S["dt"]).set_numpy(cv)
    divv = il.NodesPrimal.zeros(S["g"], S["dt"]).set_numpy(dvv)
    dvd = il.VectorData(torch.tensor(dv, dtype=S["dt"], device="cuda"))
    ref = O.vecfield_helmholtz(ovc, cv, dvv, dv)
    v = il.EdgesPrimal.zeros(S["g"], S["dt"])
    il.vecfield_helmholtz_(v, curlv, divv, dvd, None, vc, il.VectorFieldCache(vc))
    assert rel(v.numpy_components(), ref) < S["itol"]
    # uniform (Vx, Vy) and an Edges{Primal} vp
    il.vecfield_helmholtz_(v, curlv, divv, dvd, (1.5, -0.25), vc)
    assert rel(v.numpy_components(), O.vecfield_helmholtz(ovc, cv, dvv, dv, (1.5, -0.25))) < S["itol"]
    vp, vph = _rand(S, il.EdgesPrimal, 10)
    il.vecfield_helmholtz_(v, curlv, divv, dvd, vp, vc)
    assert rel(v.numpy_components(), O.vecfield_helmholtz(ovc, cv, dvv, dv, vph)) < S["itol"]
    # the building blocks compose to the same field
    vfc = il.VectorFieldCache(vc)
    psi = il.zeros_gridcurl(vc)
    phi = il.NodesPrimal.zeros(S["g"], S["dt"])
    il.vectorpotential_from_masked_curlv_(psi, curlv, dvd, vc, vfc.wcache)
    il.scalarpotential_from_masked_divv_(phi, divv, dvd, vc, vfc.dcache)
    assert rel(psi.numpy_components(), O.vectorpotential_from_masked_curlv(ovc, cv, dv)) < S["itol"]
    assert rel(phi.numpy_components(), O.scalarpotential_from_masked_divv(ovc, dvv, dv)) < S["itol"]
    v1 = il.vecfield_from_vectorpotential_(il.EdgesPrimal.zeros(S["g"], S["dt"]), psi, vc)
    v2 = il.vecfield_from_scalarpotential_(il.EdgesPrimal.zeros(S["g"], S["dt"]), phi, vc)
    assert rel(tuple(a + b_ for a, b_ in zip(v1.numpy_components(), v2.numpy_components())), ref) < S["itol"]


def test_masked_curl_div_round_trip(S):
    import torch
    il, og, b = S["il"], S["og"], S["b"]
    vc = S["vc"]
    ovc = oracle_cache(og, b, "vector")
    N = len(b)
    rng = np.random.default_rng(11)
    dv = rng.standard_normal(2 * N)
    dvd = il.VectorData(torch.tensor(dv, dtype=S["dt"], device="cuda"))
    c, ch = _rand(S, il.NodesDual, 12)
    m = il.masked_curlv_from_curlv_masked_(il.zeros_gridcurl(vc), c, dvd, vc)
    assert rel(m.numpy_components(), ch - O.regularize_normal_cross_vector(ovc, dv)) < S["tol"] * 10
    back = il.curlv_masked_from_masked_curlv_(il.zeros_gridcurl(vc), m, dvd, vc)
    assert rel(back.numpy_components(), ch) < S["tol"] * 10
    d, dh = _rand(S, il.NodesPrimal, 13)
    m = il.masked_divv_from_divv_masked_(il.NodesPrimal.zeros(S["g"], S["dt"]), d, dvd, vc)
    assert rel(m.numpy_components(), dh - O.regularize_normal_dot(ovc, dv)) < S["tol"] * 10
    back = il.divv_masked_from_masked_divv_(il.NodesPrimal.zeros(S["g"], S["dt"]), m, dvd, vc)
    assert rel(back.numpy_components(), dh) < S["tol"] * 10


def test_uniform_potentials(S):
    """The uniform-field potentials give the uniform field back through
    curl and grad (interior values)."""
    il = S["il"]
    vc = S["vc"]
    psi = il.vectorpotential_uniformvecfield_(il.zeros_gridcurl(vc), 0.8, -0.6, vc)
    phi = il.scalarpotential_uniformvecfield_(il.NodesPrimal.zeros(S["g"], S["dt"]), 0.8, -0.6, vc)
    v1 = il.vecfield_from_vectorpotential_(il.EdgesPrimal.zeros(S["g"], S["dt"]), psi, vc).numpy_components()
    v2 = il.vecfield_from_scalarpotential_(il.EdgesPrimal.zeros(S["g"], S["dt"]), phi, vc).numpy_components()
    tol = 1e-10 if S["dt"].itemsize == 8 else 1e-4
    for v in (v1, v2):
        assert np.abs(v[0][1:-1, 1:-1] - 0.8).max() < tol and np.abs(v[1][1:-1, 1:-1] + 0.6).max() < tol


def test_helmholtz_known_answer(S):
    """test/surface_ops.jl:312-341 on the device: the field from
    vecfield_helmholtz_ has masked curl w and masked divergence d at the
    interior nodes (1e-8 in FP64; 1e-2 in FP32, where the second differences
    of the potentials cancel most of their digits)."""
    import torch
    il = S["il"]
    vc = S["vc"]
    N = len(S["b"])
    w, wh = _rand(S, il.NodesDual, 31)
    d, dh = _rand(S, il.NodesPrimal, 32)
    dv = il.VectorData(torch.tensor(np.random.default_rng(33).standard_normal(2 * N), dtype=S["dt"], device="cuda"))
    v = il.vecfield_helmholtz_(il.EdgesPrimal.zeros(S["g"], S["dt"]), w, d, dv, (0.0, 0.0), vc, il.VectorFieldCache(vc))
    vfc = il.VectorFieldCache(vc)
    w2 = il.curl_(il.zeros_gridcurl(vc), v, vc)
    mw = il.masked_curlv_from_curlv_masked_(il.zeros_gridcurl(vc), w2, dv, vc, vfc.wcache).numpy_components()
    d2 = il.divergence_(il.NodesPrimal.zeros(S["g"], S["dt"]), v, vc)
    md = il.masked_divv_from_divv_masked_(il.NodesPrimal.zeros(S["g"], S["dt"]), d2, dv, vc, vfc.dcache).numpy_components()
    tol = 1e-8 if S["dt"] == torch.float64 else 1e-2
    assert np.abs(mw[1:-1, 1:-1] - wh[1:-1, 1:-1]).max() < tol
    assert np.abs(md[1:-1, 1:-1] - dh[1:-1, 1:-1]).max() < tol
