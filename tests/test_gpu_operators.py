"""Parity of every CUDA operator with the CPU oracle on the reference's unit
test geometry (h = 0.04 on [-2,2]^2, circle R = 1, ds = 1.4 h).

Tolerances: FP64 caches 1e-12 (relative to the max magnitude), FP32 caches
2e-6 for transfers/stencils and 1e-5 for the FFT-based inverse Laplacian."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import ilm_oracle as O
from geometry import angles, oracle_cache, surface_ops_case


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def relt(a, b):
    if isinstance(b, tuple):
        return max(rel(x, y) for x, y in zip(a, b))
    return rel(a, b)


@pytest.fixture(scope="module", params=["f64", "f32"])
def setup(request, cuda):
    import torch
    import immersedlayers as il
    dt = torch.float64 if request.param == "f64" else torch.float32
    og, b = surface_ops_case()
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), og.h)
    assert (g.nx, g.ny, g.i0) == (og.nx, og.ny, (og.i0x, og.i0y))
    sc = il.SurfaceScalarCache(b, g, dtype=dt)
    vc = il.SurfaceVectorCache(b, g, dtype=dt)
    tol = 1e-12 if dt == torch.float64 else 2e-6
    return dict(il=il, torch=torch, dt=dt, g=g, og=og, b=b, sc=sc, vc=vc,
                osc=oracle_cache(og, b), ovc=oracle_cache(og, b, "vector"), tol=tol,
                itol=1e-11 if dt == torch.float64 else 1e-5)


def pdata(S, cls, arr):
    return cls(S["torch"].tensor(np.asarray(arr), dtype=S["dt"], device="cuda"))


def test_regularize_interpolate(setup):
    S = setup
    il = S["il"]
    N = len(S["b"])
    rng = np.random.default_rng(1)
    f = rng.standard_normal(N)
    for cls, kind in [(il.NodesPrimal, O.NODES_PRIMAL), (il.NodesDual, O.NODES_DUAL)]:
        out = cls.zeros(S["g"], S["dt"])
        out.fill_(7.0)   # regularize! overwrites (fill 0 + mul!)
        il.regularize_(out, pdata(S, il.ScalarData, f), S["sc"])
        assert rel(out.numpy_components(), S["osc"].reg_cls(f, kind)) < S["tol"]
        s = out.numpy_components()
        fo = il.ScalarData.zeros(N, S["dt"])
        il.interpolate_(fo, out, S["sc"])
        assert rel(fo.numpy(), S["osc"].interp_cls(s, kind)) < S["tol"]
    v = rng.standard_normal(2 * N)
    q = il.EdgesPrimal.zeros(S["g"], S["dt"])
    il.regularize_(q, pdata(S, il.VectorData, v), S["sc"])
    assert relt(q.numpy_components(), O.regularize_vector(S["osc"], v)) < S["tol"]
    vo = il.VectorData.zeros(N, S["dt"])
    il.interpolate_(vo, q, S["sc"])
    assert rel(vo.numpy(), O.interpolate_vector(S["osc"], q.numpy_components())) < S["tol"]


def test_normal_transfers_scalar(setup):
    S = setup
    il = S["il"]
    N = len(S["b"])
    f = np.sin(angles(N) - math.pi / 4)
    q = il.EdgesPrimal.zeros(S["g"], S["dt"])
    il.regularize_normal_(q, pdata(S, il.ScalarData, f), S["sc"])
    assert relt(q.numpy_components(), O.regularize_normal(S["osc"], f)) < S["tol"]
    fo = il.ScalarData.zeros(N, S["dt"])
    il.normal_interpolate_(fo, q, S["sc"])
    ref = O.normal_interpolate(S["osc"], O.regularize_normal(S["osc"], f))
    assert rel(fo.numpy(), ref) < 10 * S["tol"]
    # test/surface_ops.jl:66-67 on the device result
    assert abs(fo.numpy().max() - 11) < 1.0 and abs(fo.numpy().min() + 11) < 1.0
    il.regularize_normal_cross_(q, pdata(S, il.ScalarData, f), S["sc"])
    assert relt(q.numpy_components(), O.regularize_normal_cross(S["osc"], f)) < S["tol"]
    il.normal_cross_interpolate_(fo, q, S["sc"])
    assert rel(fo.numpy(), O.normal_cross_interpolate(S["osc"], q.numpy_components())) < S["tol"]


def test_vector_transfers(setup):
    S = setup
    il = S["il"]
    N = len(S["b"])
    rng = np.random.default_rng(2)
    v = rng.standard_normal(2 * N)
    t = il.EdgeGradientPrimal.zeros(S["g"], S["dt"])
    il.regularize_normal_(t, pdata(S, il.VectorData, v), S["vc"])
    assert relt(t.numpy_components(), O.regularize_normal_tensor(S["ovc"], v)) < S["tol"]
    vo = il.VectorData.zeros(N, S["dt"])
    il.normal_interpolate_(vo, t, S["vc"])
    assert rel(vo.numpy(), O.normal_interpolate_tensor(S["ovc"], t.numpy_components())) < S["tol"]
    il.regularize_normal_symm_(t, pdata(S, il.VectorData, v), S["vc"])
    assert relt(t.numpy_components(), O.regularize_normal_symm(S["ovc"], v)) < S["tol"]
    il.normal_interpolate_symm_(vo, t, S["vc"])
    assert rel(vo.numpy(), O.normal_interpolate_symm(S["ovc"], t.numpy_components())) < 10 * S["tol"]
    # normal dot / cross with vector data
    p = il.NodesPrimal.zeros(S["g"], S["dt"])
    il.regularize_normal_dot_(p, pdata(S, il.VectorData, v), S["vc"])
    assert rel(p.numpy_components(), O.regularize_normal_dot(S["ovc"], v)) < S["tol"]
    il.normal_dot_interpolate_(vo, p, S["vc"])
    assert rel(vo.numpy(), O.normal_dot_interpolate(S["ovc"], p.numpy_components())) < S["tol"]


def test_stencils(setup):
    S = setup
    il = S["il"]
    g, og = S["g"], S["og"]
    rng = np.random.default_rng(3)
    dsc = 1.0 / og.h
    w = rng.standard_normal(og.shape(O.NODES_PRIMAL))
    wp = il.NodesPrimal.zeros(g, S["dt"]).set_numpy(w)
    q = il.EdgesPrimal.zeros(g, S["dt"])
    il.grad_(q, wp, S["sc"])
    ref = tuple(x * dsc for x in O.grad_nodes(wp.numpy_components(), og))
    assert relt(q.numpy_components(), ref) < S["tol"]
    out = il.NodesPrimal.zeros(g, S["dt"])
    il.divergence_(out, q, S["sc"])
    assert rel(out.numpy_components(), O.divergence_edges(q.numpy_components()) * dsc) < S["tol"]
    sd = il.NodesDual.zeros(g, S["dt"]).set_numpy(rng.standard_normal(og.shape(O.NODES_DUAL)))
    il.curl_(q, sd, S["sc"])
    assert relt(q.numpy_components(), tuple(x * dsc for x in O.curl_nodes_dual(sd.numpy_components(), og))) < S["tol"]
    wd = il.NodesDual.zeros(g, S["dt"])
    il.curl_(wd, q, S["sc"])
    assert rel(wd.numpy_components(), O.curl_edges(q.numpy_components(), og) * dsc) < S["tol"]
    t = il.EdgeGradientPrimal.zeros(g, S["dt"])
    il.grad_(t, q, S["vc"])
    assert relt(t.numpy_components(), tuple(x * dsc for x in O.grad_edges(q.numpy_components(), og))) < S["tol"]
    q2 = il.EdgesPrimal.zeros(g, S["dt"])
    il.divergence_(q2, t, S["vc"])
    assert relt(q2.numpy_components(),
                tuple(x * dsc for x in O.divergence_edgegrad(t.numpy_components(), og))) < S["tol"]
    lap = il.NodesPrimal.zeros(g, S["dt"])
    il.laplacian_(lap, wp, S["sc"])
    assert rel(lap.numpy_components(), O.laplacian_nodes(wp.numpy_components(), 1 / og.h ** 2)) < S["tol"]


def test_inverse_laplacian(setup):
    S = setup
    il = S["il"]
    g, og = S["g"], S["og"]
    rng = np.random.default_rng(4)
    for cls, pc in [(il.NodesPrimal, O.NODES_PRIMAL), (il.NodesDual, O.NODES_DUAL)]:
        w = np.zeros(og.shape(pc))
        w[30:70, 20:80] = rng.standard_normal((40, 60))
        src = cls.zeros(g, S["dt"]).set_numpy(w)
        out = cls.zeros(g, S["dt"])
        il.inverse_laplacian_(out, src, S["sc"])
        ref = S["osc"].inverse_laplacian(src.numpy_components())
        assert rel(out.numpy_components(), ref) < S["itol"]
        il.inverse_laplacian_(src, S["sc"])   # in place
        assert rel(src.numpy_components(), ref) < S["itol"]


def test_composite_layer_operators(setup):
    S = setup
    il = S["il"]
    g, og = S["g"], S["og"]
    c, oc = S["sc"], S["osc"]
    N = len(S["b"])
    rng = np.random.default_rng(5)
    f = rng.standard_normal(N)
    fd = pdata(S, il.ScalarData, f)
    th = il.NodesPrimal.zeros(g, S["dt"])
    il.surface_divergence_(th, fd, c)
    assert rel(th.numpy_components(), O.surface_divergence(oc, f)) < S["tol"]
    fo = il.ScalarData.zeros(N, S["dt"])
    il.surface_grad_(fo, th, c)
    assert rel(fo.numpy(), O.surface_grad(oc, th.numpy_components())) < 10 * S["tol"]
    w = il.NodesDual.zeros(g, S["dt"])
    il.surface_curl_(w, fd, c)
    assert rel(w.numpy_components(), O.surface_curl_T(oc, f)) < S["tol"]
    il.surface_curl_(fo, w, c)
    assert rel(fo.numpy(), O.surface_curl(oc, w.numpy_components())) < 10 * S["tol"]
    il.surface_curl_cross_(w, fd, c)
    assert rel(w.numpy_components(), O.surface_curl_cross_T(oc, f)) < S["tol"]
    il.surface_curl_cross_(fo, w, c)
    assert rel(fo.numpy(), O.surface_curl_cross(oc, w.numpy_components())) < 10 * S["tol"]
    il.surface_divergence_cross_(th, fd, c)
    assert rel(th.numpy_components(), O.surface_divergence_cross(oc, f)) < S["tol"]
    il.surface_grad_cross_(fo, th, c)
    assert rel(fo.numpy(), O.surface_grad_cross(oc, th.numpy_components())) < 10 * S["tol"]
    # vector cache: surface_divergence / grad (symm)
    v = rng.standard_normal(2 * N)
    vd = pdata(S, il.VectorData, v)
    q = il.EdgesPrimal.zeros(g, S["dt"])
    il.surface_divergence_symm_(q, vd, S["vc"])
    assert relt(q.numpy_components(), O.surface_divergence_symm(S["ovc"], v)) < S["tol"]
    vo = il.VectorData.zeros(N, S["dt"])
    il.surface_grad_symm_(vo, q, S["vc"])
    assert rel(vo.numpy(), O.surface_grad_symm(S["ovc"], q.numpy_components())) < 10 * S["tol"]


def test_masks_and_integrals(setup):
    S = setup
    il = S["il"]
    c = S["sc"]
    m = il.mask(c)
    ref = O.mask(S["osc"])
    assert rel(m.numpy_components(), ref) < S["itol"]
    assert abs(il.integrate(m, c) - math.pi) < 2e-3                   # test/surface_ops.jl:186
    wm = il.mask(c, il.NodesDual)
    assert abs(il.integrate(wm, c) - math.pi) < 1e-3                  # :198
    cm = il.complementary_mask(c)
    assert rel(cm.numpy_components(), 1.0 - ref) < S["itol"]
    os_ = il.ones_surface(c)
    assert abs(il.dot(os_, os_, c) - S["b"].ds.sum()) < 1e-6


def test_schur_builds_match_column_loops(setup):
    S = setup
    if S["dt"] != S["torch"].float64:
        pytest.skip("Schur builds are FP64")
    il = S["il"]
    h = S["og"].h
    c, oc = S["sc"], S["osc"]
    for fn, ofn, sc in [(il.create_RTLinvR, O.create_RTLinvR, 1.0), (il.create_CLinvCT, O.create_CLinvCT, h),
                        (il.create_GLinvD, O.create_GLinvD, h), (il.create_nRTRn, O.create_nRTRn, 1.0)]:
        A = fn(c, scale=sc).cpu().numpy()
        Ar = ofn(oc, scale=sc)
        assert rel(A, Ar) < 1e-11, fn.__name__
    A = il.create_CLinvCT(c, scale=h).cpu().numpy()
    assert abs(np.abs(np.linalg.eigvals(A)).max() - 0.2) < 0.1        # test/surface_ops.jl:71


def test_determinism(setup):
    S = setup
    il = S["il"]
    torch = S["torch"]
    N = len(S["b"])
    f = pdata(S, il.ScalarData, np.random.default_rng(6).standard_normal(N))
    a = il.NodesPrimal.zeros(S["g"], S["dt"])
    b = il.NodesPrimal.zeros(S["g"], S["dt"])
    il.surface_divergence_(a, f, S["sc"])
    il.inverse_laplacian_(a, S["sc"])
    il.surface_divergence_(b, f, S["sc"])
    il.inverse_laplacian_(b, S["sc"])
    assert torch.equal(a.data, b.data)


@pytest.mark.parametrize("n1,n2", [(32, 32), (48, 200), (64, 96), (127, 64), (192, 130), (256, 384), (383, 48),
                                   (512, 256), (40, 1100)])
def test_inverse_laplacian_fft_sizes(cuda, n1, n2):
    """FP32 LGF convolution at every padded length of the register four-step
    path (64 ... 1024, powers of two and 3 x powers of two) and at lengths
    that take the Stockham path (rows of 32 / columns of 2048)."""
    import torch
    import immersedlayers as il
    h = 0.01
    g = il.PhysicalGrid(h=h, nx=n1 + 1, ny=n2 + 1)
    og = O.Grid(n1 + 1, n2 + 1, h, (n1 + 1) // 2, (n2 + 1) // 2)
    c = il.SurfaceScalarCache(None, g, dtype=torch.float32)
    rng = np.random.default_rng(n1 * 7 + n2)
    w = rng.standard_normal((n1, n2))
    src = il.NodesPrimal.zeros(g, torch.float32).set_numpy(w)
    out = il.NodesPrimal.zeros(g, torch.float32)
    il.inverse_laplacian_(out, src, c)
    ref = O.InverseLaplacian(n1, n2, 1.0 / h ** 2)(src.numpy_components())
    assert rel(out.numpy_components(), ref) < 2e-5
