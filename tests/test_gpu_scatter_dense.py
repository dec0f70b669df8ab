"""DDF regularization with densely spaced points, where a 32 x 8 tile holds
more than 64 candidate points (the bucketed tile sum) and more than 256
(several staging chunks): a circle at ds = 0.3 h and a plate 2h thick at
ds = 0.25 h on h = 0.02, against the oracle, FP64 (1e-12) and FP32 (2e-6),
overwriting (regularize!) and accumulating (the point-forcing path)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import ilm_oracle as O


def rel(a, b):
    a = np.concatenate([np.ravel(x) for x in a]) if isinstance(a, tuple) else np.ravel(a)
    b = np.concatenate([np.ravel(x) for x in b]) if isinstance(b, tuple) else np.ravel(b)
    return np.abs(a - b).max() / np.abs(b).max()


def dense_case():
    from immersedlayers import bodies as B
    h = 0.02
    og = O.Grid.physical((-1.0, 1.0), (-1.0, 1.0), h)
    bl = B.BodyList()
    bl.append(B.circle(0.4, ds=0.3 * h, center=(-0.3, 0.2)))
    bl.append(B.rectangle(0.35, h, ds=0.25 * h, center=(0.3, -0.45)))
    return og, bl


@pytest.mark.parametrize("ddf", ["Yang3", "M4prime"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_regularize_dense_points(cuda, dtype, ddf):
    import torch
    import immersedlayers as il
    from immersedlayers import _lib as L
    from immersedlayers.core import _ptr
    dt = torch.float64 if dtype == "f64" else torch.float32
    tol = 1e-12 if dt == torch.float64 else 2e-6
    og, bl = dense_case()
    g = il.PhysicalGrid((-1.0, 1.0), (-1.0, 1.0), og.h)
    sc = il.SurfaceScalarCache(bl, g, ddftype=ddf, dtype=dt)
    vc = il.SurfaceVectorCache(bl, g, ddftype=ddf, dtype=dt)
    osc = O.SurfaceCache(bl.x, bl.y, bl.nx, bl.ny, bl.ds, og, ddftype=ddf)
    ovc = O.SurfaceCache(bl.x, bl.y, bl.nx, bl.ny, bl.ds, og, kind="vector", ddftype=ddf)
    N = len(bl)
    rng = np.random.default_rng(3)
    f = rng.standard_normal(N)
    fd = il.ScalarData(torch.tensor(f, dtype=dt, device="cuda"))
    for cls, kind in [(il.NodesPrimal, O.NODES_PRIMAL), (il.NodesDual, O.NODES_DUAL)]:
        out = cls.zeros(g, dt)
        out.fill_(5.0)
        il.regularize_(out, fd, sc)
        ref = osc.reg_cls(f, kind)
        assert rel(out.numpy_components(), ref) < tol, cls.__name__
        # accumulating scatter (occupied tiles only): out + R f
        L.call("ilm_regularize_add", sc._h, out.kind, _ptr(fd.data), _ptr(out.data), None)
        assert rel(out.numpy_components(), 2 * ref) < tol, cls.__name__
    v = rng.standard_normal(2 * N)
    q = il.EdgesPrimal.zeros(g, dt)
    il.regularize_(q, il.VectorData(torch.tensor(v, dtype=dt, device="cuda")), vc)
    assert rel(q.numpy_components(), O.regularize_vector(ovc, v)) < tol
