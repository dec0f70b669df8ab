"""Golden fixtures (tests/golden/make_golden.py): the oracle reproduces them
on the CPU, and the device solves match them on the GPU."""
import os

import numpy as np
import pytest

import ilm_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


def load(name):
    return np.load(os.path.join(HERE, "golden", name))


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max()


def test_oracle_reproduces_dirichlet_golden():
    from immersedlayers import workloads as W
    G = load("golden_dirichlet_plain.npz")
    xlim, ylim, h, b, fb = W.dirichlet_plain()
    assert np.array_equal(fb, G["fb"])
    g = O.Grid.physical(xlim, ylim, h)
    assert [g.nx, g.ny, g.i0x, g.i0y] == list(G["grid"])
    c = O.SurfaceCache(b.x, b.y, b.nx, b.ny, b.ds, g)
    f, s = O.solve_dirichlet(c, fb, np.zeros_like(fb))
    assert rel(f, G["f"]) < 1e-10 and rel(s, G["s"]) < 1e-7
    # the Schur complement has one negative (net-charge) eigenvalue
    assert G["eig"][0] < 0 < G["eig"][1]


def test_oracle_reproduces_neumann_golden():
    from immersedlayers import bodies as B
    G = load("golden_neumann_circle.npz")
    g = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), 0.04)
    b = B.circle(1.0, ds=0.056)
    c = O.SurfaceCache(b.x, b.y, b.nx, b.ny, b.ds, g)
    f, df, _, _ = O.solve_neumann(c, b.nx.copy(), np.zeros(len(b)))
    assert rel(f, G["f"]) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_device_dirichlet_matches_golden(cuda, dtype):
    import torch
    import immersedlayers as il
    from immersedlayers import workloads as W
    dt = torch.float64 if dtype == "f64" else torch.float32
    G = load("golden_dirichlet_plain.npz")
    xlim, ylim, h, b, fb = W.dirichlet_plain()
    g = il.PhysicalGrid(xlim, ylim, h)
    c = il.SurfaceScalarCache(b, g, dtype=dt)
    f, s, info = il.solve_dirichlet(c, il.ScalarData(torch.tensor(fb, dtype=dt, device="cuda")),
                                    il.ScalarData.zeros(len(b), dt), tol=1e-10)
    assert info["converged"]
    tol_f = 1e-7 if dt == torch.float64 else 1e-4
    assert rel(f.numpy_components(), G["f"]) < tol_f


@pytest.mark.gpu
def test_device_neumann_matches_golden(cuda):
    import torch
    import immersedlayers as il
    G = load("golden_neumann_circle.npz")
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), 0.04)
    b = il.circle(1.0, ds=0.056)
    c = il.SurfaceScalarCache(b, g)
    f, df, info = il.solve_neumann(c, il.ScalarData(torch.tensor(b.nx, device="cuda")), il.ScalarData.zeros(len(b)),
                                   tol=1e-10, maxiter=20000)
    assert info["converged"]
    assert rel(f.numpy_components(), G["f"]) < 1e-6
