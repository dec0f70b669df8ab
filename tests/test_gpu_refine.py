"""Parity at every grid size of the batched configuration, and the FP64
iterative refinement.

The golden fixtures (tests/golden/make_golden.py, `batched`) hold the
oracle's FP64 dense-LU solutions (test/literate/problems.jl:259-298,
neumann.jl:101-142) of one Dirichlet and one Neumann problem of the batched
configuration for each grid size 128, 192, 256, 384, 512.

Tolerances (relative, max norm; f normalised by max |f| of the oracle field,
s by max |s|):
  * refined solves (FP64 outputs after FP64 refinement): 1e-10 for f and s;
  * FP32 batched fields: 1e-5 with the right-hand-side operator and for the
    Dirichlet problems of the default path; the default path's Neumann
    problems form their Schur right-hand side from the gradient of the FP32
    potential f*, whose rounding the near-null per-body modes of the Neumann
    Schur complement amplify: 2e-5 there (the refined solve removes it);
  * FP32 surface strengths: 1e-5 with the right-hand-side operator.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def golden():
    return np.load(os.path.join(HERE, "golden", "golden_batched.npz"))


def specs_of(G):
    from immersedlayers import workloads as W
    from immersedlayers.batch import BatchProblemSpec
    out = []
    for i in G["problems"]:
        n, h, bl, kind, f = W.batch_problem(int(i))
        out.append(BatchProblemSpec(n, h, bl, kind, f))
    return out


def errors(bs, f, s, G, specs):
    st = int(G["f_stride"])
    rows = []
    for k, i in enumerate(G["problems"]):
        fg = bs.field(f, k).double().cpu().numpy().T
        sg = bs.surface(s, k).double().cpu().numpy()
        ef = np.abs(fg[::st, ::st] - G[f"f_{i}"]).max() / float(G[f"fmax_{i}"])
        sr = G[f"s_{i}"]
        es = np.abs(sg - sr).max() / np.abs(sr).max()
        rows.append((int(i), specs[k].nx, specs[k].kind, ef, es))
    return rows


def test_golden_batched_covers_every_grid_size():
    from immersedlayers import workloads as W
    G = golden()
    seen = {(int(G[f"meta_{i}"][0]), int(G[f"meta_{i}"][1])) for i in G["problems"]}
    assert seen == {(n, k) for n in W.BATCH_SIZES for k in (0, 1)}


@pytest.mark.parametrize("dtype", ["f32", "f64"])
@pytest.mark.parametrize("precond", ["none", "bjacobi"])
def test_batch_refined_matches_oracle_at_every_grid_size(cuda, dtype, precond):
    """FP64 refinement of FP32 (and FP64) batches: FP64 Schur residual
    <= 1e-12, f and s within 1e-10 of the oracle at every grid size."""
    import torch
    from immersedlayers.batch import BatchSolver
    G = golden()
    specs = specs_of(G)
    bs = BatchSolver(specs, dtype=torch.float32 if dtype == "f32" else torch.float64)
    if precond != "none":
        bs.set_precond(precond, 32)
    fp = torch.tensor(np.concatenate([s.fplus for s in specs]), dtype=torch.float64, device="cuda")
    fm = torch.tensor(np.concatenate([s.fminus for s in specs]), dtype=torch.float64, device="cuda")
    f, s = bs.solve_refined(fp, fm, tol=1e-12)
    torch.cuda.synchronize()
    assert f.dtype == torch.float64 and s.dtype == torch.float64
    its, rr = bs.info()
    assert (rr <= 1e-12).all(), (its, rr)
    for i, n, kind, ef, es in errors(bs, f, s, G, specs):
        assert ef < 1e-10 and es < 1e-10, (i, n, kind, ef, es)
    # the batch's regular solve still works after a refined one
    fp32, fm32 = bs.surface_data()
    bs.solve(fp32, fm32, tol=1e-8)
    its2, rr2 = bs.info()
    assert (rr2 <= 1e-8).all()


@pytest.mark.parametrize("rhs_operator", [False, True])
def test_batch_fp32_matches_oracle_at_every_grid_size(cuda, rhs_operator):
    import torch
    from immersedlayers.batch import BatchSolver
    G = golden()
    specs = specs_of(G)
    bs = BatchSolver(specs, dtype=torch.float32)
    if rhs_operator:
        bs.set_rhs_operator(True)
    fp, fm = bs.surface_data()
    f, s = bs.solve(fp, fm, tol=1e-8)
    torch.cuda.synchronize()
    its, rr = bs.info()
    assert (rr <= 1e-8).all(), (its, rr)
    for i, n, kind, ef, es in errors(bs, f, s, G, specs):
        tol_f = 1e-5 if (rhs_operator or kind == 0) else 2e-5
        assert ef < tol_f, (i, n, kind, ef)
        if rhs_operator:
            assert es < 1e-5, (i, n, kind, es)


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_dirichlet_refined_config1(cuda, dtype):
    """The plain Dirichlet configuration (157 points, cond(S) ~ 4e4):
    refined f and s within 1e-10 of the oracle, from an FP32 or FP64 cache;
    the FP32 cache's own solve within 1e-5 on f."""
    import torch
    import immersedlayers as il
    from immersedlayers import workloads as W
    G = np.load(os.path.join(HERE, "golden", "golden_dirichlet_plain.npz"))
    xlim, ylim, h, b, fb = W.dirichlet_plain()
    dt = torch.float32 if dtype == "f32" else torch.float64
    g = il.PhysicalGrid(xlim, ylim, h)
    c = il.SurfaceScalarCache(b, g, dtype=dt)
    fp = il.ScalarData(torch.tensor(fb, dtype=torch.float64, device="cuda"))
    fm = il.ScalarData.zeros(len(b), torch.float64)
    f, s, info = il.solve_dirichlet_refined(c, fp, fm, tol=1e-12)
    assert info["converged"] and info["rel_residual"] <= 1e-12, info
    fr, sr = G["f"], G["s"]
    ef = np.abs(f.numpy_components() - fr).max() / np.abs(fr).max()
    es = np.abs(s.numpy() - sr).max() / np.abs(sr).max()
    assert ef < 1e-10 and es < 1e-10, (ef, es, info)
    if dt == torch.float32:
        f32, s32, info32 = il.solve_dirichlet(c, il.ScalarData(fp.data.float()), il.ScalarData(fm.data.float()),
                                              tol=1e-8)
        ef32 = np.abs(f32.numpy_components() - fr).max() / np.abs(fr).max()
        assert ef32 < 1e-5, ef32


def test_neumann_refined_circle(cuda):
    import torch
    import immersedlayers as il
    from immersedlayers import bodies as B
    G = np.load(os.path.join(HERE, "golden", "golden_neumann_circle.npz"))
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), 0.04)
    b = B.circle(1.0, ds=1.4 * 0.04)
    c = il.SurfaceScalarCache(b, g, dtype=torch.float32)
    vp = il.ScalarData(torch.tensor(b.nx.copy(), dtype=torch.float64, device="cuda"))
    vm = il.ScalarData.zeros(len(b), torch.float64)
    f, df, info = il.solve_neumann_refined(c, vp, vm, tol=1e-12)
    assert info["converged"], info
    ef = np.abs(f.numpy_components() - G["f"]).max() / np.abs(G["f"]).max()
    es = np.abs(df.numpy() - G["df"]).max() / np.abs(G["df"]).max()
    assert ef < 1e-10 and es < 1e-10, (ef, es, info)


def test_refined_cache_follows_moved_points(cuda):
    """After ilm_cache_update_points the refinement's FP64 cache is rebuilt
    at the new points: the refined solve matches the oracle there."""
    import torch
    import immersedlayers as il
    import ilm_oracle as O
    from immersedlayers import bodies as B
    h = 0.04
    g = il.PhysicalGrid((-2.0, 2.0), (-2.0, 2.0), h)
    b = B.circle(0.8, ds=1.4 * h)
    c = il.SurfaceScalarCache(b, g, dtype=torch.float32)
    fb = np.cos(3 * np.arctan2(b.y, b.x))
    fp = il.ScalarData(torch.tensor(fb, dtype=torch.float64, device="cuda"))
    fm = il.ScalarData.zeros(len(b), torch.float64)
    il.solve_dirichlet_refined(c, fp, fm, tol=1e-12)
    x2, y2 = b.x + 0.13, b.y - 0.07
    t = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    c.update_points_(t(x2), t(y2), t(b.nx), t(b.ny), t(b.ds))
    f, s, info = il.solve_dirichlet_refined(c, fp, fm, tol=1e-12)
    assert info["converged"], info
    og = O.Grid(g.nx, g.ny, g.h, *g.i0)
    oc = O.SurfaceCache(x2, y2, b.nx, b.ny, b.ds, og)
    fr, sr = O.solve_dirichlet(oc, fb, np.zeros_like(fb))
    assert np.abs(f.numpy_components() - fr).max() / np.abs(fr).max() < 1e-10
    assert np.abs(s.numpy() - sr).max() / np.abs(sr).max() < 1e-10


def test_batch_coarse_correction(cuda):
    """Block-Jacobi with the per-body coarse correction on the Neumann
    problems (ilm_batch_set_coarse): the same FP32 accuracy against the
    oracle at every grid size, and fewer CG iterations on the Neumann
    problems than block-Jacobi alone; the correction can be switched off."""
    import torch
    from immersedlayers.batch import BatchSolver
    G = golden()
    specs = specs_of(G)
    bs = BatchSolver(specs, dtype=torch.float32)
    bs.set_rhs_operator(True)
    bs.set_precond("bjacobi", 64)
    fp, fm = bs.surface_data()
    neu = np.array([s.kind == 1 for s in specs])
    bs.solve(fp, fm, tol=1e-8)
    its0, rr0 = bs.info()
    bs.set_coarse(True)
    f, s = bs.solve(fp, fm, tol=1e-8)
    torch.cuda.synchronize()
    its1, rr1 = bs.info()
    assert (rr0 <= 1e-8).all() and (rr1 <= 1e-8).all(), (rr0, rr1)
    for i, n, kind, ef, es in errors(bs, f, s, G, specs):
        assert ef < 1e-5 and es < 1e-5, (i, n, kind, ef, es)
    assert (its1[~neu] == its0[~neu]).all()           # Dirichlet problems untouched
    assert its1[neu].sum() < 0.85 * its0[neu].sum(), (its0[neu], its1[neu])
    bs.set_coarse(False)
    bs.solve(fp, fm, tol=1e-8)
    its2, _ = bs.info()
    assert (its2 == its0).all()
