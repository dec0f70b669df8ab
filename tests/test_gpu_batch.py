"""Batched Dirichlet/Neumann solves (many problems, different grids, one
launch per stage) against per-problem oracle solves with dense LU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import ilm_oracle as O


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max()


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_batch_matches_oracle(cuda, dtype):
    import torch
    from immersedlayers import workloads as W
    from immersedlayers.batch import BatchSolver
    dt = torch.float64 if dtype == "f64" else torch.float32
    specs = W.batch_specs(6, sizes=(64, 96, 128))
    bs = BatchSolver(specs, dtype=dt)
    fp, fm = bs.surface_data()
    f, s = bs.solve(fp, fm, tol=1e-10, maxiter=20000)
    torch.cuda.synchronize()
    its, rr = bs.info()
    assert (rr <= 1e-10).all(), (its, rr)
    for i, sp in enumerate(specs):
        g = O.Grid(sp.nx, sp.ny, sp.h, *sp.i0)
        bl = sp.bl
        oc = O.SurfaceCache(bl.x, bl.y, bl.nx, bl.ny, bl.ds, g)
        if sp.kind == 0:
            fr, sr = O.solve_dirichlet(oc, sp.fplus, sp.fminus)
        else:
            fr, sr, _, _ = O.solve_neumann(oc, sp.fplus, sp.fminus)
        fg = bs.field(f, i).double().cpu().numpy().T
        # FP64: CG residual 1e-10; FP32: grid work in FP32 (the Neumann
        # right-hand side differentiates the FP32 potential f*)
        tol_f = 1e-9 if dt == torch.float64 else (1e-5 if sp.kind == 0 else 2e-5)
        assert rel(fg, fr) < tol_f, (i, sp.kind, rel(fg, fr))


def test_batch_split_schur_build_matches_single_kind_batches(cuda):
    """A batch with both kinds builds its Schur complements in two launches
    (the Neumann problems' first; their block inverses wait only for that
    launch).  Each problem of such a batch solves, bit for bit and in the
    same iterations, as it does in a batch of its kind alone (one launch)."""
    import torch
    from immersedlayers import workloads as W
    from immersedlayers.batch import BatchSolver
    specs = W.batch_specs(8, sizes=(64, 96))
    assert {sp.kind for sp in specs} == {0, 1}

    def run(sub):
        bs = BatchSolver(sub, dtype=torch.float32)
        bs.set_precond("bjacobi", 32)
        fp, fm = bs.surface_data()
        f, s = bs.solve(fp, fm, tol=1e-8, maxiter=20000)
        torch.cuda.synchronize()
        its, rr = bs.info()
        assert (rr <= 1e-8).all(), rr
        return [(bs.field(f, i).clone(), bs.surface(s, i).clone()) for i in range(len(sub))], its.copy()

    mixed, its_m = run(specs)
    for kind in (0, 1):
        idx = [i for i, sp in enumerate(specs) if sp.kind == kind]
        alone, its_a = run([specs[i] for i in idx])
        for j, i in enumerate(idx):
            df = (alone[j][0] - mixed[i][0]).abs().max().item()
            ds = (alone[j][1] - mixed[i][1]).abs().max().item()
            assert df == 0 and ds == 0, (kind, i, df, ds)
            assert its_a[j] == its_m[i], (kind, i, its_a[j], its_m[i])


def test_batch_block_jacobi_matches_plain(cuda):
    """Flexible CG with the block-Jacobi preconditioner reaches the same
    FP64 residual and the same solution as plain CG, in fewer iterations."""
    import torch
    from immersedlayers import workloads as W
    from immersedlayers.batch import BatchSolver
    specs = W.batch_specs(8, sizes=(96, 128, 192))
    bs = BatchSolver(specs, dtype=torch.float64)
    fp, fm = bs.surface_data()
    f0, s0 = bs.solve(fp, fm, tol=1e-10, maxiter=20000)
    it0, rr0 = bs.info()
    bs.set_precond("bjacobi", 32)
    f1, s1 = bs.solve(fp, fm, tol=1e-10, maxiter=20000)
    it1, rr1 = bs.info()
    assert (rr1 <= 1e-10).all(), rr1
    assert it1.sum() < it0.sum(), (it0, it1)
    assert rel(f1.cpu().numpy(), f0.cpu().numpy()) < 1e-7
    bs.set_precond("none")
    f2, s2 = bs.solve(fp, fm, tol=1e-10, maxiter=20000)
    assert torch.equal(f2, f0)


def test_batch_is_deterministic(cuda):
    import torch
    from immersedlayers import workloads as W
    from immersedlayers.batch import BatchSolver
    specs = W.batch_specs(4, sizes=(64, 96))
    bs = BatchSolver(specs, dtype=torch.float32)
    fp, fm = bs.surface_data()
    f1, s1 = bs.solve(fp, fm, tol=1e-8)
    f2, s2 = bs.solve(fp, fm, tol=1e-8)
    assert torch.equal(f1, f2) and torch.equal(s1, s2)


def test_batch_large_grids_match_single_solves(cuda):
    """Batched FP32 solves on the large grid sizes (padded FFT lengths 512,
    768, 1024; source boxes much smaller than the grids) against the
    single-problem FP64 device solves, which the oracle tests pin."""
    import torch
    import immersedlayers as il
    from immersedlayers import workloads as W
    from immersedlayers.batch import BatchSolver
    specs = W.batch_specs(6, sizes=(256, 384, 512))
    bs = BatchSolver(specs, dtype=torch.float32)
    fp, fm = bs.surface_data()
    f, s = bs.solve(fp, fm, tol=1e-8)
    torch.cuda.synchronize()
    its, rr = bs.info()
    assert (rr <= 1e-8).all(), (its, rr)
    st = bs.stats()
    assert st["box_cells"] < st["cells"]
    for i, sp in enumerate(specs):
        g = il.PhysicalGrid(h=sp.h, nx=sp.nx, ny=sp.ny, i0=sp.i0)
        c = il.SurfaceScalarCache(sp.bl, g, dtype=torch.float64)
        p = il.ScalarData(torch.tensor(sp.fplus, dtype=torch.float64, device="cuda"))
        m = il.ScalarData(torch.tensor(sp.fminus, dtype=torch.float64, device="cuda"))
        if sp.kind == 0:
            fr, _, info = il.solve_dirichlet(c, p, m, tol=1e-10, maxiter=20000)
        else:
            fr, _, info = il.solve_neumann(c, p, m, tol=1e-10, maxiter=20000)
        ref = fr.data.view(sp.ny - 1, sp.nx - 1).double()
        got = bs.field(f, i).double()
        err = ((got - ref).abs().max() / ref.abs().max()).item()
        assert err < (1e-5 if sp.kind == 0 else 2e-5), (i, sp.kind, sp.nx, err)


@pytest.mark.parametrize("precond", ["none", "bjacobi"])
def test_batch_cg_variants_agree(cuda, precond):
    """The row-distributed (256-, 128- and 512-thread CTAs), the
    replicated-vector and the size-split (small problems one CTA each)
    Schur CG kernels reach the tolerance and the same solution; the
    autotuner keeps one of them."""
    import torch
    from immersedlayers import workloads as W
    from immersedlayers.batch import BatchSolver
    specs = W.batch_specs(8, sizes=(96, 128, 192))
    bs = BatchSolver(specs, dtype=torch.float64)
    if precond != "none":
        bs.set_precond(precond, 32)
    fp, fm = bs.surface_data()
    out = {}
    for v in range(1, 7):
        bs.set_cg_variant(v)
        f, s = bs.solve(fp, fm, tol=1e-10, maxiter=20000)
        its, rr = bs.info()
        assert (rr <= 1e-10).all(), (v, its, rr)
        out[v] = f.clone()
    assert rel(out[2].cpu().numpy(), out[1].cpu().numpy()) < 1e-8
    for v in range(3, 7):
        assert rel(out[v].cpu().numpy(), out[1].cpu().numpy()) < 1e-8, v
    chosen, ms = bs.autotune(fp, fm, tol=1e-10, maxiter=20000, reps=1)
    assert chosen in range(1, 7) and chosen in ms and bs.cg_variant()[0] == chosen
    assert len(ms) == 6


def test_batch_graph_replay_matches_solve(cuda):
    """The captured CUDA graph of a batch solve gives bit-identical fields
    to the launch-by-launch solve, on its first (capture) and later
    (replay) calls and after a change of preconditioner (re-capture)."""
    import torch
    from immersedlayers import workloads as W
    from immersedlayers.batch import BatchSolver
    specs = W.batch_specs(6, sizes=(64, 96, 128))
    bs = BatchSolver(specs, dtype=torch.float32)
    fp, fm = bs.surface_data()
    st = torch.cuda.Stream()
    f0, s0 = bs.solve(fp, fm, tol=1e-8, stream=st)
    f1 = torch.empty_like(f0)
    s1 = torch.empty_like(s0)
    for _ in range(2):
        f1.zero_()
        bs.solve(fp, fm, f1, s1, tol=1e-8, stream=st, graph=True)
        st.synchronize()
        assert torch.equal(f1, f0) and torch.equal(s1, s0)
    bs.set_precond("bjacobi", 32)
    f2, s2 = bs.solve(fp, fm, tol=1e-8, stream=st)
    bs.solve(fp, fm, f1, s1, tol=1e-8, stream=st, graph=True)
    st.synchronize()
    assert torch.equal(f1, f2) and torch.equal(s1, s2)
    its, rr = bs.info()
    assert (rr <= 1e-8).all()


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_batch_rhs_operator_matches_default_path(cuda, dtype):
    """With the precomputed right-hand-side operator (one convolution per
    solve) the fields and surface strengths match the default two-convolution
    path, for Dirichlet and Neumann problems and through the captured graph;
    switching it off restores the default path exactly."""
    import torch
    from immersedlayers import workloads as W
    from immersedlayers.batch import BatchSolver
    dt = torch.float64 if dtype == "f64" else torch.float32
    specs = W.batch_specs(8, sizes=(64, 96, 128, 192))
    bs = BatchSolver(specs, dtype=dt)
    fp, fm = bs.surface_data()
    f0, s0 = bs.solve(fp, fm, tol=1e-10, maxiter=20000)
    f0, s0 = f0.clone(), s0.clone()
    bs.set_rhs_operator(True)
    f1, s1 = bs.solve(fp, fm, tol=1e-10, maxiter=20000)
    its, rr = bs.info()
    assert (rr <= 1e-10).all(), (its, rr)
    tol = 1e-9 if dtype == "f64" else 2e-5
    for i in range(len(specs)):
        a, b = bs.field(f1, i).double(), bs.field(f0, i).double()
        assert ((a - b).abs().max() / b.abs().max()).item() < tol, (i, specs[i].kind)
    assert rel(s1.cpu().numpy(), s0.cpu().numpy()) < (1e-8 if dtype == "f64" else 1e-4)
    st = torch.cuda.Stream()
    f2 = torch.empty_like(f1)
    s2 = torch.empty_like(s1)
    bs.solve(fp, fm, f2, s2, tol=1e-10, maxiter=20000, stream=st, graph=True)
    st.synchronize()
    assert torch.equal(f2, f1) and torch.equal(s2, s1)
    bs.set_rhs_operator(False)
    f3, s3 = bs.solve(fp, fm, tol=1e-10, maxiter=20000)
    assert torch.equal(f3, f0) and torch.equal(s3, s0)
    # repeated solves with the operator on and new surface data: the second
    # solve's fields match the default path on that data (a leftover
    # accumulation in f*'s source from the previous solve would show here)
    g = torch.Generator(device="cuda").manual_seed(3)
    fp2 = torch.randn(fp.shape, generator=g, device="cuda", dtype=dt)
    fm2 = 0.5 * torch.randn(fm.shape, generator=g, device="cuda", dtype=dt)
    f4, s4 = bs.solve(fp2, fm2, tol=1e-10, maxiter=20000)
    f4, s4 = f4.clone(), s4.clone()
    bs.set_rhs_operator(True)
    bs.solve(fp, fm, tol=1e-10, maxiter=20000)   # leaves the previous data's source behind
    f5, s5 = bs.solve(fp2, fm2, tol=1e-10, maxiter=20000)
    its, rr = bs.info()
    assert (rr <= 1e-10).all(), (its, rr)
    for i in range(len(specs)):
        a, b = bs.field(f5, i).double(), bs.field(f4, i).double()
        assert ((a - b).abs().max() / b.abs().max()).item() < tol, (i, specs[i].kind)


def test_batch_deflation_any_tolerance(cuda):
    """The deflation of the Dirichlet net-charge mode (deflated CG on the
    constants) needs S 1 and 1^T W S 1 only, formed on the device with the
    Schur build and independent of the tolerance: a solve to 1e-8 and a
    later one to 1e-11 both reach their tolerance on every problem, agree,
    and no solve adds a set-up phase of its own for it."""
    import torch
    from immersedlayers import workloads as W
    from immersedlayers.batch import BatchSolver
    specs = W.batch_specs(8, sizes=(96, 128, 192))
    bs = BatchSolver(specs, dtype=torch.float64)
    bs.set_precond("bjacobi", 32)
    fp, fm = bs.surface_data()
    f1, s1 = bs.solve(fp, fm, tol=1e-8, maxiter=20000)
    it1, rr1 = bs.info()
    assert (rr1 <= 1e-8).all(), rr1
    f2, s2 = bs.solve(fp, fm, tol=1e-11, maxiter=20000)
    it2, rr2 = bs.info()
    assert (rr2 <= 1e-11).all(), rr2
    assert torch.allclose(s1, s2, rtol=0, atol=1e-6 * float(s2.abs().max()))
    names = [n for n, _ in bs.setup_times()]
    assert not [n for n in names if "deflation" in n], names


def test_batch_calls_wait_for_the_schur_build(cuda):
    """ilm_batch_create returns while its Schur build still runs; the calls
    that read S order their device work after it.  Products, coarse set-up
    and a graph-captured solve issued straight after creation equal the same
    calls issued after a device synchronisation, bit for bit."""
    import torch
    from immersedlayers import workloads as W
    from immersedlayers.batch import BatchSolver, NEUMANN
    specs = W.batch_specs(64)
    st = torch.cuda.Stream()
    bs = BatchSolver(specs, dtype=torch.float32)
    x = torch.linspace(-1.0, 1.0, bs.total_points, dtype=torch.float64, device="cuda")
    with torch.cuda.stream(st):
        y_now = bs.schur_apply(x, stream=st)     # issued at once
    st.synchronize()
    torch.cuda.synchronize()
    with torch.cuda.stream(st):
        y_later = bs.schur_apply(x, stream=st)
    st.synchronize()
    assert torch.equal(y_now, y_later)
    del bs
    # coarse set-up and a solve (plain and captured) straight after
    # creation; the first solve also forms the block inverses on their own
    # stream, beside the deflation set-up and its stage A
    for graph in (False, True):
        outs = []
        for sync_first in (False, True):
            bs = BatchSolver(specs, dtype=torch.float32)
            if sync_first:
                torch.cuda.synchronize()
            bs.set_precond("bjacobi", 64)
            bs.set_coarse(True, kinds=(NEUMANN,))
            fp, fm = bs.surface_data()
            with torch.cuda.stream(st):
                f, s = bs.solve(fp, fm, tol=1e-8, stream=st, graph=graph)
            st.synchronize()
            its, rr = bs.info()
            assert (rr <= 1e-8).all(), rr.max()
            outs.append((f.clone(), s.clone(), its.copy()))
            del bs
        assert torch.equal(outs[0][1], outs[1][1])
        assert torch.equal(outs[0][0], outs[1][0])
        assert (outs[0][2] == outs[1][2]).all()


def test_batch_async_precond_setup_matches_synchronised(cuda):
    """The default solver's set-up issued without waiting (the learned band on
    its own stream beside the Schur build, the coarse correction's E^-1 on
    the device, the block inverses on their own stream) and a solve straight
    after it give, bit for bit, what the same calls give with the device
    synchronised after each."""
    import os
    import torch
    from immersedlayers import workloads as W
    from immersedlayers import learned as LN
    from immersedlayers.batch import BatchSolver, DIRICHLET, NEUMANN
    if not os.path.exists(LN.BATCHED_WEIGHTS[DIRICHLET]):
        pytest.skip("no trained weights for the batched configuration")
    net = LN.LearnedPreconditioner.load(LN.BATCHED_WEIGHTS[DIRICHLET])
    specs = W.batch_specs(64)
    st = torch.cuda.Stream()
    outs = []
    for sync in (False, True):
        def step():
            if sync:
                torch.cuda.synchronize()
        bs = BatchSolver(specs, dtype=torch.float32)
        step()
        bs.set_precond("bjacobi", 64)
        bs.set_learned(net, kinds=(DIRICHLET,))
        step()
        bs.set_coarse(True, kinds=(NEUMANN,))
        step()
        bs.set_precond("learned", 64)
        step()
        fp, fm = bs.surface_data()
        with torch.cuda.stream(st):
            f, s = bs.solve(fp, fm, tol=1e-8, stream=st)
        st.synchronize()
        its, rr = bs.info()
        assert (rr <= 1e-8).all(), rr.max()
        outs.append((f.clone(), s.clone(), its.copy()))
        del bs
    assert torch.equal(outs[0][1], outs[1][1])
    assert torch.equal(outs[0][0], outs[1][0])
    assert (outs[0][2] == outs[1][2]).all()


def test_batch_shared_network_across_batches(cuda):
    """One network handle serving two batches whose learned set-ups are issued
    back to back without waiting (the network's work buffers are ordered by
    its own event): each batch solves as it does set up alone."""
    import os
    import torch
    from immersedlayers import workloads as W
    from immersedlayers import learned as LN
    from immersedlayers.batch import BatchSolver, DIRICHLET
    if not os.path.exists(LN.BATCHED_WEIGHTS[DIRICHLET]):
        pytest.skip("no trained weights for the batched configuration")
    net = LN.LearnedPreconditioner.load(LN.BATCHED_WEIGHTS[DIRICHLET])
    specs_a = W.batch_specs(48)
    specs_b = W.batch_specs(48, sizes=(128, 192))
    st = torch.cuda.Stream()

    def run(bs):
        fp, fm = bs.surface_data()
        with torch.cuda.stream(st):
            f, s = bs.solve(fp, fm, tol=1e-8, stream=st)
        st.synchronize()
        its, rr = bs.info()
        assert (rr <= 1e-8).all(), rr.max()
        return f.clone(), s.clone()

    alone = []
    for specs in (specs_a, specs_b):
        bs = BatchSolver(specs, dtype=torch.float32)
        bs.set_learned(net, kinds=(DIRICHLET,))
        torch.cuda.synchronize()
        alone.append(run(bs))
        del bs
    a = BatchSolver(specs_a, dtype=torch.float32)
    b = BatchSolver(specs_b, dtype=torch.float32)
    a.set_learned(net, kinds=(DIRICHLET,))
    b.set_learned(net, kinds=(DIRICHLET,))
    for bs, ref in zip((a, b), alone):
        f, s = run(bs)
        assert torch.equal(s, ref[1]) and torch.equal(f, ref[0])
