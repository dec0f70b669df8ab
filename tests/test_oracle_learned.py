"""Pins of the oracle's learned-preconditioner pieces (CPU): the analytic
gradient against central differences, the preconditioner's symmetry and
definiteness in the ds-weighted inner product, the bf16 rounding rule and
the per-body circular neighbourhoods."""
import numpy as np
import pytest

import learned_oracle as LO


def _toy(seed=0, sizes=(23, 17)):
    rng = np.random.default_rng(seed)
    n = sum(sizes)
    starts = np.cumsum([0] + list(sizes[:-1]))
    st, ln = LO.segments(starts, n)
    F = rng.standard_normal((n, LO.NFEAT))
    w = rng.uniform(0.5, 1.5, n)
    b = rng.standard_normal(n)
    x = rng.standard_normal(n)
    return n, starts, st, ln, F, w, b, x


def test_neighbours_wrap_per_body():
    n, starts, st, ln, *_ = _toy()
    j = LO.nb(st, ln, -1)
    assert j[0] == 22 and j[23] == 39 and j[24] == 23
    assert (LO.nb(st, ln, 17) == np.arange(n))[23:].all()


def test_bf16_round_matches_definition():
    a = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.14159, 65504.0, 1e-30], dtype=np.float32)
    r = LO.bf16_round(a)
    assert r[0] == 1.0 and r[1] == 1.0            # tie -> even
    assert r[2] == np.float32(1.0 + 2 ** -7)      # above the tie -> up
    assert abs(r[3] + 3.140625) < 1e-7
    assert (r.view(np.uint32) & 0xFFFF == 0).all()


def test_gradient_matches_central_differences():
    n, starts, st, ln, F, w, b, x = _toy(1)
    theta = LO.init_params(3).astype(np.float64)
    # a last layer of ordinary size so every layer matters
    rng = np.random.default_rng(5)
    theta += 0.05 * rng.standard_normal(theta.size)
    pair_off = [0, 23, n]
    loss, g = LO.loss_and_grad(theta, F, st, ln, w, b, x, pair_off, weights_bf16=False)
    for trial in range(4):
        d = rng.standard_normal(theta.size)
        eps = 1e-6
        lp, _ = LO.loss_and_grad(theta + eps * d, F, st, ln, w, b, x, pair_off, weights_bf16=False)
        lm, _ = LO.loss_and_grad(theta - eps * d, F, st, ln, w, b, x, pair_off, weights_bf16=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g @ d) <= 1e-6 * max(1.0, abs(fd)), (trial, fd, g @ d)


def test_preconditioner_is_ds_self_adjoint_and_psd():
    n, starts, st, ln, F, w, b, x = _toy(2)
    theta = LO.init_params(4)
    c, _ = LO.forward(theta, F, st, ln)
    M = np.stack([LO.precond_apply(c, e, w, st, ln) for e in np.eye(n)], axis=1)
    WM = np.diag(w) @ M
    assert np.abs(WM - WM.T).max() < 1e-12 * np.abs(WM).max()
    assert np.linalg.eigvalsh(0.5 * (WM + WM.T)).min() > -1e-12


def test_features_on_circle():
    """Circle of radius R: curvature feature 10 h / R, unit normals."""
    import math
    R, n, h = 0.5, 200, 0.01
    th = 2 * math.pi * (np.arange(n) + 0.5) / n
    x, y = R * np.cos(th), R * np.sin(th)
    ds = np.full(n, 2 * math.pi * R / n)
    F = LO.point_features(x, y, np.cos(th), np.sin(th), ds, [0], h)
    assert np.allclose(F[:, 1], 10 * h / R, rtol=1e-3)
    assert np.allclose(F[:, 0], ds / h)
    assert np.allclose(F[:, 4] ** 2 + F[:, 5] ** 2, 1.0)


def test_library_features_match_oracle(lib_built):
    """ilm_point_features (host code in libilm) against the restatement."""
    from immersedlayers import bodies as B
    from immersedlayers import learned as LN
    from immersedlayers.workloads import learned_problem
    for i in range(3):
        n, h, bl = learned_problem(1_000_000 + i)
        bl.append(B.circle(0.2, n=40, center=(1.2, 1.1)))
        st, ln = LN.body_segments(bl)
        F = LN.point_features(bl.x, bl.y, bl.nx, bl.ny, bl.ds, st, ln, h)
        ref = LO.point_features(bl.x, bl.y, bl.nx, bl.ny, bl.ds, bl.firstindices()[:-1], h)
        assert np.abs(F - ref).max() < 1e-6
