"""Pins of the oracle's heat-conduction pieces (CPU): the lattice heat kernel
against a dense matrix exponential, the stage Schur complements' symmetry
and definiteness, and the IF-HERK step's exact constraint satisfaction
(test/literate/heatconduction.jl:87-189, ConstrainedSystems' LiskaIFHERK)."""
import numpy as np
import pytest
import scipy.linalg as sl

import ilm_oracle as O
from geometry import heat_case, oracle_cache


@pytest.mark.parametrize("a", [0.1, 0.5, 1.0 / 3.0, 1.0, 2.5])
def test_heat_kernel_matches_expm(a):
    n = 121
    L1 = -2 * np.eye(n) + np.eye(n, k=1) + np.eye(n, k=-1)
    row = sl.expm(a * L1)[n // 2]
    k = O.heat_kernel_1d(a)
    R = (k.size - 1) // 2
    assert np.abs(row[n // 2 - R:n // 2 + R + 1] - k).max() < 1e-14   # expm itself is good to ~1e-15
    assert np.abs(row).sum() - k.sum() < 1e-14   # nothing left outside the radius
    assert abs(k.sum() - 1.0) < 1e-14            # exp(aL) conserves the sum


def test_if_is_separable_exponential():
    g, b = heat_case(h=0.1, r=0.3)
    n1, n2 = g.shape(O.NODES_PRIMAL)
    rng = np.random.default_rng(3)
    w = np.zeros((n1, n2))
    w[n1 // 2 - 3:n1 // 2 + 3, n2 // 2 - 2:n2 // 2 + 4] = rng.standard_normal((6, 6))
    a = 0.7
    L5 = np.kron(np.eye(n2), -2 * np.eye(n1) + np.eye(n1, k=1) + np.eye(n1, k=-1)) + \
        np.kron(-2 * np.eye(n2) + np.eye(n2, k=1) + np.eye(n2, k=-1), np.eye(n1))
    ref = (sl.expm(a * L5) @ w.reshape(-1, order="F")).reshape((n1, n2), order="F")
    # the unbounded-lattice kernel equals the Dirichlet-box exponential while
    # the support stays far from the box edge
    assert np.abs(O.apply_if(w, a) - ref).max() < 1e-12


def test_stage_schur_is_ds_symmetric_positive():
    g, b = heat_case()
    c = oracle_cache(g, b)
    W = np.diag(c.ds)
    for a in (0.5 / 3, 1.0 / 3, 0.5, 0.0):
        S = O.heat_schur(c, a)
        WS = W @ S
        assert np.abs(WS - WS.T).max() < 1e-14 * np.abs(WS).max()
        assert np.linalg.eigvalsh(0.5 * (WS + WS.T)).min() > 0


def test_heat_march_satisfies_constraint():
    g, b = heat_case()
    c = oracle_cache(g, b)
    T0 = heat_initial_field(g)
    tp = np.zeros(c.N)
    tm = np.ones(c.N)
    h = g.h
    T, sig = O.heat_march(c, T0, tp, tm, 1.0, 0.5 * h * h, 4)
    assert np.abs(O.interpolate_scalar(c, T) - 0.5).max() < 1e-12
    assert np.isfinite(T).all() and np.abs(sig).max() > 0


def test_heat_march_without_body_is_pure_diffusion():
    g, b = heat_case()
    c = oracle_cache(g, b)
    T0 = heat_initial_field(g)
    h = g.h
    # with avg = E T of the exact diffusion the constraint force vanishes:
    # check the body-free part, exp(n a L) T0, through the integrator's IF
    a = 0.5
    T = T0.copy()
    for _ in range(3):
        T = O.apply_if(T, a)
    assert np.abs(T - O.apply_if(T0, 3 * a)).max() < 1e-13


def heat_initial_field(g):
    x, y = g.coords(O.NODES_PRIMAL)
    return np.exp(-(x[:, None] ** 2 + y[None, :] ** 2) / 0.2 ** 2)
