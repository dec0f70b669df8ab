"""Generate the golden fixtures under tests/golden/ from the CPU oracle.

The reference's own Julia path cannot run in this environment, so these
fixtures freeze the oracle's FP64 results (which are pinned by the reference's
known-answer tests) at two set-ups:

* golden_dirichlet_plain.npz: the plain Dirichlet configuration ([-2,2]^2,
  h = 0.02, circle r = 0.5 with 157 points, f+ = cos(theta) + 0.1 N(0,1) with
  numpy default_rng(1), f- = 0): f on Nodes{Primal} (x-fastest), s, and the
  extreme eigenvalues of the ds-symmetrised create_RTLinvR;
* golden_neumann_circle.npz: the Neumann problem of test/literate/neumann.jl
  at h = 0.04 ([-2,2]^2, circle R = 1, ds = 1.4h, v+ = n_x, v- = 0): f and [phi];
* golden_batched.npz: one Dirichlet and one Neumann problem of the batched
  configuration per grid size (128 ... 512), see `batched`.

Run:  python tests/golden/make_golden.py [dirichlet] [neumann] [batched]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "immersedlayers.jl_gb300"))

import ilm_oracle as O  # noqa: E402
from immersedlayers import bodies as B  # noqa: E402
from immersedlayers import workloads as W  # noqa: E402


def dirichlet_plain():
    xlim, ylim, h, b, fb = W.dirichlet_plain()
    g = O.Grid.physical(xlim, ylim, h)
    c = O.SurfaceCache(b.x, b.y, b.nx, b.ny, b.ds, g)
    S = O.create_RTLinvR(c)
    f, s = O.solve_dirichlet(c, fb, np.zeros_like(fb), S)
    d = np.sqrt(b.ds)
    ev = np.linalg.eigvalsh(0.5 * ((S * d[:, None] / d[None, :]) + (S * d[:, None] / d[None, :]).T))
    np.savez_compressed(os.path.join(HERE, "golden_dirichlet_plain.npz"), f=f, s=s, fb=fb,
                        eig=np.array([ev[0], ev[1], ev[-1]]), grid=np.array([g.nx, g.ny, g.i0x, g.i0y]), h=h)


def neumann_circle():
    h = 0.04
    g = O.Grid.physical((-2.0, 2.0), (-2.0, 2.0), h)
    b = B.circle(1.0, ds=1.4 * h)
    c = O.SurfaceCache(b.x, b.y, b.nx, b.ny, b.ds, g)
    f, df, _, _ = O.solve_neumann(c, b.nx.copy(), np.zeros(len(b)))
    np.savez_compressed(os.path.join(HERE, "golden_neumann_circle.npz"), f=f, df=df,
                        grid=np.array([g.nx, g.ny, g.i0x, g.i0y]), h=h)


# One Dirichlet and one Neumann problem of the batched configuration
# (workloads.batch_problem(i), seeds 3 + i) for every grid size it draws from.
BATCHED_PROBLEMS = (8, 11, 18, 21, 6, 3, 2, 5, 0, 15)
F_STRIDE = 4


def batched():
    """golden_batched.npz: per problem i of BATCHED_PROBLEMS, the oracle's
    dense-LU solution: s (all points; [phi] for the Neumann problems), f on
    Nodes{Primal} sampled every F_STRIDE cells in x and y (f[::4, ::4], x
    first), and max |f| over the whole field."""
    out = {"problems": np.array(BATCHED_PROBLEMS), "f_stride": F_STRIDE}
    for i in BATCHED_PROBLEMS:
        n, h, bl, kind, fb = W.batch_problem(i)
        g = O.Grid(n, n, h, n // 2, n // 2)
        c = O.SurfaceCache(bl.x, bl.y, bl.nx, bl.ny, bl.ds, g)
        fm = np.zeros_like(fb)
        if kind == 0:
            f, s = O.solve_dirichlet(c, fb, fm)
        else:
            f, s, _, _ = O.solve_neumann(c, fb, fm)
        out[f"s_{i}"] = s
        out[f"f_{i}"] = f[::F_STRIDE, ::F_STRIDE]
        out[f"fmax_{i}"] = np.abs(f).max()
        out[f"meta_{i}"] = np.array([n, kind, len(bl)])
        print(f"problem {i}: n={n} kind={kind} npts={len(bl)}", flush=True)
    np.savez_compressed(os.path.join(HERE, "golden_batched.npz"), **out)


if __name__ == "__main__":
    which = sys.argv[1:] or ["dirichlet", "neumann", "batched"]
    if "dirichlet" in which:
        dirichlet_plain()
    if "neumann" in which:
        neumann_circle()
    if "batched" in which:
        batched()
    print("written")
