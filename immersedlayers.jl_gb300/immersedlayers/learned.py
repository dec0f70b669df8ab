"""Learned preconditioner for the Schur-complement CG (libilm ilm_net_*).

A 1-D convolutional network over arc length (circular within each body; 4
layers, 64 channels, kernel 5, ReLU; BF16 weights with FP32 accumulation)
reads 8 dimensionless features per surface point and emits a band C of
2K+1 coefficients per point.  The preconditioner M r = W^-1 C^T C r
(W = diag(ds)) is linear, self-adjoint and semi-definite in the ds-weighted
inner product in which the reference's Schur operator S = R^T L^-1 R
(src/matrix_operators.jl:9-27, GridScaling) is symmetric, so the device CG
(flexible form) keeps its guarantees; plain CG stays available and the FP64
residual test decides convergence either way.

Training data are (geometry, b, x) triples that the plain device solver
generates: b is a Schur right-hand side (arc-length Fourier modes plus white
noise), x the plain-CG solution of S x = b.  Training minimises
mean |M b - x|^2 / |x|^2 with Adam, every forward and backward pass in
libilm's kernels.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import time

import numpy as np
import torch

from . import _lib as L
from .core import _ptr, _stream_ptr

NFEAT, WIDTH, NLAYERS, KSIZE, BAND = 8, 64, 4, 5, 4
DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
DEFAULT_WEIGHTS = os.path.join(DATA_DIR, "learned_star.npz")
BATCHED_WEIGHTS = {0: os.path.join(DATA_DIR, "learned_batched_dirichlet.npz"),
                   1: os.path.join(DATA_DIR, "learned_batched_neumann.npz")}


def layer_dims(width=WIDTH, nlayers=NLAYERS, band=BAND, nfeat=NFEAT):
    dims = [nfeat] + [width] * (nlayers - 1) + [2 * band + 1]
    return [(dims[l], dims[l + 1]) for l in range(nlayers)]


def initial_params(seed=0, width=WIDTH, nlayers=NLAYERS, band=BAND):
    """He-uniform weights for the ReLU layers, a small last layer (C starts
    near the identity, i.e. M near diag(1/ds)), zero biases."""
    rng = np.random.default_rng(seed)
    parts = []
    dims = layer_dims(width, nlayers, band)
    for l, (ci, co) in enumerate(dims):
        fan = ci * KSIZE
        bound = math.sqrt(6.0 / fan) if l < len(dims) - 1 else 0.01 / math.sqrt(fan)
        parts.append(rng.uniform(-bound, bound, size=co * ci * KSIZE))
        parts.append(np.zeros(co))
    return np.concatenate(parts).astype(np.float32)


def point_features(x, y, nx, ny, ds, seg_start, seg_len, h):
    """Per-point features (npts x 8, float32) computed by libilm on the host."""
    arr = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, nx, ny, ds)]
    ss = np.ascontiguousarray(seg_start, dtype=np.int32)
    sl = np.ascontiguousarray(seg_len, dtype=np.int32)
    n = arr[0].size
    out = np.empty((n, NFEAT), dtype=np.float32)
    L.call("ilm_point_features", n, *[a.ctypes.data_as(C.POINTER(C.c_double)) for a in arr],
           ss.ctypes.data_as(C.POINTER(C.c_int)), sl.ctypes.data_as(C.POINTER(C.c_int)), float(h),
           out.ctypes.data_as(C.POINTER(C.c_float)))
    return out


def body_segments(bl, offset=0):
    """(seg_start, seg_len) per point of a BodyList, start indices + offset."""
    fi = bl.firstindices()
    st, ln = [], []
    for b in range(len(fi) - 1):
        n = fi[b + 1] - fi[b]
        st.append(np.full(n, fi[b] + offset, dtype=np.int32))
        ln.append(np.full(n, n, dtype=np.int32))
    return np.concatenate(st), np.concatenate(ln)


class LearnedPreconditioner:
    """The network (device parameters, Adam state) behind ilm_net_t."""

    def __init__(self, params=None, seed=0, width=WIDTH, nlayers=NLAYERS, band=BAND):
        self.width, self.nlayers, self.band = width, nlayers, band
        h = C.c_void_p()
        L.call("ilm_net_create", NFEAT, width, nlayers, band, C.byref(h))
        self._h = h
        n = C.c_size_t()
        L.call("ilm_net_nparams", h, C.byref(n))
        self.nparams = n.value
        self.set_params(initial_params(seed, width, nlayers, band) if params is None else params)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                L.load().ilm_net_destroy(self._h)
        except Exception:
            pass

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters, got {p.size}")
        L.call("ilm_net_set_params", self._h, p.ctypes.data_as(C.POINTER(C.c_float)))

    def set_tensor_cores(self, enable=True):
        """Forward convolutions on the tcgen05 tensor cores (default) or by
        FP32 FMA (ilm_net_set_tensor_cores)."""
        L.call("ilm_net_set_tensor_cores", self._h, 1 if enable else 0)

    def get_params(self):
        p = np.empty(self.nparams, dtype=np.float32)
        L.call("ilm_net_get_params", self._h, p.ctypes.data_as(C.POINTER(C.c_float)))
        return p

    def save(self, path, **meta):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez(path, params=self.get_params(), width=self.width, nlayers=self.nlayers, band=self.band,
                 **{k: np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS):
        d = np.load(path)
        return cls(params=d["params"], width=int(d["width"]), nlayers=int(d["nlayers"]), band=int(d["band"]))

    def forward(self, feat, seg_start, seg_len, stream=None):
        """Band coefficients (npts x (2K+1)) for device features/segments."""
        n = feat.shape[0]
        out = torch.empty((n, 2 * self.band + 1), dtype=torch.float32, device=feat.device)
        L.call("ilm_net_forward", self._h, n, _ptr(feat), _ptr(seg_start), _ptr(seg_len), _ptr(out),
               _stream_ptr(stream))
        return out

    def loss_grad(self, mb, stream=None):
        """(loss, gradient) of one minibatch (a dict from TrainingSet)."""
        loss = C.c_double()
        g = np.empty(self.nparams, dtype=np.float32)
        L.call("ilm_net_loss_grad", self._h, mb["npts"], mb["npairs"], _ptr(mb["pair_off"]), _ptr(mb["feat"]),
               _ptr(mb["seg_start"]), _ptr(mb["seg_len"]), _ptr(mb["w"]), _ptr(mb["b"]), _ptr(mb["x"]),
               C.byref(loss), g.ctypes.data_as(C.POINTER(C.c_float)), _stream_ptr(stream))
        return loss.value, g

    def train_step(self, mb, lr, loss_slot=None, stream=None):
        L.call("ilm_net_train_step", self._h, mb["npts"], mb["npairs"], _ptr(mb["pair_off"]), _ptr(mb["feat"]),
               _ptr(mb["seg_start"]), _ptr(mb["seg_len"]), _ptr(mb["w"]), _ptr(mb["b"]), _ptr(mb["x"]), float(lr),
               None if loss_slot is None else C.c_void_p(loss_slot.data_ptr()), _stream_ptr(stream))


class TrainingSet:
    """(features, b, x) triples packed on the device in fixed minibatches of
    consecutive problems; segment starts and pair offsets are relative to
    each minibatch so a minibatch is a plain slice."""

    def __init__(self, minibatches):
        self.minibatches = minibatches

    def __len__(self):
        return len(self.minibatches)

    @property
    def npairs(self):
        return sum(m["npairs"] for m in self.minibatches)


def _pack_minibatch(items, device="cuda"):
    feat, ss, sl, w, b, x, off = [], [], [], [], [], [], [0]
    for it in items:
        o = off[-1]
        st, ln = it["seg"]
        feat.append(it["feat"])
        ss.append(st + o)
        sl.append(ln)
        w.append(it["w"])
        b.append(it["b"])
        x.append(it["x"])
        off.append(o + it["feat"].shape[0])
    f32 = lambda a: torch.tensor(np.concatenate(a), dtype=torch.float32, device=device)  # noqa: E731
    i32 = lambda a: torch.tensor(np.concatenate(a), dtype=torch.int32, device=device)  # noqa: E731
    return {"feat": f32(feat).reshape(-1, NFEAT).contiguous(), "seg_start": i32(ss), "seg_len": i32(sl),
            "w": f32(w), "b": f32(b), "x": f32(x), "pair_off": torch.tensor(off, dtype=torch.int32, device=device),
            "npts": off[-1], "npairs": len(items)}


def schur_rhs(bl, rng, noise=True, kind=0):
    """Schur right-hand side for training: the batched configuration's
    arc-length Fourier modes plus (optionally) white noise of random level.
    Neumann data (kind 1) get zero ds-weighted mean per body, the
    compatibility condition of the Neumann problem."""
    from .workloads import fourier_surface_data
    f = fourier_surface_data(bl, rng)
    if noise:
        f = f + rng.uniform(0.0, 1.0) * np.sqrt(np.mean(f * f)) * rng.standard_normal(f.size)
    if kind == 1:
        fi = bl.firstindices()
        ds = np.asarray(bl.ds)
        for b in range(len(fi) - 1):
            s = slice(fi[b], fi[b + 1])
            f[s] -= (f[s] * ds[s]).sum() / ds[s].sum()
    return f


def generate(problem_fn, indices, chunk=256, tol=1e-10, maxiter=5000, minibatch=64, noise=True, log=None, kind=0):
    """Triples for problems `problem_fn(i)` -> (n, h, BodyList), solved by
    the plain device CG on S x = b.  Problems the plain CG cannot bring to
    `tol` within `maxiter` (points much closer than h: S numerically
    singular) give no triple.  Returns (TrainingSet, stats)."""
    from .batch import BatchProblemSpec, BatchSolver
    items = []
    its_all = []
    t0 = time.perf_counter()
    for c0 in range(0, len(indices), chunk):
        idx = indices[c0:c0 + chunk]
        probs = [problem_fn(i) for i in idx]
        specs = [BatchProblemSpec(n, h, bl, kind, np.zeros(len(bl))) for (n, h, bl) in probs]
        bs = BatchSolver(specs, dtype=torch.float32)
        bs.set_precond("none")
        rhs = []
        for i, (n, h, bl) in zip(idx, probs):
            rng = np.random.default_rng(int(i) + 7)
            rhs.append(schur_rhs(bl, rng, noise, kind))
        b = torch.tensor(np.concatenate(rhs), dtype=torch.float64, device="cuda")
        x = bs.schur_solve(b, tol=tol, maxiter=maxiter)
        its, rr = bs.info()
        ok = rr <= tol * 1.0001
        its_all.append(its)
        xh = x.cpu().numpy()
        bh = b.cpu().numpy()
        po = bs.point_offsets
        for k, (n, h, bl) in enumerate(probs):
            if not ok[k]:
                continue
            s = slice(po[k], po[k + 1])
            st, ln = body_segments(bl)
            feat = point_features(bl.x, bl.y, bl.nx, bl.ny, bl.ds, st, ln, h)
            items.append({"feat": feat, "seg": (st, ln), "w": np.asarray(bl.ds, np.float64),
                          "b": bh[s], "x": xh[s]})
        del bs
        if log:
            log(f"generated {min(c0 + chunk, len(indices))}/{len(indices)} ({time.perf_counter() - t0:.1f}s)")
    mbs = [_pack_minibatch(items[i:i + minibatch]) for i in range(0, len(items), minibatch)]
    its = np.concatenate(its_all)
    return TrainingSet(mbs), {"plain_cg_iterations_mean": float(its.mean()), "kept": len(items),
                              "candidates": len(indices), "seconds": time.perf_counter() - t0}


def train(net, data: TrainingSet, epochs=30, lr=1e-3, lr_min=5e-5, seed=0, log=None, stream=None):
    """Adam over the minibatches (shuffled order per epoch), cosine learning
    rate from lr to lr_min.  Returns the mean loss of each epoch."""
    rng = np.random.default_rng(seed)
    nmb = len(data)
    slots = torch.zeros(nmb, dtype=torch.float64, device="cuda")
    hist = []
    total = epochs * nmb
    step = 0
    for ep in range(epochs):
        for j in rng.permutation(nmb):
            a = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * step / max(1, total)))
            net.train_step(data.minibatches[j], a, loss_slot=slots[j:j + 1], stream=stream)
            step += 1
        torch.cuda.synchronize()
        hist.append(float(slots.mean()))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4f}")
    return hist


def _timed_solves(bs, fp, fm, tol, maxiter, reps=3):
    bs.solve(fp, fm, tol=tol, maxiter=maxiter)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        f, s = bs.solve(fp, fm, tol=tol, maxiter=maxiter)
    e1.record()
    torch.cuda.synchronize()
    its, rr = bs.info()
    return e0.elapsed_time(e1) / 1000.0 / reps, its, rr, f


def evaluate(net, problem_fn, indices, tol=1e-8, maxiter=5000, fp64_errors=False):
    """Full Dirichlet Poisson solves of held-out problems (surface data:
    arc-length Fourier modes), plain CG against the learned preconditioner.

    Points closer than ~0.7 h make S numerically singular (condition numbers
    1e11-1e13): no CG reaches `tol` there.  Reported: the fraction of all
    problems each solver brings to `tol` within `maxiter`, and -- on the
    problems plain CG solves -- iterations, solves/s of the batched solve and
    the field difference between the two solvers; with `fp64_errors`, the
    learned solve's field error against the FP64 refined solution on every
    problem it solves."""
    from .batch import BatchProblemSpec, BatchSolver
    from .workloads import fourier_surface_data
    probs = [problem_fn(i) for i in indices]
    specs = [BatchProblemSpec(n, h, bl, 0, fourier_surface_data(bl, np.random.default_rng(int(i) + 11)))
             for i, (n, h, bl) in zip(indices, probs)]
    out = {"problems": len(specs), "tol": tol, "maxiter": maxiter}
    bs = BatchSolver(specs, dtype=torch.float32)
    fp, fm = bs.surface_data()
    bs.set_learned(net)
    ok = {}
    for mode in ("none", "learned"):
        bs.set_precond(mode)
        bs.solve(fp, fm, tol=tol, maxiter=maxiter)
        torch.cuda.synchronize()
        its, rr = bs.info()
        ok[mode] = rr <= tol
        out[f"converged_fraction_{mode}"] = float(ok[mode].mean())
    del bs
    sel = [k for k in range(len(specs)) if ok["none"][k]]
    sub = [specs[k] for k in sel]
    out["well_posed_problems"] = len(sub)
    out["well_posed_npts_max"] = int(max(s.npts for s in sub)) if sub else 0
    if not sub:
        return out
    bs = BatchSolver(sub, dtype=torch.float32)
    fp, fm = bs.surface_data()
    t0 = time.perf_counter()
    bs.set_learned(net)
    torch.cuda.synchronize()
    out["learned_setup_s"] = time.perf_counter() - t0
    fields = {}
    for mode in ("none", "learned"):
        bs.set_precond(mode)
        t, its, rr, f = _timed_solves(bs, fp, fm, tol, maxiter)
        out[mode] = {"solves_per_s": len(sub) / t, "ms": 1000 * t, "cg_iterations_mean": float(its.mean()),
                     "cg_iterations_max": int(its.max()), "max_rel_residual": float(rr.max()),
                     "converged": int((rr <= tol).sum())}
        fields[mode] = f.double()
    out["speedup_solves"] = out["learned"]["solves_per_s"] / out["none"]["solves_per_s"]
    out["iteration_ratio"] = out["none"]["cg_iterations_mean"] / out["learned"]["cg_iterations_mean"]
    fa, fb = fields["none"], fields["learned"]
    out["field_rel_diff"] = float((fa - fb).abs().max() / fa.abs().max())
    del bs
    if fp64_errors:
        out["error_vs_fp64"] = _errors_vs_refined(net, [specs[k] for k in range(len(specs)) if ok["learned"][k]], tol,
                                                  maxiter)
    return out


def _errors_vs_refined(net, specs, tol, maxiter):
    """Field error of the learned-preconditioned FP32 solve against the FP64
    refined solution (ilm_batch_solve_refined to a Schur residual of 1e-12,
    the path the tests hold to the oracle's dense LU at 1e-10), per problem
    relative to its max |f|, on the problems the learned solver brings to
    `tol`."""
    from .batch import BatchSolver
    if not specs:
        return {"problems": 0}
    bs = BatchSolver(specs, dtype=torch.float32)
    fp64 = torch.tensor(np.concatenate([s.fplus for s in specs]), dtype=torch.float64, device="cuda")
    fm64 = torch.tensor(np.concatenate([s.fminus for s in specs]), dtype=torch.float64, device="cuda")
    bs.set_precond("bjacobi", 64)
    fr, _ = bs.solve_refined(fp64, fm64, tol=1e-12, maxiter=20000)
    torch.cuda.synchronize()
    _, rr_ref = bs.info()
    ref_ok = rr_ref <= 1e-12
    bs.set_learned(net)
    bs.set_precond("learned")
    fp, fm = bs.surface_data()
    f, _ = bs.solve(fp, fm, tol=tol, maxiter=maxiter)
    torch.cuda.synchronize()
    errs = []
    for k in range(len(specs)):
        if not ref_ok[k]:
            continue
        a, b = bs.field(f, k).double(), bs.field(fr, k)
        errs.append(float((a - b).abs().max() / b.abs().max()))
    e = np.array(errs) if errs else np.zeros(1)
    return {"problems": len(specs), "refined_converged": int(ref_ok.sum()), "max_field_rel_err": float(e.max()),
            "median_field_rel_err": float(np.median(e)), "within_1e-5": int((e <= 1e-5).sum())}


def main(argv=None):
    """Train the preconditioner on the star-body configuration and save it:
    python -m immersedlayers.learned --train 20000 --test 1000 --epochs 30"""
    import argparse
    import json
    from .workloads import LEARNED_TEST_SEED, LEARNED_TRAIN_SEED, learned_problem
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--test", type=int, default=1000)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--minibatch", type=int, default=64)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=None)
    ap.add_argument("--report", default=None)
    ap.add_argument("--config", default="star", choices=["star", "batched"])
    ap.add_argument("--kind", default="dirichlet", choices=["dirichlet", "neumann"])
    a = ap.parse_args(argv)
    log = lambda m: print(m, flush=True)  # noqa: E731
    t0 = time.perf_counter()
    kind = 0 if a.kind == "dirichlet" else 1
    if a.config == "star":
        problem_fn, train_idx = learned_problem, [LEARNED_TRAIN_SEED + i for i in range(a.train)]
        out = a.out or DEFAULT_WEIGHTS
    else:
        from .workloads import batch_problem
        problem_fn = lambda i: batch_problem(i)[:3]  # noqa: E731
        train_idx = [10000 + i for i in range(a.train)]   # disjoint from the benchmark batch (0..255)
        out = a.out or BATCHED_WEIGHTS[kind]
    data, gstats = generate(problem_fn, train_idx, minibatch=a.minibatch, log=log, kind=kind)
    log(f"training set: {gstats}")
    net = LearnedPreconditioner(seed=a.seed)
    t1 = time.perf_counter()
    hist = train(net, data, epochs=a.epochs, lr=a.lr, seed=a.seed, log=log)
    train_s = time.perf_counter() - t1
    net.save(out, loss_history=np.asarray(hist), train_pairs=gstats["kept"], epochs=a.epochs)
    ev = evaluate(net, learned_problem, [LEARNED_TEST_SEED + i for i in range(a.test)]) if a.config == "star" \
        else None
    rep = {"generate": gstats, "train_seconds": train_s, "loss_first": hist[0], "loss_last": hist[-1],
           "held_out": ev, "total_seconds": time.perf_counter() - t0}
    log(json.dumps(rep))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
    return rep


if __name__ == "__main__":
    main()
