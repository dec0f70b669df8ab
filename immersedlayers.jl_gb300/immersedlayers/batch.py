"""Batched Dirichlet / Neumann Poisson solves (many independent problems, each
with its own grid and bodies) through libilm's ilm_batch_* entry points."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .bodies import as_bodylist
from .core import _DT, _ptr, _stream_ptr

DIRICHLET, NEUMANN = 0, 1


class BatchProblemSpec:
    """One problem of a batch: grid (n dual nodes per side, spacing h, origin
    at the centre), bodies, kind, and its plus/minus surface data."""

    def __init__(self, n, h, bodies, kind, fplus, fminus=None, ny=None):
        self.nx = int(n)
        self.ny = int(n if ny is None else ny)
        self.h = float(h)
        self.i0 = (self.nx // 2, self.ny // 2)
        self.bl = as_bodylist(bodies)
        self.kind = kind
        self.fplus = np.asarray(fplus, dtype=np.float64)
        self.fminus = np.zeros_like(self.fplus) if fminus is None else np.asarray(fminus, dtype=np.float64)

    @property
    def npts(self):
        return len(self.bl)


_PROBLEM_DTYPE = np.dtype([("nx", np.int32), ("ny", np.int32), ("h", np.float64), ("i0x", np.int32),
                           ("i0y", np.int32), ("npts", np.int32), ("kind", np.int32)], align=True)


class PackedBatch:
    """The host arrays of a batch in the C ABI's packed layout
    (ilm_batch_create): problem records, the points' coordinates, normals and
    areas concatenated in problem order, and per point the local index of its
    body's first point (ilm_batch_set_learned / ilm_batch_set_coarse).  An
    application that keeps its geometry in these arrays passes them to every
    batch it creates."""

    def __init__(self, specs):
        specs = list(specs)
        self.records = np.array([(s.nx, s.ny, s.h, s.i0[0], s.i0[1], s.npts, s.kind) for s in specs],
                                dtype=_PROBLEM_DTYPE)
        assert self.records.itemsize == C.sizeof(L.BatchProblem)
        bodies = [b for s in specs for b in s.bl.bodies]
        self.points = [np.ascontiguousarray(np.concatenate([getattr(b, a) for b in bodies]), np.float64)
                       if bodies else np.zeros(0) for a in ("x", "y", "nx", "ny", "ds")]
        starts = []
        for s in specs:
            fi = s.bl.firstindices()
            starts.append(np.repeat(fi[:-1], np.diff(fi)))
        self.body_starts = np.ascontiguousarray(np.concatenate(starts) if starts else np.zeros(0), dtype=np.int32)

    @property
    def nbytes(self):
        return self.records.nbytes + sum(a.nbytes for a in self.points)


class BatchSolver:
    """Set up (DDF windows, tile lists, FP64 Schur complements) and solve a
    batch of problems on the device.  `packed`: the specs' PackedBatch, when
    the caller already holds it (else it is built here)."""

    def __init__(self, specs, ddftype="Yang3", dtype=torch.float32, packed=None):
        self.specs = list(specs)
        self.dtype = dtype
        n = len(self.specs)
        self._packed = packed if packed is not None else PackedBatch(self.specs)
        rec = self._packed.records.ctypes.data_as(C.POINTER(L.BatchProblem))
        ptrs = [a.ctypes.data_as(C.POINTER(C.c_double)) for a in self._packed.points]
        h = C.c_void_p()
        L.call("ilm_batch_create", n, rec, *ptrs, L.DDF[ddftype], _DT[dtype], C.byref(h))
        self._h = h
        fo = (C.c_size_t * (n + 1))()
        po = (C.c_size_t * (n + 1))()
        L.call("ilm_batch_layout", h, fo, po)
        self.field_offsets = np.array(fo[:], dtype=np.int64)
        self.point_offsets = np.array(po[:], dtype=np.int64)
        self.nprob = n

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                L.load().ilm_batch_destroy(self._h)
        except Exception:
            pass

    @property
    def total_points(self):
        return int(self.point_offsets[-1])

    @property
    def total_cells(self):
        return int(self.field_offsets[-1])

    def surface_data(self, device="cuda"):
        fp = np.concatenate([s.fplus for s in self.specs])
        fm = np.concatenate([s.fminus for s in self.specs])
        return (torch.tensor(fp, dtype=self.dtype, device=device), torch.tensor(fm, dtype=self.dtype, device=device))

    def solve(self, fplus, fminus, f_out=None, s_out=None, tol=1e-8, maxiter=5000, stream=None, graph=False):
        """Solve every problem; graph=True replays a captured CUDA graph of
        the launch sequence (needs a torch.cuda.Stream, not the default)."""
        if f_out is None:
            f_out = torch.empty(self.total_cells, dtype=self.dtype, device="cuda")
        if s_out is None:
            s_out = torch.empty(self.total_points, dtype=self.dtype, device="cuda")
        L.call("ilm_batch_solve_graph" if graph else "ilm_batch_solve", self._h, _ptr(fplus), _ptr(fminus),
               _ptr(f_out), _ptr(s_out), float(tol), int(maxiter), _stream_ptr(stream))
        return f_out, s_out

    def solve_refined(self, fplus, fminus, f_out=None, s_out=None, tol=1e-12, maxiter=20000, max_refine=8,
                      stream=None):
        """Solve every problem with FP64 iterative refinement: FP64 inputs
        (converted if needed) and FP64 outputs for either batch dtype; the
        batch's own solve, then FP64 Schur residuals and preconditioned CG
        corrections until every ||b - S s|| / ||b|| <= tol, and the fields
        assembled in FP64 (ilm_batch_solve_refined)."""
        fp = fplus.to(torch.float64).contiguous()
        fm = fminus.to(torch.float64).contiguous()
        if f_out is None:
            f_out = torch.empty(self.total_cells, dtype=torch.float64, device="cuda")
        if s_out is None:
            s_out = torch.empty(self.total_points, dtype=torch.float64, device="cuda")
        L.call("ilm_batch_solve_refined", self._h, _ptr(fp), _ptr(fm), _ptr(f_out), _ptr(s_out), float(tol),
               int(maxiter), int(max_refine), _stream_ptr(stream))
        return f_out, s_out

    def info(self):
        it = (C.c_int * self.nprob)()
        rr = (C.c_double * self.nprob)()
        L.call("ilm_batch_info", self._h, it, rr)
        return np.array(it[:]), np.array(rr[:])

    def field(self, f_out, i):
        s = self.specs[i]
        a, b = self.field_offsets[i], self.field_offsets[i + 1]
        return f_out[a:b].view(s.ny - 1, s.nx - 1)

    def surface(self, s_out, i):
        return s_out[self.point_offsets[i]:self.point_offsets[i + 1]]


STAGES = ["jump/avg", "scatter (layer)", "divergence", "LGF FFT conv (f*)", "gather + rhs", "Schur CG (FP64)",
          "convert", "scatter (correction)", "divergence (corr.)", "LGF FFT conv (corr.) + f*"]


def _profiling(self, enable=True):
    L.call("ilm_batch_set_profiling", self._h, 1 if enable else 0)


def _stage_times(self):
    ms = (C.c_float * 32)()
    n = C.c_int()
    nl = C.c_int()
    L.call("ilm_batch_stage_times", self._h, ms, C.byref(n), C.byref(nl))
    return list(ms[:n.value]), nl.value


def _cg_times(self):
    """Per-problem Schur CG (start us, end us, SM) of the last profiled solve."""
    n = self.nprob
    a, b, sm = (C.c_double * n)(), (C.c_double * n)(), (C.c_int * n)()
    L.call("ilm_batch_cg_times", self._h, a, b, sm)
    return np.array(a[:]), np.array(b[:]), np.array(sm[:])


CG_VARIANTS = 6  # ILM_CG_VARIANTS of include/ilm.h


def _set_cg_variant(self, variant):
    """Schur CG kernel: 0 default (= 6, the size split; 1 when no problem is
    at or below the split), 1 row-distributed vectors (256
    threads per CTA, up to 3 per SM), 2 replicated vectors (one cluster
    barrier per iteration), 3 128-thread CTAs, 4 256-thread CTAs at most 2
    per SM, 5 512-thread CTAs one per SM, 6 size split (problems above 192
    points on variant 1's clusters, the others one CTA each beside them)."""
    L.call("ilm_batch_set_cg_variant", self._h, int(variant))


def _cg_variant(self):
    v, nc = C.c_int(), C.c_int()
    L.call("ilm_batch_get_cg_variant", self._h, C.byref(v), C.byref(nc))
    return v.value, nc.value


def _autotune(self, fplus, fminus, f_out=None, s_out=None, tol=1e-8, maxiter=5000, reps=2, stream=None):
    """Time every Schur CG kernel on this data and keep the fastest; returns
    (chosen variant, {variant: ms per solve})."""
    if f_out is None:
        f_out = torch.empty(self.total_cells, dtype=self.dtype, device="cuda")
    if s_out is None:
        s_out = torch.empty(self.total_points, dtype=self.dtype, device="cuda")
    ch = C.c_int()
    ms = (C.c_float * CG_VARIANTS)()
    L.call("ilm_batch_autotune", self._h, _ptr(fplus), _ptr(fminus), _ptr(f_out), _ptr(s_out), float(tol),
           int(maxiter), int(reps), _stream_ptr(stream), C.byref(ch), ms)
    return ch.value, {v + 1: float(ms[v]) for v in range(CG_VARIANTS) if ms[v] >= 0}


def _stats(self):
    st = (C.c_double * 6)()
    L.call("ilm_batch_stats", self._h, st)
    return dict(points=int(st[0]), cells=int(st[1]), sum_npts2=st[2], sum_fft=st[3], nprob=int(st[4]),
                box_cells=int(st[5]))


def _setup_times(self):
    """Host wall-clock (ms) of every set-up phase so far (batch creation,
    block-Jacobi inverses, learned-preconditioner inference), in order, as
    a list of (phase name, ms)."""
    n = C.c_int()
    L.call("ilm_batch_setup_times", self._h, None, 0, C.byref(n), None)
    ms = (C.c_double * max(n.value, 1))()
    names = (C.c_char_p * max(n.value, 1))()
    L.call("ilm_batch_setup_times", self._h, ms, n.value, C.byref(n), names)
    return [(names[k].decode(), float(ms[k])) for k in range(n.value)]


def _set_precond(self, mode="none", block_size=64):
    """Schur-CG preconditioner for the following solves: "none" (plain CG),
    "bjacobi" (block-Jacobi over ~block_size consecutive points) or
    "learned" (the band set by `set_learned`)."""
    L.call("ilm_batch_set_precond", self._h, {"none": 0, "bjacobi": 1, "learned": 2}[mode], int(block_size))


def _body_starts(self):
    """Per packed point, the local index of its body's first point."""
    return self._packed.body_starts


def _set_learned(self, net, kinds=(DIRICHLET, NEUMANN)):
    """Run the learned preconditioner's network over this batch's points, use
    it for the problems of the given kinds and switch the Schur CG to the
    learned preconditioner (problems of other kinds run plain CG unless
    another network is set for them)."""
    bs = _body_starts(self)
    mask = sum(1 << k for k in kinds)
    L.call("ilm_batch_set_learned", self._h, net._h, mask, bs.ctypes.data_as(C.POINTER(C.c_int)))


def _set_coarse(self, enable=True, kinds=(NEUMANN,)):
    """Coarse correction of block-Jacobi on the bodies' constant vectors for
    the problems of the given kinds (the Neumann problems, whose Schur
    complement has one near-null mode per body); enable=False removes it."""
    if not enable:
        L.call("ilm_batch_set_coarse", self._h, 0, None)
        return
    if tuple(kinds) != (NEUMANN,):
        raise ValueError("the coarse correction applies to the Neumann problems")
    bs = _body_starts(self)
    L.call("ilm_batch_set_coarse", self._h, 1 << NEUMANN, bs.ctypes.data_as(C.POINTER(C.c_int)))


def _schur_apply(self, x, y=None, stream=None):
    """y = S x for every problem (device FP64 packed vectors)."""
    if y is None:
        y = torch.empty_like(x)
    L.call("ilm_batch_schur_apply", self._h, _ptr(x), _ptr(y), _stream_ptr(stream))
    return y


def _schur_solve(self, rhs, x=None, tol=1e-10, maxiter=20000, stream=None):
    """S x = rhs for every problem with the batch's CG (device FP64)."""
    if x is None:
        x = torch.empty_like(rhs)
    L.call("ilm_batch_schur_solve", self._h, _ptr(rhs), _ptr(x), float(tol), int(maxiter), _stream_ptr(stream))
    return x


BatchSolver.body_starts = _body_starts
BatchSolver.set_learned = _set_learned
BatchSolver.set_coarse = _set_coarse
BatchSolver.schur_apply = _schur_apply
BatchSolver.schur_solve = _schur_solve


BatchSolver.set_precond = _set_precond
BatchSolver.set_profiling = _profiling
BatchSolver.stage_times = _stage_times
BatchSolver.stats = _stats
BatchSolver.setup_times = _setup_times
BatchSolver.cg_times = _cg_times
def _set_rhs_operator(self, enable=True):
    """Precompute the right-hand-side operator (E L^-1 D_s / G_s L^-1 R per
    problem; built once, as much memory as S) so that each later solve takes
    one LGF convolution instead of two; for batches solved repeatedly."""
    L.call("ilm_batch_set_rhs_operator", self._h, int(bool(enable)))


BatchSolver.set_rhs_operator = _set_rhs_operator
BatchSolver.set_cg_variant = _set_cg_variant
BatchSolver.cg_variant = _cg_variant
BatchSolver.autotune = _autotune
