"""ORACLE (test infrastructure only): FP64 NumPy restatement of the learned
Schur-complement preconditioner -- point features, the 1-D convolutional
network over arc length, the banded factor it emits, the preconditioner
M r = W^-1 C^T C r and the training loss with its gradient.  Only tests,
the smoke check and the bench's CPU leg use this module; the product runs
the CUDA kernels in libilm.

The reference has no learned component; its Schur solve is a dense LU
(test/literate/problems.jl:291).  What the preconditioner must respect is
the reference's Schur operator S = R^T L^-1 R with GridScaling
(src/matrix_operators.jl:9-27, src/cache.jl:305-316): W S is symmetric for
W = diag(ds), so M is built self-adjoint in the ds-weighted inner product.

Network (channels-last, points of one body contiguous, circular padding per
body -- the per-body segmentation of the reference's `_firstindices`,
src/cache.jl:390-391):
    a_0 = features (N x F)
    z_l[i, o] = b_l[o] + sum_{k, t=-2..2} W_l[o, k, t+2] a_l[nb(i, t), k]
    a_{l+1} = relu(z_l) for l < L-1;  out = z_{L-1}   (N x (2K+1))
    c[i, t+K] = out[i, t+K] + (t == 0)
    (C r)_j = sum_{t=-K..K} c[j, t+K] r[nb(j, t)]
    M r = W^-1 C^T C r
Loss over pairs (b, x) with S x = b:  mean_p |M b_p - x_p|^2 / |x_p|^2.
"""
from __future__ import annotations

import math

import numpy as np

NFEAT = 8
WIDTH = 64
NLAYERS = 4
KSIZE = 5
BAND = 4


def bf16_round(a):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def segments(body_starts, n):
    """Per point (start, length) of its body; body_starts ascending, first 0."""
    st = np.zeros(n, dtype=np.int64)
    ln = np.zeros(n, dtype=np.int64)
    bs = list(body_starts) + [n]
    for b in range(len(bs) - 1):
        st[bs[b]:bs[b + 1]] = bs[b]
        ln[bs[b]:bs[b + 1]] = bs[b + 1] - bs[b]
    return st, ln


def nb(st, ln, t):
    """Index of the t-th neighbour along the body (circular)."""
    i = np.arange(st.size)
    return st + np.mod(i - st + t, ln)


def point_features(x, y, nx, ny, ds, body_starts, h):
    """Dimensionless per-point features (N x 8): ds/h, 10 h * curvature,
    n_x, n_y, sin/cos(2 pi frac(x/h)), sin/cos(2 pi frac(y/h)).  The
    curvature is the turning of the normal between the two neighbours over
    the arc between them."""
    x, y, nx, ny, ds = (np.asarray(a, dtype=np.float64) for a in (x, y, nx, ny, ds))
    n = x.size
    st, ln = segments(body_starts, n)
    ip, im = nb(st, ln, 1), nb(st, ln, -1)
    th = np.arctan2(ny, nx)
    dth = np.mod(th[ip] - th[im] + math.pi, 2 * math.pi) - math.pi
    arc = 0.5 * ds[im] + ds + 0.5 * ds[ip]
    kap = dth / arc
    fx = x / h - np.floor(x / h)
    fy = y / h - np.floor(y / h)
    F = np.stack([ds / h, 10.0 * h * kap, nx, ny, np.sin(2 * math.pi * fx), np.cos(2 * math.pi * fx),
                  np.sin(2 * math.pi * fy), np.cos(2 * math.pi * fy)], axis=1)
    return F


def layer_dims(nfeat=NFEAT, width=WIDTH, nlayers=NLAYERS, band=BAND):
    dims = [nfeat] + [width] * (nlayers - 1) + [2 * band + 1]
    return [(dims[l], dims[l + 1]) for l in range(nlayers)]


def nparams(**kw):
    return sum(co * ci * KSIZE + co for ci, co in layer_dims(**kw))


def unpack(theta, **kw):
    """Flat parameters -> [(W (co, ci, 5), b (co,))] in layer order."""
    out, o = [], 0
    for ci, co in layer_dims(**kw):
        W = theta[o:o + co * ci * KSIZE].reshape(co, ci, KSIZE)
        o += co * ci * KSIZE
        b = theta[o:o + co]
        o += co
        out.append((W, b))
    return out


def init_params(seed=0, **kw):
    """He-uniform for the ReLU layers, small last layer (C starts near I)."""
    rng = np.random.default_rng(seed)
    parts = []
    dims = layer_dims(**kw)
    for l, (ci, co) in enumerate(dims):
        bound = math.sqrt(6.0 / (ci * KSIZE)) if l < len(dims) - 1 else 0.01 / math.sqrt(ci * KSIZE)
        parts.append(rng.uniform(-bound, bound, size=co * ci * KSIZE))
        parts.append(np.zeros(co))
    return np.concatenate(parts).astype(np.float32)


def conv(a, W, b, st, ln):
    """z[i, o] = b[o] + sum_{k,t} W[o,k,t+2] a[nb(i,t), k]."""
    z = np.broadcast_to(b, (a.shape[0], b.size)).astype(np.float64).copy()
    for t in range(-2, 3):
        z += a[nb(st, ln, t)] @ W[:, :, t + 2].T
    return z


def forward(theta, F, st, ln, weights_bf16=True):
    """Band coefficients c (N x (2K+1)) and the activations (for backward)."""
    layers = unpack(np.asarray(theta))
    acts = [np.asarray(F, dtype=np.float64)]
    for l, (W, b) in enumerate(layers):
        Wq = bf16_round(W) if weights_bf16 else W
        z = conv(acts[-1], Wq.astype(np.float64), b.astype(np.float64), st, ln)
        acts.append(np.maximum(z, 0.0) if l < len(layers) - 1 else z)
    c = acts[-1].copy()
    K = (c.shape[1] - 1) // 2
    c[:, K] += 1.0
    return c, acts


def band_apply(c, r, st, ln):
    K = (c.shape[1] - 1) // 2
    return sum(c[:, t + K] * r[nb(st, ln, t)] for t in range(-K, K + 1))


def band_apply_T(c, u, st, ln):
    """(C^T u)_i = sum_t c[nb(i,-t), t] u[nb(i,-t)]."""
    K = (c.shape[1] - 1) // 2
    out = np.zeros_like(u)
    for t in range(-K, K + 1):
        j = nb(st, ln, -t)
        out += c[j, t + K] * u[j]
    return out


def precond_apply(c, r, w, st, ln):
    """M r = W^-1 C^T C r."""
    return band_apply_T(c, band_apply(c, r, st, ln), st, ln) / w


def loss_and_grad(theta, F, st, ln, w, b, x, pair_off, weights_bf16=True):
    """Mean relative error of M b against x over the pairs (points
    pair_off[p]..pair_off[p+1]), and its gradient w.r.t. the FP32 master
    parameters (straight-through the bf16 rounding)."""
    c, acts = forward(theta, F, st, ln, weights_bf16)
    K = (c.shape[1] - 1) // 2
    u = band_apply(c, b, st, ln)
    z = band_apply_T(c, u, st, ln) / w
    npair = len(pair_off) - 1
    loss = 0.0
    gz = np.zeros_like(z)
    for p in range(npair):
        s = slice(pair_off[p], pair_off[p + 1])
        xx = float(np.dot(x[s], x[s]))
        e = z[s] - x[s]
        loss += float(np.dot(e, e)) / xx / npair
        gz[s] = 2.0 * e / xx / npair
    y = gz / w
    gu = band_apply(c, y, st, ln)
    gc = np.zeros_like(c)
    for t in range(-K, K + 1):
        j = nb(st, ln, t)
        gc[:, t + K] = y[j] * u + gu * b[j]
    # back through the network
    layers = unpack(np.asarray(theta))
    grads = []
    g = gc
    for l in range(len(layers) - 1, -1, -1):
        W, bias = layers[l]
        Wq = (bf16_round(W) if weights_bf16 else W).astype(np.float64)
        if l < len(layers) - 1:
            g = g * (acts[l + 1] > 0)
        a = acts[l]
        gW = np.zeros(W.shape)
        for t in range(-2, 3):
            gW[:, :, t + 2] = g.T @ a[nb(st, ln, t)]
        gb = g.sum(axis=0)
        grads.append((gW, gb))
        ga = np.zeros_like(a)
        for t in range(-2, 3):
            # a[nb(i,t)] feeds z[i]  ->  a[j] collects from i = nb(j,-t)
            ga += (g @ Wq[:, :, t + 2])[nb(st, ln, -t)]
        g = ga
    flat = []
    for gW, gb in reversed(grads):
        flat.append(gW.reshape(-1))
        flat.append(gb)
    return loss, np.concatenate(flat)


def adam_update(theta, grad, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) on FP32 master parameters."""
    m[:] = beta1 * m + (1 - beta1) * grad
    v[:] = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    theta[:] = theta - lr * mh / (np.sqrt(vh) + eps)
    return theta
