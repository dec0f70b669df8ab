// Schur complements of the immersed-layer saddle-point systems and their
// on-device Krylov solve.
//
// The reference builds each dense Schur complement column by column, with one
// regularize! + inverse_laplacian! (an FFT convolution of the whole grid) +
// interpolate! per column (src/matrix_operators.jl:9-244), then solves it with
// a dense LU on every call (test/literate/problems.jl:291, neumann.jl:123).
//
// Here every entry is evaluated directly from the lattice Green's function:
// the interpolation-side and regularization-side operators of point k are
// short separable stencils U_k (4 or 5 taps per direction, up to two terms),
// and since L^{-1} is the exact linear convolution with G,
//     (U L^{-1} V^T)_{kl} = (1/factor) sum_{a,b} U_k(a) G(a-b) V_l(b)
//                         = (1/factor) sum_{dx,dy} Cx(dx) Cy(dy) G(D + (dx,dy)),
// with Cx, Cy the 1-D correlations of the two stencils (9 values each) and D the
// offset of the stencil bases.  This is O(N^2 * 81) FP64 work instead of
// O(N * P^2 log P), and gives the same matrix (up to FP64 rounding) provided
// every stencil stays clear of the grid's ghost layer.
//
// The solve is CG in the ds-weighted inner product (the matrices are M*diag(w)
// with M symmetric), one CTA per problem, in FP64: an FP32 matvec loses the
// Krylov convergence on these ill-conditioned (cond ~ 1e4-1e5) and, for the
// Dirichlet problem, indefinite (one negative eigenvalue) systems.
// Convergence is declared on the FP64 residual ||b - A x||_2 <= tol ||b||_2.
#include <math.h>

#include <algorithm>

#include "ilm_internal.cuh"

namespace ilm {

constexpr int FW = 5;  // functional window width

struct Functional {
  // two separable terms: coef, x base, y base, 5 x-weights, 5 y-weights
  double coef[2];
  int xb[2], yb[2];
  double xw[2][FW], yw[2][FW];
  int nterm;
};

// The same functional with every weight split into a float-float (hi, lo)
// pair once per point, for the batched float-float builds (the split is an
// FP64 subtraction, which GB300 issues at a small fraction of its FP32 rate;
// split per point pair it was a large part of the build).  Written over the
// Functional buffers, so it is no larger.
struct FunctionalFF {
  float coef[2][2];
  float w[2];                  // the point's regularization weight ds (hi, lo)
  short xb[2], yb[2], nterm, pad_;  // grid base indices (|index| < 32768)
  float xw[2][FW][2], yw[2][FW][2];
};
static_assert(sizeof(FunctionalFF) <= sizeof(Functional), "FunctionalFF overlays Functional buffers");

// Build the per-point functionals for one Schur kind.  side 0 = left
// (interpolation side, no ds weight), side 1 = right (regularization side).
__global__ void k_functionals(int N, int kind, const int* __restrict__ bxP, const int* __restrict__ bxD,
                              const int* __restrict__ byP, const int* __restrict__ byD,
                              const double* __restrict__ wxP, const double* __restrict__ wxD,
                              const double* __restrict__ wyP, const double* __restrict__ wyD,
                              const double* __restrict__ nx, const double* __restrict__ ny, double invh,
                              Functional* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  Functional F;
  for (int p = 0; p < 2; ++p) {
    F.coef[p] = 0.0;
    F.xb[p] = F.yb[p] = 0;
    for (int t = 0; t < FW; ++t) F.xw[p][t] = F.yw[p][t] = 0.0;
  }
  const double* wxp = wxP + (size_t)k * NTAP;
  const double* wxd = wxD + (size_t)k * NTAP;
  const double* wyp = wyP + (size_t)k * NTAP;
  const double* wyd = wyD + (size_t)k * NTAP;
  auto at = [](const double* w, int t) { return (t >= 0 && t < NTAP) ? w[t] : 0.0; };
  if (kind == ILM_SCHUR_RTLINVR) {
    // plain E on Nodes{Primal}
    F.nterm = 1;
    F.coef[0] = 1.0;
    F.xb[0] = bxP[k];
    F.yb[0] = byP[k];
    for (int t = 0; t < NTAP; ++t) {
      F.xw[0][t] = wxp[t];
      F.yw[0][t] = wyp[t];
    }
  } else if (kind == ILM_SCHUR_CLINVCT) {
    // C_s on Nodes{Dual}: (n_x/h) [wxD (x) (wyP[t-1]-wyP[t])] + (n_y/h) [(wxP[t]-wxP[t-1]) (x) wyD]
    F.nterm = 2;
    F.coef[0] = nx[k] * invh;
    F.xb[0] = bxD[k];
    F.yb[0] = byP[k];
    for (int t = 0; t < FW; ++t) {
      F.xw[0][t] = at(wxd, t);
      F.yw[0][t] = at(wyp, t - 1) - at(wyp, t);
    }
    F.coef[1] = ny[k] * invh;
    F.xb[1] = bxP[k];
    F.yb[1] = byD[k];
    for (int t = 0; t < FW; ++t) {
      F.xw[1][t] = at(wxp, t) - at(wxp, t - 1);
      F.yw[1][t] = at(wyd, t);
    }
  } else {  // ILM_SCHUR_GLINVD: D_s functional on Nodes{Primal}
    F.nterm = 2;
    F.coef[0] = nx[k] * invh;
    F.xb[0] = bxD[k] - 1;
    F.yb[0] = byP[k];
    for (int t = 0; t < FW; ++t) {
      F.xw[0][t] = at(wxd, t) - at(wxd, t - 1);
      F.yw[0][t] = at(wyp, t);
    }
    F.coef[1] = ny[k] * invh;
    F.xb[1] = bxP[k];
    F.yb[1] = byD[k] - 1;
    for (int t = 0; t < FW; ++t) {
      F.xw[1][t] = at(wxp, t);
      F.yw[1][t] = at(wyd, t) - at(wyd, t - 1);
    }
  }
  out[k] = F;
}

// A[k + N l] = sgn * sum_{p,q} cL_kp cR_lq w_l sum_{dx,dy} Cx Cy G(...)
__global__ void __launch_bounds__(256) k_schur_pairs(int N, const Functional* __restrict__ F,
                                                     const double* __restrict__ w, const double* __restrict__ G,
                                                     int ld, int M, double sgn, double* __restrict__ A) {
  const int k = blockIdx.y * 16 + threadIdx.y;
  const int l = blockIdx.x * 16 + threadIdx.x;
  if (k >= N || l >= N) return;
  const Functional& Fk = F[k];
  const Functional& Fl = F[l];
  double total = 0.0;
  for (int p = 0; p < Fk.nterm; ++p) {
    for (int q = 0; q < Fl.nterm; ++q) {
      double cx[2 * FW - 1], cy[2 * FW - 1];
#pragma unroll
      for (int d = 0; d < 2 * FW - 1; ++d) {
        cx[d] = 0.0;
        cy[d] = 0.0;
      }
#pragma unroll
      for (int t = 0; t < FW; ++t) {
#pragma unroll
        for (int u = 0; u < FW; ++u) {
          cx[t - u + FW - 1] += Fk.xw[p][t] * Fl.xw[q][u];
          cy[t - u + FW - 1] += Fk.yw[p][t] * Fl.yw[q][u];
        }
      }
      const int Dx = Fk.xb[p] - Fl.xb[q] - (FW - 1);
      const int Dy = Fk.yb[p] - Fl.yb[q] - (FW - 1);
      double acc = 0.0;
#pragma unroll
      for (int dy = 0; dy < 2 * FW - 1; ++dy) {
        int my = abs(Dy + dy);
        my = my > M ? M : my;
        const double* Grow = G + (size_t)my;
        double racc = 0.0;
#pragma unroll
        for (int dx = 0; dx < 2 * FW - 1; ++dx) {
          int mx = abs(Dx + dx);
          mx = mx > M ? M : mx;
          racc += cx[dx] * __ldg(Grow + (size_t)mx * ld);
        }
        acc += cy[dy] * racc;
      }
      total += Fk.coef[p] * Fl.coef[q] * acc;
    }
  }
  A[(size_t)l * N + k] = sgn * w[l] * total;
}

// nRTRn: A[k + N l] = scale * w_l * (nx_k nx_l <phiU_k,phiU_l> + ny_k ny_l <phiV_k,phiV_l>)
__global__ void k_nrtrn(int N, const int* __restrict__ bxP, const int* __restrict__ bxD, const int* __restrict__ byP,
                        const int* __restrict__ byD, const double* __restrict__ wxP, const double* __restrict__ wxD,
                        const double* __restrict__ wyP, const double* __restrict__ wyD, const double* __restrict__ nx,
                        const double* __restrict__ ny, const double* __restrict__ w, double scale,
                        double* __restrict__ A) {
  const int k = blockIdx.y * 16 + threadIdx.y;
  const int l = blockIdx.x * 16 + threadIdx.x;
  if (k >= N || l >= N) return;
  auto ov = [&](const int* b, const double* wv) {
    const int d = b[k] - b[l];
    double s = 0.0;
    for (int t = 0; t < NTAP; ++t) {
      const int u = t + d;
      if (u >= 0 && u < NTAP) s += wv[(size_t)k * NTAP + t] * wv[(size_t)l * NTAP + u];
    }
    return s;
  };
  const double su = ov(bxD, wxD) * ov(byP, wyP);
  const double sv = ov(bxP, wxP) * ov(byD, wyD);
  A[(size_t)l * N + k] = scale * w[l] * (nx[k] * nx[l] * su + ny[k] * ny[l] * sv);
}

int schur_build(ilm_cache_s* c, int which, double scale, double* A, cudaStream_t st, bool any_cache) {
  const int N = c->npts;
  if (N == 0) return ILM_OK;
  const ilm_grid_s& g = c->grid;
  dim3 blk(16, 16), grd((N + 15) / 16, (N + 15) / 16);
  if (which == ILM_SCHUR_NRTRN) {
    // R_f = diag(ds/h^2) phi (GridScaling) or phi (IndexScaling); E = phi
    DevBuf W;
    ILM_TRY(W.alloc((size_t)N * sizeof(double)));
    if (c->scaling == ILM_GRID_SCALING) {
      ILM_TRY(st_axpby(N, ILM_F64, 1.0 / (g.h * g.h), c->ds64.p, 0.0, nullptr, W.p, st));
    } else {
      ILM_TRY(st_fill(N, ILM_F64, 1.0, W.p, st));
    }
    k_nrtrn<<<grd, blk, 0, st>>>(N, c->bx[0].as<int>(), c->bx[1].as<int>(), c->by[0].as<int>(), c->by[1].as<int>(),
                                 c->wx64[0].as<double>(), c->wx64[1].as<double>(), c->wy64[0].as<double>(),
                                 c->wy64[1].as<double>(), c->nx64.as<double>(), c->ny64.as<double>(),
                                 W.as<double>(), scale, A);
    ILM_CHECK_LAUNCH();
    ILM_CHECK_CUDA(cudaStreamSynchronize(st));
    return ILM_OK;
  }
  if (c->kind == ILM_CACHE_VECTOR && !any_cache) {
    set_error("dense Schur build for vector caches not supported");
    return ILM_ERR_UNSUPPORTED;
  }
  const double* G = nullptr;
  int ld = 0;
  const int M = std::max(g.nx, g.ny) + 16;
  ILM_TRY(lgf_table_device(M, &G, &ld, st));
  DevBuf F, W;
  ILM_TRY(F.alloc((size_t)N * sizeof(Functional)));
  ILM_TRY(W.alloc((size_t)N * sizeof(double)));
  const double invh = c->scaling == ILM_GRID_SCALING ? 1.0 / g.h : 1.0;
  // w_l = regularization weight / factor : GridScaling ds_l/h^2 * h^2 = ds_l
  const double h2 = g.h * g.h;
  (void)h2;
  k_functionals<<<(N + 127) / 128, 128, 0, st>>>(N, which, c->bx[0].as<int>(), c->bx[1].as<int>(), c->by[0].as<int>(),
                                                 c->by[1].as<int>(), c->wx64[0].as<double>(), c->wx64[1].as<double>(),
                                                 c->wy64[0].as<double>(), c->wy64[1].as<double>(),
                                                 c->nx64.as<double>(), c->ny64.as<double>(), invh, F.as<Functional>());
  ILM_CHECK_LAUNCH();
  if (c->scaling == ILM_GRID_SCALING) {
    ILM_CHECK_CUDA(cudaMemcpyAsync(W.p, c->ds64.p, N * sizeof(double), cudaMemcpyDeviceToDevice, st));
  } else {
    ILM_TRY(st_fill(N, ILM_F64, 1.0, W.p, st));
  }
  // RTLinvR: -scale ; CLinvCT: -scale ; GLinvD: +scale (G_s = -D_s^T)
  const double sgn = (which == ILM_SCHUR_GLINVD) ? scale : -scale;
  k_schur_pairs<<<grd, blk, 0, st>>>(N, F.as<Functional>(), W.as<double>(), G, ld, ld - 1, sgn, A);
  ILM_CHECK_LAUNCH();
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  return ILM_OK;
}

// ---------------------------------------------------------------------------
// batched CG, one CTA per problem
// ---------------------------------------------------------------------------
constexpr int CG_THREADS = 512;

__device__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    red[32] = s;
  }
  __syncthreads();
  return red[32];
}

// y = A x (A column-major n x n, FP64), rows distributed over the block
__device__ __forceinline__ void gemv64(const double* __restrict__ A, const double* __restrict__ x,
                                       double* __restrict__ y, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double* __restrict__ col = A + i;
    double a0 = 0.0, a1 = 0.0;
    int j = 0;
    for (; j + 1 < n; j += 2) {
      a0 = fma(__ldg(col + (size_t)j * n), x[j], a0);
      a1 = fma(__ldg(col + (size_t)(j + 1) * n), x[j + 1], a1);
    }
    if (j < n) a0 = fma(__ldg(col + (size_t)j * n), x[j], a0);
    y[i] = a0 + a1;
  }
}

// CG in the w-weighted inner product (A = M diag(w), M symmetric), FP64.
// The recursive residual decides when to check; convergence is declared on
// the true residual ||b - A x||_2 <= tol ||b||_2, which is also recomputed
// (and substituted) every 100 iterations.  Bounded by maxiter: no waits.
__global__ void __launch_bounds__(CG_THREADS) k_cg(const CGParams* __restrict__ P) {
  const CGParams pr = P[blockIdx.x];
  const int n = pr.n;
  extern __shared__ __align__(16) unsigned char smraw[];
  double* red = reinterpret_cast<double*>(smraw);  // 40 doubles
  double* x = red + 40;
  double* r = x + n;
  double* p = r + n;
  double* q = p + n;
  double* w = q + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    x[i] = 0.0;
    r[i] = pr.b[i];
    p[i] = r[i];
    w[i] = pr.w ? pr.w[i] : 1.0;
  }
  __syncthreads();
  double bb = 0.0, rz = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    bb += r[i] * r[i];
    rz += w[i] * r[i] * r[i];
  }
  bb = block_sum(bb, red);
  rz = block_sum(rz, red);
  const double bnorm = sqrt(bb);
  const double thr = pr.tol * bnorm;
  int it = 0;
  double relres = bnorm > 0 ? 1.0 : 0.0;
  bool done = bnorm == 0.0;
  while (!done && it < pr.maxiter) {
    gemv64(pr.A64, p, q, n);
    __syncthreads();
    double pq = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) pq += w[i] * p[i] * q[i];
    pq = block_sum(pq, red);
    if (pq == 0.0) break;
    const double alpha = rz / pq;
    double rr = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      rr += r[i] * r[i];
    }
    rr = block_sum(rr, red);
    ++it;
    relres = bnorm > 0 ? sqrt(rr) / bnorm : 0.0;
    if (sqrt(rr) <= thr || (it % 100) == 0 || it == pr.maxiter) {
      gemv64(pr.A64, x, q, n);
      __syncthreads();
      double tr = 0.0;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        r[i] = pr.b[i] - q[i];
        tr += r[i] * r[i];
      }
      tr = block_sum(tr, red);
      relres = bnorm > 0 ? sqrt(tr) / bnorm : 0.0;
      if (sqrt(tr) <= thr) {
        done = true;
        break;
      }
    }
    double rzn = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) rzn += w[i] * r[i] * r[i];
    rzn = block_sum(rzn, red);
    const double beta = rzn / rz;
    rz = rzn;
    for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = r[i] + beta * p[i];
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) pr.x[i] = x[i];
  if (threadIdx.x == 0) {
    if (pr.iters) *pr.iters = it;
    if (pr.relres) *pr.relres = relres;
  }
}

int launch_cg_batched(const CGParams* probs_dev, int nprob, int max_n, cudaStream_t st) {
  const size_t smem = 40 * sizeof(double) + (size_t)max_n * 5 * sizeof(double) + 64;
  if (smem > 227 * 1024) {
    set_error("CG: problem of %d unknowns exceeds the shared-memory solver", max_n);
    return ILM_ERR_SIZE_LIMIT;
  }
  ILM_CHECK_CUDA(cudaFuncSetAttribute(k_cg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_cg<<<nprob, CG_THREADS, smem, st>>>(probs_dev);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

}  // namespace ilm

// ---------------------------------------------------------------------------
// batched Schur builds: all problems of a batch in one launch
// ---------------------------------------------------------------------------
namespace ilm {

__global__ void k_functionals_batched(int Ptot, const int* __restrict__ pt2prob, const SchurProbDev* __restrict__ pr,
                                      const int* __restrict__ bxP, const int* __restrict__ bxD,
                                      const int* __restrict__ byP, const int* __restrict__ byD,
                                      const double* __restrict__ wxP, const double* __restrict__ wxD,
                                      const double* __restrict__ wyP, const double* __restrict__ wyD,
                                      const double* __restrict__ nx, const double* __restrict__ ny,
                                      const double* __restrict__ w, Functional* __restrict__ out, int force_kind) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= Ptot) return;
  SchurProbDev P = pr[pt2prob[g]];
  if (force_kind >= 0) P.kind = force_kind;
  // reuse the single-problem kernel body on a one-point view
  const int k = g;
  Functional F;
  for (int p = 0; p < 2; ++p) {
    F.coef[p] = 0.0;
    F.xb[p] = F.yb[p] = 0;
    for (int t = 0; t < FW; ++t) F.xw[p][t] = F.yw[p][t] = 0.0;
  }
  const double* wxp = wxP + (size_t)k * NTAP;
  const double* wxd = wxD + (size_t)k * NTAP;
  const double* wyp = wyP + (size_t)k * NTAP;
  const double* wyd = wyD + (size_t)k * NTAP;
  auto at = [](const double* w, int t) { return (t >= 0 && t < NTAP) ? w[t] : 0.0; };
  if (P.kind == ILM_SCHUR_RTLINVR) {
    F.nterm = 1;
    F.coef[0] = 1.0;
    F.xb[0] = bxP[k];
    F.yb[0] = byP[k];
    for (int t = 0; t < NTAP; ++t) {
      F.xw[0][t] = wxp[t];
      F.yw[0][t] = wyp[t];
    }
  } else if (P.kind == ILM_SCHUR_GLINVD) {  // D_s functional on Nodes{Primal} (as k_functionals)
    F.nterm = 2;
    F.coef[0] = nx[k] * P.invh;
    F.xb[0] = bxD[k] - 1;
    F.yb[0] = byP[k];
    for (int t = 0; t < FW; ++t) {
      F.xw[0][t] = at(wxd, t) - at(wxd, t - 1);
      F.yw[0][t] = at(wyp, t);
    }
    F.coef[1] = ny[k] * P.invh;
    F.xb[1] = bxP[k];
    F.yb[1] = byD[k] - 1;
    for (int t = 0; t < FW; ++t) {
      F.xw[1][t] = at(wxp, t);
      F.yw[1][t] = at(wyd, t) - at(wyd, t - 1);
    }
  } else {  // CLinvCT
    F.nterm = 2;
    F.coef[0] = nx[k] * P.invh;
    F.xb[0] = bxD[k];
    F.yb[0] = byP[k];
    for (int t = 0; t < FW; ++t) {
      F.xw[0][t] = at(wxd, t);
      F.yw[0][t] = at(wyp, t - 1) - at(wyp, t);
    }
    F.coef[1] = ny[k] * P.invh;
    F.xb[1] = bxP[k];
    F.yb[1] = byD[k];
    for (int t = 0; t < FW; ++t) {
      F.xw[1][t] = at(wxp, t) - at(wxp, t - 1);
      F.yw[1][t] = at(wyd, t);
    }
  }
  FunctionalFF Q;
  Q.nterm = (short)F.nterm;
  Q.pad_ = 0;
  {
    const double wk = w ? w[g] : 0.0;
    const float wh = (float)wk;
    Q.w[0] = wh;
    Q.w[1] = (float)(wk - (double)wh);
  }
  for (int p = 0; p < 2; ++p) {
    Q.xb[p] = (short)F.xb[p];
    Q.yb[p] = (short)F.yb[p];
    const float ch = (float)F.coef[p];
    Q.coef[p][0] = ch;
    Q.coef[p][1] = (float)(F.coef[p] - (double)ch);
    for (int t = 0; t < FW; ++t) {
      const float xh = (float)F.xw[p][t], yh = (float)F.yw[p][t];
      Q.xw[p][t][0] = xh;
      Q.xw[p][t][1] = (float)(F.xw[p][t] - (double)xh);
      Q.yw[p][t][0] = yh;
      Q.yw[p][t][1] = (float)(F.yw[p][t] - (double)yh);
    }
  }
  reinterpret_cast<FunctionalFF*>(out)[g] = Q;
}


// Batched Schur entries in float-float on the FP32 pipes (~2^-44 relative
// per operation; GB300 issues FP64 at a small fraction of its FP32 rate):
// the same 1-D weight correlations and LGF contractions as k_schur_pairs,
// with the weights read as float-float pairs (split once per point) and the
// LGF read from its float-float copy.
//
// T_kl = sum_{p,q} c_p c_q sum_{dx,dy} Cx(dx) Cy(dy) G(|Dx + dx|, |Dy + dy|)
// for the functionals of points k and l (Cx, Cy the 1-D correlations of their
// weights).
__device__ __forceinline__ FF pair_sum(const FunctionalFF& Fk, const FunctionalFF& Fl, const float2* __restrict__ G,
                                       int ld, int M) {
  FF total{0.f, 0.f};
  for (int p = 0; p < Fk.nterm; ++p) {
    FF xk[FW], yk[FW];
#pragma unroll
    for (int a = 0; a < FW; ++a) {
      xk[a] = FF{Fk.xw[p][a][0], Fk.xw[p][a][1]};
      yk[a] = FF{Fk.yw[p][a][0], Fk.yw[p][a][1]};
    }
    for (int q = 0; q < Fl.nterm; ++q) {
      FF cx[2 * FW - 1], cy[2 * FW - 1];
#pragma unroll
      for (int d = 0; d < 2 * FW - 1; ++d) cx[d] = cy[d] = FF{0.f, 0.f};
#pragma unroll
      for (int b = 0; b < FW; ++b) {
        const float xbh = Fl.xw[q][b][0], xbl = Fl.xw[q][b][1];
        const float ybh = Fl.yw[q][b][0], ybl = Fl.yw[q][b][1];
#pragma unroll
        for (int a = 0; a < FW; ++a) {
          ff_fma(cx[a - b + FW - 1], xk[a].hi, xk[a].lo, xbh, xbl);
          ff_fma(cy[a - b + FW - 1], yk[a].hi, yk[a].lo, ybh, ybl);
        }
      }
#pragma unroll
      for (int d = 0; d < 2 * FW - 1; ++d) {
        cx[d] = ff_renorm(cx[d].hi, cx[d].lo);
        cy[d] = ff_renorm(cy[d].hi, cy[d].lo);
      }
      const int Dx = Fk.xb[p] - Fl.xb[q] - (FW - 1);
      const int Dy = Fk.yb[p] - Fl.yb[q] - (FW - 1);
      FF acc{0.f, 0.f};
#pragma unroll
      for (int dy = 0; dy < 2 * FW - 1; ++dy) {
        int my = abs(Dy + dy);
        my = my > M ? M : my;
        const float2* Grow = G + (size_t)my;
        FF racc{0.f, 0.f};
#pragma unroll
        for (int dx = 0; dx < 2 * FW - 1; ++dx) {
          int mx = abs(Dx + dx);
          mx = mx > M ? M : mx;
          const float2 g = __ldg(Grow + (size_t)mx * ld);
          ff_fma(racc, g.x, g.y, cx[dx].hi, cx[dx].lo);
        }
        racc = ff_renorm(racc.hi, racc.lo);
        ff_fma(acc, cy[dy].hi, cy[dy].lo, racc.hi, racc.lo);
      }
      acc = ff_renorm(acc.hi, acc.lo);
      const FF cc = ff_mul(FF{Fk.coef[p][0], Fk.coef[p][1]}, FF{Fl.coef[q][0], Fl.coef[q][1]});
      ff_fma(total, cc.hi, cc.lo, acc.hi, acc.lo);
    }
  }
  return ff_renorm(total.hi, total.lo);
}

__global__ void __launch_bounds__(256) k_schur_pairs_batched(int nprob, const SchurProbDev* __restrict__ pr,
                                                             const FunctionalFF* __restrict__ F,
                                                             const double* __restrict__ w,
                                                             const float2* __restrict__ G, int ld, int M,
                                                             float* __restrict__ Shi, float* __restrict__ Slo) {
  int lo = 0, hi = nprob - 1;
  const int u = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pr[mid].tile0 <= u) lo = mid; else hi = mid - 1;
  }
  const SchurProbDev P = pr[lo];
  const int N = P.n;
  const int nt = (N + 15) / 16;
  // the tile sum T_kl = sum U_k(a) G(a - b) U_l(b) is symmetric (G depends on
  // |a - b| only and both sides use the same functionals): one CTA per tile
  // of the upper triangle (ti <= tj) in row-major order, writing S_kl = -w_l
  // T_kl and, off the diagonal tiles, S_lk = -w_k T_kl
  const int t = u - P.tile0;
  // tile row of triangle index t (FP32 estimate, corrected exactly below)
  const float tn = 2.0f * nt + 1.0f;
  int ti = (int)((tn - sqrtf(fmaxf(tn * tn - 8.0f * t, 0.0f))) * 0.5f);
  auto row0 = [nt](int i) { return i * nt - i * (i - 1) / 2; };  // first triangle tile of tile row i
  while (ti > 0 && row0(ti) > t) --ti;
  while (ti + 1 < nt && row0(ti + 1) <= t) ++ti;
  const int tj = ti + (t - row0(ti));
  const int k = ti * 16 + threadIdx.y;
  const int l = tj * 16 + threadIdx.x;
  if (k >= N || l >= N) return;
  const FunctionalFF& Fk = F[P.poff + k];
  const FunctionalFF& Fl = F[P.poff + l];
  const FF total = pair_sum(Fk, Fl, G, ld, M);
  // row-major float-float pair: S[k][l] = hi + lo
  const FF wl{-Fl.w[0], -Fl.w[1]};
  const FF v = ff_mul(wl, total);
  Shi[P.soff + (size_t)k * schur_ld(N) + l] = v.hi;
  Slo[P.soff + (size_t)k * schur_ld(N) + l] = v.lo;
  if (ti != tj) {
    const FF wk{-Fk.w[0], -Fk.w[1]};
    const FF vt = ff_mul(wk, total);
    Shi[P.soff + (size_t)l * schur_ld(N) + k] = vt.hi;
    Slo[P.soff + (size_t)l * schur_ld(N) + k] = vt.lo;
  }
}

int schur_build_batched(int nprob, const SchurProbDev* probs_dev, int total_tiles, int Ptot, const int* pt2prob,
                        const BatchWin& W, const double* w, Functional* F, float* Shi, float* Slo, int max_grid,
                        cudaStream_t st, const SchurProbDev* order, int nfirst, int tiles_first,
                        cudaEvent_t mid) {
  if (Ptot == 0) return ILM_OK;
  const float2* G = nullptr;
  int ld = 0;
  ILM_TRY(lgf_table_ff_device(max_grid + 16, &G, &ld, st));
  k_functionals_batched<<<(Ptot + 127) / 128, 128, 0, st>>>(Ptot, pt2prob, probs_dev, W.bx[0], W.bx[1], W.by[0],
                                                            W.by[1], W.wx64[0], W.wx64[1], W.wy64[0], W.wy64[1],
                                                            W.nx64, W.ny64, w, F, -1);
  ILM_CHECK_LAUNCH();
  // the pair tiles: one launch over probs_dev, or two over the build order
  // (the functionals above index probs_dev by problem, so it stays in
  // problem order)
  const FunctionalFF* FF_ = reinterpret_cast<const FunctionalFF*>(F);
  if (!order) {
    if (total_tiles > 0)
      k_schur_pairs_batched<<<total_tiles, dim3(16, 16), 0, st>>>(nprob, probs_dev, FF_, w, G, ld, ld - 1, Shi, Slo);
    ILM_CHECK_LAUNCH();
    return ILM_OK;
  }
  if (tiles_first > 0)
    k_schur_pairs_batched<<<tiles_first, dim3(16, 16), 0, st>>>(nfirst, order, FF_, w, G, ld, ld - 1, Shi, Slo);
  ILM_CHECK_LAUNCH();
  if (mid) ILM_CHECK_CUDA(cudaEventRecord(mid, st));
  const int tiles_second = total_tiles - tiles_first;
  if (tiles_second > 0)
    k_schur_pairs_batched<<<tiles_second, dim3(16, 16), 0, st>>>(nprob - nfirst, order + nfirst, FF_, w, G, ld,
                                                                 ld - 1, Shi, Slo);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

// The right-hand-side operator of the batched solves, built from the same
// LGF point-point sums as S: Dirichlet M = E L^-1 D_s (the Schur right-hand
// side E f*, f* = L^-1 D_s [f]), Neumann M = G_s L^-1 R (G_s f*, f* =
// L^-1 R [v_n]).  With the plain-interpolation functionals U and the double-
// layer functionals D of k_functionals, E L^-1 R = w_l U G U and
// G_s = -D^T, so M_kl = +w_l (U G D)_kl (Dirichlet) and -w_l (D G U)_kl
// (Neumann).  Full n x n tiles (M is not symmetric), one CTA per 16 x 16
// tile, float-float as k_schur_pairs_batched; the tiles of problem p start at
// pr[p].tile0 (the caller's full-tile numbering).
__global__ void __launch_bounds__(256) k_rhsop_pairs_batched(int nprob, const SchurProbDev* __restrict__ pr,
                                                             const FunctionalFF* __restrict__ FU,
                                                             const FunctionalFF* __restrict__ FD,
                                                             const double* __restrict__ w,
                                                             const float2* __restrict__ G, int ld, int M,
                                                             float* __restrict__ Mhi, float* __restrict__ Mlo) {
  int lo = 0, hi = nprob - 1;
  const int u = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pr[mid].tile0 <= u) lo = mid; else hi = mid - 1;
  }
  const SchurProbDev P = pr[lo];
  const int N = P.n;
  const int nt = (N + 15) / 16;
  const int t = u - P.tile0;
  const int ti = t / nt, tj = t - (t / nt) * nt;
  const int k = ti * 16 + threadIdx.y;
  const int l = tj * 16 + threadIdx.x;
  if (k >= N || l >= N) return;
  const bool dir = P.kind == ILM_SCHUR_RTLINVR;
  const FunctionalFF& Fl = dir ? FD[P.poff + l] : FU[P.poff + l];
  const FF total = pair_sum(dir ? FU[P.poff + k] : FD[P.poff + k], Fl, G, ld, M);
  const FF wl = dir ? FF{Fl.w[0], Fl.w[1]} : FF{-Fl.w[0], -Fl.w[1]};
  const FF v = ff_mul(wl, total);
  Mhi[P.soff + (size_t)k * schur_ld(N) + l] = v.hi;
  Mlo[P.soff + (size_t)k * schur_ld(N) + l] = v.lo;
}

int rhsop_build_batched(int nprob, const SchurProbDev* probs_full_dev, int total_tiles, int Ptot, const int* pt2prob,
                        const BatchWin& W, const double* w, Functional* FU, Functional* FD, float* Mhi, float* Mlo,
                        int max_grid, cudaStream_t st) {
  if (Ptot == 0) return ILM_OK;
  const float2* G = nullptr;
  int ld = 0;
  ILM_TRY(lgf_table_ff_device(max_grid + 16, &G, &ld, st));
  k_functionals_batched<<<(Ptot + 127) / 128, 128, 0, st>>>(Ptot, pt2prob, probs_full_dev, W.bx[0], W.bx[1], W.by[0],
                                                            W.by[1], W.wx64[0], W.wx64[1], W.wy64[0], W.wy64[1],
                                                            W.nx64, W.ny64, w, FU, ILM_SCHUR_RTLINVR);
  ILM_CHECK_LAUNCH();
  k_functionals_batched<<<(Ptot + 127) / 128, 128, 0, st>>>(Ptot, pt2prob, probs_full_dev, W.bx[0], W.bx[1], W.by[0],
                                                            W.by[1], W.wx64[0], W.wx64[1], W.wy64[0], W.wy64[1],
                                                            W.nx64, W.ny64, w, FD, ILM_SCHUR_GLINVD);
  ILM_CHECK_LAUNCH();
  k_rhsop_pairs_batched<<<total_tiles, dim3(16, 16), 0, st>>>(nprob, probs_full_dev,
                                                              reinterpret_cast<const FunctionalFF*>(FU),
                                                              reinterpret_cast<const FunctionalFF*>(FD), w, G, ld,
                                                              ld - 1, Mhi, Mlo);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

size_t functional_size() { return sizeof(Functional); }

}  // namespace ilm
