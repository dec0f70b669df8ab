// Stokes flow with no-slip surfaces on a vector cache: the reference's
// StokesFlowProblem `solve` (test/literate/stokes.jl:101-166) on the device,
// for one or several velocity right-hand sides at once.
//
//   psi*  = L^-2 (-C D_s^symm [v])            (surface viscous flux, twice inverted)
//   phi   = L^-1 R (n . [v]);  v_phi = G phi   (normal-velocity jump)
//   v'    = avg(v_b) - E v_phi - E C psi*
//   S sigma = v',  S = -C_s L^-2 C_s^T         (create_CL2invCT, :102-128)
//   psi   = psi* + L^-2 (-C_s^T sigma);  v = C psi + v_phi
//   psi  += L^-1 (-C^x_s^T Ss^-1 G^x_s phi),  Ss = -C_s L^-1 C_s^T (scalar, :71-93)
//   sigma <- F^2 sigma  (surface filter, :247-262)
//
// The reference forms S and Ss densely (2N and N columns of operator
// applications) and LU-solves them.  L^-2 is two grid-truncated LGF
// convolutions, which is not translation invariant, so S has no point-pair
// closed form.  Both Schur systems are solved matrix-free, in the symmetric
// form y = W sigma (W = diag(ds)): -S W^-1 and Ss W^-1 are symmetric
// positive semi-definite.  All right-hand sides are solved together by block
// CG: each iteration applies the operator to every column of the direction
// block, A-orthonormalises the block (eigen-decomposition of its s x s Gram
// matrix; directions that have become dependent are dropped), and forms the
// step and the next direction block from s x s products.  The right-hand
// sides share the slowly converging modes (the near-null modes of thin
// bodies), which the block recurrence resolves for all of them at once.
//
// Preconditioner of S: -C_s L^-2 C_s^T and the single layer -E L^-1 E^T are
// pseudo-differential operators of the same order (the Stokeslet and the
// log kernel), so the inverse of the Nodes{Primal} Schur complement
// P = -E L^-1 E^T (LGF point-point sums, as create_RTLinvR), applied to each
// velocity component, bounds the condition number independently of the
// point count on smooth bodies.  P is indefinite in its constant mode (the
// LGF's logarithm changes sign at large distances); adding c 1 1^T with
// c = 2 |1^T P 1| / N^2 makes it positive definite.  Its inverse is formed
// once per cache by Gauss-Jordan elimination on the device (positive pivots
// are checked; c grows if one is not) and applied as a dense product.
//
// The filter F = W^-1 E R, W = diag(E R 1): the filtered interpolation of
// CartesianGrids' Regularize(filter = true) (un-vendored) restated from
// Goza, Liska, Morley & Colonius (2016).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <vector>

#include "ilm_internal.cuh"

namespace ilm {
namespace {

inline void* elem_ptr(const void* base, size_t elems, int dtype) {
  return (void*)((const unsigned char*)base + elems * (dtype == ILM_F64 ? 8 : 4));
}

template <typename T>
__global__ void k_ndot(int n, const T* __restrict__ nx, const T* __restrict__ ny, const T* __restrict__ v,
                       T* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = nx[k] * v[k] + ny[k] * v[n + k];
}

constexpr int STOKES_PC_MAX = 4096;  // largest N with a preconditioner (N x N FP64 inverse)

template <typename T>
__global__ void k_to_op(int n, int N, const double* __restrict__ y, const double* __restrict__ ds,
                        T* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (T)(y[i] / ds[i % N]);
}

template <typename T>
__global__ void k_from_op(int n, const T* __restrict__ in, double sgn, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = sgn * (double)in[i];
}

// G[i + j sa] = sum_k A[k + i lda] B[k + j ldb]; one CTA per entry
// (deterministic order)
__global__ void __launch_bounds__(256) k_gram(int n, const double* __restrict__ A, int lda, int sa,
                                              const double* __restrict__ B, int ldb, double* __restrict__ G) {
  __shared__ double red[8];
  const int i = blockIdx.x % sa, j = blockIdx.x / sa;
  const double* a = A + (size_t)i * lda;
  const double* b = B + (size_t)j * ldb;
  double acc = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) acc = fma(a[k], b[k], acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    G[blockIdx.x] = t;
  }
}

// C (n x t) = alpha A (n x k) B (k x t) + beta C, column-major; one thread
// per row, eight columns of C per pass.  beta = 0 does not read C.
__global__ void __launch_bounds__(256) k_gemm_rows(int n, int k, int t, const double* __restrict__ A, int lda,
                                                   const double* __restrict__ B, int ldb, double alpha, double beta,
                                                   double* C, int ldc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int j0 = 0; j0 < t; j0 += 8) {
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    const int nj = min(8, t - j0);
    for (int kk = 0; kk < k; ++kk) {
      const double a = A[i + (size_t)kk * lda];
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < nj) acc[q] = fma(a, __ldg(B + kk + (size_t)(j0 + q) * ldb), acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (q >= nj) break;
      double* cp = C + i + (size_t)(j0 + q) * ldc;
      *cp = beta == 0.0 ? alpha * acc[q] : fma(alpha, acc[q], beta * *cp);
    }
  }
}

// T = sym(Sp diag(1/ds)) + shift (N x N)
__global__ void k_pc_form(int N, const double* __restrict__ Sp, const double* __restrict__ ds, double shift,
                          double* __restrict__ T) {
  const size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (idx >= (size_t)N * N) return;
  const int i = (int)(idx % N), j = (int)(idx / N);
  T[idx] = 0.5 * (Sp[idx] / ds[j] + Sp[j + (size_t)i * N] / ds[i]) + shift;
}

// out[j] = sum_i Sp[i][j] / ds[j] (column sums of Sp diag(1/ds), for the shift)
__global__ void __launch_bounds__(256) k_pc_sum(int N, const double* __restrict__ Sp, const double* __restrict__ ds,
                                                double* __restrict__ out) {
  __shared__ double red[8];
  const int j = blockIdx.x;  // one CTA per column, deterministic
  double acc = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) acc += Sp[i + (size_t)j * N];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    out[j] = t / ds[j];
  }
}

// Gauss-Jordan inversion in place without pivoting (T symmetric positive
// definite): step k turns column k into a column of the inverse.  The pivot
// column and row of step k (old values) come from colk / rowk; the new
// column and row k + 1 are written to coln / rown for the next step.  A
// non-positive pivot records k + 1 in *bad (first one wins) and is replaced
// by 1 so that the remaining steps stay finite.
__global__ void k_gj_init(int N, const double* __restrict__ T, double* __restrict__ col, double* __restrict__ row) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) {
    col[i] = T[i];
    row[i] = T[(size_t)i * N];
  }
}

__global__ void k_gj_step(int N, int k, double* __restrict__ T, const double* __restrict__ colk,
                          const double* __restrict__ rowk, double* __restrict__ coln, double* __restrict__ rown,
                          int* __restrict__ bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= N || j >= N) return;
  double p = rowk[k];
  if (!(p > 0.0)) {
    if (i == 0 && j == 0) atomicCAS(bad, 0, k + 1);
    p = 1.0;
  }
  const double ip = 1.0 / p;
  double v;
  if (i == k)
    v = j == k ? ip : rowk[j] * ip;
  else if (j == k)
    v = -colk[i] * ip;
  else
    v = T[i + (size_t)j * N] - colk[i] * rowk[j] * ip;
  T[i + (size_t)j * N] = v;
  if (j == k + 1) coln[i] = v;
  if (i == k + 1) rown[j] = v;
}

int ensure_stokes_pc(ilm_cache_s* c, cudaStream_t st) {
  if (c->stokes_pc_ready) return ILM_OK;
  const int N = c->npts;
  const size_t nn = (size_t)N * N;
  DevBuf Sp, sums, gj, bad;
  ILM_TRY(Sp.alloc(nn * sizeof(double)));
  ILM_TRY(c->stokes_pc.alloc(nn * sizeof(double)));
  ILM_TRY(sums.alloc((size_t)N * sizeof(double)));
  ILM_TRY(gj.alloc((size_t)4 * N * sizeof(double)));
  ILM_TRY(bad.alloc(sizeof(int)));
  ILM_TRY(schur_build(c, ILM_SCHUR_RTLINVR, 1.0, Sp.as<double>(), st, true));
  k_pc_sum<<<N, 256, 0, st>>>(N, Sp.as<double>(), c->ds64.as<double>(), sums.as<double>());
  ILM_CHECK_LAUNCH();
  std::vector<double> hs(N);
  ILM_CHECK_CUDA(cudaMemcpyAsync(hs.data(), sums.p, N * sizeof(double), cudaMemcpyDeviceToHost, st));
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  double tot = 0.0;
  for (double v : hs) tot += v;
  double shift = 2.0 * fabs(tot) / ((double)N * N);
  if (!(shift > 0.0)) shift = 1e-300;
  double* T = c->stokes_pc.as<double>();
  double* cb[2] = {gj.as<double>(), gj.as<double>() + N};
  double* rb[2] = {gj.as<double>() + 2 * N, gj.as<double>() + 3 * N};
  const dim3 blk(32, 8), grd((N + 31) / 32, (N + 7) / 8);
  for (int attempt = 0; attempt < 4; ++attempt, shift *= 8.0) {
    k_pc_form<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(N, Sp.as<double>(), c->ds64.as<double>(), shift, T);
    ILM_CHECK_LAUNCH();
    ILM_CHECK_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
    k_gj_init<<<(N + 255) / 256, 256, 0, st>>>(N, T, cb[0], rb[0]);
    ILM_CHECK_LAUNCH();
    for (int k = 0; k < N; ++k) {
      k_gj_step<<<grd, blk, 0, st>>>(N, k, T, cb[k & 1], rb[k & 1], cb[(k + 1) & 1], rb[(k + 1) & 1],
                                     bad.as<int>());
      ILM_CHECK_LAUNCH();
    }
    int hb = 0;
    ILM_CHECK_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    ILM_CHECK_CUDA(cudaStreamSynchronize(st));
    if (hb == 0) {
      c->stokes_pc_ready = true;
      return ILM_OK;
    }
  }
  set_error("solve_stokes: preconditioner not positive definite after 4 shifts");
  return ILM_ERR_NOT_CONVERGED;
}

// eigen-decomposition of a symmetric s x s matrix (cyclic Jacobi rotations);
// A (row-major) is destroyed, lam[j] and column j of V (row-major) are the
// eigenpairs
void sym_eig(int s, std::vector<double>& A, std::vector<double>& lam, std::vector<double>& V) {
  V.assign((size_t)s * s, 0.0);
  for (int i = 0; i < s; ++i) V[i * s + i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < s; ++i)
      for (int j = 0; j < s; ++j) {
        tot += A[i * s + j] * A[i * s + j];
        if (i != j) off += A[i * s + j] * A[i * s + j];
      }
    if (off <= 1e-30 * tot || tot == 0.0) break;
    for (int p = 0; p < s; ++p)
      for (int q = p + 1; q < s; ++q) {
        const double apq = A[p * s + q];
        if (apq == 0.0) continue;
        const double theta = (A[q * s + q] - A[p * s + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < s; ++k) {  // A <- A J  (columns p, q)
          const double akp = A[k * s + p], akq = A[k * s + q];
          A[k * s + p] = cs * akp - sn * akq;
          A[k * s + q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < s; ++k) {  // A <- J^T A  (rows p, q)
          const double apk = A[p * s + k], aqk = A[q * s + k];
          A[p * s + k] = cs * apk - sn * aqk;
          A[q * s + k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < s; ++k) {
          const double vkp = V[k * s + p], vkq = V[k * s + q];
          V[k * s + p] = cs * vkp - sn * vkq;
          V[k * s + q] = sn * vkp + cs * vkq;
        }
      }
  }
  lam.resize(s);
  for (int i = 0; i < s; ++i) lam[i] = A[i * s + i];
}

// Q (n x s) = B Y (n x s), the operator applied column by column
using BlockApply = std::function<int(const double*, double*, int)>;
// Z (n x s) = M R (n x s)
using BlockPrec = std::function<int(const double*, double*, int)>;

struct BlockCG {
  int n = 0, s = 0;
  DevBuf R, Z, P, Q, Pn, Qn, G1, G2, small;
};

int gram(const double* A, int sa, const double* B, int sb, int n, double* dG, std::vector<double>& hG,
         cudaStream_t st, bool sync = true) {
  k_gram<<<sa * sb, 256, 0, st>>>(n, A, n, sa, B, n, dG);
  ILM_CHECK_LAUNCH();
  hG.resize((size_t)sa * sb);
  ILM_CHECK_CUDA(cudaMemcpyAsync(hG.data(), dG, (size_t)sa * sb * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (sync) ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  return ILM_OK;
}

int gemm(int n, int k, int t, const double* A, const double* B, double alpha, double beta, double* C,
         cudaStream_t st) {
  if (n == 0 || t == 0) return ILM_OK;
  k_gemm_rows<<<(n + 255) / 256, 256, 0, st>>>(n, k, t, A, n, B, k, alpha, beta, C, n);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

// Block CG on B Y = Bb (n x s, FP64 device, column-major); Y = 0 at start.
// relres[j] = ||Bb_j - B Y_j|| / ||Bb_j|| (recomputed from B Y at the end).
// `drop`: directions whose A-norm^2 falls below drop x the largest are
// discarded (the operator's rounding level: an FP32 operator is only
// symmetric to ~1e-7).  The iterate with the smallest worst-column residual
// is kept; the recurrence stops when that residual grows a thousandfold
// (an FP32 operator below its attainable accuracy), or with a stall window
// when it has not improved by 10% for `stall` iterations, and returns the
// kept one.
int block_cg(int n, int s, const BlockApply& A, const BlockPrec* M, const double* Bb, double* Y, double tol,
             int maxiter, double drop, int* iters, double* relres, cudaStream_t st, int stall = 0) {
  const size_t nb = (size_t)n * s * sizeof(double);
  BlockCG w;
  DevBuf Ybest;
  for (DevBuf* b : {&w.R, &w.Z, &w.P, &w.Q, &w.Pn, &w.Qn, &Ybest}) ILM_TRY(b->alloc(std::max<size_t>(nb, 8)));
  ILM_TRY(w.G1.alloc((size_t)s * s * sizeof(double)));
  ILM_TRY(w.G2.alloc((size_t)s * s * sizeof(double)));
  ILM_TRY(w.small.alloc((size_t)s * s * sizeof(double)));
  double *R = w.R.as<double>(), *Z = w.Z.as<double>(), *P = w.P.as<double>(), *Q = w.Q.as<double>();
  double *Pn = w.Pn.as<double>(), *Qn = w.Qn.as<double>(), *dsm = w.small.as<double>();
  ILM_CHECK_CUDA(cudaMemsetAsync(Y, 0, nb, st));
  ILM_CHECK_CUDA(cudaMemcpyAsync(R, Bb, nb, cudaMemcpyDeviceToDevice, st));
  std::vector<double> hg, hr, bn(s);
  ILM_TRY(gram(Bb, s, Bb, s, n, w.G1.as<double>(), hg, st));
  bool all_zero = true;
  for (int j = 0; j < s; ++j) {
    bn[j] = sqrt(std::max(hg[j + (size_t)j * s], 0.0));
    relres[j] = bn[j] > 0.0 ? 1.0 : 0.0;
    all_zero = all_zero && bn[j] == 0.0;
  }
  *iters = 0;
  if (all_zero || n == 0) return ILM_OK;
  auto precond = [&](const double* r, double* z) -> int {
    if (M) return (*M)(r, z, s);
    ILM_CHECK_CUDA(cudaMemcpyAsync(z, r, nb, cudaMemcpyDeviceToDevice, st));
    return ILM_OK;
  };
  auto residual_norms = [&](std::vector<double>& out) -> int {
    std::vector<double> d;
    ILM_TRY(gram(R, s, R, s, n, w.G2.as<double>(), d, st));
    out.resize(s);
    for (int j = 0; j < s; ++j)
      out[j] = bn[j] > 0.0 ? sqrt(std::max(d[j + (size_t)j * s], 0.0)) / bn[j] : 0.0;
    return ILM_OK;
  };
  ILM_TRY(precond(R, P));
  int sp = s;  // columns of the direction block
  std::vector<double> lam, V, Tm, hab;
  int it = 0;
  bool done = false, have_best = false;
  double best = 1.0;  // worst-column residual of Ybest (Y = 0 at start)
  int last_gain = 0;
  auto worst = [&](const std::vector<double>& r) {
    double m = 0.0;
    for (double v : r) m = (v > m || v != v) ? v : m;
    return m;
  };
  while (it < maxiter && !done) {
    ILM_TRY(A(P, Q, sp));
    // A-orthonormalise the direction block: G = P^T Q = V diag(lam) V^T
    ILM_TRY(gram(P, sp, Q, sp, n, w.G1.as<double>(), hg, st));
    std::vector<double> Gs((size_t)sp * sp);
    for (int i = 0; i < sp; ++i)
      for (int j = 0; j < sp; ++j) Gs[i * sp + j] = 0.5 * (hg[i + (size_t)j * sp] + hg[j + (size_t)i * sp]);
    sym_eig(sp, Gs, lam, V);
    double lmax = 0.0;
    for (double l : lam) lmax = std::max(lmax, l);
    std::vector<int> keep;
    for (int j = 0; j < sp; ++j)
      if (lam[j] > drop * lmax && lam[j] > 0.0) keep.push_back(j);
    const int sk = (int)keep.size();
    if (sk == 0) break;  // no direction left (stagnation)
    Tm.assign((size_t)sp * sk, 0.0);  // column-major sp x sk
    for (int q = 0; q < sk; ++q)
      for (int i = 0; i < sp; ++i) Tm[i + (size_t)q * sp] = V[i * sp + keep[q]] / sqrt(lam[keep[q]]);
    ILM_CHECK_CUDA(cudaMemcpyAsync(dsm, Tm.data(), Tm.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    ILM_TRY(gemm(n, sp, sk, P, dsm, 1.0, 0.0, Pn, st));
    ILM_TRY(gemm(n, sp, sk, Q, dsm, 1.0, 0.0, Qn, st));
    // alpha = Pn^T R; Y += Pn alpha; R -= Qn alpha
    ILM_TRY(gram(Pn, sk, R, s, n, w.G1.as<double>(), hab, st));
    ILM_CHECK_CUDA(cudaMemcpyAsync(dsm, hab.data(), hab.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    ILM_TRY(gemm(n, sk, s, Pn, dsm, 1.0, 1.0, Y, st));
    ILM_TRY(gemm(n, sk, s, Qn, dsm, -1.0, 1.0, R, st));
    ++it;
    ILM_TRY(residual_norms(hr));
    const double wr = worst(hr);
    if (wr < 0.9 * best) last_gain = it;  // a 10% gain restarts the stall window
    if (wr < best) {
      best = wr;
      have_best = true;
      ILM_CHECK_CUDA(cudaMemcpyAsync(Ybest.p, Y, nb, cudaMemcpyDeviceToDevice, st));
    }
    // diverging, or (with a stall window) no 10% gain for `stall` iterations:
    // return the best iterate
    const bool diverged = !(wr <= 1e3 * best) || (stall > 0 && it - last_gain >= stall);
    bool conv = true;
    for (int j = 0; j < s; ++j) conv = conv && hr[j] <= tol;
    if (diverged) {  // back to the best iterate; its true residual
      if (have_best)
        ILM_CHECK_CUDA(cudaMemcpyAsync(Y, Ybest.p, nb, cudaMemcpyDeviceToDevice, st));
      else
        ILM_CHECK_CUDA(cudaMemsetAsync(Y, 0, nb, st));
      ILM_TRY(A(Y, Q, s));
      ILM_TRY(st_axpby((size_t)n * s, ILM_F64, 1.0, Bb, -1.0, Q, R, st));
      ILM_TRY(residual_norms(hr));
      for (int j = 0; j < s; ++j) relres[j] = hr[j];
      break;
    }
    if (conv || it == maxiter) {  // true residual
      ILM_TRY(A(Y, Q, s));
      ILM_TRY(st_axpby((size_t)n * s, ILM_F64, 1.0, Bb, -1.0, Q, R, st));  // R = Bb - B Y
      ILM_TRY(residual_norms(hr));
      conv = true;
      for (int j = 0; j < s; ++j) conv = conv && hr[j] <= tol;
      if (conv) done = true;
      if (!conv && it == maxiter && have_best && worst(hr) > best) {  // the kept iterate, if better
        std::vector<double> hb;
        ILM_CHECK_CUDA(cudaMemcpyAsync(Pn, Ybest.p, nb, cudaMemcpyDeviceToDevice, st));
        ILM_TRY(A(Pn, Q, s));
        ILM_TRY(st_axpby((size_t)n * s, ILM_F64, 1.0, Bb, -1.0, Q, Qn, st));
        std::swap(R, Qn);
        ILM_TRY(residual_norms(hb));
        std::swap(R, Qn);
        if (worst(hb) < worst(hr)) {
          ILM_CHECK_CUDA(cudaMemcpyAsync(Y, Pn, nb, cudaMemcpyDeviceToDevice, st));
          hr = hb;
        }
      }
    }
    for (int j = 0; j < s; ++j) relres[j] = hr[j];
    if (done || it == maxiter) break;
    // Z = M R; beta = -Qn^T Z; P = Z + Pn beta
    ILM_TRY(precond(R, Z));
    ILM_TRY(gram(Qn, sk, Z, s, n, w.G1.as<double>(), hab, st));
    for (double& v : hab) v = -v;
    ILM_CHECK_CUDA(cudaMemcpyAsync(dsm, hab.data(), hab.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    ILM_CHECK_CUDA(cudaMemcpyAsync(P, Z, nb, cudaMemcpyDeviceToDevice, st));
    ILM_TRY(gemm(n, sk, s, Pn, dsm, 1.0, 1.0, P, st));
    sp = s;
  }
  *iters = it;
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  return ILM_OK;
}

// Work buffers and operators of the Stokes solves on one cache (any dtype;
// Krylov vectors in FP64, converted at the operator boundary).
struct StokesWork {
  ilm_cache_s* c = nullptr;
  int N = 0, dt = 0;
  size_t es = 0, ne = 0, nd = 0, np = 0, n2 = 0;
  DevBuf e1, d1, d2, p1, p2, v1, v2, v4, s1;

  int init(ilm_cache_s* cache) {
    c = cache;
    N = c->npts;
    dt = c->dtype;
    es = dt == ILM_F64 ? 8 : 4;
    ne = c->grid.shape(PC_U).numel() + c->grid.shape(PC_V).numel();
    nd = c->grid.shape(PC_D).numel();
    np = c->grid.shape(PC_P).numel();
    n2 = 2 * (size_t)N;
    ILM_TRY(e1.alloc(ne * es));
    ILM_TRY(d1.alloc(nd * es));
    ILM_TRY(d2.alloc(nd * es));
    ILM_TRY(p1.alloc(np * es));
    ILM_TRY(p2.alloc(np * es));
    for (DevBuf* b : {&v1, &v2, &v4}) ILM_TRY(b->alloc(std::max<size_t>(n2, 1) * es));
    return s1.alloc(std::max<size_t>(N, 1) * es);
  }
  void* at(const void* base, size_t per, int j) const { return elem_ptr(base, per * j, dt); }

  int to_op(const double* y, void* out, int n, cudaStream_t st) const {
    if (n == 0) return ILM_OK;
    if (dt == ILM_F64)
      k_to_op<double><<<(n + 255) / 256, 256, 0, st>>>(n, N, y, c->ds64.as<double>(), static_cast<double*>(out));
    else
      k_to_op<float><<<(n + 255) / 256, 256, 0, st>>>(n, N, y, c->ds64.as<double>(), static_cast<float*>(out));
    ILM_CHECK_LAUNCH();
    return ILM_OK;
  }
  int from_op(const void* in, double sgn, double* out, int n, cudaStream_t st) const {
    if (n == 0) return ILM_OK;
    if (dt == ILM_F64)
      k_from_op<double><<<(n + 255) / 256, 256, 0, st>>>(n, static_cast<const double*>(in), sgn, out);
    else
      k_from_op<float><<<(n + 255) / 256, 256, 0, st>>>(n, static_cast<const float*>(in), sgn, out);
    ILM_CHECK_LAUNCH();
    return ILM_OK;
  }

  // psi* (into s_out), v_phi (into v_out), v' and the Ss right-hand side
  // G^x_s phi of one right-hand side (cache dtype)
  int prepare(const void* vpl, const void* vmi, void* vo, void* so, void* vp, void* ssr, cudaStream_t st) {
    ilm_stream_t stream = st;
    void* dv = v1.p;  // [v]
    void* vb = v2.p;  // avg
    ILM_TRY(st_axpby(n2, dt, 1.0, vpl, -1.0, vmi, dv, st));
    ILM_TRY(st_axpby(n2, dt, 0.5, vpl, 0.5, vmi, vb, st));
    // psi* = L^-2 (-C D_s^symm [v])
    ILM_TRY(ilm_surface_divergence_symm(c, dv, e1.p, stream));
    ILM_TRY(ilm_curl(c, ILM_EDGES_PRIMAL, e1.p, d1.p, stream));
    ILM_TRY(st_affine(nd, dt, -1.0, d1.p, 0.0, d1.p, st));
    ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, d1.p, d2.p, stream));
    ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, d2.p, so, stream));
    // phi = L^-1 R (n . [v]),  v_phi = G phi  (kept in v_out)
    if (N > 0) {
      if (dt == ILM_F64)
        k_ndot<double><<<(N + 255) / 256, 256, 0, st>>>(N, c->nx.as<double>(), c->ny.as<double>(),
                                                        static_cast<const double*>(dv), s1.as<double>());
      else
        k_ndot<float><<<(N + 255) / 256, 256, 0, st>>>(N, c->nx.as<float>(), c->ny.as<float>(),
                                                       static_cast<const float*>(dv), s1.as<float>());
      ILM_CHECK_LAUNCH();
    }
    ILM_TRY(ilm_regularize(c, ILM_NODES_PRIMAL, s1.p, p1.p, stream));
    ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_PRIMAL, p1.p, p2.p, stream));
    void* phi = p2.p;
    ILM_TRY(ilm_grad(c, ILM_NODES_PRIMAL, phi, vo, stream));
    // v' = avg - E v_phi - E C psi*
    ILM_TRY(ilm_interpolate(c, ILM_EDGES_PRIMAL, vo, v4.p, stream));
    ILM_TRY(st_axpby(n2, dt, 1.0, vb, -1.0, v4.p, vp, st));
    ILM_TRY(ilm_curl(c, ILM_NODES_DUAL, so, e1.p, stream));
    ILM_TRY(ilm_interpolate(c, ILM_EDGES_PRIMAL, e1.p, v4.p, stream));
    ILM_TRY(st_axpby(n2, dt, 1.0, vp, -1.0, v4.p, vp, st));
    return ilm_surface_grad_cross(c, phi, ssr, stream);
  }

  // Q = (-S W^-1) Y = C_s L^-2 C_s^T W^-1 Y, column by column (n2 x s)
  int applyB(const double* Yb, double* Qb, int s, cudaStream_t st) {
    ilm_stream_t stream = st;
    for (int j = 0; j < s; ++j) {
      ILM_TRY(to_op(Yb + n2 * j, v4.p, (int)n2, st));
      ILM_TRY(ilm_surface_curl(c, 0, ILM_VECTOR_DATA, v4.p, d1.p, stream));
      ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, d1.p, d2.p, stream));
      ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, d2.p, d1.p, stream));
      ILM_TRY(ilm_surface_curl(c, 1, ILM_VECTOR_DATA, d1.p, v4.p, stream));
      ILM_TRY(from_op(v4.p, 1.0, Qb + n2 * j, (int)n2, st));
    }
    return ILM_OK;
  }
  // Q = (Ss W^-1) Y, Ss = -C_s L^-1 C_s^T on scalars (N x s)
  int applyBs(const double* Yb, double* Qb, int s, cudaStream_t st) {
    ilm_stream_t stream = st;
    for (int j = 0; j < s; ++j) {
      ILM_TRY(to_op(Yb + (size_t)N * j, s1.p, N, st));
      ILM_TRY(ilm_surface_curl(c, 0, ILM_SCALAR_DATA, s1.p, d1.p, stream));
      ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, d1.p, d2.p, stream));
      ILM_TRY(ilm_surface_curl(c, 1, ILM_SCALAR_DATA, d2.p, s1.p, stream));
      ILM_TRY(from_op(s1.p, -1.0, Qb + (size_t)N * j, N, st));
    }
    return ILM_OK;
  }
  // each velocity component: Z_comp = P^-1 R_comp (leading dimension 2N)
  int applyM(const double* Rb, double* Zb, int s, cudaStream_t st) const {
    const double* Ti = c->stokes_pc.as<double>();
    for (int comp = 0; comp < 2; ++comp)
      for (int j0 = 0; j0 < s; j0 += 8) {
        const int t = std::min(8, s - j0);
        k_gemm_rows<<<(N + 255) / 256, 256, 0, st>>>(N, N, t, Ti, N, Rb + comp * N + n2 * j0, (int)n2, 1.0, 0.0,
                                                     Zb + comp * N + n2 * j0, (int)n2);
        ILM_CHECK_LAUNCH();
      }
    return ILM_OK;
  }

  // sigma = W^-1 y; psi = psi* + L^-2 (-C_s^T sigma); v = C psi + v_phi
  int fields(const double* Yr, void* sig, void* vo, void* so, cudaStream_t st) {
    ilm_stream_t stream = st;
    ILM_TRY(to_op(Yr, sig, (int)n2, st));
    ILM_TRY(ilm_surface_curl(c, 0, ILM_VECTOR_DATA, sig, d1.p, stream));
    ILM_TRY(st_affine(nd, dt, -1.0, d1.p, 0.0, d1.p, st));
    ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, d1.p, d2.p, stream));
    ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, d2.p, d1.p, stream));
    ILM_TRY(st_axpby(nd, dt, 1.0, d1.p, 1.0, so, so, st));
    ILM_TRY(ilm_curl(c, ILM_NODES_DUAL, so, e1.p, stream));
    return st_axpby(ne, dt, 1.0, e1.p, 1.0, vo, vo, st);
  }
  // psi += L^-1 (-C^x_s^T W^-1 ys); sigma <- F^2 sigma
  int finish(const double* Ysr, void* sig, void* so, cudaStream_t st) {
    ilm_stream_t stream = st;
    ILM_TRY(to_op(Ysr, s1.p, N, st));
    ILM_TRY(ilm_surface_curl_cross(c, 0, s1.p, d1.p, stream));
    ILM_TRY(st_affine(nd, dt, -1.0, d1.p, 0.0, d1.p, st));
    ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, d1.p, d2.p, stream));
    ILM_TRY(st_axpby(nd, dt, 1.0, d2.p, 1.0, so, so, st));
    return ilm_surface_filter(c, 2, sig, sig, stream);
  }
};

int stokes_check(ilm_cache_s* c, int nrhs, double tol, int maxiter) {
  ILM_REQUIRE(c, "null cache");
  ILM_REQUIRE(c->kind == ILM_CACHE_VECTOR, "solve_stokes: vector cache required");
  ILM_REQUIRE(c->scaling == ILM_GRID_SCALING, "solve_stokes: GridScaling cache required");
  ILM_REQUIRE(tol > 0 && maxiter > 0, "solve_stokes: bad tolerance / iteration limit");
  ILM_REQUIRE(nrhs >= 1 && nrhs <= ILM_STOKES_MAX_RHS, "solve_stokes: nrhs %d outside 1..%d", nrhs,
              ILM_STOKES_MAX_RHS);
  return ILM_OK;
}

}  // namespace
}  // namespace ilm

using namespace ilm;

extern "C" {

int ilm_solve_stokes_multi(ilm_cache_t c, int nrhs, const void* vplus, const void* vminus, void* v_out,
                           void* s_out, void* sigma_out, double tol, int maxiter, int precond,
                           ilm_solve_info_t* info, ilm_stream_t stream) {
  ILM_TRY(stokes_check(c, nrhs, tol, maxiter));
  ILM_REQUIRE(vplus && vminus && v_out && s_out && sigma_out, "solve_stokes: null argument");
  ILM_REQUIRE(precond == 0 || precond == 1, "solve_stokes: precond must be 0 or 1");
  cudaStream_t st = as_stream(stream);
  StokesWork w;
  ILM_TRY(w.init(c));
  const int N = w.N;
  const size_t n2 = w.n2, ne = w.ne, nd = w.nd;
  DevBuf Bb, Y, Bs, Ys, vp_all, ss_all;
  ILM_TRY(vp_all.alloc(std::max<size_t>(n2 * nrhs, 1) * w.es));
  ILM_TRY(ss_all.alloc(std::max<size_t>((size_t)N * nrhs, 1) * w.es));
  for (DevBuf* b : {&Bb, &Y}) ILM_TRY(b->alloc(std::max<size_t>(n2 * nrhs, 1) * sizeof(double)));
  for (DevBuf* b : {&Bs, &Ys}) ILM_TRY(b->alloc(std::max<size_t>((size_t)N * nrhs, 1) * sizeof(double)));
  for (int r = 0; r < nrhs; ++r) {
    ILM_TRY(w.prepare(w.at(vplus, n2, r), w.at(vminus, n2, r), w.at(v_out, ne, r), w.at(s_out, nd, r),
                      w.at(vp_all.p, n2, r), w.at(ss_all.p, N, r), st));
    ILM_TRY(w.from_op(w.at(vp_all.p, n2, r), -1.0, Bb.as<double>() + n2 * r, (int)n2, st));
    ILM_TRY(w.from_op(w.at(ss_all.p, N, r), 1.0, Bs.as<double>() + (size_t)N * r, N, st));
  }
  // S sigma = v' in y = W sigma: (-S W^-1) y = -v'
  BlockApply applyB = [&](const double* Yb, double* Qb, int s) { return w.applyB(Yb, Qb, s, st); };
  BlockApply applyBs = [&](const double* Yb, double* Qb, int s) { return w.applyBs(Yb, Qb, s, st); };
  BlockPrec applyM = [&](const double* Rb, double* Zb, int s) { return w.applyM(Rb, Zb, s, st); };
  const bool use_pc = precond == 1 && N > 0 && N <= STOKES_PC_MAX;
  if (use_pc) ILM_TRY(ensure_stokes_pc(c, st));
  std::vector<double> rr1(nrhs, 0.0), rr2(nrhs, 0.0);
  int it1 = 0, it2 = 0;
  const double drop = w.dt == ILM_F64 ? 1e-13 : 1e-6;
  ILM_TRY(block_cg((int)n2, nrhs, applyB, use_pc ? &applyM : nullptr, Bb.as<double>(), Y.as<double>(), tol, maxiter,
                   drop, &it1, rr1.data(), st));
  for (int r = 0; r < nrhs; ++r)
    ILM_TRY(w.fields(Y.as<double>() + n2 * r, w.at(sigma_out, n2, r), w.at(v_out, ne, r), w.at(s_out, nd, r), st));
  // Ss d = G^x_s phi in y = W d: (Ss W^-1) y = rhs
  ILM_TRY(block_cg(N, nrhs, applyBs, nullptr, Bs.as<double>(), Ys.as<double>(), tol, maxiter, drop, &it2, rr2.data(),
                   st));
  for (int r = 0; r < nrhs; ++r)
    ILM_TRY(w.finish(Ys.as<double>() + (size_t)N * r, w.at(sigma_out, n2, r), w.at(s_out, nd, r), st));
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  bool ok = true;
  for (int r = 0; r < nrhs; ++r) {
    const bool cr = rr1[r] <= tol && rr2[r] <= tol;
    ok = ok && cr;
    if (info) {
      info[r].iterations = it1 + it2;
      info[r].converged = cr ? 1 : 0;
      info[r].rel_residual = std::max(rr1[r], rr2[r]);
    }
  }
  if (!ok) set_error("solve_stokes: rel. residual %g not reached in %d block iterations", tol, maxiter);
  return ok ? ILM_OK : ILM_ERR_NOT_CONVERGED;
}

int ilm_solve_stokes(ilm_cache_t c, const void* vplus, const void* vminus, void* v_out, void* s_out, void* sigma_out,
                     double tol, int maxiter, ilm_solve_info_t* info, ilm_stream_t stream) {
  return ilm_solve_stokes_multi(c, 1, vplus, vminus, v_out, s_out, sigma_out, tol, maxiter, 1, info, stream);
}

// FP64-refined Stokes solves (see ilm.h).  The pre-step, the FP64 residuals
// and the field assembly run on the FP64 twin cache; each correction is a
// block CG with the cache's own operator (FP32 for an FP32 cache) to
// kStokesInnerTol of its residual, stopped early when it stalls.
int ilm_solve_stokes_multi_refined(ilm_cache_t c, int nrhs, const double* vplus, const double* vminus,
                                   double* v_out, double* s_out, double* sigma_out, double tol, int maxiter,
                                   int max_refine, ilm_solve_info_t* info, ilm_stream_t stream) {
  constexpr double kStokesInnerTol = 1e-4;
  constexpr int kStokesStall = 40;  // block iterations without a 10% gain end a correction
  ILM_TRY(stokes_check(c, nrhs, tol, maxiter));
  ILM_REQUIRE(vplus && vminus && v_out && s_out && sigma_out, "solve_stokes_refined: null argument");
  ILM_REQUIRE(max_refine >= 1, "solve_stokes_refined: max_refine must be >= 1");
  cudaStream_t st = as_stream(stream);
  ilm_cache_s* c64 = nullptr;
  ILM_TRY(ensure_twin(c, &c64));
  StokesWork w64, wb;
  ILM_TRY(w64.init(c64));
  const bool sep = c64 != c;
  if (sep) ILM_TRY(wb.init(c));
  StokesWork& wk = sep ? wb : w64;  // the corrections' operator
  const int N = w64.N;
  const size_t n2 = w64.n2, ne = w64.ne, nd = w64.nd;
  DevBuf vp_all, ss_all, Bb, Y, R, D, Q, Bs, Ys, Rs, Ds, Qs;
  ILM_TRY(vp_all.alloc(std::max<size_t>(n2 * nrhs, 1) * 8));
  ILM_TRY(ss_all.alloc(std::max<size_t>((size_t)N * nrhs, 1) * 8));
  for (DevBuf* b : {&Bb, &Y, &R, &D, &Q}) ILM_TRY(b->alloc(std::max<size_t>(n2 * nrhs, 1) * sizeof(double)));
  for (DevBuf* b : {&Bs, &Ys, &Rs, &Ds, &Qs}) ILM_TRY(b->alloc(std::max<size_t>((size_t)N * nrhs, 1) * sizeof(double)));
  for (int r = 0; r < nrhs; ++r) {
    ILM_TRY(w64.prepare(vplus + n2 * r, vminus + n2 * r, v_out + ne * r, s_out + nd * r, vp_all.as<double>() + n2 * r,
                        ss_all.as<double>() + (size_t)N * r, st));
    ILM_TRY(w64.from_op(vp_all.as<double>() + n2 * r, -1.0, Bb.as<double>() + n2 * r, (int)n2, st));
    ILM_TRY(w64.from_op(ss_all.as<double>() + (size_t)N * r, 1.0, Bs.as<double>() + (size_t)N * r, N, st));
  }
  const bool use_pc = N > 0 && N <= STOKES_PC_MAX;
  if (use_pc) ILM_TRY(ensure_stokes_pc(c, st));
  BlockPrec applyM = [&](const double* Rb, double* Zb, int s) { return wk.applyM(Rb, Zb, s, st); };
  const double drop = wk.dt == ILM_F64 ? 1e-13 : 1e-6;
  // y += B^-1 (b - B y) with B in the corrections' precision, b - B y in FP64
  auto refine = [&](size_t n, bool vec, const double* b, double* y, double* res, double* d, double* q,
                    std::vector<double>& rel, int* iters) -> int {
    BlockApply A64 = [&](const double* Yb, double* Qb, int s) {
      return vec ? w64.applyB(Yb, Qb, s, st) : w64.applyBs(Yb, Qb, s, st);
    };
    BlockApply Ak = [&](const double* Yb, double* Qb, int s) {
      return vec ? wk.applyB(Yb, Qb, s, st) : wk.applyBs(Yb, Qb, s, st);
    };
    const size_t nb = n * nrhs * sizeof(double);
    ILM_CHECK_CUDA(cudaMemsetAsync(y, 0, nb, st));
    ILM_CHECK_CUDA(cudaMemcpyAsync(res, b, nb, cudaMemcpyDeviceToDevice, st));
    std::vector<double> bn(nrhs), g;
    DevBuf G;
    ILM_TRY(G.alloc((size_t)nrhs * nrhs * sizeof(double)));
    ILM_TRY(gram(b, nrhs, b, nrhs, (int)n, G.as<double>(), g, st));
    for (int j = 0; j < nrhs; ++j) bn[j] = sqrt(std::max(g[j + (size_t)j * nrhs], 0.0));
    rel.assign(nrhs, 1.0);
    *iters = 0;
    std::vector<double> rin(nrhs), relk(nrhs);
    double worst_prev = 1.0;
    for (int k = 0; k < max_refine; ++k) {
      int it = 0;
      ILM_TRY(block_cg((int)n, nrhs, Ak, vec && use_pc ? &applyM : nullptr, res, d, kStokesInnerTol, maxiter, drop,
                       &it, rin.data(), st, kStokesStall));
      *iters += it;
      ILM_TRY(st_axpby(n * nrhs, ILM_F64, 1.0, y, 1.0, d, y, st));
      ILM_TRY(A64(y, q, nrhs));
      ILM_TRY(st_axpby(n * nrhs, ILM_F64, 1.0, b, -1.0, q, q, st));  // q = b - B y (candidate residual)
      ILM_TRY(gram(q, nrhs, q, nrhs, (int)n, G.as<double>(), g, st));
      bool all = true;
      double worst = 0.0;
      for (int j = 0; j < nrhs; ++j) {
        relk[j] = bn[j] > 0.0 ? sqrt(std::max(g[j + (size_t)j * nrhs], 0.0)) / bn[j] : 0.0;
        all = all && relk[j] <= tol;
        worst = std::max(worst, relk[j]);
      }
      if (!(worst < worst_prev)) {
        // the correction did not reduce the FP64 residual (the corrections'
        // operator cannot resolve the slowest modes): keep the previous y
        ILM_TRY(st_axpby(n * nrhs, ILM_F64, 1.0, y, -1.0, d, y, st));
        break;
      }
      worst_prev = worst;
      rel = relk;
      ILM_CHECK_CUDA(cudaMemcpyAsync(res, q, nb, cudaMemcpyDeviceToDevice, st));
      if (all) break;
    }
    return ILM_OK;
  };
  std::vector<double> rr1, rr2;
  int it1 = 0, it2 = 0;
  ILM_TRY(refine(n2, true, Bb.as<double>(), Y.as<double>(), R.as<double>(), D.as<double>(), Q.as<double>(), rr1, &it1));
  for (int r = 0; r < nrhs; ++r)
    ILM_TRY(w64.fields(Y.as<double>() + n2 * r, sigma_out + n2 * r, v_out + ne * r, s_out + nd * r, st));
  ILM_TRY(refine(N, false, Bs.as<double>(), Ys.as<double>(), Rs.as<double>(), Ds.as<double>(), Qs.as<double>(), rr2,
                 &it2));
  for (int r = 0; r < nrhs; ++r)
    ILM_TRY(w64.finish(Ys.as<double>() + (size_t)N * r, sigma_out + n2 * r, s_out + nd * r, st));
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  bool ok = true;
  for (int r = 0; r < nrhs; ++r) {
    const bool cr = rr1[r] <= tol && rr2[r] <= tol;
    ok = ok && cr;
    if (info) {
      info[r].iterations = it1 + it2;
      info[r].converged = cr ? 1 : 0;
      info[r].rel_residual = std::max(rr1[r], rr2[r]);
    }
  }
  if (!ok) set_error("solve_stokes_refined: rel. residual %g not reached in %d refinement steps", tol, max_refine);
  return ok ? ILM_OK : ILM_ERR_NOT_CONVERGED;
}

}  // extern "C"
