// Batched Schur CG on thread-block clusters with float-float matvecs.
//
// One cluster of CG_CLUSTER CTAs per problem.  Each CTA owns a contiguous
// slice of the rows: it keeps its slices of x, r, p, q, w, b in shared memory,
// assembles the full search direction from the other CTAs' slices through
// distributed shared memory once per iteration, and computes its rows of
// S p.  Reductions publish one partial per CTA and every CTA sums the
// partials in rank order after a hardware cluster barrier, so all CTAs see
// bit-identical scalars and take identical branches (no CTA can wait on a
// barrier the others skip).
//
// GB300 issues FP64 FMAs at a small fraction of its FP32 rate, so the matvec
// runs in float-float ("double-single") arithmetic on the FP32 pipes: the
// FP64 Schur complement is stored as S_hi + S_lo (two FP32 matrices, row
// major), the direction as p_hi + p_lo, products are split exactly with fmaf
// and accumulated with TwoSum.  The result carries ~48 bits, enough for an
// FP64-quality Krylov iteration; the CG scalars and vectors stay FP64.
#include <cooperative_groups.h>

#include <algorithm>

#include "ilm_internal.cuh"

namespace cg = cooperative_groups;

namespace ilm {

constexpr int CG_CLUSTER = 8;
constexpr int CG_RED_K = 8;       // values per cluster reduction (csum_t0)
constexpr int CG_BC = 24;         // broadcast scalars: [0, 16) CG, [16, 20) coarse coefficients
constexpr int CGC_THREADS = 256;
constexpr int CGC_WARPS = CGC_THREADS / 32;

// a / b to ~2^-46 relative: an FP32 reciprocal and one FP64 correction.
// GB300 issues FP64 at a small fraction of its FP32 rate and the divide is a
// long FP64 sequence; every thread of a CTA evaluates the CG scalars, so the
// full-precision divide cost more than the rest of an iteration.
__device__ __forceinline__ double fdiv(double a, double b) {
  const double ab = fabs(b);
  if (!(ab > 1e-30 && ab < 1e30)) return a / b;
  const double r = (double)(1.0f / (float)b);
  const double q = a * r;
  return fma(fma(-q, b, a), r, q);
}

// Block-wide sums of two doubles in fixed order; result valid in all
// threads.  `red` holds 2 * blockDim + 2 doubles.  The per-thread partials go
// through shared memory and only warp 0 adds them: GB300 issues FP64 at a
// small fraction of its FP32 rate, and an add tree in every warp followed by
// every thread summing the warp totals cost more FP64 issue slots than the
// whole CG iteration's vector arithmetic.
__device__ void block_sum2(double& a, double& b, double* red) {
  const int nt = blockDim.x, t = threadIdx.x;
  red[t] = a;
  red[nt + t] = b;
  __syncthreads();
  if (t < 32) {
    double sa = 0.0, sb = 0.0;
    for (int i = t; i < nt; i += 32) {
      sa += red[i];
      sb += red[nt + i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sa += __shfl_down_sync(0xffffffffu, sa, o);
      sb += __shfl_down_sync(0xffffffffu, sb, o);
    }
    if (t == 0) {
      red[2 * nt] = sa;
      red[2 * nt + 1] = sb;
    }
  }
  __syncthreads();
  a = red[2 * nt];
  b = red[2 * nt + 1];
  __syncthreads();
}

struct CGFFParams {
  const float* Shi;   // n x n row-major
  const float* Slo;
  const double* b;
  double* x;
  const double* w;
  int n;
  int maxiter;
  double tol;
  int* iters;
  double* relres;
  // optional block-Jacobi preconditioner (blk == nullptr: plain CG)
  const int* blk;      // block of each point
  const int* bstart;   // first point of each block
  const int* bsize;    // points in each block
  const int* boff;     // offset of each block's inverse (row-major bsize^2)
  const float* binv_hi;  // block inverses as float-float pairs
  const float* binv_lo;
  // optional sparse matrix (CSR over rows; Shi/Slo hold the nnz values)
  const int* rowptr;
  const int* colidx;
  // optional initial guess (warm start)
  const double* x0;
  // optional learned banded preconditioner M r = W^-1 C^T C r: C has
  // 2 band_k + 1 coefficients per row (row-major), circular within each
  // body; seg_start / seg_len give each point's body (local indices)
  const float* band;
  int band_k;
  const int* seg_start;
  const int* seg_len;
  // optional deflation of the negative (net-charge) mode of the Dirichlet
  // Schur complement by deflated CG on Z = 1 (Nicolaides 1987; Saad, Yeung,
  // Erhel and Guyomarc'h 2000): sz = S 1 (this problem's rows) and
  // *inv_e = 1 / E, E = 1^T W S 1 < 0 (device memory, formed after the
  // Schur build; 0 makes the deflation a no-op).  S has one negative
  // eigenvalue and E
  // takes it, so S is positive definite on the S-orthogonal complement of 1
  // (inertia additivity of the Schur complement).  x0 is corrected by
  // (1^T W r0 / E) 1 so that 1^T W r0 = 0, and every search direction is
  // kept S-orthogonal to 1, p <- p - ((S 1)^T W p / E) 1, which keeps
  // 1^T W r = 0.  sz == nullptr: off.
  const double* sz;
  const double* inv_e;
  // optional: global-timer stamps (ns) when the problem is taken and done,
  // and the SM of the cluster's first CTA (profiling)
  unsigned long long* tspan;
  // optional coarse correction of the block-Jacobi preconditioner on the
  // bodies' constant vectors: z = M_bj r + Z E^-1 Z^T W r, Z the indicator
  // vectors of the cnb bodies (points [cstart[b], cstart[b+1])), E = Z^T W S Z
  // (cnb = 0: off)
  int cnb;
  int cstart[CG_COARSE_MAX + 1];
  const double* cEinv;  // CG_COARSE_MAX^2, row-major (device memory)
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned sm_id() {
  unsigned r;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
  return r;
}

// y[i - r0] = (S v)_i for a CSR matrix (float-float values), one warp per row
__device__ void ff_spmv_rows(const CGFFParams& pr, int r0, int r1, const float* __restrict__ vhi,
                             const float* __restrict__ vlo, double* __restrict__ y) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = r0 + warp; i < r1; i += CGC_WARPS) {
    const int e0 = pr.rowptr[i], e1 = pr.rowptr[i + 1];
    FF a0{0.f, 0.f}, a1{0.f, 0.f};
    int e = e0 + lane;
    for (; e + 32 < e1; e += 64) {
      const int c0 = __ldg(pr.colidx + e), c1 = __ldg(pr.colidx + e + 32);
      ff_fma(a0, __ldg(pr.Shi + e), __ldg(pr.Slo + e), vhi[c0], vlo[c0]);
      ff_fma(a1, __ldg(pr.Shi + e + 32), __ldg(pr.Slo + e + 32), vhi[c1], vlo[c1]);
    }
    if (e < e1) {
      const int c0 = __ldg(pr.colidx + e);
      ff_fma(a0, __ldg(pr.Shi + e), __ldg(pr.Slo + e), vhi[c0], vlo[c0]);
    }
    FF acc = ff_add(a0, a1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      FF other;
      other.hi = __shfl_down_sync(0xffffffffu, acc.hi, o);
      other.lo = __shfl_down_sync(0xffffffffu, acc.lo, o);
      acc = ff_add(acc, other);
    }
    if (lane == 0) y[i - r0] = (double)acc.hi + (double)acc.lo;
  }
}

// z[i - r0] = (M r)_i for rows i in [r0, r1): float-float block-Jacobi (the
// diagonal blocks of the Dirichlet Schur complement are indefinite with
// condition numbers up to ~1e6, so an FP32 application loses most of the gain)
__device__ void apply_bjacobi(const CGFFParams& pr, int r0, int r1, const float* __restrict__ rhi,
                              const float* __restrict__ rlo, double* __restrict__ z) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = r0 + warp; i < r1; i += CGC_WARPS) {
    const int b = pr.blk[i];
    const int s = pr.bstart[b], sz = pr.bsize[b];
    const float* __restrict__ rh = pr.binv_hi + pr.boff[b] + (size_t)(i - s) * sz;
    const float* __restrict__ rl = pr.binv_lo + pr.boff[b] + (size_t)(i - s) * sz;
    FF acc{0.f, 0.f};
    for (int t = lane; t < sz; t += 32) ff_fma(acc, __ldg(rh + t), __ldg(rl + t), rhi[s + t], rlo[s + t]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      FF other;
      other.hi = __shfl_down_sync(0xffffffffu, acc.hi, o);
      other.lo = __shfl_down_sync(0xffffffffu, acc.lo, o);
      acc = ff_add(acc, other);
    }
    if (lane == 0) z[i - r0] = (double)acc.hi + (double)acc.lo;
  }
}

__device__ __forceinline__ int seg_nb(int j, int s, int L, int t) {
  if (L < 1) return j;
  int q = (j - s + t) % L;
  q += q < 0 ? L : 0;
  return s + q;
}

// ---------------------------------------------------------------------------
// Replicated-vector cluster CG (systems of up to a few thousand unknowns).
//
// Every CTA of the cluster keeps the whole of x, r, p, z and W in shared
// memory and runs the vector updates, the dot products and the
// preconditioner redundantly: the same data and the same fixed reduction
// order keep the CTAs' copies bit-identical, so they take the same branches.
// Only the matrix-vector product is split by rows: each CTA writes its rows
// into its own full-length exchange buffer, one cluster barrier publishes
// them, and every CTA copies the other CTAs' rows out of their buffers
// through distributed shared memory.  That is one cluster barrier per
// iteration (two when the true residual is refreshed), where the
// row-distributed kernel above needs three barriers and two vector gathers.
// The two exchange buffers alternate, so a CTA never overwrites rows another
// CTA may still be reading: between two uses of one buffer lies the barrier
// of an exchange through the other.
// ---------------------------------------------------------------------------
constexpr int CGR_THREADS = 256;
constexpr int CGR_WARPS = CGR_THREADS / 32;

__device__ __forceinline__ void ff_fma4(FF& acc, float4 h, float4 l, float4 ph, float4 pl) {
  ff_fma(acc, h.x, l.x, ph.x, pl.x);
  ff_fma(acc, h.y, l.y, ph.y, pl.y);
  ff_fma(acc, h.z, l.z, ph.z, pl.z);
  ff_fma(acc, h.w, l.w, ph.w, pl.w);
}

// y[i] = (S v)_i for rows i in [r0, r1) of a dense float-float matrix whose
// rows start on 16-byte boundaries (stride schur_ld(n), zero padding; v
// zero-padded to the same length): one warp per two rows, 16-byte loads of
// four consecutive columns.
__device__ void ff_gemv_rows_v4(const float* __restrict__ Shi, const float* __restrict__ Slo, int n, int r0, int r1,
                                const float* __restrict__ vhi, const float* __restrict__ vlo, double* __restrict__ y) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ld = schur_ld(n), nq = ld >> 2;
  const float4* vh4 = reinterpret_cast<const float4*>(vhi);
  const float4* vl4 = reinterpret_cast<const float4*>(vlo);
  for (int i = r0 + 2 * warp; i < r1; i += 2 * CGR_WARPS) {
    const bool two = i + 1 < r1;
    const float4* h0 = reinterpret_cast<const float4*>(Shi + (size_t)i * ld);
    const float4* l0 = reinterpret_cast<const float4*>(Slo + (size_t)i * ld);
    const float4* h1 = reinterpret_cast<const float4*>(Shi + (size_t)(two ? i + 1 : i) * ld);
    const float4* l1 = reinterpret_cast<const float4*>(Slo + (size_t)(two ? i + 1 : i) * ld);
    FF a{0.f, 0.f}, b{0.f, 0.f};
    for (int j = lane; j < nq; j += 32) {
      const float4 x0 = __ldg(h0 + j), y0 = __ldg(l0 + j), x1 = __ldg(h1 + j), y1 = __ldg(l1 + j);
      const float4 ph = vh4[j], pl = vl4[j];
      ff_fma4(a, x0, y0, ph, pl);
      ff_fma4(b, x1, y1, ph, pl);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      FF oa, ob;
      oa.hi = __shfl_down_sync(0xffffffffu, a.hi, o);
      oa.lo = __shfl_down_sync(0xffffffffu, a.lo, o);
      ob.hi = __shfl_down_sync(0xffffffffu, b.hi, o);
      ob.lo = __shfl_down_sync(0xffffffffu, b.lo, o);
      a = ff_add(a, oa);
      b = ff_add(b, ob);
    }
    if (lane == 0) {
      y[i] = (double)a.hi + (double)a.lo;
      if (two) y[i + 1] = (double)b.hi + (double)b.lo;
    }
  }
}

// rows [r0, r1) of S v into y (full-length indexing)
__device__ __forceinline__ void matvec_rows_full(const CGFFParams& pr, int n, int r0, int r1, const float* vhi,
                                                 const float* vlo, double* y) {
  if (pr.rowptr) ff_spmv_rows(pr, r0, r1, vhi, vlo, y + r0);
  else ff_gemv_rows_v4(pr.Shi, pr.Slo, n, r0, r1, vhi, vlo, y);
}

// neighbour of point j at band offset t within its body [s, s + L) (circular)
__device__ __forceinline__ int seg_nb_near(int j, int s, int L, int t) {
  if (L < 1) return j;
  int q = j + t;
  if (q < s) q += L;
  else if (q >= s + L) q -= L;
  if (q < s || q >= s + L) return seg_nb(j, s, L, t);  // body shorter than the band
  return q;
}

// z = W^-1 C^T C r over all n points (float-float): u = C r for every point
// first (one thread per point), then z from u, so every thread has work and
// each product is formed once
__device__ void apply_band_full(const CGFFParams& pr, int n, const float* __restrict__ rhi,
                                const float* __restrict__ rlo, float* __restrict__ uhi, float* __restrict__ ulo,
                                const double* __restrict__ w, double* __restrict__ z) {
  const int K = pr.band_k, P = 2 * K + 1;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const int s = __ldg(pr.seg_start + j), L = __ldg(pr.seg_len + j);
    const float* __restrict__ cj = pr.band + (size_t)j * P;
    FF u{0.f, 0.f};
    for (int t2 = -K; t2 <= K; ++t2) {
      const int q = seg_nb_near(j, s, L, t2);
      ff_fma(u, __ldg(cj + t2 + K), 0.f, rhi[q], rlo[q]);
    }
    uhi[j] = u.hi;
    ulo[j] = u.lo;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int s = __ldg(pr.seg_start + i), L = __ldg(pr.seg_len + i);
    FF acc{0.f, 0.f};
    for (int t = -K; t <= K; ++t) {
      const int j = seg_nb_near(i, s, L, -t);
      ff_fma(acc, __ldg(pr.band + (size_t)j * P + t + K), 0.f, uhi[j], ulo[j]);
    }
    z[i] = fdiv((double)acc.hi + (double)acc.lo, w[i]);
  }
}

struct CGRShared {
  double* red;
  double* work;
  double *x, *r, *p, *z, *w, *xb[2];
  float *vhi, *vlo, *uhi, *ulo;
};

__device__ __forceinline__ void split_full(const double* v, int n, int ld, float* vhi, float* vlo) {
  for (int j = threadIdx.x; j < ld; j += blockDim.x) {
    const double a = j < n ? v[j] : 0.0;
    const float h = (float)a;
    vhi[j] = h;
    vlo[j] = (float)(a - (double)h);
  }
}

// sum_j w_j a_j b_j and sum_j w2_j c_j d_j over the whole vectors (fixed order)
__device__ __forceinline__ double wsum(const double* w, const double* a, const double* b, int n, double* red) {
  double s = 0.0, unused = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) s += w[j] * a[j] * b[j];
  block_sum2(s, unused, red);
  return s;
}

// y = S v (full vector in every CTA): rows [r0, r1) here, the rest from the
// other CTAs' exchange buffers after one cluster barrier.  v must be split
// into vhi / vlo (zero-padded) and visible to the whole CTA.
__device__ __forceinline__ double* exchange_matvec(cg::cluster_group& cl, const CGFFParams& pr, const CGRShared& S, int& xsel, int n,
                                   int rows, int rank, int r0, int r1) {
  double* buf = S.xb[xsel];
  xsel ^= 1;
  matvec_rows_full(pr, n, r0, r1, S.vhi, S.vlo, buf);
  cl.sync();
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const int c = j / rows;
    if (c != rank) buf[j] = cl.map_shared_rank(buf, c)[j];
  }
  __syncthreads();
  return buf;
}

__device__ __forceinline__ void apply_precond_full(const CGFFParams& pr, int n, const CGRShared& S, double* z) {
  if (pr.band) apply_band_full(pr, n, S.vhi, S.vlo, S.uhi, S.ulo, S.w, z);
  else apply_bjacobi(pr, 0, n, S.vhi, S.vlo, z);
}

// deflation of a whole search direction (sz = S 1, inv_e = 1 / 1^T W S 1):
// p -= ((S 1)^T W p / E) 1, each thread its own entries (no-op without sz)
__device__ __forceinline__ void deflate_full(const double* sz, double inv_e, const double* w, double* p, int n,
                                             double* red) {
  if (!sz) return;
  double m = 0.0, unused = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) m += w[j] * __ldg(sz + j) * p[j];
  block_sum2(m, unused, red);
  m *= inv_e;
  for (int j = threadIdx.x; j < n; j += blockDim.x) p[j] -= m;
}

__global__ void __cluster_dims__(CG_CLUSTER, 1, 1) __launch_bounds__(CGR_THREADS, 3)
    k_cg_rep(const CGFFParams* __restrict__ P, const int* __restrict__ order, int nprob, int* counter, int max_n) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int ldm = schur_ld(max_n);
  extern __shared__ __align__(16) unsigned char smraw[];
  CGRShared S;
  S.red = reinterpret_cast<double*>(smraw);  // 2 * threads + 2
  S.work = S.red + 2 * CGR_THREADS + 2;       // 4: [0] queue index taken by rank 0
  S.x = S.work + 4;
  S.r = S.x + ldm;
  S.p = S.r + ldm;
  S.z = S.p + ldm;
  S.w = S.z + ldm;
  S.xb[0] = S.w + ldm;
  S.xb[1] = S.xb[0] + ldm;
  S.vhi = reinterpret_cast<float*>(S.xb[1] + ldm);
  S.vlo = S.vhi + ldm;
  S.uhi = S.vlo + ldm;
  S.ulo = S.uhi + ldm;
  double* x = S.x;
  double* r = S.r;
  double* p = S.p;
  double* z = S.z;
  double* w = S.w;
  double* red = S.red;
  int xsel = 0;
  while (true) {
    if (rank == 0 && threadIdx.x == 0) S.work[0] = (double)atomicAdd(counter, 1);
    cl.sync();
    const int q = (int)cl.map_shared_rank(S.work, 0)[0];
    if (q >= nprob) break;
    const CGFFParams& pr = P[order[q]];
    if (pr.tspan && rank == 0 && threadIdx.x == 0) {
      pr.tspan[0] = global_ns();
      pr.tspan[2] = sm_id();
    }
    const int n = pr.n, ld = schur_ld(n);
    const int rows = (n + CG_CLUSTER - 1) / CG_CLUSTER;
    const int r0 = min(n, rank * rows), r1 = min(n, r0 + rows);
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      x[j] = pr.x0 ? pr.x0[j] : 0.0;
      w[j] = pr.w ? pr.w[j] : 1.0;
    }
    __syncthreads();
    if (pr.x0) {  // warm start: r = b - S x0
      split_full(x, n, ld, S.vhi, S.vlo);
      __syncthreads();
      const double* t = exchange_matvec(cl, pr, S, xsel, n, rows, rank, r0, r1);
      for (int j = threadIdx.x; j < n; j += blockDim.x) r[j] = pr.b[j] - t[j];
    } else {
      for (int j = threadIdx.x; j < n; j += blockDim.x) r[j] = pr.b[j];
    }
    __syncthreads();
    const double* sz = pr.sz;  // deflation (as k_cg_cluster): S 1, whole vector
    const double inv_e = sz ? __ldg(pr.inv_e) : 0.0;
    if (sz) {  // x += c 1, r -= c S 1, c = 1^T W r / E
      double c = 0.0, unused = 0.0;
      for (int j = threadIdx.x; j < n; j += blockDim.x) c += w[j] * r[j];
      block_sum2(c, unused, red);
      c *= inv_e;
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        x[j] += c;
        r[j] -= c * __ldg(sz + j);
      }
      __syncthreads();
    }
    const bool pre = pr.blk != nullptr || pr.band != nullptr;
    double bb = 0.0, rz = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      const double bj = pr.b[j];
      bb += bj * bj;
      rz += w[j] * r[j] * r[j];
    }
    block_sum2(bb, rz, red);
    if (pre) {
      split_full(r, n, ld, S.vhi, S.vlo);
      __syncthreads();
      apply_precond_full(pr, n, S, z);
      __syncthreads();
    }
    for (int j = threadIdx.x; j < n; j += blockDim.x) p[j] = pre ? z[j] : r[j];
    deflate_full(sz, inv_e, w, p, n, red);
    const double bnorm = sqrt(bb);
    const double thr = pr.tol * bnorm;
    const double thr2 = thr * thr;
    double rlast = bb;  // latest squared residual norm (recursive or true)
    int it = 0;
    double relres = bnorm > 0 ? 1.0 : 0.0;
    bool done = bnorm == 0.0;
    // stagnation guard (as in k_cg_cluster): the best true-residual iterate
    // is kept in pr.x (each CTA its rows)
    double best = 1e300;
    int stall = 0;
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) pr.x[i] = x[i];
    __syncthreads();
    while (!done && it < pr.maxiter) {
      split_full(p, n, ld, S.vhi, S.vlo);
      __syncthreads();
      double* qv = exchange_matvec(cl, pr, S, xsel, n, rows, rank, r0, r1);
      double pq = 0.0, pr_ = 0.0;
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        pq += w[j] * p[j] * qv[j];
        pr_ += w[j] * p[j] * r[j];
      }
      block_sum2(pq, pr_, red);
      if (pq == 0.0) break;
      const double alpha = fdiv(pre ? pr_ : rz, pq);
      double rr = 0.0, rzn = 0.0;
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        x[j] += alpha * p[j];
        const double rj = r[j] - alpha * qv[j];
        r[j] = rj;
        rr += rj * rj;
        rzn += w[j] * rj * rj;
      }
      block_sum2(rr, rzn, red);
      ++it;
      rlast = rr;
      if (rr <= thr2 || (it % 50) == 0 || it == pr.maxiter) {
        // true residual b - S x (exchange through the other buffer: q = S p stays)
        split_full(x, n, ld, S.vhi, S.vlo);
        __syncthreads();
        const double* t = exchange_matvec(cl, pr, S, xsel, n, rows, rank, r0, r1);
        double tr = 0.0, tz = 0.0;
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
          const double rj = pr.b[j] - t[j];
          r[j] = rj;
          tr += rj * rj;
          tz += w[j] * rj * rj;
        }
        block_sum2(tr, tz, red);
        relres = bnorm > 0 ? sqrt(tr) / bnorm : 0.0;
        rlast = tr;
        rzn = tz;
        if (tr <= thr2) {
          done = true;
          break;
        }
        if (relres < best) {
          best = relres;
          stall = 0;
          for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) pr.x[i] = x[i];
        } else if (++stall >= 8) {
          break;
        }
      }
      if (!pre) {
        const double beta = fdiv(rzn, rz);
        rz = rzn;
        for (int j = threadIdx.x; j < n; j += blockDim.x) p[j] = r[j] + beta * p[j];
        deflate_full(sz, inv_e, w, p, n, red);
        __syncthreads();
      } else {
        // flexible CG: z = M r, beta = -(z, q) / (p, q), p = z + beta p
        split_full(r, n, ld, S.vhi, S.vlo);
        __syncthreads();
        apply_precond_full(pr, n, S, z);
        __syncthreads();
        const double zq = wsum(w, z, qv, n, red);
        const double beta = fdiv(-zq, pq);
        for (int j = threadIdx.x; j < n; j += blockDim.x) p[j] = z[j] + beta * p[j];
        deflate_full(sz, inv_e, w, p, n, red);
        __syncthreads();
      }
    }
    relres = bnorm > 0 ? sqrt(rlast) / bnorm : 0.0;
    if (best < relres) {  // stopped past the best iterate: return that one
      relres = best;
      cl.sync();  // every CTA's rows of the best iterate are in pr.x
      for (int j = threadIdx.x; j < n; j += blockDim.x) x[j] = __ldcg(pr.x + j);
      __syncthreads();
    }
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) pr.x[i] = x[i];
    if (rank == 0 && threadIdx.x == 0) {
      if (pr.iters) *pr.iters = it;
      if (pr.relres) *pr.relres = relres;
      if (pr.tspan) pr.tspan[1] = global_ns();
    }
  }
  cl.sync();  // keep shared memory alive until every CTA is done reading it
}

// ---------------------------------------------------------------------------
// Row-distributed cluster CG (any size that fits the slices in shared memory).
//
// Each CTA owns rows [r0, r1) of every vector (FP64 slices of x, r, p, q, z,
// W, b) and of the matrix.  Vectors that the whole cluster needs (p for the
// product, r for the preconditioner, x for the true residual) are exchanged
// as float-float splits: every CTA writes the split of its slice into its own
// full-length buffer, a cluster barrier publishes it, and every CTA copies the
// other CTAs' parts through distributed shared memory (FP32 loads; no FP64
// work over the full length).  Reductions sum per-thread partials in warp 0
// only and publish one value per CTA; the CG scalars are formed once, by
// thread 0, and broadcast.  GB300's FP64 issue rate is a small fraction of
// its FP32 rate, so FP64 work is kept to the owned rows.  Two exchange
// buffers alternate; between two writes of one buffer lies the barrier of
// an exchange through the other, so no CTA overwrites rows that another CTA
// may still be copying.
// ---------------------------------------------------------------------------

// rows [r0, r1) of S v as float-float pairs yh/yl[i - r0] (dense rows with
// 16-byte alignment, or CSR)
__device__ void matvec_rows_ff(const CGFFParams& pr, int n, int r0, int r1, const float* __restrict__ vhi,
                               const float* __restrict__ vlo, float* __restrict__ yh, float* __restrict__ yl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (pr.rowptr) {
    for (int i = r0 + warp; i < r1; i += nwarps) {
      const int e0 = pr.rowptr[i], e1 = pr.rowptr[i + 1];
      FF a{0.f, 0.f};
      for (int e = e0 + lane; e < e1; e += 32) {
        const int c = __ldg(pr.colidx + e);
        ff_fma(a, __ldg(pr.Shi + e), __ldg(pr.Slo + e), vhi[c], vlo[c]);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        FF oa;
        oa.hi = __shfl_down_sync(0xffffffffu, a.hi, o);
        oa.lo = __shfl_down_sync(0xffffffffu, a.lo, o);
        a = ff_add(a, oa);
      }
      if (lane == 0) {
        yh[i - r0] = a.hi;
        yl[i - r0] = a.lo;
      }
    }
    return;
  }
  const int ld = schur_ld(n), nq = ld >> 2;
  const float4* vh4 = reinterpret_cast<const float4*>(vhi);
  const float4* vl4 = reinterpret_cast<const float4*>(vlo);
  for (int i = r0 + 2 * warp; i < r1; i += 2 * nwarps) {
    const bool two = i + 1 < r1;
    const float4* h0 = reinterpret_cast<const float4*>(pr.Shi + (size_t)i * ld);
    const float4* l0 = reinterpret_cast<const float4*>(pr.Slo + (size_t)i * ld);
    const float4* h1 = reinterpret_cast<const float4*>(pr.Shi + (size_t)(two ? i + 1 : i) * ld);
    const float4* l1 = reinterpret_cast<const float4*>(pr.Slo + (size_t)(two ? i + 1 : i) * ld);
    FF a{0.f, 0.f}, b{0.f, 0.f};
    int j = lane;
    for (; j + 32 < nq; j += 64) {  // eight 16-byte loads in flight per lane
      const float4 x0 = __ldg(h0 + j), y0 = __ldg(l0 + j), x1 = __ldg(h1 + j), y1 = __ldg(l1 + j);
      const float4 x2 = __ldg(h0 + j + 32), y2 = __ldg(l0 + j + 32), x3 = __ldg(h1 + j + 32),
                   y3 = __ldg(l1 + j + 32);
      ff_fma4(a, x0, y0, vh4[j], vl4[j]);
      ff_fma4(b, x1, y1, vh4[j], vl4[j]);
      ff_fma4(a, x2, y2, vh4[j + 32], vl4[j + 32]);
      ff_fma4(b, x3, y3, vh4[j + 32], vl4[j + 32]);
    }
    if (j < nq) {
      const float4 x0 = __ldg(h0 + j), y0 = __ldg(l0 + j), x1 = __ldg(h1 + j), y1 = __ldg(l1 + j);
      ff_fma4(a, x0, y0, vh4[j], vl4[j]);
      ff_fma4(b, x1, y1, vh4[j], vl4[j]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      FF oa, ob;
      oa.hi = __shfl_down_sync(0xffffffffu, a.hi, o);
      oa.lo = __shfl_down_sync(0xffffffffu, a.lo, o);
      ob.hi = __shfl_down_sync(0xffffffffu, b.hi, o);
      ob.lo = __shfl_down_sync(0xffffffffu, b.lo, o);
      a = ff_add(a, oa);
      b = ff_add(b, ob);
    }
    if (lane == 0) {
      yh[i - r0] = a.hi;
      yl[i - r0] = a.lo;
      if (two) {
        yh[i + 1 - r0] = b.hi;
        yl[i + 1 - r0] = b.lo;
      }
    }
  }
}

// z[i - r0] = (W^-1 C^T C r)_i for the owned rows (float-float).  u = C r is
// formed for every point (one thread per point, coefficient rows read from
// L2; the same values in every CTA), so the owned rows, including those
// whose band wraps around their body, read their neighbours' u from shared
// memory.
__device__ void apply_band_rows(const CGFFParams& pr, int n, int r0, int r1, const float* __restrict__ rhi,
                                const float* __restrict__ rlo, float* __restrict__ uhi, float* __restrict__ ulo,
                                const double* __restrict__ ws, double* __restrict__ z) {
  const int K = pr.band_k, P = 2 * K + 1;
  // half-width 4 (the shipped networks): fixed trip counts, so every
  // coefficient load of a point is issued before the first product
  constexpr int K4 = 4, P4 = 9;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const int s = __ldg(pr.seg_start + j), L = __ldg(pr.seg_len + j);
    const float* __restrict__ cj = pr.band + (size_t)j * P;
    FF u{0.f, 0.f};
    if (K == K4) {
      float c[P4];
#pragma unroll
      for (int t = 0; t < P4; ++t) c[t] = __ldg(cj + t);
#pragma unroll
      for (int t2 = -K4; t2 <= K4; ++t2) {
        const int q = seg_nb_near(j, s, L, t2);
        ff_fma(u, c[t2 + K4], 0.f, rhi[q], rlo[q]);
      }
    } else {
      for (int t2 = -K; t2 <= K; ++t2) {
        const int q = seg_nb_near(j, s, L, t2);
        ff_fma(u, __ldg(cj + t2 + K), 0.f, rhi[q], rlo[q]);
      }
    }
    uhi[j] = u.hi;
    ulo[j] = u.lo;
  }
  __syncthreads();
  for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
    const int s = __ldg(pr.seg_start + i), L = __ldg(pr.seg_len + i);
    FF acc{0.f, 0.f};
    if (K == K4) {
      int jn[P4];
      float c[P4];
#pragma unroll
      for (int t = -K4; t <= K4; ++t) {
        jn[t + K4] = seg_nb_near(i, s, L, -t);
        c[t + K4] = __ldg(pr.band + (size_t)jn[t + K4] * P4 + t + K4);
      }
#pragma unroll
      for (int t = 0; t < P4; ++t) ff_fma(acc, c[t], 0.f, uhi[jn[t]], ulo[jn[t]]);
    } else {
      for (int t = -K; t <= K; ++t) {
        const int j = seg_nb_near(i, s, L, -t);
        ff_fma(acc, __ldg(pr.band + (size_t)j * P + t + K), 0.f, uhi[j], ulo[j]);
      }
    }
    z[i - r0] = fdiv((double)acc.hi + (double)acc.lo, ws[i - r0]);
  }
}

// zh/zl[i - r0] = (M r)_i for the owned rows, block-Jacobi in float-float:
// one warp per four rows so that four rows' loads are in flight together
__device__ void apply_bjacobi_rows(const CGFFParams& pr, int r0, int r1, const float* __restrict__ rhi,
                                   const float* __restrict__ rlo, float* __restrict__ zh, float* __restrict__ zl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i0 = r0 + 4 * warp; i0 < r1; i0 += 4 * nw) {
    FF acc[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      acc[u] = FF{0.f, 0.f};
      const int i = i0 + u;
      if (i < r1) {
        const int b = pr.blk[i];
        const int s = pr.bstart[b], sz = pr.bsize[b];
        const float* __restrict__ rh = pr.binv_hi + pr.boff[b] + (size_t)(i - s) * sz;
        const float* __restrict__ rl = pr.binv_lo + pr.boff[b] + (size_t)(i - s) * sz;
        int t = lane;
        for (; t + 32 < sz; t += 64) {  // two columns per lane per trip, loads first
          const float h0 = __ldg(rh + t), l0 = __ldg(rl + t), h1 = __ldg(rh + t + 32), l1 = __ldg(rl + t + 32);
          ff_fma(acc[u], h0, l0, rhi[s + t], rlo[s + t]);
          ff_fma(acc[u], h1, l1, rhi[s + t + 32], rlo[s + t + 32]);
        }
        if (t < sz) ff_fma(acc[u], __ldg(rh + t), __ldg(rl + t), rhi[s + t], rlo[s + t]);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        FF other;
        other.hi = __shfl_down_sync(0xffffffffu, acc[u].hi, o);
        other.lo = __shfl_down_sync(0xffffffffu, acc[u].lo, o);
        acc[u] = ff_add(acc[u], other);
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u < r1) {
          zh[i0 + u - r0] = acc[u].hi;
          zl[i0 + u - r0] = acc[u].lo;
        }
    }
  }
}

// Cluster-wide sums of K <= 4 values, partials held by threads [0, nact).
// On return the totals are in v[] of thread 0 only; thread 0 derives what
// the other threads need, stores it in the broadcast area and the caller
// synchronises the CTA before reading it.  Each FP64 partial is split into a
// float-float pair (hi exact, lo rounded: ~48 bits) and the sums run in FP32
// float-float arithmetic: GB300 issues FP64 at a small fraction of the FP32
// rate and a chain of dependent FP64 adds costs far more latency than the
// same chain of FP32 two-sums.  `red` holds 2 K blockDim floats (K blockDim
// doubles), `pub` 8 slots of 4 float-float values; the published slot
// rotates over seven values so that a CTA never overwrites a slot another
// CTA may still be reading.  K <= CG_RED_K.
template <int K, int CS = CG_CLUSTER>
__device__ void csum_t0(cg::cluster_group& cl, double (&v)[K], int nact, double* red, double* pub, int& slot) {
  static_assert(K <= CG_RED_K, "too many values in one cluster reduction");
  constexpr int PS = 2 * CG_RED_K;  // floats per published slot
  const int t = threadIdx.x, nt = blockDim.x;
  float* rf = reinterpret_cast<float*>(red);
  float* pf = reinterpret_cast<float*>(pub);
  nact = min(nact, nt);  // threads beyond hold zero partials (or none)
  if (t < nact)
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const float h = (float)v[k];
      rf[(2 * k) * nt + t] = h;
      rf[(2 * k + 1) * nt + t] = (float)(v[k] - (double)h);
    }
  __syncthreads();
  if (t < 32) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      FF a{0.f, 0.f};
      for (int i = t; i < nact; i += 32) a = ff_add(a, FF{rf[(2 * k) * nt + i], rf[(2 * k + 1) * nt + i]});
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        FF b;
        b.hi = __shfl_down_sync(0xffffffffu, a.hi, o);
        b.lo = __shfl_down_sync(0xffffffffu, a.lo, o);
        a = ff_add(a, b);
      }
      if (t == 0) {
        pf[PS * slot + 2 * k] = a.hi;
        pf[PS * slot + 2 * k + 1] = a.lo;
      }
    }
  }
  cl.sync();
  if (t < 32) {
    float rh[K], rl[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      rh[k] = t < CS ? cl.map_shared_rank(pf, t)[PS * slot + 2 * k] : 0.f;
      rl[k] = t < CS ? cl.map_shared_rank(pf, t)[PS * slot + 2 * k + 1] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      FF a{rh[k], rl[k]};
#pragma unroll
      for (int o = CS / 2; o > 0; o >>= 1) {
        FF b;
        b.hi = __shfl_down_sync(0xffffffffu, a.hi, o);
        b.lo = __shfl_down_sync(0xffffffffu, a.lo, o);
        a = ff_add(a, b);
      }
      v[k] = (double)a.hi + (double)a.lo;
    }
  }
  slot = slot == 7 ? 1 : slot + 1;
}

// body of local point i under the coarse correction (cnb >= 1)
__device__ __forceinline__ int coarse_body(const CGFFParams& pr, int i) {
  int b = 0;
#pragma unroll
  for (int k = 1; k < CG_COARSE_MAX; ++k) b += (k < pr.cnb && i >= pr.cstart[k]) ? 1 : 0;
  return b;
}

// csum_t0 of v[0, K0) and, with the coarse correction, of the per-body sums
// sum_{i in body b} w_i r_i of the owned rows; thread 0 then forms the
// coarse coefficients c = E^-1 Z^T W r into bc[16 + b] (read after the
// caller's next CTA barrier).
template <int K0, int CS>
__device__ void csum_coarse(cg::cluster_group& cl, const CGFFParams& pr, double (&v)[K0], const double* ws,
                            const double* rs, int r0, int nr, double* red, double* pub, int& slot, double* bc) {
  if (pr.cnb <= 0) {
    csum_t0<K0, CS>(cl, v, nr, red, pub, slot);
    return;
  }
  double u[K0 + CG_COARSE_MAX];
#pragma unroll
  for (int k = 0; k < K0; ++k) u[k] = v[k];
#pragma unroll
  for (int b = 0; b < CG_COARSE_MAX; ++b) u[K0 + b] = 0.0;
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    const int bi = coarse_body(pr, r0 + i);
    const double wr = ws[i] * rs[i];
#pragma unroll
    for (int b = 0; b < CG_COARSE_MAX; ++b) u[K0 + b] += b == bi ? wr : 0.0;
  }
  csum_t0<K0 + CG_COARSE_MAX, CS>(cl, u, nr, red, pub, slot);
#pragma unroll
  for (int k = 0; k < K0; ++k) v[k] = u[k];
  if (threadIdx.x == 0)  // entries of E^-1 beyond the bodies are zero
#pragma unroll
    for (int a = 0; a < CG_COARSE_MAX; ++a) {
      double c = 0.0;
#pragma unroll
      for (int b = 0; b < CG_COARSE_MAX; ++b) c += pr.cEinv[a * CG_COARSE_MAX + b] * u[K0 + b];
      bc[16 + a] = c;
    }
}

// z_i += c[body(i)] on the owned rows (coarse coefficients in bc[16..])
__device__ __forceinline__ void add_coarse(const CGFFParams& pr, int r0, int nr, double* zs, const double* bc) {
  if (pr.cnb <= 0) return;
  for (int i = threadIdx.x; i < nr; i += blockDim.x) zs[i] += bc[16 + coarse_body(pr, r0 + i)];
}

// split of the owned slice into the exchange buffer's owned part
__device__ __forceinline__ void publish_slice(const double* s, int r0, int nr, float* eh, float* el) {
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    const double v = s[i];
    const float h = (float)v;
    eh[r0 + i] = h;
    el[r0 + i] = (float)(v - (double)h);
  }
}

// copy the other CTAs' parts of an exchange buffer (after the barrier that
// published them)
__device__ __forceinline__ void gather_parts(cg::cluster_group& cl, float* eh, float* el, int n, int rows, int rank) {
  // four elements per thread and trip, all remote loads issued before the stores
  const int nt = blockDim.x;
  for (int j0 = threadIdx.x; j0 < n; j0 += 4 * nt) {
    float h[4], l[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = j0 + u * nt;
      const int c = j < n ? j / rows : rank;
      h[u] = c != rank ? cl.map_shared_rank(eh, c)[j] : 0.f;
      l[u] = c != rank ? cl.map_shared_rank(el, c)[j] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = j0 + u * nt;
      if (j < n && j / rows != rank) {
        eh[j] = h[u];
        el[j] = l[u];
      }
    }
  }
  __syncthreads();
}

// p = v + b p in float-float (b = bh + bl); ~2^-46 relative
__device__ __forceinline__ FF ff_axpy(float bh, float bl, FF p, FF v) {
  const float m = bh * p.hi;
  float me = fmaf(bh, p.hi, -m);
  me = fmaf(bh, p.lo, fmaf(bl, p.hi, me));
  float s, e;
  two_sum(v.hi, m, s, e);
  e += v.lo + me;
  const float hi = s + e;
  return FF{hi, e - (hi - s)};
}

// a - (mh + ml) in float-float
__device__ __forceinline__ FF ff_sub_const(FF a, float mh, float ml) {
  float s, e;
  two_sum(a.hi, -mh, s, e);
  e += a.lo - ml;
  const float hi = s + e;
  return FF{hi, e - (hi - s)};
}

// The search direction p is kept whole in every CTA as a float-float vector
// (ph/pl) and updated there (p = z + beta p over all n points in FP32
// float-float arithmetic), so the product S p needs no exchange: only r
// (and z with a preconditioner) cross the cluster, each with the barrier of
// the reduction that needs it anyway.  Plain CG takes two cluster barriers
// per iteration, flexible CG three.  The owned slice of p is read back as
// (double)hi + (double)lo, so x, r and the product all use the same p.
// With the deflation (pr.sz) the projection of p rides in the reduction of
// z (or r) that the update needs anyway: no barrier is added.
template <int NT, int MINB, int CS = CG_CLUSTER>
__global__ void __cluster_dims__(CS, 1, 1) __launch_bounds__(NT, MINB)
    k_cg_cluster(const CGFFParams* __restrict__ P, const int* __restrict__ order, int nprob, int* counter,
                 int max_n) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int rmax = (max_n + CS - 1) / CS;
  const int ldm = schur_ld(max_n);
  extern __shared__ __align__(16) unsigned char smraw[];
  double* red = reinterpret_cast<double*>(smraw);  // CG_RED_K * threads (2 K floats per thread)
  double* bc = red + CG_RED_K * NT;                // CG_BC: scalars broadcast by thread 0
  double* pub = bc + CG_BC;                        // 8 slots x CG_RED_K float-float: published CTA sums
  double* work = pub + 8 * CG_RED_K;               // 4: [0] queue index taken by rank 0
  double* xs = work + 4;                           // owned slices (rmax each)
  double* rs = xs + rmax;
  double* ps = rs + rmax;
  double* qs = ps + rmax;
  double* zs = qs + rmax;
  double* ws = zs + rmax;
  double* bs = ws + rmax;
  // float arrays, 16-byte aligned: p (whole), exchange buffers for r (A) and
  // for z / x (B), band intermediate, product rows, staged band and segments
  float* ph = reinterpret_cast<float*>(bs + rmax + (rmax & 1));
  float* pl = ph + ldm;
  float* ah = pl + ldm;
  float* al = ah + ldm;
  float* bh = al + ldm;
  float* bl = bh + ldm;
  float* uhi = bl + ldm;  // band intermediate u = C r (every point)
  float* ulo = uhi + ldm;
  float* yh = ulo + ldm;  // product rows
  float* yl = yh + rmax;
  int slot = 1;
  while (true) {
    if (rank == 0 && threadIdx.x == 0) work[0] = (double)atomicAdd(counter, 1);
    cl.sync();
    const int q = (int)cl.map_shared_rank(work, 0)[0];
    if (q >= nprob) break;
    const CGFFParams& pr = P[order[q]];  // fields read through L1 as needed
    if (pr.tspan && rank == 0 && threadIdx.x == 0) {
      pr.tspan[0] = global_ns();
      pr.tspan[2] = sm_id();
    }
    const int n = pr.n, ld = schur_ld(n);
    const int rows = (n + CS - 1) / CS;
    const int r0 = min(n, rank * rows), r1 = min(n, r0 + rows);
    const int nr = r1 - r0;
    const bool sz = pr.sz != nullptr;  // deflation: S 1 read from pr.sz (owned rows from r0)
    // 1 / E (deflation) is read by thread 0 where it forms the scalars
    const bool pre = pr.blk != nullptr || pr.band != nullptr;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      xs[i] = pr.x0 ? pr.x0[r0 + i] : 0.0;
      bs[i] = pr.b[r0 + i];
      ws[i] = pr.w ? pr.w[r0 + i] : 1.0;
    }
    for (int j = n + threadIdx.x; j < ld; j += blockDim.x) {  // padding of the product's vectors
      ph[j] = pl[j] = bh[j] = bl[j] = 0.f;
    }
    __syncthreads();
    if (pr.x0) {  // warm start: r = b - S x0 (x through buffer B)
      double v[1] = {0.0};
      publish_slice(xs, r0, nr, bh, bl);
      csum_t0<1, CS>(cl, v, nr, red, pub, slot);  // the barrier that publishes x
      gather_parts(cl, bh, bl, n, rows, rank);
      matvec_rows_ff(pr, n, r0, r1, bh, bl, yh, yl);
      __syncthreads();
      for (int i = threadIdx.x; i < nr; i += blockDim.x) rs[i] = bs[i] - ((double)yh[i] + (double)yl[i]);
      __syncthreads();
    } else {
      for (int i = threadIdx.x; i < nr; i += blockDim.x) rs[i] = bs[i];
      __syncthreads();
    }
    if (sz) {  // deflation: x += c 1, r -= c S 1, c = 1^T W r / E (then 1^T W r = 0)
      double v[1] = {0.0};
      for (int i = threadIdx.x; i < nr; i += blockDim.x) v[0] += ws[i] * rs[i];
      csum_t0<1, CS>(cl, v, nr, red, pub, slot);
      if (threadIdx.x == 0) bc[0] = v[0] * __ldg(pr.inv_e);
      __syncthreads();
      const double c = bc[0];
      for (int i = threadIdx.x; i < nr; i += blockDim.x) {
        xs[i] += c;
        rs[i] -= c * __ldg(pr.sz + r0 + i);
      }
      __syncthreads();
    }
    // |b|^2, (r, r)_W and (S 1)^T W r (the deflation's projection of p = r);
    // r published with the same barrier
    double rz, bnorm, mu;
    {
      double v[3] = {0.0, 0.0, 0.0};
      for (int i = threadIdx.x; i < nr; i += blockDim.x) {
        v[0] += bs[i] * bs[i];
        v[1] += ws[i] * rs[i] * rs[i];
        if (sz) v[2] += ws[i] * __ldg(pr.sz + r0 + i) * rs[i];
      }
      publish_slice(rs, r0, nr, ah, al);
      csum_coarse<3, CS>(cl, pr, v, ws, rs, r0, nr, red, pub, slot, bc);
      if (threadIdx.x == 0) {
        bc[0] = sqrt(v[0]);
        bc[1] = v[1];
        bc[2] = sz ? v[2] * __ldg(pr.inv_e) : 0.0;
      }
      gather_parts(cl, ah, al, n, rows, rank);
      bnorm = bc[0];
      rz = bc[1];
      mu = bc[2];
    }
    if (pre) {  // p = z = M r (- mu 1), exchanged through buffer B (with (S 1)^T W z)
      if (pr.band) {
        apply_band_rows(pr, n, r0, r1, ah, al, uhi, ulo, ws, zs);
      } else {
        apply_bjacobi_rows(pr, r0, r1, ah, al, yh, yl);
        __syncthreads();
        for (int i = threadIdx.x; i < nr; i += blockDim.x) zs[i] = (double)yh[i] + (double)yl[i];
        add_coarse(pr, r0, nr, zs, bc);
      }
      __syncthreads();
      double v[1] = {0.0};
      if (sz)
        for (int i = threadIdx.x; i < nr; i += blockDim.x) v[0] += ws[i] * __ldg(pr.sz + r0 + i) * zs[i];
      publish_slice(zs, r0, nr, bh, bl);
      csum_t0<1, CS>(cl, v, nr, red, pub, slot);
      if (threadIdx.x == 0) bc[2] = sz ? v[0] * __ldg(pr.inv_e) : 0.0;
      gather_parts(cl, bh, bl, n, rows, rank);
      mu = bc[2];
      const float mh = (float)mu, ml = (float)(mu - (double)mh);
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const FF pj = sz ? ff_sub_const(FF{bh[j], bl[j]}, mh, ml) : FF{bh[j], bl[j]};
        ph[j] = pj.hi;
        pl[j] = pj.lo;
      }
    } else {
      const float mh = (float)mu, ml = (float)(mu - (double)mh);
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const FF pj = sz ? ff_sub_const(FF{ah[j], al[j]}, mh, ml) : FF{ah[j], al[j]};
        ph[j] = pj.hi;
        pl[j] = pj.lo;
      }
    }
    __syncthreads();
    const double thr = pr.tol * bnorm;
    const double thr2 = thr * thr;
    double rlast = bnorm * bnorm;
    int it = 0;
    double relres = bnorm > 0 ? 1.0 : 0.0;
    bool done = bnorm == 0.0;
    // stagnation guard: past the attainable accuracy (float-float products on
    // a Schur complement of condition ~1e6 floor near 1e-10) CG drifts and
    // eventually diverges; stop after 8 refreshes without a better true
    // residual and return the best iterate (kept in pr.x, owned rows)
    double best = 1e300;
    int stall = 0;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) pr.x[r0 + i] = xs[i];
    while (!done && it < pr.maxiter) {
      // q = S p on the owned rows (p whole in this CTA)
      matvec_rows_ff(pr, n, r0, r1, ph, pl, yh, yl);
      __syncthreads();
      double alpha, pq;
      {
        double v[2] = {0.0, 0.0};
        for (int i = threadIdx.x; i < nr; i += blockDim.x) {
          const double pi = (double)ph[r0 + i] + (double)pl[r0 + i];
          const double qi = (double)yh[i] + (double)yl[i];
          ps[i] = pi;
          qs[i] = qi;
          v[0] += ws[i] * pi * qi;
          v[1] += ws[i] * pi * rs[i];
        }
        csum_t0<2, CS>(cl, v, nr, red, pub, slot);
        if (threadIdx.x == 0) {
          bc[3] = v[0];
          bc[4] = v[0] != 0.0 ? fdiv(pre ? v[1] : rz, v[0]) : 0.0;
        }
        __syncthreads();
        pq = bc[3];
        alpha = bc[4];
      }
      if (pq == 0.0) break;
      double rr, rzn, mur;  // mur: the deflation's projection of p = r + beta p
      {
        double v[3] = {0.0, 0.0, 0.0};
        for (int i = threadIdx.x; i < nr; i += blockDim.x) {
          xs[i] += alpha * ps[i];
          const double ri = rs[i] - alpha * qs[i];
          rs[i] = ri;
          v[0] += ri * ri;
          v[1] += ws[i] * ri * ri;
          if (sz) v[2] += ws[i] * __ldg(pr.sz + r0 + i) * ri;
        }
        publish_slice(rs, r0, nr, ah, al);
        csum_coarse<3, CS>(cl, pr, v, ws, rs, r0, nr, red, pub, slot, bc);
        if (threadIdx.x == 0) {
          bc[5] = v[0];
          bc[6] = v[1];
          bc[7] = sz ? v[2] * __ldg(pr.inv_e) : 0.0;
        }
        __syncthreads();
        rr = bc[5];
        rzn = bc[6];
        mur = bc[7];
      }
      ++it;
      rlast = rr;
      if (rr <= thr2 || (it % 50) == 0 || it == pr.maxiter) {
        // true residual b - S x (x through buffer B; the r published above
        // is superseded by the refreshed one)
        {
          double v[1] = {0.0};
          publish_slice(xs, r0, nr, bh, bl);
          csum_t0<1, CS>(cl, v, nr, red, pub, slot);  // the barrier that publishes x
          gather_parts(cl, bh, bl, n, rows, rank);
          matvec_rows_ff(pr, n, r0, r1, bh, bl, yh, yl);
          __syncthreads();
        }
        double v[3] = {0.0, 0.0, 0.0};
        for (int i = threadIdx.x; i < nr; i += blockDim.x) {
          const double ri = bs[i] - ((double)yh[i] + (double)yl[i]);
          rs[i] = ri;
          v[0] += ri * ri;
          v[1] += ws[i] * ri * ri;
          if (sz) v[2] += ws[i] * __ldg(pr.sz + r0 + i) * ri;
        }
        publish_slice(rs, r0, nr, ah, al);
        csum_coarse<3, CS>(cl, pr, v, ws, rs, r0, nr, red, pub, slot, bc);
        if (threadIdx.x == 0) {
          bc[9] = v[0];
          bc[10] = v[1];
          bc[11] = sz ? v[2] * __ldg(pr.inv_e) : 0.0;
        }
        __syncthreads();
        const double tr = bc[9];
        rzn = bc[10];
        mur = bc[11];
        rlast = tr;
        if (tr <= thr2) {
          done = true;
          break;
        }
        relres = bnorm > 0 ? sqrt(tr) / bnorm : 0.0;
        if (relres < best) {
          best = relres;
          stall = 0;
          for (int i = threadIdx.x; i < nr; i += blockDim.x) pr.x[r0 + i] = xs[i];
        } else if (++stall >= 8) {
          break;
        }
      }
      // r of every CTA (buffer A), published with the reduction above
      gather_parts(cl, ah, al, n, rows, rank);
      // with the deflation the new p is projected: p -= ((S 1)^T W p / E) 1,
      // where (S 1)^T W p = (S 1)^T W (r or z) (the old p is S-orthogonal to 1)
      double beta;
      if (!pre) {
        beta = fdiv(rzn, rz);
        rz = rzn;
        // p = r + beta p (- mur 1)
        const float bh_ = (float)beta, bl_ = (float)(beta - (double)bh_);
        const float mh = (float)mur, ml = (float)(mur - (double)mh);
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
          FF pn = ff_axpy(bh_, bl_, FF{ph[j], pl[j]}, FF{ah[j], al[j]});
          if (sz) pn = ff_sub_const(pn, mh, ml);
          ph[j] = pn.hi;
          pl[j] = pn.lo;
        }
      } else {
        // flexible CG: z = M r, beta = -(z, q) / (p, q), p = z + beta p
        if (pr.band) {
          apply_band_rows(pr, n, r0, r1, ah, al, uhi, ulo, ws, zs);
        } else {
          apply_bjacobi_rows(pr, r0, r1, ah, al, yh, yl);
          __syncthreads();
          for (int i = threadIdx.x; i < nr; i += blockDim.x) zs[i] = (double)yh[i] + (double)yl[i];
          add_coarse(pr, r0, nr, zs, bc);
        }
        __syncthreads();
        double v[2] = {0.0, 0.0};
        for (int i = threadIdx.x; i < nr; i += blockDim.x) {
          v[0] += ws[i] * zs[i] * qs[i];
          if (sz) v[1] += ws[i] * __ldg(pr.sz + r0 + i) * zs[i];
        }
        publish_slice(zs, r0, nr, bh, bl);
        csum_t0<2, CS>(cl, v, nr, red, pub, slot);
        if (threadIdx.x == 0) {
          bc[13] = fdiv(-v[0], pq);
          bc[14] = sz ? v[1] * __ldg(pr.inv_e) : 0.0;
        }
        gather_parts(cl, bh, bl, n, rows, rank);
        beta = bc[13];
        const double muz = bc[14];
        const float bh_ = (float)beta, bl_ = (float)(beta - (double)bh_);
        const float mh = (float)muz, ml = (float)(muz - (double)mh);
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
          FF pn = ff_axpy(bh_, bl_, FF{ph[j], pl[j]}, FF{bh[j], bl[j]});
          if (sz) pn = ff_sub_const(pn, mh, ml);
          ph[j] = pn.hi;
          pl[j] = pn.lo;
        }
      }
      __syncthreads();
    }
    relres = bnorm > 0 ? sqrt(rlast) / bnorm : 0.0;
    if (best < relres) {  // stopped past the best iterate: return that one
      relres = best;
      for (int i = threadIdx.x; i < nr; i += blockDim.x) xs[i] = pr.x[r0 + i];
      __syncthreads();
    }
    for (int i = threadIdx.x; i < nr; i += blockDim.x) pr.x[r0 + i] = xs[i];
    if (rank == 0 && threadIdx.x == 0) {
      if (pr.iters) *pr.iters = it;
      if (pr.relres) *pr.relres = relres;
      if (pr.tspan) pr.tspan[1] = global_ns();
    }
  }
  cl.sync();  // keep shared memory alive until every CTA is done reading it
}

size_t cg_cluster_smem(int max_n, int nt, int cs) {
  const size_t rmax = (size_t)(max_n + cs - 1) / cs;
  const size_t ldm = (size_t)schur_ld(max_n);
  return (CG_RED_K * (size_t)nt + CG_BC + 8 * CG_RED_K + 4 + 7 * rmax + 1) * sizeof(double) +
         (8 * ldm + 2 * rmax) * sizeof(float) + 64;
}

size_t cg_rep_smem(int max_n) {
  const size_t ldm = (size_t)schur_ld(max_n);
  return (2 * CGR_THREADS + 2 + 4 + 7 * ldm) * sizeof(double) + 4 * ldm * sizeof(float);
}


// Kernel variants (the batch autotuner picks among them): 0 (default) and 1 =
// row-distributed over 8-CTA clusters, 256 threads per CTA, up to 3 CTAs per
// SM; 3 = 128 threads, up to 6 CTAs per SM (more problems in flight); 4 =
// 256 threads, at most 2 CTAs per SM (more registers, less sharing of an SM
// between clusters); 5 = 512 threads, one CTA per SM (each cluster alone on
// its SMs); 2 = replicated vectors, when they fit in shared memory.  The
// cluster size stays 8: clusters of 1, 2, 4 and 16 CTAs (the template's CS)
// were measured 2.7x, 2.0x, 1.2x and 1.5x slower on the batched
// configuration with the learned preconditioner (fewer CTAs cannot keep
// enough of a large problem's matrix rows in flight; 16 pays 16-way
// barriers).
static bool use_rep(int variant, int max_n) { return variant == 2 && cg_rep_smem(max_n) <= 200 * 1024; }
static int dist_threads(int variant) { return variant == 3 ? 128 : variant == 5 ? 512 : 256; }
static int dist_cluster(int) { return CG_CLUSTER; }

size_t cg_variant_smem(int max_n, int variant) {
  return use_rep(variant, max_n) ? cg_rep_smem(max_n)
                                 : cg_cluster_smem(max_n, dist_threads(variant), dist_cluster(variant));
}

template <int NT, int MINB, int CS>
static int launch_dist(const CGFFParams* prm, const int* order, int nprob, int* counter, int max_n, int nclusters,
                       size_t smem, cudaStream_t st) {
  ILM_CHECK_CUDA(
      cudaFuncSetAttribute(k_cg_cluster<NT, MINB, CS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_cg_cluster<NT, MINB, CS><<<nclusters * CS, NT, smem, st>>>(prm, order, nprob, counter, max_n);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

template <int NT, int MINB, int CS>
static cudaError_t clusters_dist(int* nc, cudaLaunchConfig_t* cfg, size_t smem) {
  cudaError_t e =
      cudaFuncSetAttribute(k_cg_cluster<NT, MINB, CS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(nc, k_cg_cluster<NT, MINB, CS>, cfg);
  return e;
}

int launch_cg_cluster(const void* params_dev, const int* order, int nprob, int* counter, int max_n, int nclusters,
                      cudaStream_t st, int variant) {
  const CGFFParams* prm = static_cast<const CGFFParams*>(params_dev);
  ILM_CHECK_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
  if (use_rep(variant, max_n)) {  // replicated vectors: one cluster barrier per iteration
    const size_t rsm = cg_rep_smem(max_n);
    ILM_CHECK_CUDA(cudaFuncSetAttribute(k_cg_rep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsm));
    k_cg_rep<<<nclusters * CG_CLUSTER, CGR_THREADS, rsm, st>>>(prm, order, nprob, counter, max_n);
    ILM_CHECK_LAUNCH();
    return ILM_OK;
  }
  const size_t smem = cg_variant_smem(max_n, variant);
  if (smem > 200 * 1024) {
    set_error("cluster CG: %d unknowns exceed the shared-memory layout of CG variant %d", max_n, variant);
    return ILM_ERR_SIZE_LIMIT;
  }
  switch (variant) {
    case 3: return launch_dist<128, 6, CG_CLUSTER>(prm, order, nprob, counter, max_n, nclusters, smem, st);
    case 4: return launch_dist<256, 2, CG_CLUSTER>(prm, order, nprob, counter, max_n, nclusters, smem, st);
    case 5: return launch_dist<512, 1, CG_CLUSTER>(prm, order, nprob, counter, max_n, nclusters, smem, st);
    default: return launch_dist<256, 3, CG_CLUSTER>(prm, order, nprob, counter, max_n, nclusters, smem, st);
  }
}

// One CTA per problem (no cluster): the small problems of a size-split CG
// launch (batch CG variant 6), run beside the 8-CTA clusters of the large
// ones in the CTA slots those leave free.
int launch_cg_single(const void* params_dev, const int* order, int nprob, int* counter, int max_n, int nctas,
                     cudaStream_t st) {
  const CGFFParams* prm = static_cast<const CGFFParams*>(params_dev);
  ILM_CHECK_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
  const size_t smem = cg_cluster_smem(max_n, 256, 1);
  if (smem > 200 * 1024) {
    set_error("single-CTA CG: %d unknowns exceed its shared-memory layout", max_n);
    return ILM_ERR_SIZE_LIMIT;
  }
  return launch_dist<256, 3, 1>(prm, order, nprob, counter, max_n, nctas, smem, st);
}

// co-resident CTAs of the single-CTA CG kernel on the whole device
int cg_single_slots(int max_n) {
  int dev = 0, nsm = 148, nb = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = cg_cluster_smem(max_n, 256, 1);
  if (smem > 200 * 1024) return 0;
  if (cudaFuncSetAttribute(k_cg_cluster<256, 3, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_cg_cluster<256, 3, 1>, 256, smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return nb * nsm;
}

int cg_cluster_count(int nprob, int max_n, int variant) {
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // co-resident clusters of the kernel launch_cg_cluster will pick (the
  // persistent clusters beyond that would only find the queue empty)
  const bool rep = use_rep(variant, max_n);
  const int nt = rep ? CGR_THREADS : dist_threads(variant);
  const int cs = rep ? CG_CLUSTER : dist_cluster(variant);
  const size_t smem = cg_variant_smem(max_n, variant);
  int nc = 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cs * nsm);
  cfg.blockDim = dim3(nt);
  cfg.dynamicSmemBytes = smem;
  cudaError_t e;
  if (rep) {
    e = cudaFuncSetAttribute(k_cg_rep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(&nc, k_cg_rep, &cfg);
  } else if (smem > 200 * 1024) {
    e = cudaErrorInvalidValue;  // the launch refuses this variant; any count will do
  } else {
    switch (variant) {
      case 3: e = clusters_dist<128, 6, CG_CLUSTER>(&nc, &cfg, smem); break;
      case 4: e = clusters_dist<256, 2, CG_CLUSTER>(&nc, &cfg, smem); break;
      case 5: e = clusters_dist<512, 1, CG_CLUSTER>(&nc, &cfg, smem); break;
      default: e = clusters_dist<256, 3, CG_CLUSTER>(&nc, &cfg, smem); break;
    }
  }
  if (e != cudaSuccess || nc <= 0) {
    (void)cudaGetLastError();
    const int per_sm = variant == 3 ? 6 : variant == 4 ? 2 : variant == 5 ? 1 : 3;
    nc = std::max(1, per_sm * nsm / cs);
  }
  return std::min(nc, nprob);
}

size_t cgff_params_size() { return sizeof(CGFFParams); }

void cgff_params_fill(void* dst, const float* Shi, const float* Slo, const double* b, double* x, const double* w,
                      int n, int maxiter, double tol, int* iters, double* relres, const int* blk,
                      const int* bstart, const int* bsize, const int* boff, const float* binv_hi,
                      const float* binv_lo) {
  CGFFParams p{Shi, Slo, b, x, w, n, maxiter, tol, iters, relres, blk, bstart, bsize, boff, binv_hi, binv_lo};
  *static_cast<CGFFParams*>(dst) = p;
}

void cgff_params_fill_csr(void* dst, const float* vhi, const float* vlo, const int* rowptr, const int* colidx,
                          const double* b, double* x, const double* x0, const double* w, int n, int maxiter,
                          double tol, int* iters, double* relres) {
  CGFFParams p{vhi, vlo, b, x, w, n, maxiter, tol, iters, relres,
               nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, rowptr, colidx, x0};
  *static_cast<CGFFParams*>(dst) = p;
}

void cgff_params_set_deflation(void* dst, const double* sz, const double* inv_e) {
  CGFFParams* p = static_cast<CGFFParams*>(dst);
  p->sz = sz;
  p->inv_e = inv_e;
}

void cgff_params_set_timing(void* dst, unsigned long long* tspan) {
  static_cast<CGFFParams*>(dst)->tspan = tspan;
}

void cgff_params_set_x0(void* dst, const double* x0) { static_cast<CGFFParams*>(dst)->x0 = x0; }

void cgff_params_set_coarse(void* dst, int nb, const int* starts, const double* Einv) {
  CGFFParams* p = static_cast<CGFFParams*>(dst);
  p->cnb = nb;
  for (int b = 0; b <= CG_COARSE_MAX; ++b) p->cstart[b] = b <= nb ? starts[b] : 0;
  p->cEinv = Einv;
}

void cgff_params_set_band(void* dst, const float* band, int band_k, const int* seg_start, const int* seg_len) {
  CGFFParams* p = static_cast<CGFFParams*>(dst);
  p->band = band;
  p->band_k = band_k;
  p->seg_start = seg_start;
  p->seg_len = seg_len;
}

// ---------------------------------------------------------------------------
// block-Jacobi set-up: inverse of each diagonal block of S by Gauss-Jordan
// elimination in place with partial pivoting on S_hi + S_lo (+ a tiny
// shift * mean|diag| I against exact singularity), one CTA per block.  The
// elimination runs in float-float on the FP32 pipes (each update a - f b to
// ~2^-44 relative): GB300 issues FP64 at a small fraction of its FP32 rate.
// In place (no augmented identity: half the work and the shared memory of
// [A | I], so several blocks share an SM), rows at an odd stride (column
// reads free of bank conflicts), the pivot reciprocal an FP32 reciprocal and
// one float-float Newton step (~2^-44), the row swaps undone as a column
// permutation when the inverse is written.  The pivot search is a warp
// argmax (ties to the lower row, deterministic).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_block_inverse(const BJBlockTask* __restrict__ tasks, double shift) {
  const BJBlockTask T = tasks[blockIdx.x];
  const int sz = T.sz;
  const int ld = sz | 1;  // odd row stride
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  extern __shared__ __align__(16) float smf[];  // hi and lo of sz x ld, pivot column, scalars, pivots, columns
  float* Ah = smf;
  float* Al = Ah + (size_t)sz * ld;
  float* fh = Al + (size_t)sz * ld;
  float* fl = fh + sz;
  float* sc = fl + sz;  // [0..1] reciprocal of the pivot (hi, lo), [2] pivot row (int bits), [3] shift
  int* piv = reinterpret_cast<int*>(sc + 4);
  int* src = piv + sz;
  const int ldS = schur_ld(T.n);
  for (int i = warp; i < sz; i += nw)
    for (int j = lane; j < sz; j += 32) {
      const size_t g = (size_t)(T.s + i) * ldS + T.s + j;
      Ah[(size_t)i * ld + j] = T.Shi[g];
      Al[(size_t)i * ld + j] = T.Slo[g];
    }
  __syncthreads();
  if (warp == 0) {
    float m = 0.f;
    for (int i = lane; i < sz; i += 32) m += fabsf(Ah[(size_t)i * ld + i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
    if (lane == 0) sc[3] = (float)(shift * (double)m / (double)sz);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < sz; i += blockDim.x) {
    const FF d = ff_add(FF{Ah[(size_t)i * ld + i], Al[(size_t)i * ld + i]}, FF{sc[3], 0.f});
    const FF r = ff_renorm(d.hi, d.lo);
    Ah[(size_t)i * ld + i] = r.hi;
    Al[(size_t)i * ld + i] = r.lo;
  }
  __syncthreads();
  for (int k = 0; k < sz; ++k) {
    if (warp == 0) {  // argmax |A[i][k]| over i >= k, ties to the lower row
      float best = -1.f;
      int bi = k;
      for (int i = k + lane; i < sz; i += 32) {
        const float v = fabsf(Ah[(size_t)i * ld + k]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (lane == 0) {
        sc[2] = __int_as_float(bi);
        piv[k] = bi;
        const float dh = Ah[(size_t)bi * ld + k], dl = Al[(size_t)bi * ld + k];
        if (dh != 0.f) {  // 1/d: r = 1/d_hi, then r (1 + e), e = 1 - d r
          const float r = 1.0f / dh;
          const float p = dh * r;
          float pe = fmaf(dh, r, -p);
          pe = fmaf(dl, r, pe);
          const float e = (1.0f - p) - pe;
          const FF inv = ff_renorm(r, r * e);
          sc[0] = inv.hi;
          sc[1] = inv.lo;
        } else {
          sc[0] = sc[1] = 0.f;
        }
      }
    }
    __syncthreads();
    const int p = __float_as_int(sc[2]);
    const FF inv{sc[0], sc[1]};
    // swap rows k and p; new row k = (row with A[k][k] set to 1) x 1/pivot
    for (int j = threadIdx.x; j < sz; j += blockDim.x) {
      const FF rk{Ah[(size_t)k * ld + j], Al[(size_t)k * ld + j]};
      const FF rp{Ah[(size_t)p * ld + j], Al[(size_t)p * ld + j]};
      if (p != k) {
        Ah[(size_t)p * ld + j] = rk.hi;
        Al[(size_t)p * ld + j] = rk.lo;
      }
      const FF v = j == k ? inv : ff_mul(p != k ? rp : rk, inv);
      Ah[(size_t)k * ld + j] = v.hi;
      Al[(size_t)k * ld + j] = v.lo;
    }
    __syncthreads();
    // factors f_i = A[i][k] (i != k); column k of those rows becomes 0 - f_i x row k
    for (int i = threadIdx.x; i < sz; i += blockDim.x) {
      fh[i] = i == k ? 0.f : Ah[(size_t)i * ld + k];
      fl[i] = i == k ? 0.f : Al[(size_t)i * ld + k];
      if (i != k) {
        Ah[(size_t)i * ld + k] = 0.f;
        Al[(size_t)i * ld + k] = 0.f;
      }
    }
    __syncthreads();
    for (int i = warp; i < sz; i += nw) {
      if (i == k) continue;
      const FF f{fh[i], fl[i]};
      for (int j = lane; j < sz; j += 32) {
        const FF a{Ah[(size_t)i * ld + j], Al[(size_t)i * ld + j]};
        const FF r = ff_sub_mul(a, f, FF{Ah[(size_t)k * ld + j], Al[(size_t)k * ld + j]});
        Ah[(size_t)i * ld + j] = r.hi;
        Al[(size_t)i * ld + j] = r.lo;
      }
    }
    __syncthreads();
  }
  // the row swaps of the elimination are column swaps of the inverse, undone
  // in reverse order: column c of the inverse is column src[c] of A
  if (threadIdx.x == 0) {
    for (int c = 0; c < sz; ++c) src[c] = c;
    for (int k = sz - 1; k >= 0; --k) {
      const int q = piv[k];
      if (q != k) {
        const int t = src[k];
        src[k] = src[q];
        src[q] = t;
      }
    }
  }
  __syncthreads();
  for (int i = warp; i < sz; i += nw)
    for (int j = lane; j < sz; j += 32) {
      T.out_hi[(size_t)i * sz + j] = Ah[(size_t)i * ld + src[j]];
      T.out_lo[(size_t)i * sz + j] = Al[(size_t)i * ld + src[j]];
    }
}

int launch_block_inverse(const BJBlockTask* tasks_dev, int ntasks, int max_sz, cudaStream_t st) {
  if (ntasks == 0) return ILM_OK;
  const size_t smem = ((size_t)max_sz * (max_sz | 1) * 2 + 2 * max_sz + 4 + 2 * max_sz) * sizeof(float);
  if (smem > 200 * 1024) {
    set_error("block-Jacobi block of %d points too large", max_sz);
    return ILM_ERR_SIZE_LIMIT;
  }
  ILM_CHECK_CUDA(cudaFuncSetAttribute(k_block_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_block_inverse<<<ntasks, 256, smem, st>>>(tasks_dev, 1e-12);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

}  // namespace ilm
