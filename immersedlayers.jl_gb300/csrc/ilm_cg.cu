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
constexpr int CGC_THREADS = 256;
constexpr int CGC_WARPS = CGC_THREADS / 32;

struct FF {
  float hi, lo;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float v = s - a;
  e = (a - (s - v)) + (b - v);
}

// acc += S * (p_hi + p_lo) with S = s_hi + s_lo
__device__ __forceinline__ void ff_fma(FF& acc, float s_hi, float s_lo, float p_hi, float p_lo) {
  const float ph = s_hi * p_hi;
  const float pe = fmaf(s_hi, p_hi, -ph);                 // exact error of the product
  const float t = fmaf(s_hi, p_lo, fmaf(s_lo, p_hi, pe));  // low-order terms
  float s, e;
  two_sum(acc.hi, ph, s, e);
  acc.hi = s;
  acc.lo += e + t;
}

__device__ __forceinline__ FF ff_add(FF a, FF b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  FF r;
  r.hi = s;
  r.lo = e + a.lo + b.lo;
  return r;
}

// y[i - r0] = sum_j S[i][j] v[j] for rows i in [r0, r1); one warp per row,
// lanes stride the columns (coalesced row-major reads) with four independent
// accumulators so that eight loads per lane are in flight.
__device__ void ff_gemv_rows(const float* __restrict__ Shi, const float* __restrict__ Slo, int n, int r0, int r1,
                             const float* __restrict__ vhi, const float* __restrict__ vlo, double* __restrict__ y) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = r0 + warp; i < r1; i += CGC_WARPS) {
    const float* __restrict__ rh = Shi + (size_t)i * n;
    const float* __restrict__ rl = Slo + (size_t)i * n;
    FF a0{0.f, 0.f}, a1{0.f, 0.f}, a2{0.f, 0.f}, a3{0.f, 0.f};
    int j = lane;
    for (; j + 96 < n; j += 128) {
      const float h0 = __ldg(rh + j), h1 = __ldg(rh + j + 32), h2 = __ldg(rh + j + 64), h3 = __ldg(rh + j + 96);
      const float l0 = __ldg(rl + j), l1 = __ldg(rl + j + 32), l2 = __ldg(rl + j + 64), l3 = __ldg(rl + j + 96);
      ff_fma(a0, h0, l0, vhi[j], vlo[j]);
      ff_fma(a1, h1, l1, vhi[j + 32], vlo[j + 32]);
      ff_fma(a2, h2, l2, vhi[j + 64], vlo[j + 64]);
      ff_fma(a3, h3, l3, vhi[j + 96], vlo[j + 96]);
    }
    for (; j < n; j += 32) ff_fma(a0, __ldg(rh + j), __ldg(rl + j), vhi[j], vlo[j]);
    FF acc = ff_add(ff_add(a0, a1), ff_add(a2, a3));
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

// block-wide sums of two doubles in fixed order; result valid in all threads
__device__ void block_sum2(double& a, double& b, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  __syncthreads();
  if (lane == 0) {
    red[wid] = a;
    red[CGC_WARPS + wid] = b;
  }
  __syncthreads();
  double sa = 0.0, sb = 0.0;
  for (int w = 0; w < CGC_WARPS; ++w) {
    sa += red[w];
    sb += red[CGC_WARPS + w];
  }
  a = sa;
  b = sb;
  __syncthreads();
}

// publish two partials of this CTA in slot `slot`, cluster barrier, and sum
// every CTA's partials in rank order (identical result in all CTAs)
// Only warp 0 touches remote shared memory (lane c reads CTA c's partials);
// the fixed shuffle tree makes the sum bit-identical in every CTA.
__device__ void cluster_sum2(cg::cluster_group& cl, double* pub, double* bcast, int slot, double& a, double& b) {
  if (threadIdx.x == 0) {
    pub[2 * slot] = a;
    pub[2 * slot + 1] = b;
  }
  cl.sync();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    double sa = 0.0, sb = 0.0;
    if (lane < CG_CLUSTER) {
      const double* rp = cl.map_shared_rank(pub, lane);
      sa = rp[2 * slot];
      sb = rp[2 * slot + 1];
    }
#pragma unroll
    for (int o = CG_CLUSTER / 2; o > 0; o >>= 1) {
      sa += __shfl_down_sync(0xffffffffu, sa, o);
      sb += __shfl_down_sync(0xffffffffu, sb, o);
    }
    if (lane == 0) {
      bcast[0] = sa;
      bcast[1] = sb;
    }
  }
  __syncthreads();
  a = bcast[0];
  b = bcast[1];
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
  // optional rank-one deflation of the negative (net-charge) mode of the
  // Dirichlet Schur complement: CG runs on S' = S + gamma 1 1^T W (SPD) and
  // x = y + gamma t z, t = 1^T W y / (1 - gamma 1^T W z), z = S'^-1 1
  // (Sherman-Morrison); gamma = 0: off.  zdef == nullptr: no correction
  // (the solve for z itself).
  double gamma;
  const double* zdef;
  double uz;
};

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

__device__ __forceinline__ void matvec_rows(const CGFFParams& pr, int n, int r0, int r1, const float* vhi,
                                            const float* vlo, double* y) {
  if (pr.rowptr) ff_spmv_rows(pr, r0, r1, vhi, vlo, y);
  else ff_gemv_rows(pr.Shi, pr.Slo, n, r0, r1, vhi, vlo, y);
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

// sum_j w_j v_j over the whole problem from the split vector in shared
// memory; every CTA computes the same value (fixed order)
__device__ double full_wdot(const CGFFParams& pr, int n, const float* vhi, const float* vlo, double* red) {
  double a = 0.0, unused = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) a += __ldg(pr.w + j) * ((double)vhi[j] + (double)vlo[j]);
  block_sum2(a, unused, red);
  return a;
}

__device__ double full_wdot_d(const CGFFParams& pr, int n, const double* v, double* red) {
  double a = 0.0, unused = 0.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) a += __ldg(pr.w + j) * v[j];
  block_sum2(a, unused, red);
  return a;
}

__device__ __forceinline__ int seg_nb(int j, int s, int L, int t) {
  if (L < 1) return j;
  int q = (j - s + t) % L;
  q += q < 0 ? L : 0;
  return s + q;
}

// z[i - r0] = (W^-1 C^T C r)_i for rows i in [r0, r1), in float-float
// arithmetic (an FP32 application changes M from one iteration to the next
// by rounding and stalls flexible CG near 1e-7 on these indefinite Schur
// complements).  Each row needs u_j = (C r)_j at its 2K+1 band neighbours
// j; they are formed on the fly (same body, circular), two threads per row.
__device__ void apply_band(const CGFFParams& pr, int r0, int r1, const float* __restrict__ rhi,
                           const float* __restrict__ rlo, const double* __restrict__ ws, double* __restrict__ z) {
  const int K = pr.band_k, P = 2 * K + 1;
  const int half = threadIdx.x & 1;
  const int nrow = r1 - r0;
  for (int base = 0; base < nrow; base += blockDim.x / 2) {
    const int row = base + (threadIdx.x >> 1);
    FF zacc{0.f, 0.f};
    if (row < nrow) {
      const int i = r0 + row;
      const int s = __ldg(pr.seg_start + i), L = __ldg(pr.seg_len + i);
      // thread `half` takes t = -K + half, -K + half + 2, ...
      for (int t = -K + half; t <= K; t += 2) {
        const int j = seg_nb(i, s, L, -t);
        const float* __restrict__ cj = pr.band + (size_t)j * P;
        FF u{0.f, 0.f};
        for (int t2 = -K; t2 <= K; ++t2) {
          const int q = seg_nb(j, s, L, t2);
          ff_fma(u, __ldg(cj + t2 + K), 0.f, rhi[q], rlo[q]);
        }
        ff_fma(zacc, __ldg(cj + t + K), 0.f, u.hi, u.lo);
      }
    }
    FF other;
    other.hi = __shfl_xor_sync(0xffffffffu, zacc.hi, 1);
    other.lo = __shfl_xor_sync(0xffffffffu, zacc.lo, 1);
    zacc = ff_add(zacc, other);
    if (row < nrow && half == 0) z[row] = ((double)zacc.hi + (double)zacc.lo) / ws[row];
  }
}

__device__ __forceinline__ void apply_precond(const CGFFParams& pr, int r0, int r1, const float* rhi,
                                              const float* rlo, const double* ws, double* z) {
  if (pr.band) apply_band(pr, r0, r1, rhi, rlo, ws, z);
  else apply_bjacobi(pr, r0, r1, rhi, rlo, z);
}

// Persistent: each cluster takes problems from a work queue (largest first,
// `order`) until the queue is empty.  `counter` must be 0 at launch.
__global__ void __cluster_dims__(CG_CLUSTER, 1, 1) __launch_bounds__(CGC_THREADS, 4)
    k_cg_cluster(const CGFFParams* __restrict__ P, const int* __restrict__ order, int nprob, int* counter,
                 int max_n) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int rmax = (max_n + CG_CLUSTER - 1) / CG_CLUSTER;
  extern __shared__ __align__(16) unsigned char smraw[];
  double* pub = reinterpret_cast<double*>(smraw);   // 16 doubles: published partials (8 slots x 2)
  double* red = pub + 16;                           // 2 * warps
  double* work = red + 2 * CGC_WARPS;               // [0] queue index taken by rank 0, [2..3] broadcast
  double* xs = work + 4;                            // slices (rmax each)
  double* rs = xs + rmax;
  double* qs = rs + rmax;
  double* ws = qs + rmax;
  double* bs = ws + rmax;
  double* ts = bs + rmax;                           // S x of the residual refresh (q stays S p)
  double* xb = ts + rmax;                           // best iterate so far (true residual)
  double* pf = xb + rmax;                           // full direction (max_n)
  double* zs = pf + max_n;                          // preconditioned residual slice (rmax)
  float* vhi = reinterpret_cast<float*>(zs + max_n); // split vector (max_n each)
  float* vlo = vhi + max_n;
  int slot = 1;
  while (true) {
    if (rank == 0 && threadIdx.x == 0) work[0] = (double)atomicAdd(counter, 1);
    cl.sync();
    const int q = (int)cl.map_shared_rank(work, 0)[0];
    if (q >= nprob) break;
    const CGFFParams& pr = P[order[q]];  // fields read through L1 as needed (a copy spills)
    const int n = pr.n;
    const int rows = (n + CG_CLUSTER - 1) / CG_CLUSTER;
    const int r0 = min(n, rank * rows), r1 = min(n, r0 + rows);
    const int nr = r1 - r0;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      xs[i] = pr.x0 ? pr.x0[r0 + i] : 0.0;
      bs[i] = pr.b[r0 + i];
      ws[i] = pr.w ? pr.w[r0 + i] : 1.0;
    }
    if (pr.x0) {  // warm start: r = b - S x0
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double v = pr.x0[j];
        const float h = (float)v;
        vhi[j] = h;
        vlo[j] = (float)(v - (double)h);
      }
      __syncthreads();
      matvec_rows(pr, n, r0, r1, vhi, vlo, qs);
      const double c0 = pr.gamma != 0.0 ? pr.gamma * full_wdot(pr, n, vhi, vlo, red) : 0.0;
      __syncthreads();
      for (int i = threadIdx.x; i < nr; i += blockDim.x) rs[i] = bs[i] - qs[i] - c0;
    } else {
      for (int i = threadIdx.x; i < nr; i += blockDim.x) rs[i] = bs[i];
    }
    __syncthreads();
    const bool pre = pr.blk != nullptr || pr.band != nullptr;
    double bb = 0.0, rz = 0.0;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      bb += bs[i] * bs[i];
      rz += ws[i] * rs[i] * rs[i];
    }
    block_sum2(bb, rz, red);
    cluster_sum2(cl, pub, work + 2, slot, bb, rz);
    slot = slot == 7 ? 1 : slot + 1;
    // p = r (gathered from every CTA's final slice)
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      const int c = j / rows;
      const double v = cl.map_shared_rank(rs, c)[j - c * rows];
      pf[j] = v;
      const float h = (float)v;
      vhi[j] = h;
      vlo[j] = (float)(v - (double)h);
    }
    __syncthreads();
    if (pre) {
      apply_precond(pr, r0, r1, vhi, vlo, ws, zs);
      __syncthreads();
      cl.sync();
    }
    if (pre) {  // p = z = M r, gathered from every CTA's (final) z slice
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const int c = j / rows;
        pf[j] = cl.map_shared_rank(zs, c)[j - c * rows];
      }
      __syncthreads();
    }
    const double bnorm = sqrt(bb);
    const double thr = pr.tol * bnorm;
    int it = 0;
    double relres = bnorm > 0 ? 1.0 : 0.0;
    bool done = bnorm == 0.0;
    // stagnation guard: past the attainable accuracy (float-float products on
    // a Schur complement of condition ~1e6 floor near 1e-10) CG drifts and
    // eventually diverges; stop after 8 refreshes without a better true
    // residual and return the best iterate
    double best = 1e300;
    int stall = 0;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) xb[i] = xs[i];
    while (!done && it < pr.maxiter) {
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double v = pf[j];
        const float h = (float)v;
        vhi[j] = h;
        vlo[j] = (float)(v - (double)h);
      }
      __syncthreads();
      matvec_rows(pr, n, r0, r1, vhi, vlo, qs);
      if (pr.gamma != 0.0) {  // q = S' p
        const double cp = pr.gamma * full_wdot_d(pr, n, pf, red);
        for (int i = threadIdx.x; i < nr; i += blockDim.x) qs[i] += cp;
      }
      __syncthreads();
      double pq = 0.0, pr_ = 0.0;
      for (int i = threadIdx.x; i < nr; i += blockDim.x) {
        pq += ws[i] * pf[r0 + i] * qs[i];
        pr_ += ws[i] * pf[r0 + i] * rs[i];
      }
      block_sum2(pq, pr_, red);
      cluster_sum2(cl, pub, work + 2, slot, pq, pr_);
      slot = slot == 7 ? 1 : slot + 1;
      if (pq == 0.0) break;
      const double alpha = pre ? pr_ / pq : rz / pq;
      double rr = 0.0, rzn = 0.0;
      for (int i = threadIdx.x; i < nr; i += blockDim.x) {
        xs[i] += alpha * pf[r0 + i];
        rs[i] -= alpha * qs[i];
        rr += rs[i] * rs[i];
        rzn += ws[i] * rs[i] * rs[i];
      }
      block_sum2(rr, rzn, red);
      cluster_sum2(cl, pub, work + 2, slot,rr, rzn);
      slot = slot == 7 ? 1 : slot + 1;
      ++it;
      relres = bnorm > 0 ? sqrt(rr) / bnorm : 0.0;
      if (sqrt(rr) <= thr || (it % 50) == 0 || it == pr.maxiter) {
        // true residual b - S x from every CTA's (final) x slice
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
          const int c = j / rows;
          const double v = cl.map_shared_rank(xs, c)[j - c * rows];
          const float h = (float)v;
          vhi[j] = h;
          vlo[j] = (float)(v - (double)h);
        }
        __syncthreads();
        matvec_rows(pr, n, r0, r1, vhi, vlo, ts);
        const double cx = pr.gamma != 0.0 ? pr.gamma * full_wdot(pr, n, vhi, vlo, red) : 0.0;
        __syncthreads();
        double tr = 0.0, tz = 0.0;
        for (int i = threadIdx.x; i < nr; i += blockDim.x) {
          rs[i] = bs[i] - ts[i] - cx;
          tr += rs[i] * rs[i];
          tz += ws[i] * rs[i] * rs[i];
        }
        block_sum2(tr, tz, red);
        cluster_sum2(cl, pub, work + 2, slot,tr, tz);
        slot = slot == 7 ? 1 : slot + 1;
        relres = bnorm > 0 ? sqrt(tr) / bnorm : 0.0;
        rzn = tz;
        if (sqrt(tr) <= thr) {
          done = true;
          break;
        }
        if (relres < best) {
          best = relres;
          stall = 0;
          for (int i = threadIdx.x; i < nr; i += blockDim.x) xb[i] = xs[i];
        } else if (++stall >= 8) {
          break;
        }
      }
      if (!pre) {
        const double beta = rzn / rz;
        rz = rzn;
        // p = r + beta p over the full vector, r gathered from every CTA's
        // (final) slice: identical in all CTAs, no extra barrier
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
          const int c = j / rows;
          pf[j] = cl.map_shared_rank(rs, c)[j - c * rows] + beta * pf[j];
        }
        __syncthreads();
      } else {
        // flexible CG: z = M r on this CTA's rows (r gathered from every
        // CTA's final slice), beta = -(z, q) / (p, q), p = z + beta p
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
          const int c = j / rows;
          const double v = cl.map_shared_rank(rs, c)[j - c * rows];
          const float h = (float)v;
          vhi[j] = h;
          vlo[j] = (float)(v - (double)h);
        }
        __syncthreads();
        apply_precond(pr, r0, r1, vhi, vlo, ws, zs);
        __syncthreads();
        double zq = 0.0, d1 = 0.0;
        for (int i = threadIdx.x; i < nr; i += blockDim.x) zq += ws[i] * zs[i] * qs[i];
        block_sum2(zq, d1, red);
        cluster_sum2(cl, pub, work + 2, slot, zq, d1);
        slot = slot == 7 ? 1 : slot + 1;
        const double beta = -zq / pq;
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
          const int c = j / rows;
          pf[j] = cl.map_shared_rank(zs, c)[j - c * rows] + beta * pf[j];
        }
        __syncthreads();
      }
    }
    if (best < relres) {  // stopped past the best iterate: return that one
      for (int i = threadIdx.x; i < nr; i += blockDim.x) xs[i] = xb[i];
      relres = best;
      __syncthreads();
    }
    if (pr.zdef != nullptr && pr.gamma != 0.0) {
      // Sherman-Morrison back to S: x = y + gamma t z, t = 1^T W y / (1 - gamma 1^T W z)
      double wy = 0.0, unused = 0.0;
      for (int i = threadIdx.x; i < nr; i += blockDim.x) wy += ws[i] * xs[i];
      block_sum2(wy, unused, red);
      cluster_sum2(cl, pub, work + 2, slot, wy, unused);
      slot = slot == 7 ? 1 : slot + 1;
      const double t = wy / (1.0 - pr.gamma * pr.uz);
      for (int i = threadIdx.x; i < nr; i += blockDim.x) xs[i] += pr.gamma * t * pr.zdef[r0 + i];
      __syncthreads();
      cl.sync();
      // reported residual: the true one of S x = b (the deflated operator's
      // residual equals it up to the accuracy of z)
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const int c = j / rows;
        const double v = cl.map_shared_rank(xs, c)[j - c * rows];
        const float h = (float)v;
        vhi[j] = h;
        vlo[j] = (float)(v - (double)h);
      }
      __syncthreads();
      matvec_rows(pr, n, r0, r1, vhi, vlo, ts);
      __syncthreads();
      double tr = 0.0;
      for (int i = threadIdx.x; i < nr; i += blockDim.x) {
        const double d = bs[i] - ts[i];
        tr += d * d;
      }
      block_sum2(tr, unused, red);
      cluster_sum2(cl, pub, work + 2, slot, tr, unused);
      slot = slot == 7 ? 1 : slot + 1;
      relres = bnorm > 0 ? sqrt(tr) / bnorm : 0.0;
    }
    for (int i = threadIdx.x; i < nr; i += blockDim.x) pr.x[r0 + i] = xs[i];
    if (rank == 0 && threadIdx.x == 0) {
      if (pr.iters) *pr.iters = it;
      if (pr.relres) *pr.relres = relres;
    }
    cl.sync();  // every CTA done with this problem's shared data
  }
  cl.sync();  // keep shared memory alive until every CTA is done reading it
}

size_t cg_cluster_smem(int max_n) {
  const int rmax = (max_n + CG_CLUSTER - 1) / CG_CLUSTER;
  return (16 + 2 * CGC_WARPS + 4 + 7 * (size_t)rmax + 2 * (size_t)max_n) * sizeof(double) +
         2 * (size_t)max_n * sizeof(float) + 64;
}

int launch_cg_cluster(const void* params_dev, const int* order, int nprob, int* counter, int max_n, int nclusters,
                      cudaStream_t st) {
  const size_t smem = cg_cluster_smem(max_n);
  if (smem > 200 * 1024) {
    set_error("cluster CG: %d unknowns exceed the shared-memory layout", max_n);
    return ILM_ERR_SIZE_LIMIT;
  }
  ILM_CHECK_CUDA(cudaFuncSetAttribute(k_cg_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  ILM_CHECK_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
  k_cg_cluster<<<nclusters * CG_CLUSTER, CGC_THREADS, smem, st>>>(static_cast<const CGFFParams*>(params_dev), order,
                                                                  nprob, counter, max_n);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int cg_cluster_count(int nprob, int max_n) {
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // four 256-thread CTAs per SM: about 4 nsm / 8 resident clusters
  int nc = std::max(1, 4 * nsm / CG_CLUSTER);
  (void)max_n;
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

void cgff_params_set_deflation(void* dst, double gamma, const double* zdef, double uz) {
  CGFFParams* p = static_cast<CGFFParams*>(dst);
  p->gamma = gamma;
  p->zdef = zdef;
  p->uz = uz;
}

void cgff_params_set_band(void* dst, const float* band, int band_k, const int* seg_start, const int* seg_len) {
  CGFFParams* p = static_cast<CGFFParams*>(dst);
  p->band = band;
  p->band_k = band_k;
  p->seg_start = seg_start;
  p->seg_len = seg_len;
}

// ---------------------------------------------------------------------------
// block-Jacobi set-up: inverse of each diagonal block of S, FP64 Gauss-Jordan
// with partial pivoting on S_hi + S_lo (+ a tiny shift * mean|diag| I against
// exact singularity), stored as float-float pairs; one CTA per block
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_block_inverse(const BJBlockTask* __restrict__ tasks, double shift) {
  const BJBlockTask T = tasks[blockIdx.x];
  const int sz = T.sz;
  const int ld = 2 * sz;
  extern __shared__ __align__(16) double Ad[];  // sz x 2sz, then fcol[sz], scal[2]
  double* fcol = Ad + (size_t)sz * ld;
  double* scal = fcol + sz;
  for (int idx = threadIdx.x; idx < sz * ld; idx += blockDim.x) {
    const int i = idx / ld, j = idx - i * ld;
    const size_t g = (size_t)(T.s + i) * T.n + T.s + j;
    Ad[idx] = j < sz ? (double)T.Shi[g] + (double)T.Slo[g] : (j - sz == i ? 1.0 : 0.0);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int i = 0; i < sz; ++i) m += fabs(Ad[(size_t)i * ld + i]);
    scal[0] = shift * m / (double)sz;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < sz; i += blockDim.x) Ad[(size_t)i * ld + i] += scal[0];
  __syncthreads();
  for (int k = 0; k < sz; ++k) {
    if (threadIdx.x == 0) {
      int p = k;
      double best = fabs(Ad[(size_t)k * ld + k]);
      for (int i = k + 1; i < sz; ++i) {
        const double v = fabs(Ad[(size_t)i * ld + k]);
        if (v > best) {
          best = v;
          p = i;
        }
      }
      scal[1] = (double)p;
    }
    __syncthreads();
    const int p = (int)scal[1];
    if (p != k)
      for (int j = threadIdx.x; j < ld; j += blockDim.x) {
        const double t = Ad[(size_t)k * ld + j];
        Ad[(size_t)k * ld + j] = Ad[(size_t)p * ld + j];
        Ad[(size_t)p * ld + j] = t;
      }
    __syncthreads();
    const double piv = Ad[(size_t)k * ld + k];
    const double inv = piv != 0.0 ? 1.0 / piv : 0.0;
    __syncthreads();
    for (int j = threadIdx.x; j < ld; j += blockDim.x) Ad[(size_t)k * ld + j] *= inv;
    for (int i = threadIdx.x; i < sz; i += blockDim.x) fcol[i] = Ad[(size_t)i * ld + k];
    __syncthreads();
    for (int idx = threadIdx.x; idx < sz * ld; idx += blockDim.x) {
      const int i = idx / ld, j = idx - i * ld;
      if (i != k) Ad[idx] -= fcol[i] * Ad[(size_t)k * ld + j];
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < sz * sz; idx += blockDim.x) {
    const int i = idx / sz, j = idx - i * sz;
    const double v = Ad[(size_t)i * ld + sz + j];
    const float h = (float)v;
    T.out_hi[idx] = h;
    T.out_lo[idx] = (float)(v - (double)h);
  }
}

int launch_block_inverse(const BJBlockTask* tasks_dev, int ntasks, int max_sz, cudaStream_t st) {
  if (ntasks == 0) return ILM_OK;
  const size_t smem = ((size_t)max_sz * 2 * max_sz + max_sz + 2) * sizeof(double);
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
