// Batched Poisson solves: hundreds of independent Dirichlet / Neumann problems
// of different grid sizes and geometries advanced together in a fixed
// sequence of launches (one launch per stage for the whole batch).
//
// Per problem this is the reference's block-LU solve (Dirichlet:
// test/literate/problems.jl:259-298; Neumann: test/literate/neumann.jl:101-127)
// with its dense LU `S \ s` replaced by device CG on the LGF-assembled Schur
// complement.  All per-problem descriptors ("tasks") are built on the host
// once, at batch creation, and live in device memory, so a solve issues no
// host<->device traffic and can be captured in a CUDA graph.
#include <array>
#include <climits>
#include <string.h>

#include <math.h>

#include <algorithm>
#include <chrono>
#include <memory>
#include <mutex>
#include <new>

#include "ilm_internal.cuh"

namespace ilm {

// One DDF scatter of a problem: the tiles of the box [tx0, tx0 + ntxb) x
// [ty0, ...) of its tile grid (ntx tiles per row); cells of other tiles are
// not written
struct BScatterTask {
  int n1, n2, ntx, tile0;
  int tx0, ty0, ntxb, pad_;
  int xa, xb, ya, yb, fill0, nne;  // box cells [xa, xb) x [ya, yb), first zero-fill block, occupied tiles
  const int* ne;                    // the box's tiles that hold candidate points (tile ids of the problem)
  const int* tptr;
  const int* tpts;
  const int* bx;
  const int* by;
  const void* wx;
  const void* wy;
  const void* wsc;
  const void* nx;
  const void* ny;
  const void* in;
  int coef;
  int accum;  // 1: add the sums to the output (no zero fill of its box)
  void* out;
};

// a stencil over the box [i0, i0 + bw) x [j0, j0 + bh) of its output array
struct BStencilTask {
  int NX, NY, blk0;
  int i0, j0, bw, bh;
  const void* in;
  void* out;
  double scale;
  int accum = 0;  // 1: add to the output
};

struct BGatherTask {
  int npts, pt0, nterms, pad;
  const int* bx[2];
  const int* by[2];
  const void* wx[2];
  const void* wy[2];
  const void* nx;
  const void* ny;
  const void* arr[2];
  int n1[2], n2[2], xs[2], ys[2], coef[2];
  // 0: arr is the sampled field (n1 x n2); 1: the field is the x-difference
  // of the cell array arr ((n1 - 1) x n2, u faces, zero on the ghost
  // columns); 2: the y-difference (n1 x (n2 - 1), v faces, zero on the ghost
  // rows) -- the Nodes -> Edges gradient fused into the gather
  int gmode[2];
  void* out;
  double scale;
};

constexpr int SB_X = 32, SB_Y = 8;

template <typename Task>
__device__ __forceinline__ int find_task(const Task* t, int n, int u, int Task::*field) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (t[mid].*field <= u) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <typename T>
__device__ __forceinline__ T bcoef(int code, const T* nx, const T* ny, int k) {
  switch (code) {
    case CF_ONE: return (T)1;
    case CF_NX: return nx[k];
    case CF_NY: return ny[k];
    case CF_MNX: return -nx[k];
    case CF_MNY: return -ny[k];
    case CF_MONE: return (T)-1;
  }
  return (T)0;
}

// Zero fill of every task's box, one block per box row (the scatter below
// then visits only the tiles that hold points)
// one warp per box row (box rows are tens to a few hundred cells wide)
template <typename T>
__global__ void __launch_bounds__(256)
    k_bfill(const BScatterTask* __restrict__ tasks, int nrows, const int* __restrict__ bmap) {
  const int r = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (r >= nrows) return;
  const BScatterTask& S = tasks[bmap[r]];
  const int j = S.ya + r - S.fill0;
  T* row = static_cast<T*>(S.out) + (size_t)j * S.n1;
  for (int i = S.xa + (threadIdx.x & 31); i < S.xb; i += 32) row[i] = (T)0;
}

// Deterministic scatter: one thread per output cell of an occupied 32 x 8
// tile; the tile's candidate points (index order) are staged in shared
// memory 256 at a time, one point per thread, and every cell sums the points
// of its window buckets (tile_sum_bucketed) in a fixed order.
template <typename T>
__global__ void __launch_bounds__(SB_X* SB_Y, 6)
    k_bscatter(const BScatterTask* __restrict__ tasks, int ntasks, const int* __restrict__ bmap) {
  static_assert(SB_X == TILE_X && SB_Y == TILE_Y, "batched scatter tiles are the cache tiles");
  __shared__ ScatterSmem<T> sm;
  const int ti = bmap[blockIdx.x];
  const BScatterTask& S = tasks[ti];
  const int tile = S.ne[blockIdx.x - S.tile0];
  const int x0 = (tile % S.ntx) * SB_X, y0 = (tile / S.ntx) * SB_Y;
  const int i = x0 + threadIdx.x;
  const int j = y0 + threadIdx.y;
  const int tid = threadIdx.y * SB_X + threadIdx.x;
  const int p0 = S.tptr[tile], p1 = S.tptr[tile + 1];
  const T* __restrict__ wx = static_cast<const T*>(S.wx);
  const T* __restrict__ wy = static_cast<const T*>(S.wy);
  const T* __restrict__ wsc = static_cast<const T*>(S.wsc);
  const T* __restrict__ in = static_cast<const T*>(S.in);
  const T* nx = static_cast<const T*>(S.nx);
  const T* ny = static_cast<const T*>(S.ny);
  T acc = (T)0;
  for (int c0 = p0; c0 < p1; c0 += SCAT_NB) {
    const int nc = min(SCAT_NB, p1 - c0);
    if (tid < nc) {
      const int k = S.tpts[c0 + tid];
      sm.bx[tid] = S.bx[k];
      sm.by[tid] = S.by[k];
      sm.amp[tid] = wsc[k] * (bcoef<T>(S.coef, nx, ny, k) * in[k]);
#pragma unroll
      for (int q = 0; q < NTAP; ++q) {
        sm.wx[tid * NTAP + q] = wx[k * NTAP + q];
        sm.wy[tid * NTAP + q] = wy[k * NTAP + q];
      }
    }
    acc += tile_sum_bucketed<T>(sm, nc, x0, i, j);
    __syncthreads();
  }
  if (i < S.n1 && j < S.n2) {
    T* o = static_cast<T*>(S.out) + (size_t)j * S.n1 + i;
    *o = S.accum ? *o + acc : acc;
  }
}

// Edges{Primal} -> Nodes{Primal} divergence
template <typename T>
__global__ void k_bdiv(const BStencilTask* __restrict__ tasks, int ntasks, const int* __restrict__ bmap) {
  const int ti = bmap[blockIdx.x];
  const BStencilTask& S = tasks[ti];
  const int NX = S.NX, NY = S.NY;
  const int nbx = (S.bw + SB_X - 1) / SB_X;
  const int b = blockIdx.x - S.blk0;
  const int i = S.i0 + (b % nbx) * SB_X + threadIdx.x, j = S.j0 + (b / nbx) * SB_Y + threadIdx.y;
  if (i >= S.i0 + S.bw || j >= S.j0 + S.bh) return;
  const T* u = static_cast<const T*>(S.in);
  const T* v = u + (size_t)NX * (NY - 1);
  const T du = u[(size_t)j * NX + i + 1] - u[(size_t)j * NX + i];
  const T dv = v[(size_t)(j + 1) * (NX - 1) + i] - v[(size_t)j * (NX - 1) + i];
  T* o = static_cast<T*>(S.out) + (size_t)j * (NX - 1) + i;
  *o = S.accum ? *o + (du + dv) * (T)S.scale : (du + dv) * (T)S.scale;
}

// Schur right-hand side from the precomputed operator M (one warp per point):
// rhs = M [jump] - avg, the same quantity as the gather of f* minus avg
template <typename T>
__global__ void k_rhsop_matvec(int Ptot, const int* __restrict__ pt2prob, const SchurProbDev* __restrict__ pr,
                               const float* __restrict__ Mhi, const float* __restrict__ Mlo,
                               const T* __restrict__ jump, const T* __restrict__ avg, double* __restrict__ out) {
  const int r = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (r >= Ptot) return;
  const SchurProbDev P = pr[pt2prob[r]];
  const int k = r - P.poff, n = P.n;
  const float* __restrict__ mh = Mhi + P.soff + (size_t)k * schur_ld(n);
  const float* __restrict__ ml = Mlo + P.soff + (size_t)k * schur_ld(n);
  const T* __restrict__ jp = jump + P.poff;
  FF a{0.f, 0.f};
  for (int l = lane; l < n; l += 32) {
    const double v = (double)jp[l];
    const float vh = (float)v;
    ff_fma(a, __ldg(mh + l), __ldg(ml + l), vh, (float)(v - (double)vh));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    FF b;
    b.hi = __shfl_down_sync(0xffffffffu, a.hi, o);
    b.lo = __shfl_down_sync(0xffffffffu, a.lo, o);
    a = ff_add(a, b);
  }
  if (lane == 0) out[r] = ((double)a.hi + (double)a.lo) - (double)avg[r];
}

template <typename T>
__global__ void k_bgather(const BGatherTask* __restrict__ tasks, int ntasks, int Ptot) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= Ptot) return;
  const int ti = find_task(tasks, ntasks, g, &BGatherTask::pt0);
  const BGatherTask& G = tasks[ti];
  const int k = g - G.pt0;
  if (k >= G.npts) return;
  T total = (T)0;
  for (int q = 0; q < G.nterms; ++q) {
    const int xs = G.xs[q], ys = G.ys[q];
    const int b0 = G.bx[xs][k], e0 = G.by[ys][k];
    const T* wx = static_cast<const T*>(G.wx[xs]) + k * NTAP;
    const T* wy = static_cast<const T*>(G.wy[ys]) + k * NTAP;
    const T* a = static_cast<const T*>(G.arr[q]);
    const int n1 = G.n1[q], n2 = G.n2[q], gm = G.gmode[q];
    T acc = (T)0;
#pragma unroll
    for (int jj = 0; jj < NTAP; ++jj) {
      const int j = e0 + jj;
      if ((unsigned)j >= (unsigned)n2) continue;
      T racc = (T)0;
#pragma unroll
      for (int ii = 0; ii < NTAP; ++ii) {
        const int i = b0 + ii;
        if ((unsigned)i >= (unsigned)n1) continue;
        T v;
        if (gm == 0) {
          v = a[(size_t)j * n1 + i];
        } else if (gm == 1) {
          v = (i >= 1 && i <= n1 - 2) ? a[(size_t)j * (n1 - 1) + i] - a[(size_t)j * (n1 - 1) + i - 1] : (T)0;
        } else {
          v = (j >= 1 && j <= n2 - 2) ? a[(size_t)j * n1 + i] - a[(size_t)(j - 1) * n1 + i] : (T)0;
        }
        racc += wx[ii] * v;
      }
      acc += wy[jj] * racc;
    }
    total += bcoef<T>(G.coef[q], static_cast<const T*>(G.nx), static_cast<const T*>(G.ny), k) * acc;
  }
  static_cast<T*>(G.out)[k] = total * (T)G.scale;
}

// dst[k][0..P) = src[k][0..P) for the selected points k
__global__ void k_select_rows(int N, int P, const unsigned char* __restrict__ sel, const float* __restrict__ src,
                              float* __restrict__ dst) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N * P; e += gridDim.x * blockDim.x)
    if (sel[e / P]) dst[e] = src[e];
}

// rhs64 = (double)g - (double)avg
template <typename T>
__global__ void k_rhs64(int n, const T* __restrict__ g, const T* __restrict__ avg, double* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = (double)g[i] - (double)avg[i];
}

template <typename T>
__global__ void k_jump_avg(int n, const T* __restrict__ p, const T* __restrict__ m, T* __restrict__ jump,
                           T* __restrict__ avg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    jump[i] = p[i] - m[i];
    avg[i] = (T)0.5 * (p[i] + m[i]);
  }
}

}  // namespace ilm

using namespace ilm;

struct ilm_batch_s {
  int nprob = 0, dtype = ILM_F64, ddf = ILM_DDF_YANG3, Ptot = 0, maxN = 0, max_grid = 0;
  std::vector<ilm_batch_problem_t> probs;
  std::vector<size_t> foff, poff, soff;   // nprob + 1 offsets (fields, points, Schur)
  size_t ftot = 0, etot = 0, stot = 0;
  // packed point data
  DevBuf bx[2], by[2], wx[2], wy[2], wx64[2], wy64[2];
  DevBuf nx, ny, wsc, nx64, ny64, ds64, pt2prob;
  DevBuf tptr[4], tpts[4];
  // work
  DevBuf fstar, corr, edges, convwork, Shi, Slo, F;
  DevBuf jump, avg, g, s, rhs64, x64;
  DevBuf cgp, iters, relres, order, counter;
  int nclusters = 1;
  int cg_variant = 0;  // Schur CG kernel (0 default = the size split of 6, 1..ILM_CG_VARIANTS)
  // tasks
  DevBuf scatA, divA, gathA, scatB, divB, convA, convB, schurP;
  int n_scatA = 0, n_divA = 0, n_gathA = 0, n_scatB = 0, n_divB = 0;
  int blk_scatA = 0, blk_divA = 0, blk_scatB = 0, blk_divB = 0, blk_fillA = 0, blk_fillB = 0;
  DevBuf scat_ne;  // occupied tiles of the scatter tasks
  // task of every block of the batched launches (no per-block search)
  DevBuf mfillA, mscatA, mdivA, mfillB, mscatB, mdivB, mconv[3];
  // precomputed right-hand-side operator (ilm_batch_set_rhs_operator): M per
  // problem (float-float, the layout of S), the functionals it is built from,
  // and the stage-B tasks that add the correction source to f*'s source so
  // that one convolution gives the field
  bool rhs_op = false, rhs_op_ready = false;
  DevBuf Mhi, Mlo, FU, FD, schurPfull, scatB2, divB2, convC, mfillB2;
  int blk_fillB2 = 0, rhs_tiles = 0;
  std::vector<SchurProbDev> schur_host;
  int n_conv = 0;
  size_t box_cells = 0;  // cells of all source boxes
  ConvLaunch convL;
  int schur_tiles = 0;
  double cg_tol = -1.0;
  int cg_maxiter = -1;
  // optional stage timing (CUDA events on the solve stream)
  // preconditioner of the Schur CG: 0 none, 1 block-Jacobi
  int precond = 0, bj_block = 0;
  bool params_dirty = false;
  DevBuf bj_blk, bj_start, bj_size, bj_off, bj_inv, bj_inv_lo, bj_tasks;
  std::vector<BJBlockTask> bj_tasks_host;  // every block's inversion task
  std::vector<char> bj_have;               // problems whose block inverses are formed
  int bj_max_sz = 1;
  std::vector<int> bj_first;  // first block of each problem
  // learned banded preconditioner (mode 2): coefficients per packed point,
  // body segments as local indices
  int band_k = -1;
  DevBuf band, lseg_start, lseg_len;
  DevBuf arena_learned;      // body segments of the learned preconditioner
  DevBuf arena_learned_tmp;  // its set-up's scratch (features, band before the scatter), kept for reuse
  std::vector<char> has_band;  // problems whose kind a network was set for
  // coarse correction of block-Jacobi on the bodies' constants
  // (ilm_batch_set_coarse): per problem the bodies (0: off), their
  // CG_COARSE_MAX + 1 local starts and E^-1 (CG_COARSE_MAX^2, row-major)
  std::vector<int> coarse_nb, coarse_start;  // E^-1 in coarse_Einv (device)
  // deflation of the Dirichlet net-charge mode, formed on the device right
  // after the Schur build (k_defl_rows, k_defl_e): S 1 for every point of a
  // Dirichlet problem, and per problem 1 / (1^T W S 1) when that is
  // negative (0: the deflation is a no-op)
  DevBuf defl_sz, defl_ie;
  // host copies of the points (features of the learned preconditioner)
  std::vector<double> hx, hy, hnx, hny, hds;
  DevBuf dpoff;  // point offsets on the device (Schur products)
  int profiling = 0;
  DevBuf cgtime;  // per problem: CG start / end (global timer ns), SM (profiling)
  cudaEvent_t ev[32] = {};
  int nev = 0, launches = 0;
  // captured solve (ilm_batch_solve_graph): the launch sequence of one
  // solve for one set of buffers, tolerance and CG parameter generation
  cudaGraphExec_t gexec = nullptr;
  const void* gkey[4] = {};
  double gtol = -1.0;
  int gmaxiter = -1, ggen = -1;
  int param_gen = 0;  // bumped whenever the device CG parameters or the CG launch change
  // FP64 iterative refinement (ilm_batch_solve_refined): an FP64 copy of the
  // pipeline (same problems and points, no Schur matrices of its own) for the
  // accurate Schur right-hand side and the field assembly, and FP64 vectors
  // CG variant 6 (size split): problems above kSplitN points on the 8-CTA
  // clusters, the others one CTA each on a second stream, joined by events
  bool split_ready = false;
  int n_large = 0, n_small = 0, max_small = 0, nctas_small = 0;
  DevBuf order_large, order_small, counter2;
  cudaStream_t s2 = nullptr;
  // lazy set-up of the first solve (block-Jacobi inverses, deflation
  // vectors): its own non-blocking stream, so that it overlaps the solve's
  // stage A, and its scratch allocated before stage A is issued (cudaMalloc
  // and cudaFree may synchronise the device)
  cudaStream_t s_setup = nullptr;
  DevBuf lz_bjtasks;
  // block-Jacobi inverses: formed on their own stream beside the first
  // solve's stage A and deflation set-up; the CG launches that read them
  // wait for bj_ready (wait_precond)
  cudaStream_t s_bj = nullptr;
  cudaEvent_t bj_ready = nullptr;
  // asynchronous preconditioner set-up: the learned band on its own stream
  // (band_ready; the network's timeout flag is copied to band_err there and
  // checked on the host before the first solve that reads the band) and the
  // coarse correction's E^-1 on the set-up stream (coarse_ready); the CG
  // launches wait for both (wait_precond)
  cudaStream_t s_learn = nullptr;
  cudaEvent_t band_ready = nullptr, coarse_ready = nullptr;
  bool band_check = false;
  DevBuf band_err, coarse_tasks, coarse_tprob, coarse_part, coarse_Einv;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  ilm_batch_s* twin = nullptr;
  DevBuf ref_in, ref_b, ref_x, ref_r, ref_y, ref_norm, dsoff;
  // host wall-clock of the set-up phases (ilm_batch_setup_times), ms
  std::vector<std::pair<const char*, double>> setup_ms;
  // the set-up's device memory: geometry, work buffers and task tables are
  // views into two arenas (one allocation and one host->device copy each)
  DevBuf arena_geom, arena_tasks;
  DevBuf px, py, ph;  // point coordinates (FP64) and per-problem h on the device
  // set while the Schur build of ilm_batch_create may still be running: it
  // continues past the call's return, and every launch that reads S waits
  // for this event (wait_schur)
  cudaEvent_t schur_ready = nullptr;
  // The build runs as two launches when the batch holds both kinds, the
  // Neumann problems' matrices first: schur_first is recorded between them,
  // and set-up work that reads only those matrices (their block inverses and
  // coarse E) waits for it instead of schur_ready (wait_schur_for).
  // in_first[p]: problem p's S is built by the first launch.
  cudaEvent_t schur_first = nullptr;
  std::vector<char> in_first;
  ~ilm_batch_s() {
    if (schur_ready) {
      cudaEventSynchronize(schur_ready);
      cudaEventDestroy(schur_ready);
    }
    if (schur_first) {
      cudaEventSynchronize(schur_first);
      cudaEventDestroy(schur_first);
    }
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    if (gexec) cudaGraphExecDestroy(gexec);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (s2) cudaStreamDestroy(s2);
    if (s_setup) cudaStreamDestroy(s_setup);
    for (cudaEvent_t e : {bj_ready, band_ready, coarse_ready})
      if (e) {
        cudaEventSynchronize(e);
        cudaEventDestroy(e);
      }
    if (s_bj) cudaStreamDestroy(s_bj);
    if (s_learn) cudaStreamDestroy(s_learn);
    delete twin;
  }
};

namespace {

size_t es(int dtype) { return dtype == ILM_F64 ? 8 : 4; }

template <typename V>
int up(DevBuf& b, const std::vector<V>& v) {
  ILM_TRY(b.alloc(std::max<size_t>(v.size(), 1) * sizeof(V)));
  if (!v.empty()) ILM_CHECK_CUDA(cudaMemcpy(b.p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice));
  return ILM_OK;
}

#define BDISPATCH(dtype, ...)  \
  do {                         \
    if ((dtype) == ILM_F64) {  \
      using T = double;        \
      __VA_ARGS__;             \
    } else {                   \
      using T = float;         \
      __VA_ARGS__;             \
    }                          \
  } while (0)


int ensure_split(ilm_batch_s* b);  // CG variant 6's queues (defined with batch_cg)

struct CoarseTask {
  const float* Shi;  // n x n row-major float-float (leading dimension schur_ld(n))
  const float* Slo;
  const double* w;   // ds of the problem's points
  int n, nb;
  int cst[CG_COARSE_MAX + 1];
};

// Partial E = Z^T W S Z over rows [c n / COARSE_SPLIT, (c + 1) n / COARSE_SPLIT)
// of task t into E[(t COARSE_SPLIT + c) 16 ...] (row-major nb x nb): a warp
// per row, each body's column range summed in FP32 (the hi parts; E only
// preconditions), per-warp partials summed in warp order.  The host adds
// the COARSE_SPLIT partials in order (deterministic).
constexpr int COARSE_SPLIT = 8;
__global__ void __launch_bounds__(256) k_coarse_E(const CoarseTask* __restrict__ tasks, double* __restrict__ E) {
  constexpr int NB2 = CG_COARSE_MAX * CG_COARSE_MAX;
  __shared__ double part[8][NB2];
  const int t = blockIdx.x / COARSE_SPLIT, c = blockIdx.x % COARSE_SPLIT;
  const CoarseTask T = tasks[t];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, ld = schur_ld(T.n);
  for (int k = lane; k < NB2; k += 32) part[warp][k] = 0.0;
  __syncwarp();
  const int i0 = (int)((long long)T.n * c / COARSE_SPLIT), i1 = (int)((long long)T.n * (c + 1) / COARSE_SPLIT);
  for (int i = i0 + warp; i < i1; i += 8) {
    const float* h = T.Shi + (size_t)i * ld;
    int a = 0;
    for (int k = 1; k < T.nb; ++k) a += i >= T.cst[k] ? 1 : 0;
    for (int b = 0; b < T.nb; ++b) {
      float acc = 0.f;
      for (int j = T.cst[b] + lane; j < T.cst[b + 1]; j += 32) acc += h[j];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
      if (lane == 0) part[warp][a * CG_COARSE_MAX + b] += T.w[i] * (double)acc;
    }
  }
  __syncthreads();
  if (threadIdx.x < NB2) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += part[w][threadIdx.x];
    E[(size_t)blockIdx.x * NB2 + threadIdx.x] = s;
  }
}

// E^-1 of each coarse task: the COARSE_SPLIT partials of k_coarse_E summed in
// order, the symmetric part taken (W S is symmetric up to rounding), then
// Gauss-Jordan with partial pivoting, one thread per task in FP64 (at most
// CG_COARSE_MAX bodies); a singular E leaves zeros, and the correction then
// adds nothing.  Written to Einv[tprob[t]] (row-major, CG_COARSE_MAX^2).
__global__ void k_coarse_inv(int ntask, const CoarseTask* __restrict__ tasks, const int* __restrict__ tprob,
                             const double* __restrict__ part, double* __restrict__ Einv) {
  constexpr int M = CG_COARSE_MAX, NB2 = M * M;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntask) return;
  const int k = tasks[t].nb;
  double Ef[NB2];
  for (int q = 0; q < NB2; ++q) Ef[q] = 0.0;
  for (int c = 0; c < COARSE_SPLIT; ++c)
    for (int q = 0; q < NB2; ++q) Ef[q] += part[((size_t)t * COARSE_SPLIT + c) * NB2 + q];
  double a[M][2 * M];
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < 2 * M; ++j) a[i][j] = 0.0;
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) {
      a[i][j] = 0.5 * (Ef[i * M + j] + Ef[j * M + i]);
      a[i][k + j] = i == j ? 1.0 : 0.0;
    }
  double* out = Einv + (size_t)tprob[t] * NB2;
  for (int c = 0; c < k; ++c) {
    int piv = c;
    for (int r = c + 1; r < k; ++r)
      if (fabs(a[r][c]) > fabs(a[piv][c])) piv = r;
    if (!(fabs(a[piv][c]) > 0.0)) {
      for (int q = 0; q < NB2; ++q) out[q] = 0.0;
      return;
    }
    for (int j = 0; j < 2 * k; ++j) {
      const double tmp = a[c][j];
      a[c][j] = a[piv][j];
      a[piv][j] = tmp;
    }
    const double ip = 1.0 / a[c][c];
    for (int j = 0; j < 2 * k; ++j) a[c][j] *= ip;
    for (int r = 0; r < k; ++r) {
      if (r == c) continue;
      const double f = a[r][c];
      for (int j = 0; j < 2 * k; ++j) a[r][j] -= f * a[c][j];
    }
  }
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j) out[i * M + j] = i < k && j < k ? a[i][k + j] : 0.0;
}

// Order work on stream st after the batch's Schur build (ilm_batch_create
// returns while it runs): a device-side wait on its event, or a host wait
// when st is being captured (the capture takes no dependency on work outside
// it).  Once the build is known to be done the event is dropped.
int wait_schur_host(ilm_batch_s* b) {
  if (!b->schur_ready) return ILM_OK;
  ILM_CHECK_CUDA(cudaEventSynchronize(b->schur_ready));
  cudaEventDestroy(b->schur_ready);
  b->schur_ready = nullptr;
  return ILM_OK;
}

int wait_schur(ilm_batch_s* b, cudaStream_t st) {
  if (!b->schur_ready) return ILM_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  ILM_CHECK_CUDA(cudaStreamIsCapturing(st, &cs));
  if (cs != cudaStreamCaptureStatusNone) return wait_schur_host(b);
  const cudaError_t q = cudaEventQuery(b->schur_ready);
  if (q == cudaSuccess) {
    cudaEventDestroy(b->schur_ready);
    b->schur_ready = nullptr;
    return ILM_OK;
  }
  if (q != cudaErrorNotReady) ILM_CHECK_CUDA(q);
  if (cudaPeekAtLastError() == cudaErrorNotReady) (void)cudaGetLastError();  // a status, not a launch error
  ILM_CHECK_CUDA(cudaStreamWaitEvent(st, b->schur_ready, 0));
  return ILM_OK;
}

int wait_event(cudaEvent_t ev, cudaStream_t st);

// Order work on stream st after the Schur build of the problems probs: the
// first launch's event when all of them are built by it, else the whole build
int wait_schur_for(ilm_batch_s* b, cudaStream_t st, const std::vector<int>& probs) {
  bool first = b->schur_first != nullptr && b->schur_ready != nullptr && !probs.empty();
  for (int p : probs) first = first && b->in_first[p];
  return first ? wait_event(b->schur_first, st) : wait_schur(b, st);
}

// Order work on stream st after the work recorded by event ev (a host wait
// when st is being captured: the capture takes no dependency on work outside
// it); ev == nullptr: nothing to wait for
int wait_event(cudaEvent_t ev, cudaStream_t st) {
  if (!ev) return ILM_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  ILM_CHECK_CUDA(cudaStreamIsCapturing(st, &cs));
  if (cs != cudaStreamCaptureStatusNone) {
    ILM_CHECK_CUDA(cudaEventSynchronize(ev));
    return ILM_OK;
  }
  ILM_CHECK_CUDA(cudaStreamWaitEvent(st, ev, 0));
  return ILM_OK;
}

// the preconditioner set-up issued so far: block inverses, learned band,
// coarse E^-1
int wait_precond(ilm_batch_s* b, cudaStream_t st) {
  ILM_TRY(wait_event(b->bj_ready, st));
  ILM_TRY(wait_event(b->band_ready, st));
  return wait_event(b->coarse_ready, st);
}

// the network's completion status of the last learned set-up, once (the
// set-up does not synchronise; its flag was copied to band_err on its stream)
int check_band(ilm_batch_s* b) {
  if (!b->band_check) return ILM_OK;
  b->band_check = false;
  int e = 0;
  ILM_CHECK_CUDA(cudaMemcpyAsync(&e, b->band_err.p, sizeof(int), cudaMemcpyDeviceToHost, b->s_learn));
  ILM_CHECK_CUDA(cudaStreamSynchronize(b->s_learn));
  if (e) {
    set_error("learned preconditioner: a tensor-core convolution of its network did not complete in time");
    return ILM_ERR_TIMEOUT;
  }
  return ILM_OK;
}

int ensure_setup_stream(ilm_batch_s* b) {
  if (!b->s_setup) ILM_CHECK_CUDA(cudaStreamCreateWithFlags(&b->s_setup, cudaStreamNonBlocking));
  return ILM_OK;
}

// Block-Jacobi inverses (Gauss-Jordan, float-float) of the problems whose
// preconditioner uses them: every problem under block-Jacobi, the problems
// without a network under the learned preconditioner
int ensure_block_inverses(ilm_batch_s* b) {
  if (b->bj_block <= 0 || b->precond == 0) return ILM_OK;
  std::vector<BJBlockTask> todo;
  std::vector<int> todo_probs;
  for (int p = 0; p < b->nprob; ++p) {
    const bool need = b->precond == 1 || (b->precond == 2 && (b->has_band.empty() || !b->has_band[p]));
    if (!need || b->bj_have[p]) continue;
    for (int t = b->bj_first[p]; t < b->bj_first[p + 1]; ++t) todo.push_back(b->bj_tasks_host[t]);
    b->bj_have[p] = 1;
    todo_probs.push_back(p);
  }
  if (todo.empty()) return ILM_OK;
  const auto t0 = std::chrono::steady_clock::now();
  if (!b->s_bj) ILM_CHECK_CUDA(cudaStreamCreateWithFlags(&b->s_bj, cudaStreamNonBlocking));
  if (!b->bj_ready) ILM_CHECK_CUDA(cudaEventCreateWithFlags(&b->bj_ready, cudaEventDisableTiming));
  ILM_TRY(wait_schur_for(b, b->s_bj, todo_probs));
  ILM_TRY(b->lz_bjtasks.alloc(todo.size() * sizeof(BJBlockTask)));
  // (from pageable memory: the copy has read todo when the call returns)
  ILM_CHECK_CUDA(cudaMemcpyAsync(b->lz_bjtasks.p, todo.data(), todo.size() * sizeof(BJBlockTask),
                                 cudaMemcpyHostToDevice, b->s_bj));
  ILM_TRY(launch_block_inverse(b->lz_bjtasks.as<BJBlockTask>(), (int)todo.size(), b->bj_max_sz, b->s_bj));
  ILM_CHECK_CUDA(cudaEventRecord(b->bj_ready, b->s_bj));
  b->setup_ms.emplace_back("block-Jacobi inverses (issued; formed on their own stream)",
                           std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
  return ILM_OK;
}

// CG parameter records for the current preconditioner, tolerance and limit
int ensure_cg_params(ilm_batch_s* b, double tol, int maxiter) {
  if (tol == b->cg_tol && maxiter == b->cg_maxiter && !b->params_dirty) return ILM_OK;
  ILM_TRY(check_band(b));
  // the size split's queues and stream, built here (outside any stream
  // capture) for the default variant and variant 6
  if (b->cg_variant == 0 || b->cg_variant == 6) ILM_TRY(ensure_split(b));
  ILM_TRY(ensure_block_inverses(b));
  b->params_dirty = false;
  std::vector<unsigned char> cg((size_t)b->nprob * cgff_params_size());
  const int P = 2 * b->band_k + 1;
  const bool bj_ready = b->bj_block > 0;
  for (int p = 0; p < b->nprob; ++p) {
    const size_t o = b->poff[p];
    void* dst = cg.data() + (size_t)p * cgff_params_size();
    // block-Jacobi when selected, and for the problems the learned
    // preconditioner has no network for (when block-Jacobi is set up)
    const bool pre = b->precond == 1 || (b->precond == 2 && !b->has_band[p] && bj_ready);
    cgff_params_fill(dst, b->Shi.as<float>() + b->soff[p], b->Slo.as<float>() + b->soff[p],
                     b->rhs64.as<double>() + o, b->x64.as<double>() + o, b->ds64.as<double>() + o, b->probs[p].npts,
                     maxiter, tol, b->iters.as<int>() + p, b->relres.as<double>() + p,
                     pre ? b->bj_blk.as<int>() + o : nullptr, pre ? b->bj_start.as<int>() + b->bj_first[p] : nullptr,
                     pre ? b->bj_size.as<int>() + b->bj_first[p] : nullptr,
                     pre ? b->bj_off.as<int>() + b->bj_first[p] : nullptr, pre ? b->bj_inv.as<float>() : nullptr,
                     pre ? b->bj_inv_lo.as<float>() : nullptr);
    if (b->probs[p].kind == 0 && b->defl_sz.p)
      cgff_params_set_deflation(dst, b->defl_sz.as<double>() + o, b->defl_ie.as<double>() + p);
    cgff_params_set_timing(dst, b->profiling ? b->cgtime.as<unsigned long long>() + 3 * (size_t)p : nullptr);
    if (b->precond == 2 && b->has_band[p])
      cgff_params_set_band(dst, b->band.as<float>() + o * P, b->band_k, b->lseg_start.as<int>() + o,
                           b->lseg_len.as<int>() + o);
    if (pre && !b->coarse_nb.empty() && b->coarse_nb[p] > 0)
      cgff_params_set_coarse(dst, b->coarse_nb[p], &b->coarse_start[(size_t)p * (CG_COARSE_MAX + 1)],
                             b->coarse_Einv.as<double>() + (size_t)p * CG_COARSE_MAX * CG_COARSE_MAX);
  }
  ILM_TRY(up(b->cgp, cg));
  b->cg_tol = tol;
  b->cg_maxiter = maxiter;
  b->param_gen++;
  return ILM_OK;
}

// y = S x for every problem (float-float S, FP64 accumulation), one warp per row
__global__ void k_batch_schur_apply(int Ptot, const int* __restrict__ pt2prob, const size_t* __restrict__ poff,
                                    const float* __restrict__ Shi, const float* __restrict__ Slo,
                                    const size_t* __restrict__ soff, const double* __restrict__ x,
                                    double* __restrict__ y) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= Ptot) return;
  const int p = pt2prob[row];
  const size_t o = poff[p];
  const int n = (int)(poff[p + 1] - o);
  const int i = row - (int)o;
  const float* sh = Shi + soff[p] + (size_t)i * schur_ld(n);
  const float* sl = Slo + soff[p] + (size_t)i * schur_ld(n);
  double acc = 0.0;
  for (int j = lane; j < n; j += 32) acc += ((double)sh[j] + (double)sl[j]) * x[o + j];
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, s);
  if (lane == 0) y[row] = acc;
}

// Scratch of the lazy set-up, allocated before a solve issues its stage A
// (cudaMalloc and cudaFree may synchronise the device)
int prepare_lazy_setup(ilm_batch_s* b) {
  if (!b->dpoff.p) ILM_TRY(up(b->dpoff, b->poff));
  if (b->bj_block > 0) ILM_TRY(b->lz_bjtasks.alloc(std::max<size_t>(b->bj_tasks_host.size(), 1) * sizeof(BJBlockTask)));
  return ILM_OK;
}

// Deflation data of the Dirichlet problems (see CGFFParams::sz).  The
// Dirichlet Schur complement S = -E L^-1 R has one negative eigenvalue, the
// net-charge mode (the lattice Green's function is normalised with
// G(0,0) = 0, the logarithmic energy is positive only for neutral charge);
// plain CG on it can break down.  Where E = 1^T W S 1 < 0 the constants see
// that mode and the CG deflates them: S is positive definite on the
// S-orthogonal complement of 1 because E takes the one negative eigenvalue
// (inertia additivity).  k_defl_rows: sz = S 1, one warp per row of the
// Dirichlet problems (float-float entries summed in FP64, lanes striding the
// row, then a shuffle tree: a fixed order); other rows 0.
__global__ void k_defl_rows(int Ptot, const int* __restrict__ pt2prob, const SchurProbDev* __restrict__ pr,
                            const float* __restrict__ Shi, const float* __restrict__ Slo, double* __restrict__ sz) {
  const int row = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= Ptot) return;
  const SchurProbDev P = pr[pt2prob[row]];
  if (P.kind != ILM_SCHUR_RTLINVR) {
    if (lane == 0) sz[row] = 0.0;
    return;
  }
  const int i = row - P.poff;
  const float* sh = Shi + P.soff + (size_t)i * schur_ld(P.n);
  const float* sl = Slo + P.soff + (size_t)i * schur_ld(P.n);
  double acc = 0.0;
  for (int j = lane; j < P.n; j += 32) acc += (double)sh[j] + (double)sl[j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) sz[row] = acc;
}

// k_defl_e: per Dirichlet problem (one block each) E = sum_i w_i sz_i in a
// fixed order and inv_e = 1 / E when E < 0, else 0 (no deflation)
__global__ void __launch_bounds__(256) k_defl_e(const SchurProbDev* __restrict__ pr, const double* __restrict__ w,
                                                const double* __restrict__ sz, double* __restrict__ inv_e) {
  __shared__ double part[256];
  const SchurProbDev P = pr[blockIdx.x];
  if (P.kind != ILM_SCHUR_RTLINVR) {
    if (threadIdx.x == 0) inv_e[blockIdx.x] = 0.0;
    return;
  }
  double s = 0.0;
  for (int i = threadIdx.x; i < P.n; i += blockDim.x) s += w[P.poff + i] * sz[P.poff + i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) inv_e[blockIdx.x] = part[0] < 0.0 ? 1.0 / part[0] : 0.0;
}

// optional stage timing: one CUDA event per stage boundary on the solve stream
int batch_mark(ilm_batch_s* b, cudaStream_t st) {
  if (b->profiling && b->nev < 32) {
    if (!b->ev[b->nev]) ILM_CHECK_CUDA(cudaEventCreate(&b->ev[b->nev]));
    ILM_CHECK_CUDA(cudaEventRecord(b->ev[b->nev], st));
    b->nev++;
  }
  return ILM_OK;
}

// Stage A of a solve: surface jump / average, the source of f* (double layer
// for Dirichlet, single layer for Neumann), f* = L^-1 source and the Schur
// right-hand side in rhs64 (or, with the right-hand-side operator, rhs64 from
// M [jump] - avg and f*'s source left unconvolved in fstar).
int batch_stage_a(ilm_batch_s* b, const void* fplus, const void* fminus, cudaStream_t st) {
  const int dt = b->dtype;
  const int Ptot = b->Ptot;
  const int pb = std::min(1024, (Ptot + 255) / 256);
  BDISPATCH(dt, {
    k_jump_avg<T><<<pb, 256, 0, st>>>(Ptot, static_cast<const T*>(fplus), static_cast<const T*>(fminus),
                                      b->jump.as<T>(), b->avg.as<T>());
    ILM_CHECK_LAUNCH();
    b->launches++;
    ILM_TRY(batch_mark(b, st));  // 1: surface data jump/average
    if (b->blk_fillA)
      k_bfill<T><<<(b->blk_fillA + 7) / 8, 256, 0, st>>>(b->scatA.as<BScatterTask>(), b->blk_fillA, b->mfillA.as<int>());
    ILM_CHECK_LAUNCH();
    if (b->blk_scatA) k_bscatter<T><<<b->blk_scatA, dim3(SB_X, SB_Y), 0, st>>>(b->scatA.as<BScatterTask>(), b->n_scatA,
                                                                    b->mscatA.as<int>());
    ILM_CHECK_LAUNCH();
    b->launches += (b->blk_fillA ? 1 : 0) + (b->blk_scatA ? 1 : 0);
    ILM_TRY(batch_mark(b, st));  // 2: DDF scatter (double layer / single layer)
    if (b->n_divA) k_bdiv<T><<<b->blk_divA, dim3(SB_X, SB_Y), 0, st>>>(b->divA.as<BStencilTask>(), b->n_divA, b->mdivA.as<int>());
    ILM_CHECK_LAUNCH();
    b->launches += b->n_divA ? 1 : 0;
    ILM_TRY(batch_mark(b, st));  // 3: divergence stencil
  });
  if (!b->rhs_op) {
    ILM_TRY(conv_jobs_launch(b->convA.as<ConvJobDev>(), b->n_conv, b->convL, dt, st));
    b->launches += 3;
  }
  ILM_TRY(batch_mark(b, st));  // 4: LGF FFT convolution (f*; with the rhs operator f* stays a source)
  BDISPATCH(dt, {
    if (b->rhs_op) {
      if (Ptot > 0)
        k_rhsop_matvec<T><<<(Ptot + 7) / 8, 256, 0, st>>>(Ptot, b->pt2prob.as<int>(), b->schurPfull.as<SchurProbDev>(),
                                                       b->Mhi.as<float>(), b->Mlo.as<float>(), b->jump.as<T>(),
                                                       b->avg.as<T>(), b->rhs64.as<double>());
      ILM_CHECK_LAUNCH();
      b->launches += 1;
    } else {
      k_bgather<T><<<(Ptot + 127) / 128, 128, 0, st>>>(b->gathA.as<BGatherTask>(), b->n_gathA, Ptot);
      ILM_CHECK_LAUNCH();
      k_rhs64<T><<<pb, 256, 0, st>>>(Ptot, b->g.as<T>(), b->avg.as<T>(), b->rhs64.as<double>());
      ILM_CHECK_LAUNCH();
      b->launches += 2;
    }
  });
  return batch_mark(b, st);  // 5: DDF gather (Neumann: with the gradient) + Schur right-hand side
}

// CG variant 6: the two queues (largest first each), the second stream and
// its events (built on first use)
constexpr int kSplitN = 192;
int ensure_split(ilm_batch_s* b) {
  if (b->split_ready) return ILM_OK;
  std::vector<int> ord(b->nprob), large, small;
  for (int p = 0; p < b->nprob; ++p) ord[p] = p;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return b->probs[a].npts > b->probs[c].npts; });
  int max_small = 0;
  for (int p : ord) {
    if (b->probs[p].npts > kSplitN) {
      large.push_back(p);
    } else {
      small.push_back(p);
      max_small = std::max(max_small, b->probs[p].npts);
    }
  }
  ILM_TRY(up(b->order_large, large));
  ILM_TRY(up(b->order_small, small));
  ILM_TRY(b->counter2.alloc(sizeof(int)));
  if (!b->s2) ILM_CHECK_CUDA(cudaStreamCreateWithFlags(&b->s2, cudaStreamNonBlocking));
  // timing-enabled fork / join events: with cudaEventDisableTiming the two
  // launches of the split measured as if serialised on GB300 (2.77 against
  // 2.44 ms per batched solve of the bench configuration, CUDA events around
  // whole solves; the same 2.44 ms with timing-enabled events recorded
  // between the stages, which is how the difference was found)
  if (!b->ev_fork) ILM_CHECK_CUDA(cudaEventCreate(&b->ev_fork));
  if (!b->ev_join) ILM_CHECK_CUDA(cudaEventCreate(&b->ev_join));
  b->n_large = (int)large.size();
  b->n_small = (int)small.size();
  b->max_small = max_small;
  // the CTA slots the large problems' clusters leave free (at least 8)
  const int slots = small.empty() ? 0 : cg_single_slots(max_small);
  b->nctas_small = std::max(8, std::min(b->n_small, slots - 8 * cg_cluster_count(b->nprob, b->maxN, 1)));
  b->split_ready = true;
  return ILM_OK;
}

// The Schur CG of every problem: rhs64 -> x64 (parameters set by ensure_cg_params)
int batch_cg(ilm_batch_s* b, cudaStream_t st) {
  ILM_TRY(wait_schur(b, st));
  ILM_TRY(wait_precond(b, st));
  if (b->cg_variant == 6 || b->cg_variant == 0) {  // the default is the size split
    ILM_TRY(ensure_split(b));
    if (b->n_small > 0 && b->n_large > 0) {
      ILM_CHECK_CUDA(cudaEventRecord(b->ev_fork, st));
      ILM_CHECK_CUDA(cudaStreamWaitEvent(b->s2, b->ev_fork, 0));
      ILM_TRY(launch_cg_cluster(b->cgp.p, b->order_large.as<int>(), b->n_large, b->counter.as<int>(), b->maxN,
                                b->nclusters, st, 1));
      ILM_TRY(launch_cg_single(b->cgp.p, b->order_small.as<int>(), b->n_small, b->counter2.as<int>(), b->max_small,
                               b->nctas_small, b->s2));
      ILM_CHECK_CUDA(cudaEventRecord(b->ev_join, b->s2));
      ILM_CHECK_CUDA(cudaStreamWaitEvent(st, b->ev_join, 0));
      b->launches += 2;
      return batch_mark(b, st);  // 6: Schur CG
    }
  }
  ILM_TRY(launch_cg_cluster(b->cgp.p, b->order.as<int>(), b->nprob, b->counter.as<int>(), b->maxN, b->nclusters, st,
                            b->cg_variant));
  b->launches += 1;
  return batch_mark(b, st);  // 6: Schur CG
}

// Stage B of a solve: f = f* + L^-1 (correction source of the surface
// strength in b->s), written into f_out by the last convolution pass.
int batch_stage_b(ilm_batch_s* b, void* f_out, cudaStream_t st) {
  const int dt = b->dtype;
  BDISPATCH(dt, {
    // with the rhs operator the correction's source is added to f*'s
    // source (scatB2 / divB2 accumulate into it) and one convolution follows
    const BScatterTask* sBt = (b->rhs_op ? b->scatB2 : b->scatB).as<BScatterTask>();
    const int fillB = b->rhs_op ? b->blk_fillB2 : b->blk_fillB;
    if (fillB)
      k_bfill<T><<<(fillB + 7) / 8, 256, 0, st>>>(sBt, fillB, (b->rhs_op ? b->mfillB2 : b->mfillB).as<int>());
    ILM_CHECK_LAUNCH();
    if (b->blk_scatB) k_bscatter<T><<<b->blk_scatB, dim3(SB_X, SB_Y), 0, st>>>(sBt, b->n_scatB, b->mscatB.as<int>());
    ILM_CHECK_LAUNCH();
    b->launches += (fillB ? 1 : 0) + (b->blk_scatB ? 1 : 0);
    ILM_TRY(batch_mark(b, st));  // 8: DDF scatter (correction)
    if (b->n_divB)
      k_bdiv<T><<<b->blk_divB, dim3(SB_X, SB_Y), 0, st>>>((b->rhs_op ? b->divB2 : b->divB).as<BStencilTask>(),
                                                         b->n_divB, b->mdivB.as<int>());
    ILM_CHECK_LAUNCH();
    b->launches += b->n_divB ? 1 : 0;
    ILM_TRY(batch_mark(b, st));  // 9: divergence stencil
  });
  // f = f* + L^-1 (correction source), written into f_out by the inverse row pass
  ILM_TRY(conv_jobs_launch((b->rhs_op ? b->convC : b->convB).as<ConvJobDev>(), b->n_conv, b->convL, dt, st, f_out));
  b->launches += 3;
  return batch_mark(b, st);  // 10: LGF FFT convolution (correction) + f*
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {

// learned-preconditioner features of the selected points (compacted order:
// point i of the selection is point c2o[i] of the batch; its body is
// [sst[i], sst[i] + sln[i]) in the selection)
__global__ void k_batch_features(int Nsel, const int* __restrict__ c2o, const int* __restrict__ sst,
                                 const int* __restrict__ sln, const double* __restrict__ x,
                                 const double* __restrict__ y, const double* __restrict__ nx,
                                 const double* __restrict__ ny, const double* __restrict__ ds,
                                 const int* __restrict__ pt2prob, const double* __restrict__ hprob,
                                 float* __restrict__ feat) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Nsel) return;
  const int s = sst[i], L = sln[i];
  const int k = c2o[i], kp = c2o[s + (i - s + 1) % L], km = c2o[s + (i - s + L - 1) % L];
  point_feature(x[k], y[k], nx[k], ny[k], ds[k], nx[kp], ny[kp], ds[kp], nx[km], ny[km], ds[km], hprob[pt2prob[k]],
                feat + (size_t)i * 8);
}

// band[c2o[i]] = rows[i] (P coefficients per point)
__global__ void k_scatter_rows(int Nsel, int P, const int* __restrict__ c2o, const float* __restrict__ rows,
                               float* __restrict__ band) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < Nsel * P; e += gridDim.x * blockDim.x)
    band[(size_t)c2o[e / P] * P + e % P] = rows[e];
}

// Many small device arrays carved out of one allocation; the ones with host
// data are filled by one host->device copy through pinned staging memory
// (kept by the library and grown on demand; one batch set-up at a time
// uses it).  g_stage_done marks the end of the last copy out of it: the next
// set-up waits for it before writing the staging memory again, so a copy's
// stream need not be synchronised (work after it on that stream is ordered
// after it anyway).
std::mutex g_stage_mu;
void* g_stage = nullptr;
size_t g_stage_bytes = 0;
cudaEvent_t g_stage_done = nullptr;

struct ArenaBuilder {
  struct Item {
    DevBuf* dst;
    size_t off, bytes;
    const void* src;
  };
  std::vector<Item> items;
  size_t total = 0, copy_end = 0;
  void add(DevBuf* dst, size_t bytes, const void* src = nullptr) {
    const size_t off = (total + 255) & ~(size_t)255;
    items.push_back({dst, off, bytes, src});
    total = off + std::max<size_t>(bytes, 1);
    if (src && bytes) copy_end = off + bytes;
  }
  template <typename V>
  void add(DevBuf* dst, const std::vector<V>& v) {
    add(dst, v.size() * sizeof(V), v.data());
  }
  int commit(DevBuf& arena, cudaStream_t st) {
    ILM_TRY(commit_layout(arena));
    return commit_upload(arena, st);
  }
  // allocate the arena and point every buffer at its part
  int commit_layout(DevBuf& arena) {
    ILM_TRY(arena.alloc(std::max<size_t>(total, 256)));
    for (const Item& it : items) it.dst->view(static_cast<unsigned char*>(arena.p) + it.off, it.bytes);
    return ILM_OK;
  }
  // one copy of every buffer's host data (read now, so the host arrays may
  // have been edited after commit_layout)
  int commit_upload(DevBuf& arena, cudaStream_t st) {
    if (!copy_end) return ILM_OK;
    std::lock_guard<std::mutex> lk(g_stage_mu);
    if (!g_stage_done) ILM_CHECK_CUDA(cudaEventCreateWithFlags(&g_stage_done, cudaEventDisableTiming));
    ILM_CHECK_CUDA(cudaEventSynchronize(g_stage_done));  // the last copy out of the staging memory
    if (g_stage_bytes < copy_end) {
      if (g_stage) cudaFreeHost(g_stage);
      g_stage = nullptr;
      g_stage_bytes = 0;
      ILM_CHECK_CUDA(cudaMallocHost(&g_stage, copy_end));
      g_stage_bytes = copy_end;
    }
    for (const Item& it : items)
      if (it.src && it.bytes) memcpy(static_cast<unsigned char*>(g_stage) + it.off, it.src, it.bytes);
    ILM_CHECK_CUDA(cudaMemcpyAsync(arena.p, g_stage, copy_end, cudaMemcpyHostToDevice, st));
    ILM_CHECK_CUDA(cudaEventRecord(g_stage_done, st));
    return ILM_OK;
  }
};

// Set-up of a batch; without `build_schur` the Schur matrices are neither
// allocated nor built (the FP64 refinement copy uses its parent's).
int batch_create_impl(int nprob, const ilm_batch_problem_t* probs, const double* x, const double* y,
                      const double* nrmx, const double* nrmy, const double* ds, int ddf, int dtype, bool build_schur,
                      ilm_batch_t* out) {
  ILM_REQUIRE(out && probs && nprob > 0, "batch: bad arguments");
  ILM_REQUIRE(dtype == ILM_F64 || dtype == ILM_F32, "batch: bad dtype %d", dtype);
  ILM_REQUIRE(ddf >= ILM_DDF_YANG3 && ddf <= ILM_DDF_M3, "batch: bad ddf %d", ddf);
  auto* B = new (std::nothrow) ilm_batch_s();
  if (!B) return ILM_ERR_NO_MEMORY;
  std::unique_ptr<ilm_batch_s> guard(B);
  auto clk = std::chrono::steady_clock::now();
  auto phase = [&](const char* name) {
    const auto now = std::chrono::steady_clock::now();
    B->setup_ms.emplace_back(name, std::chrono::duration<double, std::milli>(now - clk).count());
    clk = now;
  };
  B->nprob = nprob;
  B->dtype = dtype;
  B->ddf = ddf;
  B->probs.assign(probs, probs + nprob);
  B->foff.assign(nprob + 1, 0);
  B->poff.assign(nprob + 1, 0);
  B->soff.assign(nprob + 1, 0);
  std::vector<size_t> eoff(nprob + 1, 0);
  for (int p = 0; p < nprob; ++p) {
    const ilm_batch_problem_t& P = probs[p];
    ILM_REQUIRE(P.nx >= 8 && P.ny >= 8 && P.nx <= 8192 && P.ny <= 8192 && P.h > 0, "batch: bad grid of problem %d", p);
    ILM_REQUIRE(P.npts >= 1, "batch: problem %d has no points", p);
    ILM_REQUIRE(P.kind == 0 || P.kind == 1, "batch: bad kind of problem %d", p);
    B->foff[p + 1] = B->foff[p] + (size_t)(P.nx - 1) * (P.ny - 1);
    eoff[p + 1] = eoff[p] + (size_t)P.nx * (P.ny - 1) + (size_t)(P.nx - 1) * P.ny;
    B->poff[p + 1] = B->poff[p] + P.npts;
    B->soff[p + 1] = B->soff[p] + (size_t)P.npts * schur_ld(P.npts);
    B->maxN = std::max(B->maxN, P.npts);
    B->max_grid = std::max(B->max_grid, std::max(P.nx, P.ny));
  }
  const int Ptot = (int)B->poff[nprob];
  B->Ptot = Ptot;
  B->ftot = B->foff[nprob];
  B->etot = eoff[nprob];
  B->stot = B->soff[nprob];
  for (int k = 0; k < Ptot; ++k)
    ILM_REQUIRE(isfinite(x[k]) && isfinite(y[k]) && isfinite(nrmx[k]) && isfinite(nrmy[k]) && isfinite(ds[k]),
                "batch: non-finite point data at %d", k);

  phase("validate point data");
  // ---- geometry and work buffers: one arena; DDF windows and tile lists on
  // the device -----------------------------------------------------------
  const size_t e = es(dtype);
  std::vector<int> hp2p(Ptot), hpoff(nprob + 1), hgrid(4 * (size_t)nprob);
  std::vector<double> hh(nprob);
  std::vector<int> tpo[4], tso[4];   // per problem offsets into the packed tile arrays
  std::vector<int> ntx[4];            // tiles per row, per problem and class
  int tp_tot[4] = {0, 0, 0, 0}, ts_tot[4] = {0, 0, 0, 0};
  for (int c = 0; c < 4; ++c) {
    tpo[c].assign(nprob, 0);
    tso[c].assign(nprob, 0);
    ntx[c].assign(nprob, 0);
  }
  for (int p = 0; p < nprob; ++p) {
    const ilm_batch_problem_t& P = probs[p];
    hpoff[p] = (int)B->poff[p];
    for (int k = 0; k < P.npts; ++k) hp2p[B->poff[p] + k] = p;
    hgrid[4 * p] = P.nx;
    hgrid[4 * p + 1] = P.ny;
    hgrid[4 * p + 2] = P.i0x;
    hgrid[4 * p + 3] = P.i0y;
    hh[p] = P.h;
    const ilm_grid_s g{P.nx, P.ny, P.h, P.i0x, P.i0y};
    for (int c = 0; c < 4; ++c) {
      const Shape2 sh = g.shape(c);
      ntx[c][p] = (sh.n1 + TILE_X - 1) / TILE_X;
      const int nt = ntx[c][p] * ((sh.n2 + TILE_Y - 1) / TILE_Y);
      tpo[c][p] = tp_tot[c];
      tp_tot[c] += nt + 1;
      tso[c][p] = ts_tot[c];
      ts_tot[c] += 4 * P.npts;   // a 4 x 4 window touches at most 2 x 2 tiles
    }
  }
  hpoff[nprob] = Ptot;
  // Schur complement descriptors (float-float LGF point-point sums)
  std::vector<SchurProbDev> sp(nprob);
  {
    int tiles = 0;
    for (int p = 0; p < nprob; ++p) {
      sp[p].kind = probs[p].kind == 0 ? ILM_SCHUR_RTLINVR : ILM_SCHUR_CLINVCT;
      sp[p].n = probs[p].npts;
      sp[p].poff = (int)B->poff[p];
      sp[p].tile0 = tiles;
      const int nt = (probs[p].npts + 15) / 16;
      tiles += nt * (nt + 1) / 2;  // upper triangle (the pair sums are symmetric)
      sp[p].soff = B->soff[p];
      sp[p].invh = 1.0 / probs[p].h;
    }
    B->schur_tiles = tiles;
    B->schur_host = sp;
  }
  // build order of a batch with both kinds: the Neumann problems' matrices
  // first (two launches, schur_first recorded between them); each group's
  // descriptors number its tiles from zero
  std::vector<SchurProbDev> sp_build;
  int nfirst = 0, tiles_first = 0, tiles_second = 0;  // (tiles_first + tiles_second = schur_tiles)
  B->in_first.assign(nprob, 0);
  for (int p = 0; p < nprob; ++p) nfirst += probs[p].kind != 0;
  if (nfirst > 0 && nfirst < nprob) {
    sp_build.reserve(nprob);
    for (int pass = 0; pass < 2; ++pass)
      for (int p = 0; p < nprob; ++p) {
        if ((probs[p].kind != 0) != (pass == 0)) continue;
        SchurProbDev q = sp[p];
        int& t = pass == 0 ? tiles_first : tiles_second;
        const int nt = (q.n + 15) / 16;
        q.tile0 = t;
        t += nt * (nt + 1) / 2;
        sp_build.push_back(q);
        if (pass == 0) B->in_first[p] = 1;
      }
  }
  // set-up streams (non-blocking: independent of the legacy stream): the
  // geometry and task tables on sg, the Schur build on ss, overlapping the
  // host's task building
  struct Streams {
    cudaStream_t g = nullptr, s = nullptr;
    ~Streams() {
      if (g) cudaStreamDestroy(g);
      if (s) cudaStreamDestroy(s);
    }
  } SS;
  ILM_CHECK_CUDA(cudaStreamCreateWithFlags(&SS.g, cudaStreamNonBlocking));
  ILM_CHECK_CUDA(cudaStreamCreateWithFlags(&SS.s, cudaStreamNonBlocking));
  cudaStream_t sg = SS.g, ss = SS.s;
  DevBuf d_in[5], d_poff, d_grid, d_tpo[4], d_tso[4], d_cnt, d_spb;
  {
    ArenaBuilder A;
    const double* src[5] = {x, y, nrmx, nrmy, ds};
    DevBuf* dst[5] = {&B->px, &B->py, &d_in[2], &d_in[3], &d_in[4]};
    for (int q = 0; q < 5; ++q) A.add(dst[q], (size_t)Ptot * 8, src[q]);
    A.add(&B->pt2prob, hp2p);
    A.add(&d_poff, hpoff);
    A.add(&d_grid, hgrid);
    A.add(&B->ph, hh);
    A.add(&B->schurP, sp);
    if (!sp_build.empty()) A.add(&d_spb, sp_build);
    for (int c = 0; c < 4; ++c) {
      A.add(&d_tpo[c], tpo[c]);
      A.add(&d_tso[c], tso[c]);
    }
    for (int d = 0; d < 2; ++d) {
      A.add(&B->bx[d], (size_t)Ptot * 4);
      A.add(&B->by[d], (size_t)Ptot * 4);
      A.add(&B->wx[d], (size_t)Ptot * NTAP * e);
      A.add(&B->wy[d], (size_t)Ptot * NTAP * e);
      A.add(&B->wx64[d], (size_t)Ptot * NTAP * 8);
      A.add(&B->wy64[d], (size_t)Ptot * NTAP * 8);
    }
    A.add(&B->nx, (size_t)Ptot * e);
    A.add(&B->ny, (size_t)Ptot * e);
    A.add(&B->wsc, (size_t)Ptot * e);
    A.add(&B->nx64, (size_t)Ptot * 8);
    A.add(&B->ny64, (size_t)Ptot * 8);
    A.add(&B->ds64, (size_t)Ptot * 8);
    int cnt_tot = 0;
    for (int c = 0; c < 4; ++c) {
      A.add(&B->tptr[c], (size_t)tp_tot[c] * 4);
      A.add(&B->tpts[c], (size_t)std::max(ts_tot[c], 1) * 4);
      cnt_tot += tp_tot[c];
    }
    A.add(&d_cnt, (size_t)cnt_tot * 4);
    // work buffers
    A.add(&B->fstar, B->ftot * e);
    A.add(&B->corr, B->ftot * e);
    A.add(&B->edges, B->etot * e);
    A.add(&B->jump, (size_t)Ptot * e);
    A.add(&B->avg, (size_t)Ptot * e);
    A.add(&B->g, (size_t)Ptot * e);
    A.add(&B->s, (size_t)Ptot * e);
    A.add(&B->rhs64, (size_t)Ptot * 8);
    A.add(&B->x64, (size_t)Ptot * 8);
    if (build_schur) {
      A.add(&B->Shi, std::max<size_t>(B->stot, 1) * 4);
      A.add(&B->Slo, std::max<size_t>(B->stot, 1) * 4);
      A.add(&B->F, (size_t)Ptot * functional_size());
      A.add(&B->defl_sz, (size_t)Ptot * 8);
      A.add(&B->defl_ie, (size_t)nprob * 8);
    }
    A.add(&B->iters, (size_t)nprob * sizeof(int));
    A.add(&B->relres, (size_t)nprob * sizeof(double));
    A.add(&B->counter, sizeof(int));
    ILM_TRY(A.commit(B->arena_geom, sg));
    phase("upload points, allocate buffers (one arena)");
    BatchGeomDev G;
    memset(&G, 0, sizeof(G));
    G.x = B->px.as<double>();
    G.y = B->py.as<double>();
    G.nx = d_in[2].as<double>();
    G.ny = d_in[3].as<double>();
    G.ds = d_in[4].as<double>();
    G.pt2prob = B->pt2prob.as<int>();
    G.poff = d_poff.as<int>();
    G.grid = d_grid.as<int>();
    G.h = B->ph.as<double>();
    for (int d = 0; d < 2; ++d) {
      G.bx[d] = B->bx[d].as<int>();
      G.by[d] = B->by[d].as<int>();
      G.wx64[d] = B->wx64[d].as<double>();
      G.wy64[d] = B->wy64[d].as<double>();
      G.wx[d] = B->wx[d].p;
      G.wy[d] = B->wy[d].p;
    }
    G.nxo = B->nx.p;
    G.nyo = B->ny.p;
    G.wsc = B->wsc.p;
    G.nx64 = B->nx64.as<double>();
    G.ny64 = B->ny64.as<double>();
    G.ds64 = B->ds64.as<double>();
    int co = 0;
    for (int c = 0; c < 4; ++c) {
      G.tptr[c] = B->tptr[c].as<int>();
      G.tpts[c] = B->tpts[c].as<int>();
      G.tp_off[c] = d_tpo[c].as<int>();
      G.ts_off[c] = d_tso[c].as<int>();
      G.cnt_off[c] = co;
      co += tp_tot[c];
    }
    G.cnt = d_cnt.as<int>();
    G.cnt_total = co;
    ILM_TRY(batch_windows_and_tiles(nprob, Ptot, G, ddf, dtype, 1, sg));
    if (build_schur) {
      cudaEvent_t geo_done = nullptr;
      ILM_CHECK_CUDA(cudaEventCreateWithFlags(&geo_done, cudaEventDisableTiming));
      const cudaError_t e1 = cudaEventRecord(geo_done, sg);
      const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(ss, geo_done, 0) : e1;
      cudaEventDestroy(geo_done);
      ILM_CHECK_CUDA(e2);
      // the row padding of every matrix stays zero
      ILM_CHECK_CUDA(cudaMemsetAsync(B->Shi.p, 0, std::max<size_t>(B->stot, 1) * 4, ss));
      ILM_CHECK_CUDA(cudaMemsetAsync(B->Slo.p, 0, std::max<size_t>(B->stot, 1) * 4, ss));
      BatchWin BW;
      for (int d = 0; d < 2; ++d) {
        BW.bx[d] = B->bx[d].as<int>();
        BW.by[d] = B->by[d].as<int>();
        BW.wx64[d] = B->wx64[d].as<double>();
        BW.wy64[d] = B->wy64[d].as<double>();
      }
      BW.nx64 = B->nx64.as<double>();
      BW.ny64 = B->ny64.as<double>();
      const bool split = !sp_build.empty();
      if (split) ILM_CHECK_CUDA(cudaEventCreateWithFlags(&B->schur_first, cudaEventDisableTiming));
      const SchurProbDev* spb = split ? d_spb.as<SchurProbDev>() : nullptr;
      ILM_TRY(schur_build_batched(nprob, B->schurP.as<SchurProbDev>(), B->schur_tiles, Ptot, B->pt2prob.as<int>(),
                                  BW, B->ds64.as<double>(), static_cast<Functional*>(B->F.p), B->Shi.as<float>(),
                                  B->Slo.as<float>(), B->max_grid, ss, spb, nfirst, tiles_first, B->schur_first));
      // the deflation data of the Dirichlet problems, after S on its stream
      k_defl_rows<<<(unsigned)(((size_t)Ptot * 32 + 255) / 256), 256, 0, ss>>>(
          Ptot, B->pt2prob.as<int>(), B->schurP.as<SchurProbDev>(), B->Shi.as<float>(), B->Slo.as<float>(),
          B->defl_sz.as<double>());
      ILM_CHECK_LAUNCH();
      k_defl_e<<<nprob, 256, 0, ss>>>(B->schurP.as<SchurProbDev>(), B->ds64.as<double>(), B->defl_sz.as<double>(),
                                       B->defl_ie.as<double>());
      ILM_CHECK_LAUNCH();
    }
  }
  // the host's copy of the point data (read by the FP64 refinement copy of
  // the batch), taken while the windows kernels and the Schur build run: the
  // device copy above read the caller's arrays
  B->hx.assign(x, x + Ptot);
  B->hy.assign(y, y + Ptot);
  B->hnx.assign(nrmx, nrmx + Ptot);
  B->hny.assign(nrmy, nrmy + Ptot);
  B->hds.assign(ds, ds + Ptot);
  // the windows' base indices and the tile pointers, for the boxes and task
  // tables built on the host (the copies to pageable memory return once done)
  std::vector<int> hbx[2], hby[2], htp[4];
  for (int d = 0; d < 2; ++d) {
    hbx[d].resize(Ptot);
    hby[d].resize(Ptot);
    ILM_CHECK_CUDA(cudaMemcpyAsync(hbx[d].data(), B->bx[d].p, (size_t)Ptot * 4, cudaMemcpyDeviceToHost, sg));
    ILM_CHECK_CUDA(cudaMemcpyAsync(hby[d].data(), B->by[d].p, (size_t)Ptot * 4, cudaMemcpyDeviceToHost, sg));
  }
  for (int c = 0; c < 4; ++c) {
    htp[c].resize(tp_tot[c]);
    ILM_CHECK_CUDA(cudaMemcpyAsync(htp[c].data(), B->tptr[c].p, (size_t)tp_tot[c] * 4, cudaMemcpyDeviceToHost, sg));
  }
  ILM_CHECK_CUDA(cudaStreamSynchronize(sg));
  phase("DDF windows and tile lists (device) + read-back; host copy of the points");
  std::vector<int> ord(nprob);
  {
    // CG work queue: largest problems first (cost ~ npts^2 * sqrt(npts))
    for (int p = 0; p < nprob; ++p) ord[p] = p;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) {
      const double ca = pow((double)probs[a].npts, 2.5), cc = pow((double)probs[c].npts, 2.5);
      return ca > cc;
    });
    B->nclusters = cg_cluster_count(nprob, B->maxN);
  }

  // FFT convolution jobs (fstar and corr in place); one work area per problem
  std::vector<size_t> woff(nprob + 1, 0);
  std::vector<int> P1(nprob), P2(nprob);
  for (int p = 0; p < nprob; ++p) {
    const int n1 = probs[p].nx - 1, n2 = probs[p].ny - 1;
    P1[p] = good_fft_size(2 * n1 - 1);
    P2[p] = good_fft_size(2 * n2 - 1);
    woff[p + 1] = woff[p] + (size_t)n2 * (P1[p] / 2 + 1) * 2 * e;
  }
  ILM_TRY(B->convwork.alloc(woff[nprob]));
  // Source box of each problem: every cell of the two convolution inputs that
  // can be non-zero (DDF windows of all points, both staggerings, widened by
  // the divergence stencil) lies in [ca, cb) x [ra, rb).  The scatters and
  // divergences write only this box and the FFT row pass reads only it.
  std::vector<std::array<int, 4>> box(nprob);
  for (int p = 0; p < nprob; ++p) {
    const size_t o = B->poff[p];
    int xmin = INT_MAX, xmax = INT_MIN, ymin = INT_MAX, ymax = INT_MIN;
    for (int k = 0; k < probs[p].npts; ++k)
      for (int d = 0; d < 2; ++d) {
        xmin = std::min(xmin, hbx[d][o + k]);
        xmax = std::max(xmax, hbx[d][o + k] + NTAP - 1);
        ymin = std::min(ymin, hby[d][o + k]);
        ymax = std::max(ymax, hby[d][o + k] + NTAP - 1);
      }
    const int n1 = probs[p].nx - 1, n2 = probs[p].ny - 1;
    int ca = std::max(0, xmin - 3), cb = std::min(n1, xmax + 4);
    int ra = std::max(0, ymin - 3), rb = std::min(n2, ymax + 4);
    if (ca >= cb) ca = 0, cb = 1;  // every window off the grid: nothing is scattered
    if (ra >= rb) ra = 0, rb = 1;
    box[p] = {ca, cb, ra, rb};
    B->box_cells += (size_t)(cb - ca) * (rb - ra);
  }
  std::vector<ConvJobDev> jobsA(nprob), jobsB(nprob), jobsC(nprob);
  for (int p = 0; p < nprob; ++p) {
    ConvJobDev J;
    memset(&J, 0, sizeof(J));
    J.has_box = 1;
    J.ca = box[p][0];
    J.cb = box[p][1];
    J.ra = box[p][2];
    J.rb = box[p][3];
    ILM_TRY(conv_resources(P1[p], P2[p], dtype, &J.spec, &J.tw1, &J.tw2, nullptr));
    J.work = static_cast<unsigned char*>(B->convwork.p) + woff[p];
    J.n1 = probs[p].nx - 1;
    J.n2 = probs[p].ny - 1;
    J.n2out = J.n2;
    J.P1 = P1[p];
    J.P2 = P2[p];
    J.scale = probs[p].h * probs[p].h;  // L^{-1} = h^2 G* under GridScaling
    J.in = J.out = static_cast<unsigned char*>(B->fstar.p) + B->foff[p] * e;
    jobsA[p] = J;
    // correction: f = f* + L^-1 q_B, written straight into the caller's
    // field (out_base at launch)
    J.in = static_cast<unsigned char*>(B->corr.p) + B->foff[p] * e;
    J.out = nullptr;
    J.out_off = B->foff[p] * e;
    J.add = static_cast<unsigned char*>(B->fstar.p) + B->foff[p] * e;
    jobsB[p] = J;
    // rhs-operator path: the combined source (in fstar) convolved straight
    // into the caller's field
    J.in = static_cast<unsigned char*>(B->fstar.p) + B->foff[p] * e;
    J.add = nullptr;
    jobsC[p] = J;
  }
  ILM_TRY(conv_jobs_finalize(jobsA, dtype, &B->convL));
  ILM_TRY(conv_jobs_finalize(jobsB, dtype, &B->convL));
  ILM_TRY(conv_jobs_finalize(jobsC, dtype, &B->convL));
  // every task table goes to the device in one arena (laid out below, the
  // device addresses resolved, then one copy)
  ArenaBuilder TA;
  if (B->convL.fast) {  // CTA -> job maps (the two job tables share their geometry)
    TA.add(&B->mconv[0], B->convL.mrows);
    TA.add(&B->mconv[1], B->convL.mcols);
    TA.add(&B->mconv[2], B->convL.mirows);
  }
  B->n_conv = nprob;
  TA.add(&B->convA, jobsA);
  TA.add(&B->convB, jobsB);
  TA.add(&B->convC, jobsC);
  TA.add(&B->order, ord);

  phase("source boxes and convolution jobs");
  // ---- tasks ---------------------------------------------------------------
  auto ptr_at = [&](const DevBuf& b, size_t off) { return (void*)(static_cast<unsigned char*>(b.p) + off * e); };
  std::vector<int> nelist;  // occupied tiles of every scatter task, packed
  auto scat = [&](int p, int pc, const DevBuf& in, int coef, void* outp, int& tiles, int& fills) {
    BScatterTask T;
    memset(&T, 0, sizeof(T));
    ilm_grid_s g{probs[p].nx, probs[p].ny, probs[p].h, probs[p].i0x, probs[p].i0y};
    const Shape2 sh = g.shape(pc);
    const int dx = pc_dx(pc), dy = pc_dy(pc);
    const size_t o = B->poff[p];
    T.n1 = sh.n1;
    T.n2 = sh.n2;
    T.ntx = ntx[pc][p];
    // cells written: the source box (faces: one more column / row, which the
    // divergence of the box reads)
    const int ext = pc == PC_P ? 0 : 1;
    const int xa = std::min(box[p][0], sh.n1 - 1), xb = std::min(box[p][1] + ext, sh.n1);
    const int ya = std::min(box[p][2], sh.n2 - 1), yb = std::min(box[p][3] + ext, sh.n2);
    T.tx0 = xa / SB_X;
    T.ty0 = ya / SB_Y;
    T.ntxb = (xb - 1) / SB_X - T.tx0 + 1;
    const int ntyb = (yb - 1) / SB_Y - T.ty0 + 1;
    T.xa = xa;
    T.xb = xb;
    T.ya = ya;
    T.yb = yb;
    T.fill0 = fills;
    fills += yb - ya;
    // occupied tiles of the box (ids into the problem's tile grid), packed
    const int* tp = htp[pc].data() + tpo[pc][p];
    T.pad_ = (int)nelist.size();  // offset into the packed list, resolved after upload
    for (int ty = T.ty0; ty < T.ty0 + ntyb; ++ty)
      for (int tx = T.tx0; tx < T.tx0 + T.ntxb; ++tx) {
        const int t = ty * T.ntx + tx;
        if (tp[t + 1] > tp[t]) nelist.push_back(t);
      }
    T.nne = (int)nelist.size() - T.pad_;
    T.tile0 = tiles;
    tiles += T.nne;
    T.tptr = B->tptr[pc].as<int>() + tpo[pc][p];
    T.tpts = B->tpts[pc].as<int>() + tso[pc][p];
    T.bx = B->bx[dx].as<int>() + o;
    T.by = B->by[dy].as<int>() + o;
    T.wx = static_cast<unsigned char*>(B->wx[dx].p) + o * NTAP * e;
    T.wy = static_cast<unsigned char*>(B->wy[dy].p) + o * NTAP * e;
    T.wsc = ptr_at(B->wsc, o);
    T.nx = ptr_at(B->nx, o);
    T.ny = ptr_at(B->ny, o);
    T.in = ptr_at(in, o);
    T.coef = coef;
    T.out = outp;
    return T;
  };
  auto edge_u = [&](int p) { return ptr_at(B->edges, eoff[p]); };
  auto edge_v = [&](int p) { return ptr_at(B->edges, eoff[p] + (size_t)probs[p].nx * (probs[p].ny - 1)); };
  auto field = [&](const DevBuf& b, int p) { return ptr_at(b, B->foff[p]); };
  // divergence Edges -> Nodes{Primal} over the source box
  auto stencil = [&](int p, const void* in, void* outp, int& blks) {
    BStencilTask T;
    T.NX = probs[p].nx;
    T.NY = probs[p].ny;
    T.blk0 = blks;
    T.i0 = box[p][0];
    T.bw = box[p][1] - box[p][0];
    T.j0 = box[p][2];
    T.bh = box[p][3] - box[p][2];
    blks += ((T.bw + SB_X - 1) / SB_X) * ((T.bh + SB_Y - 1) / SB_Y);
    T.in = in;
    T.out = outp;
    T.scale = 1.0 / probs[p].h;
    return T;
  };
  auto gath = [&](int p, int& pts) {
    BGatherTask G;
    memset(&G, 0, sizeof(G));
    const size_t o = B->poff[p];
    G.npts = probs[p].npts;
    G.pt0 = pts;
    pts += G.npts;
    for (int d = 0; d < 2; ++d) {
      G.bx[d] = B->bx[d].as<int>() + o;
      G.by[d] = B->by[d].as<int>() + o;
      G.wx[d] = static_cast<unsigned char*>(B->wx[d].p) + o * NTAP * e;
      G.wy[d] = static_cast<unsigned char*>(B->wy[d].p) + o * NTAP * e;
    }
    G.nx = ptr_at(B->nx, o);
    G.ny = ptr_at(B->ny, o);
    G.out = ptr_at(B->g, o);
    return G;
  };
  std::vector<BScatterTask> sA, sB;
  std::vector<BStencilTask> dA, dB;
  std::vector<BGatherTask> hA;
  int tA = 0, tB = 0, bdA = 0, bdB = 0, ptsA = 0;
  int fillA = 0, fillB = 0;
  for (int p = 0; p < nprob; ++p) {
    const int nx_ = probs[p].nx, ny_ = probs[p].ny;
    if (probs[p].kind == 0) {  // Dirichlet: f* = L^-1 D_s [f]; correction R s
      sA.push_back(scat(p, PC_U, B->jump, CF_NX, edge_u(p), tA, fillA));
      sA.push_back(scat(p, PC_V, B->jump, CF_NY, edge_v(p), tA, fillA));
      dA.push_back(stencil(p, edge_u(p), field(B->fstar, p), bdA));
      BGatherTask G = gath(p, ptsA);
      G.nterms = 1;
      G.arr[0] = field(B->fstar, p);
      G.n1[0] = nx_ - 1;
      G.n2[0] = ny_ - 1;
      G.xs[0] = 0;
      G.ys[0] = 0;
      G.coef[0] = CF_ONE;
      G.scale = 1.0;
      hA.push_back(G);
      sB.push_back(scat(p, PC_P, B->s, CF_ONE, field(B->corr, p), tB, fillB));
    } else {  // Neumann: f* = L^-1 R [vn]; rhs from G_s f* (gradient fused into the gather); correction D_s [phi]
      sA.push_back(scat(p, PC_P, B->jump, CF_ONE, field(B->fstar, p), tA, fillA));
      BGatherTask G = gath(p, ptsA);
      G.nterms = 2;
      G.arr[0] = field(B->fstar, p);
      G.gmode[0] = 1;
      G.n1[0] = nx_;
      G.n2[0] = ny_ - 1;
      G.xs[0] = 1;
      G.ys[0] = 0;
      G.coef[0] = CF_NX;
      G.arr[1] = field(B->fstar, p);
      G.gmode[1] = 2;
      G.n1[1] = nx_ - 1;
      G.n2[1] = ny_;
      G.xs[1] = 0;
      G.ys[1] = 1;
      G.coef[1] = CF_NY;
      G.scale = 1.0 / probs[p].h;
      hA.push_back(G);
      sB.push_back(scat(p, PC_U, B->s, CF_NX, edge_u(p), tB, fillB));
      sB.push_back(scat(p, PC_V, B->s, CF_NY, edge_v(p), tB, fillB));
      dB.push_back(stencil(p, edge_u(p), field(B->corr, p), bdB));
    }
  }
  B->n_scatA = (int)sA.size();
  B->blk_scatA = tA;
  B->n_scatB = (int)sB.size();
  B->blk_scatB = tB;
  B->n_divA = (int)dA.size();
  B->blk_divA = bdA;
  B->n_divB = (int)dB.size();
  B->blk_divB = bdB;
  B->n_gathA = (int)hA.size();
  TA.add(&B->scat_ne, nelist);
  B->blk_fillA = fillA;
  B->blk_fillB = fillB;
  std::vector<int> maps[7];
  std::vector<BScatterTask> sB2;
  std::vector<BStencilTask> dB2;
  {
    // block -> task maps
    auto mk_scat = [&](const std::vector<BScatterTask>& v, int nblk, bool fill) {
      std::vector<int> m(std::max(nblk, 1), 0);
      for (size_t t = 0; t < v.size(); ++t) {
        const int b0 = fill ? v[t].fill0 : v[t].tile0;
        const int nb = fill ? v[t].yb - v[t].ya : v[t].nne;
        for (int k = 0; k < nb; ++k) m[b0 + k] = (int)t;
      }
      return m;
    };
    auto mk_div = [&](const std::vector<BStencilTask>& v, int nblk) {
      std::vector<int> m(std::max(nblk, 1), 0);
      for (size_t t = 0; t < v.size(); ++t) {
        const int nb = ((v[t].bw + SB_X - 1) / SB_X) * ((v[t].bh + SB_Y - 1) / SB_Y);
        for (int k = 0; k < nb; ++k) m[v[t].blk0 + k] = (int)t;
      }
      return m;
    };
    maps[0] = mk_scat(sA, fillA, true);
    maps[1] = mk_scat(sA, tA, false);
    maps[2] = mk_scat(sB, fillB, true);
    maps[3] = mk_scat(sB, tB, false);
    maps[4] = mk_div(dA, bdA);
    maps[5] = mk_div(dB, bdB);
    DevBuf* dst[6] = {&B->mfillA, &B->mscatA, &B->mfillB, &B->mscatB, &B->mdivA, &B->mdivB};
    for (int k = 0; k < 6; ++k) TA.add(dst[k], maps[k]);
  }
  TA.add(&B->scatA, sA);
  TA.add(&B->scatB, sB);
  TA.add(&B->divA, dA);
  TA.add(&B->divB, dB);
  {
    // stage-B tasks of the rhs-operator path: the single layer (Dirichlet
    // R s) and the divergence of the double layer (Neumann D_s [phi]) add
    // into f*'s source (same per-problem offset in fstar as in corr); only
    // the Neumann edge scatters still zero their boxes
    auto in_corr = [&](const void* q) {
      const unsigned char* c0 = static_cast<const unsigned char*>(B->corr.p);
      const unsigned char* c = static_cast<const unsigned char*>(q);
      return c >= c0 && c < c0 + B->ftot * e;
    };
    auto to_fstar = [&](void* q) {
      return (void*)(static_cast<unsigned char*>(B->fstar.p) + (static_cast<unsigned char*>(q) -
                                                                 static_cast<unsigned char*>(B->corr.p)));
    };
    sB2 = sB;
    int fill2 = 0;
    for (auto& T : sB2) {
      if (in_corr(T.out)) {
        T.out = to_fstar(T.out);
        T.accum = 1;
        T.fill0 = 0;
      } else {
        T.fill0 = fill2;
        fill2 += T.yb - T.ya;
      }
    }
    std::vector<int>& m2 = maps[6];
    m2.assign(std::max(fill2, 1), 0);
    for (size_t t = 0; t < sB2.size(); ++t)
      if (!sB2[t].accum)
        for (int k = 0; k < sB2[t].yb - sB2[t].ya; ++k) m2[sB2[t].fill0 + k] = (int)t;
    dB2 = dB;
    for (auto& T : dB2) {
      T.out = to_fstar(T.out);
      T.accum = 1;
    }
    B->blk_fillB2 = fill2;
    TA.add(&B->mfillB2, m2);
    TA.add(&B->scatB2, sB2);
    TA.add(&B->divB2, dB2);
  }
  TA.add(&B->gathA, hA);
  // lay out the arena, resolve the device addresses the tables hold, copy
  ILM_TRY(TA.commit_layout(B->arena_tasks));
  for (auto* v : {&sA, &sB, &sB2})
    for (auto& T : *v) T.ne = B->scat_ne.as<int>() + T.pad_;
  if (B->convL.fast)
    for (int k = 0; k < 3; ++k) B->convL.dmap[k] = B->mconv[k].as<int>();
  ILM_TRY(TA.commit_upload(B->arena_tasks, sg));

  phase("stage tasks (build and upload)");
  ILM_CHECK_CUDA(cudaStreamSynchronize(sg));
  if (build_schur) {
    // the Schur build runs on past the return (its stream is released once
    // the build ends); the launches that read S wait for this event
    ILM_CHECK_CUDA(cudaEventCreateWithFlags(&B->schur_ready, cudaEventDisableTiming));
    ILM_CHECK_CUDA(cudaEventRecord(B->schur_ready, ss));
  }
  *out = guard.release();
  return ILM_OK;
}

// r = b - y per problem, with |r|^2 and |b|^2 (one block per problem, fixed
// reduction order)
__global__ void __launch_bounds__(256) k_ref_residual(const size_t* __restrict__ poff, const double* __restrict__ bv,
                                                      const double* __restrict__ y, double* __restrict__ r,
                                                      double* __restrict__ norms) {
  __shared__ double sr[256], sb[256];
  const int p = blockIdx.x;
  const size_t o = poff[p];
  const int n = (int)(poff[p + 1] - o);
  double rr = 0.0, bb = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double bi = bv[o + i];
    const double ri = bi - y[o + i];
    r[o + i] = ri;
    rr += ri * ri;
    bb += bi * bi;
  }
  sr[threadIdx.x] = rr;
  sb[threadIdx.x] = bb;
  __syncthreads();
  for (int s2 = blockDim.x / 2; s2 > 0; s2 >>= 1) {
    if (threadIdx.x < s2) {
      sr[threadIdx.x] += sr[threadIdx.x + s2];
      sb[threadIdx.x] += sb[threadIdx.x + s2];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    norms[2 * p] = sr[0];
    norms[2 * p + 1] = sb[0];
  }
}

// The FP64 copy of an FP32 batch used by the refinement (built on first use)
int ensure_twin(ilm_batch_s* b) {
  if (b->twin) return ILM_OK;
  ilm_batch_t t = nullptr;
  ILM_TRY(batch_create_impl(b->nprob, b->probs.data(), b->hx.data(), b->hy.data(), b->hnx.data(), b->hny.data(),
                            b->hds.data(), b->ddf, ILM_F64, false, &t));
  b->twin = t;
  return ILM_OK;
}

}  // namespace

extern "C" {

int ilm_batch_create(int nprob, const ilm_batch_problem_t* probs, const double* x, const double* y,
                     const double* nrmx, const double* nrmy, const double* ds, int ddf, int dtype, ilm_batch_t* out) {
  return batch_create_impl(nprob, probs, x, y, nrmx, nrmy, ds, ddf, dtype, true, out);
}

int ilm_batch_destroy(ilm_batch_t b) {
  delete b;
  return ILM_OK;
}

int ilm_batch_layout(ilm_batch_t b, size_t* field_offsets, size_t* point_offsets) {
  ILM_REQUIRE(b, "null batch");
  for (int p = 0; p <= b->nprob; ++p) {
    if (field_offsets) field_offsets[p] = b->foff[p];
    if (point_offsets) point_offsets[p] = b->poff[p];
  }
  return ILM_OK;
}

int ilm_batch_solve(ilm_batch_t b, const void* fplus, const void* fminus, void* f_out, void* s_out, double tol,
                    int maxiter, ilm_stream_t stream) {
  ILM_REQUIRE(b && fplus && fminus && f_out && s_out, "batch_solve: null argument");
  ILM_REQUIRE(tol > 0 && maxiter > 0, "batch_solve: bad tolerance / iteration limit");
  cudaStream_t st = as_stream(stream);
  // new CG parameters (and, for the first solve, the lazy set-up on the
  // set-up stream) are prepared after stage A is issued, so the set-up
  // kernels overlap stage A; the stream is drained first so that no earlier
  // solve still reads the parameters that get replaced
  const bool rebuild = !(tol == b->cg_tol && maxiter == b->cg_maxiter && !b->params_dirty);
  if (rebuild) {
    ILM_CHECK_CUDA(cudaStreamSynchronize(st));
    ILM_TRY(prepare_lazy_setup(b));
  }
  b->nev = 0;
  b->launches = 0;
  ILM_TRY(batch_mark(b, st));
  ILM_TRY(batch_stage_a(b, fplus, fminus, st));
  ILM_TRY(ensure_cg_params(b, tol, maxiter));
  ILM_TRY(batch_cg(b, st));
  ILM_TRY(st_convert(b->Ptot, ILM_F64, b->x64.p, b->dtype, s_out, st));
  ILM_CHECK_CUDA(cudaMemcpyAsync(b->s.p, s_out, (size_t)b->Ptot * es(b->dtype), cudaMemcpyDeviceToDevice, st));
  b->launches += 1;
  ILM_TRY(batch_mark(b, st));  // 7: convert
  return batch_stage_b(b, f_out, st);
}

// FP64 iterative refinement of a batched solve.  The batch's own pipeline
// (FP32 grid work for an FP32 batch) gives the first surface strengths; the
// Schur right-hand side is then formed in FP64 by an FP64 copy of the
// pipeline, and every refinement step forms the FP64 Schur residual
// r = b - S x (float-float S, FP64 sums), solves S d = r with the batch's
// preconditioned CG to kRefineInnerTol and adds d in FP64, until every
// problem's |r| / |b| <= tol or max_refine steps are taken.  The field is
// assembled from the refined strengths by the FP64 pipeline.
int ilm_batch_solve_refined(ilm_batch_t b, const double* fplus, const double* fminus, double* f_out, double* s_out,
                            double tol, int maxiter, int max_refine, ilm_stream_t stream) {
  constexpr double kRefineFirstTol = 1e-8;  // first (bulk-precision) solve
  constexpr double kRefineInnerTol = 1e-6;  // each correction solve, relative to its residual
  ILM_REQUIRE(b && fplus && fminus && f_out && s_out, "batch_solve_refined: null argument");
  ILM_REQUIRE(tol > 0 && maxiter > 0 && max_refine >= 0 && max_refine <= 100,
              "batch_solve_refined: bad tolerance / iteration limit / refinement steps");
  cudaStream_t st = as_stream(stream);
  const int Ptot = b->Ptot, np = b->nprob;
  ilm_batch_s* T64 = b;
  if (b->dtype != ILM_F64) {
    ILM_TRY(ensure_twin(b));
    T64 = b->twin;
  }
  const size_t pv = (size_t)std::max(Ptot, 1) * sizeof(double);
  ILM_TRY(b->ref_b.alloc(pv));
  ILM_TRY(b->ref_x.alloc(pv));
  ILM_TRY(b->ref_r.alloc(pv));
  ILM_TRY(b->ref_y.alloc(pv));
  ILM_TRY(b->ref_norm.alloc((size_t)2 * np * sizeof(double)));
  if (!b->dpoff.p) ILM_TRY(up(b->dpoff, b->poff));
  if (!b->dsoff.p) ILM_TRY(up(b->dsoff, b->soff));
  b->nev = 0;
  b->launches = 0;
  // first solve in the batch's precision, and the FP64 right-hand side
  ILM_TRY(ensure_cg_params(b, std::max(tol, kRefineFirstTol), maxiter));
  if (b->dtype == ILM_F64) {
    ILM_TRY(batch_stage_a(b, fplus, fminus, st));
  } else {
    ILM_TRY(b->ref_in.alloc((size_t)2 * std::max(Ptot, 1) * es(b->dtype)));
    void* in_p = b->ref_in.p;
    void* in_m = static_cast<unsigned char*>(b->ref_in.p) + (size_t)Ptot * es(b->dtype);
    ILM_TRY(st_convert(Ptot, ILM_F64, fplus, b->dtype, in_p, st));
    ILM_TRY(st_convert(Ptot, ILM_F64, fminus, b->dtype, in_m, st));
    ILM_TRY(batch_stage_a(b, in_p, in_m, st));
    T64->nev = 0;
    ILM_TRY(batch_stage_a(T64, fplus, fminus, st));
  }
  ILM_CHECK_CUDA(cudaMemcpyAsync(b->ref_b.p, T64->rhs64.p, (size_t)Ptot * 8, cudaMemcpyDeviceToDevice, st));
  ILM_TRY(batch_cg(b, st));
  ILM_CHECK_CUDA(cudaMemcpyAsync(b->ref_x.p, b->x64.p, (size_t)Ptot * 8, cudaMemcpyDeviceToDevice, st));
  std::vector<int> its(np, 0), it1(np);
  std::vector<double> rel(np, 0.0), nrm(2 * (size_t)np);
  auto add_iters = [&]() -> int {
    ILM_CHECK_CUDA(cudaMemcpyAsync(it1.data(), b->iters.p, (size_t)np * sizeof(int), cudaMemcpyDeviceToHost, st));
    ILM_CHECK_CUDA(cudaStreamSynchronize(st));
    for (int p = 0; p < np; ++p) its[p] += it1[p];
    return ILM_OK;
  };
  ILM_TRY(add_iters());
  for (int k = 0;; ++k) {
    // FP64 Schur residual of every problem
    if (Ptot > 0)
      k_batch_schur_apply<<<(Ptot * 32 + 255) / 256, 256, 0, st>>>(Ptot, b->pt2prob.as<int>(), b->dpoff.as<size_t>(),
                                                                   b->Shi.as<float>(), b->Slo.as<float>(),
                                                                   b->dsoff.as<size_t>(), b->ref_x.as<double>(),
                                                                   b->ref_y.as<double>());
    ILM_CHECK_LAUNCH();
    k_ref_residual<<<np, 256, 0, st>>>(b->dpoff.as<size_t>(), b->ref_b.as<double>(), b->ref_y.as<double>(),
                                       b->ref_r.as<double>(), b->ref_norm.as<double>());
    ILM_CHECK_LAUNCH();
    b->launches += 2;
    ILM_CHECK_CUDA(cudaMemcpyAsync(nrm.data(), b->ref_norm.p, nrm.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                   st));
    ILM_CHECK_CUDA(cudaStreamSynchronize(st));
    double worst = 0.0;
    for (int p = 0; p < np; ++p) {
      rel[p] = nrm[2 * p + 1] > 0.0 ? std::sqrt(nrm[2 * p] / nrm[2 * p + 1]) : 0.0;
      worst = std::max(worst, rel[p]);
    }
    if (worst <= tol || k >= max_refine) break;
    // correction: S d = r (FP64 vectors, float-float S), x += d
    ILM_TRY(ensure_cg_params(b, kRefineInnerTol, maxiter));
    ILM_CHECK_CUDA(cudaMemcpyAsync(b->rhs64.p, b->ref_r.p, (size_t)Ptot * 8, cudaMemcpyDeviceToDevice, st));
    ILM_TRY(batch_cg(b, st));
    ILM_TRY(st_axpby(Ptot, ILM_F64, 1.0, b->ref_x.p, 1.0, b->x64.p, b->ref_x.p, st));
    b->launches += 1;
    ILM_TRY(add_iters());
  }
  // outputs: the refined strengths and the FP64 field assembled from them
  ILM_CHECK_CUDA(cudaMemcpyAsync(s_out, b->ref_x.p, (size_t)Ptot * 8, cudaMemcpyDeviceToDevice, st));
  ILM_CHECK_CUDA(cudaMemcpyAsync(T64->s.p, b->ref_x.p, (size_t)Ptot * 8, cudaMemcpyDeviceToDevice, st));
  T64->nev = 0;
  ILM_TRY(batch_stage_b(T64, f_out, st));
  if (T64 != b) b->launches += T64->launches;
  // per-problem totals for ilm_batch_info: CG iterations of all solves, final FP64 residual
  ILM_CHECK_CUDA(cudaMemcpyAsync(b->iters.p, its.data(), (size_t)np * sizeof(int), cudaMemcpyHostToDevice, st));
  ILM_CHECK_CUDA(cudaMemcpyAsync(b->relres.p, rel.data(), (size_t)np * sizeof(double), cudaMemcpyHostToDevice, st));
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  return ILM_OK;
}

int ilm_batch_set_precond(ilm_batch_t b, int mode, int block_size) {
  ILM_REQUIRE(b, "null batch");
  ILM_REQUIRE(mode == 0 || mode == 1 || mode == 2, "batch: unknown preconditioner %d", mode);
  ILM_REQUIRE(mode != 2 || b->band_k >= 0, "batch: no learned preconditioner set (ilm_batch_set_learned)");
  if (mode == 1) {
    ILM_REQUIRE(block_size >= 4 && block_size <= 72, "batch: block size %d outside [4, 72]", block_size);
    if (b->bj_block != block_size) {
      // inverses still being formed write into the arrays rebuilt here
      if (b->bj_ready) ILM_CHECK_CUDA(cudaEventSynchronize(b->bj_ready));
      // blocks of ~block_size consecutive points (at most 1.5 x block_size);
      // their inverses are formed by the next solve, for the problems whose
      // preconditioner uses them (ensure_block_inverses)
      std::vector<int> blk(b->Ptot), bst, bsz, boff;
      b->bj_tasks_host.clear();
      b->bj_first.assign(b->nprob + 1, 0);
      size_t total = 0;
      int max_sz = 1;
      for (int p = 0; p < b->nprob; ++p) {
        const int n = b->probs[p].npts;
        const int nb = std::max(1, (int)lround((double)n / block_size));
        b->bj_first[p] = (int)bst.size();
        for (int k = 0; k < nb; ++k) {
          const int s = (int)((long long)n * k / nb), e = (int)((long long)n * (k + 1) / nb);
          for (int j = s; j < e; ++j) blk[b->poff[p] + j] = k;
          bst.push_back(s);
          bsz.push_back(e - s);
          boff.push_back((int)total);
          max_sz = std::max(max_sz, e - s);
          BJBlockTask T;
          T.Shi = b->Shi.as<float>() + b->soff[p];
          T.Slo = b->Slo.as<float>() + b->soff[p];
          T.n = n;
          T.s = s;
          T.sz = e - s;
          T.out_hi = T.out_lo = nullptr;  // set after allocation
          b->bj_tasks_host.push_back(T);
          total += (size_t)(e - s) * (e - s);
        }
      }
      b->bj_first[b->nprob] = (int)bst.size();
      ILM_REQUIRE(max_sz <= 144, "batch: preconditioner block of %d points", max_sz);
      ILM_TRY(b->bj_inv.alloc(std::max<size_t>(total, 1) * sizeof(float)));
      ILM_TRY(b->bj_inv_lo.alloc(std::max<size_t>(total, 1) * sizeof(float)));
      for (size_t t = 0; t < b->bj_tasks_host.size(); ++t) {
        b->bj_tasks_host[t].out_hi = b->bj_inv.as<float>() + boff[t];
        b->bj_tasks_host[t].out_lo = b->bj_inv_lo.as<float>() + boff[t];
      }
      ILM_TRY(up(b->bj_blk, blk));
      ILM_TRY(up(b->bj_start, bst));
      ILM_TRY(up(b->bj_size, bsz));
      ILM_TRY(up(b->bj_off, boff));
      b->bj_max_sz = max_sz;
      b->bj_have.assign(b->nprob, 0);
      b->bj_block = block_size;
    }
  }
  b->precond = mode;
  b->params_dirty = true;
  // the learned mode fixes which problems need block inverses (those without
  // a network): issue them now, on their own stream, so that they form while
  // the caller prepares the first solve
  if (mode == 2 && b->bj_block > 0) ILM_TRY(ensure_block_inverses(b));
  return ILM_OK;
}

int ilm_batch_set_profiling(ilm_batch_t b, int enable) {
  ILM_REQUIRE(b, "null batch");
  const int e = enable ? 1 : 0;
  if (e && !b->cgtime.p) {
    ILM_TRY(b->cgtime.alloc((size_t)b->nprob * 3 * sizeof(unsigned long long)));
    ILM_CHECK_CUDA(cudaMemset(b->cgtime.p, 0, (size_t)b->nprob * 3 * sizeof(unsigned long long)));
  }
  if (e != b->profiling) b->params_dirty = true;
  b->profiling = e;
  return ILM_OK;
}

int ilm_batch_set_rhs_operator(ilm_batch_t b, int enable) {
  ILM_REQUIRE(b, "null batch");
  if (enable && !b->rhs_op_ready && b->Ptot > 0) {
    // full-tile numbering of every problem's n x n operator
    std::vector<SchurProbDev> sp = b->schur_host;
    int tiles = 0;
    for (auto& P : sp) {
      const int nt = (P.n + 15) / 16;
      P.tile0 = tiles;
      tiles += nt * nt;
    }
    b->rhs_tiles = tiles;
    ILM_TRY(up(b->schurPfull, sp));
    ILM_TRY(b->Mhi.alloc(std::max<size_t>(b->stot, 1) * 4));
    ILM_TRY(b->Mlo.alloc(std::max<size_t>(b->stot, 1) * 4));
    // set-up work on a stream of its own (not the legacy stream, which
    // would wait for and block every other stream of the device)
    cudaStream_t st = nullptr;
    ILM_CHECK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
      cudaStream_t s;
      ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{st};
    ILM_CHECK_CUDA(cudaMemsetAsync(b->Mhi.p, 0, std::max<size_t>(b->stot, 1) * 4, st));
    ILM_CHECK_CUDA(cudaMemsetAsync(b->Mlo.p, 0, std::max<size_t>(b->stot, 1) * 4, st));
    ILM_TRY(b->FU.alloc((size_t)b->Ptot * functional_size()));
    ILM_TRY(b->FD.alloc((size_t)b->Ptot * functional_size()));
    BatchWin BW;
    for (int d = 0; d < 2; ++d) {
      BW.bx[d] = b->bx[d].as<int>();
      BW.by[d] = b->by[d].as<int>();
      BW.wx64[d] = b->wx64[d].as<double>();
      BW.wy64[d] = b->wy64[d].as<double>();
    }
    BW.nx64 = b->nx64.as<double>();
    BW.ny64 = b->ny64.as<double>();
    ILM_TRY(rhsop_build_batched(b->nprob, b->schurPfull.as<SchurProbDev>(), tiles, b->Ptot, b->pt2prob.as<int>(), BW,
                                b->ds64.as<double>(), static_cast<Functional*>(b->FU.p),
                                static_cast<Functional*>(b->FD.p), b->Mhi.as<float>(), b->Mlo.as<float>(),
                                b->max_grid, st));
    ILM_CHECK_CUDA(cudaStreamSynchronize(st));
    b->rhs_op_ready = true;
  }
  if (b->rhs_op != (enable != 0)) b->param_gen++;
  b->rhs_op = enable != 0;
  return ILM_OK;
}

int ilm_batch_set_cg_variant(ilm_batch_t b, int variant) {
  ILM_REQUIRE(b, "null batch");
  ILM_REQUIRE(variant >= 0 && variant <= ILM_CG_VARIANTS, "batch: unknown CG variant %d", variant);
  b->cg_variant = variant;
  b->nclusters = cg_cluster_count(b->nprob, b->maxN, variant);
  if (variant == 6) ILM_TRY(ensure_split(b));  // queues and stream built here, outside any stream capture
  b->param_gen++;
  return ILM_OK;
}

// The whole solve as one CUDA graph launch: the first call for a set of
// buffers / tolerance / CG configuration captures ilm_batch_solve on the
// stream (every per-problem descriptor already lives in device memory, so
// the sequence is fixed) and later calls replay it.  The CG parameter table
// is rebuilt before the capture, outside it.
int ilm_batch_solve_graph(ilm_batch_t b, const void* fplus, const void* fminus, void* f_out, void* s_out,
                          double tol, int maxiter, ilm_stream_t stream) {
  ILM_REQUIRE(b && fplus && fminus && f_out && s_out, "batch_solve_graph: null argument");
  ILM_REQUIRE(tol > 0 && maxiter > 0, "batch_solve_graph: bad tolerance / iteration limit");
  cudaStream_t st = as_stream(stream);
  ILM_REQUIRE(st != nullptr, "batch_solve_graph: needs a created stream (the legacy default stream cannot be captured)");
  ILM_TRY(ensure_cg_params(b, tol, maxiter));
  ILM_TRY(wait_schur_host(b));
  for (cudaEvent_t e : {b->bj_ready, b->band_ready, b->coarse_ready})
    if (e) ILM_CHECK_CUDA(cudaEventSynchronize(e));
  const void* key[4] = {fplus, fminus, f_out, s_out};
  bool reuse = b->gexec && b->gtol == tol && b->gmaxiter == maxiter && b->ggen == b->param_gen;
  for (int i = 0; i < 4 && reuse; ++i) reuse = key[i] == b->gkey[i];
  if (!reuse) {
    if (b->gexec) {
      cudaGraphExecDestroy(b->gexec);
      b->gexec = nullptr;
    }
    const int prof = b->profiling;
    b->profiling = 0;
    ILM_CHECK_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    const int rc = ilm_batch_solve(b, fplus, fminus, f_out, s_out, tol, maxiter, stream);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    b->profiling = prof;
    if (rc != ILM_OK || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (rc != ILM_OK) return rc;
      set_error("batch_solve_graph: stream capture failed: %s", cudaGetErrorString(e));
      return ILM_ERR_CUDA;
    }
    const cudaError_t ei = cudaGraphInstantiate(&b->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
      b->gexec = nullptr;
      set_error("batch_solve_graph: graph instantiation failed: %s", cudaGetErrorString(ei));
      return ILM_ERR_CUDA;
    }
    for (int i = 0; i < 4; ++i) b->gkey[i] = key[i];
    b->gtol = tol;
    b->gmaxiter = maxiter;
    b->ggen = b->param_gen;
  }
  ILM_CHECK_CUDA(cudaGraphLaunch(b->gexec, st));
  return ILM_OK;
}

int ilm_batch_get_cg_variant(ilm_batch_t b, int* variant, int* nclusters) {
  ILM_REQUIRE(b && variant && nclusters, "null argument");
  *variant = b->cg_variant;
  *nclusters = b->nclusters;
  return ILM_OK;
}

// Autotuner: every candidate Schur CG kernel solves the given data once
// untimed (plans, deflation set-up) and `reps` times timed with CUDA events
// on the stream; the fastest is kept.  Candidates whose shared-memory layout
// does not fit are skipped.
int ilm_batch_autotune(ilm_batch_t b, const void* fplus, const void* fminus, void* f_out, void* s_out, double tol,
                       int maxiter, int reps, ilm_stream_t stream, int* chosen, float* ms_per_variant) {
  ILM_REQUIRE(b && reps >= 1, "batch_autotune: bad arguments");
  cudaStream_t st = as_stream(stream);
  cudaEvent_t e0, e1;
  ILM_CHECK_CUDA(cudaEventCreate(&e0));
  ILM_CHECK_CUDA(cudaEventCreate(&e1));
  const int old_prof = b->profiling;
  b->profiling = 0;
  int best = 0;
  float best_ms = 0.f;
  int rc = ILM_OK;
  for (int v = 1; v <= ILM_CG_VARIANTS && rc == ILM_OK; ++v) {
    if (ms_per_variant) ms_per_variant[v - 1] = -1.f;
    if (v == 2 && cg_rep_smem(b->maxN) > 200 * 1024) continue;
    if (v != 2 && cg_variant_smem(b->maxN, v) > 200 * 1024) continue;
    if ((rc = ilm_batch_set_cg_variant(b, v)) != ILM_OK) break;
    if ((rc = ilm_batch_solve(b, fplus, fminus, f_out, s_out, tol, maxiter, stream)) != ILM_OK) {
      // a variant the device refuses to launch (cluster size, shared memory)
      // is skipped; the default variant must run
      if (v == 1 || rc != ILM_ERR_CUDA || cudaStreamSynchronize(st) != cudaSuccess) break;
      (void)cudaGetLastError();
      rc = ILM_OK;
      continue;
    }
    // each timed solve between its own events, the least kept (a solve that
    // waited for the host's launches does not decide the choice)
    float ms = -1.f;
    for (int k = 0; k < reps && rc == ILM_OK; ++k) {
      if (cudaEventRecord(e0, st) != cudaSuccess) {
        rc = ILM_ERR_CUDA;
        break;
      }
      if ((rc = ilm_batch_solve(b, fplus, fminus, f_out, s_out, tol, maxiter, stream)) != ILM_OK) break;
      float mk = 0.f;
      if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&mk, e0, e1) != cudaSuccess) {
        rc = ILM_ERR_CUDA;
        break;
      }
      if (ms < 0.f || mk < ms) ms = mk;
    }
    if (rc != ILM_OK) break;
    if (ms_per_variant) ms_per_variant[v - 1] = ms;
    if (best == 0 || ms < best_ms) {
      best = v;
      best_ms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->profiling = old_prof;
  if (rc != ILM_OK) return rc;
  ILM_TRY(ilm_batch_set_cg_variant(b, best));
  if (chosen) *chosen = best;
  return ILM_OK;
}

int ilm_batch_cg_times(ilm_batch_t b, double* start_us, double* end_us, int* sm) {
  ILM_REQUIRE(b && start_us && end_us && sm, "null argument");
  ILM_REQUIRE(b->cgtime.p, "batch: profiling was never enabled");
  std::vector<unsigned long long> t((size_t)b->nprob * 3);
  ILM_CHECK_CUDA(cudaMemcpy(t.data(), b->cgtime.p, t.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  unsigned long long t0 = ~0ull;
  for (int p = 0; p < b->nprob; ++p) t0 = std::min(t0, t[3 * p]);
  for (int p = 0; p < b->nprob; ++p) {
    start_us[p] = 1e-3 * (double)(t[3 * p] - t0);
    end_us[p] = 1e-3 * (double)(t[3 * p + 1] - t0);
    sm[p] = (int)t[3 * p + 2];
  }
  return ILM_OK;
}

int ilm_batch_stage_times(ilm_batch_t b, float* ms, int* nstages, int* launches) {
  ILM_REQUIRE(b, "null batch");
  const int n = b->nev > 0 ? b->nev - 1 : 0;
  if (nstages) *nstages = n;
  if (launches) *launches = b->launches;
  if (ms && n > 0) {
    ILM_CHECK_CUDA(cudaEventSynchronize(b->ev[b->nev - 1]));
    for (int i = 0; i < n; ++i) ILM_CHECK_CUDA(cudaEventElapsedTime(&ms[i], b->ev[i], b->ev[i + 1]));
  }
  return ILM_OK;
}

int ilm_batch_setup_times(ilm_batch_t b, double* ms, int max_phases, int* nphases, const char** names) {
  ILM_REQUIRE(b && nphases, "batch_setup_times: null argument");
  const int n = (int)b->setup_ms.size();
  *nphases = n;
  for (int k = 0; k < std::min(n, max_phases); ++k) {
    if (ms) ms[k] = b->setup_ms[k].second;
    if (names) names[k] = b->setup_ms[k].first;
  }
  return ILM_OK;
}

int ilm_batch_stats(ilm_batch_t b, double* stats) {
  ILM_REQUIRE(b && stats, "null argument");
  // total points, total Nodes{Primal} cells, sum of npts^2, sum over problems of
  // the padded FFT extent P1*P2, number of problems
  double p2 = 0.0, fft = 0.0;
  for (int p = 0; p < b->nprob; ++p) {
    const auto& P = b->probs[p];
    p2 += (double)P.npts * P.npts;
    fft += (double)good_fft_size(2 * (P.nx - 1) - 1) * good_fft_size(2 * (P.ny - 1) - 1);
  }
  stats[0] = b->Ptot;
  stats[1] = (double)b->ftot;
  stats[2] = p2;
  stats[3] = fft;
  stats[4] = b->nprob;
  stats[5] = (double)b->box_cells;
  return ILM_OK;
}

int ilm_batch_info(ilm_batch_t b, int* iterations, double* rel_residual) {
  ILM_REQUIRE(b, "null batch");
  if (iterations)
    ILM_CHECK_CUDA(cudaMemcpy(iterations, b->iters.p, (size_t)b->nprob * sizeof(int), cudaMemcpyDeviceToHost));
  if (rel_residual)
    ILM_CHECK_CUDA(cudaMemcpy(rel_residual, b->relres.p, (size_t)b->nprob * sizeof(double), cudaMemcpyDeviceToHost));
  return ILM_OK;
}

int ilm_batch_set_coarse(ilm_batch_t b, int kind_mask, const int* body_start) {
  ILM_REQUIRE(b, "null batch");
  ILM_REQUIRE(kind_mask >= 0 && kind_mask <= 2 && kind_mask != 1,
              "batch_set_coarse: kind mask %d (0 off, 2 Neumann)", kind_mask);
  constexpr int M = CG_COARSE_MAX, M1 = CG_COARSE_MAX + 1;
  b->coarse_nb.assign(b->nprob, 0);
  b->coarse_start.assign((size_t)b->nprob * M1, 0);
  b->params_dirty = true;
  if (kind_mask == 0) return ILM_OK;
  ILM_REQUIRE(body_start, "batch_set_coarse: null body starts");
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<CoarseTask> tasks;
  std::vector<int> tprob;
  for (int p = 0; p < b->nprob; ++p) {
    const int o = (int)b->poff[p], n = b->probs[p].npts;
    std::vector<int> st;
    for (int k = 0; k < n; ++k) {
      const int s = body_start[o + k];
      ILM_REQUIRE(s >= 0 && s <= k && (k == 0 ? s == 0 : (s == body_start[o + k - 1] || s == k)),
                  "batch_set_coarse: body starts of problem %d are not contiguous at point %d", p, k);
      if (s == k) st.push_back(k);
    }
    if (!((kind_mask >> b->probs[p].kind) & 1) || st.empty() || (int)st.size() > M) continue;
    CoarseTask T;
    T.Shi = b->Shi.as<float>() + b->soff[p];
    T.Slo = b->Slo.as<float>() + b->soff[p];
    T.w = b->ds64.as<double>() + o;
    T.n = n;
    T.nb = (int)st.size();
    for (int q = 0; q < M1; ++q) T.cst[q] = q < T.nb ? st[q] : n;
    tasks.push_back(T);
    tprob.push_back(p);
  }
  if (tasks.empty()) return ILM_OK;
  // E and E^-1 on the device, on the set-up stream after the Schur build; no
  // host synchronisation (the CG launches wait for coarse_ready).  The
  // buffers stay with the batch: freeing device memory would wait for the
  // whole device.
  const int nt = (int)tasks.size();
  ILM_TRY(ensure_setup_stream(b));
  cudaStream_t ss = b->s_setup;
  if (!b->coarse_ready) ILM_CHECK_CUDA(cudaEventCreateWithFlags(&b->coarse_ready, cudaEventDisableTiming));
  ILM_TRY(b->coarse_tasks.alloc((size_t)nt * sizeof(CoarseTask)));
  ILM_TRY(b->coarse_tprob.alloc((size_t)nt * sizeof(int)));
  ILM_TRY(b->coarse_part.alloc((size_t)nt * COARSE_SPLIT * M * M * sizeof(double)));
  ILM_TRY(b->coarse_Einv.alloc((size_t)b->nprob * M * M * sizeof(double)));
  // (from pageable memory: the copies have read the vectors when they return)
  ILM_CHECK_CUDA(cudaMemcpyAsync(b->coarse_tasks.p, tasks.data(), (size_t)nt * sizeof(CoarseTask),
                                 cudaMemcpyHostToDevice, ss));
  ILM_CHECK_CUDA(cudaMemcpyAsync(b->coarse_tprob.p, tprob.data(), (size_t)nt * sizeof(int), cudaMemcpyHostToDevice,
                                 ss));
  ILM_TRY(wait_schur_for(b, ss, tprob));
  k_coarse_E<<<(unsigned)(nt * COARSE_SPLIT), 256, 0, ss>>>(b->coarse_tasks.as<CoarseTask>(),
                                                            b->coarse_part.as<double>());
  ILM_CHECK_LAUNCH();
  k_coarse_inv<<<(nt + 127) / 128, 128, 0, ss>>>(nt, b->coarse_tasks.as<CoarseTask>(), b->coarse_tprob.as<int>(),
                                                 b->coarse_part.as<double>(), b->coarse_Einv.as<double>());
  ILM_CHECK_LAUNCH();
  ILM_CHECK_CUDA(cudaEventRecord(b->coarse_ready, ss));
  for (int t = 0; t < nt; ++t) {
    const int p = tprob[t];
    b->coarse_nb[p] = tasks[t].nb;
    for (int q = 0; q < M1; ++q) b->coarse_start[(size_t)p * M1 + q] = tasks[t].cst[q];
  }
  b->setup_ms.emplace_back("coarse correction (issued; E and E^-1 on the device)",
                           std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
  return ILM_OK;
}

int ilm_batch_set_learned(ilm_batch_t b, ilm_net_t net, int kind_mask, const int* body_start) {
  ILM_REQUIRE(b && net && body_start, "batch_set_learned: null argument");
  ILM_REQUIRE(kind_mask >= 1 && kind_mask <= 3, "batch_set_learned: kind mask %d (1 Dirichlet, 2 Neumann, 3 both)",
              kind_mask);
  ILM_REQUIRE(net_nfeat(net) == 8, "batch_set_learned: the network must read the 8 point features");
  const int K = net_band(net), P = 2 * K + 1;
  ILM_REQUIRE(b->band_k < 0 || b->band_k == K, "batch_set_learned: all networks of a batch must share the band width");
  ILM_REQUIRE(K >= 0 && K <= 8, "batch_set_learned: band half-width %d (at most 8)", K);
  const int Ptot = b->Ptot;
  std::vector<int> ls(Ptot), ll(Ptot), as(Ptot);
  for (int p = 0; p < b->nprob; ++p) {
    const int o = (int)b->poff[p], n = b->probs[p].npts;
    for (int k = 0; k < n; ++k) {
      const int s = body_start[o + k];
      ILM_REQUIRE(s >= 0 && s <= k && (k == 0 ? s == 0 : (s == body_start[o + k - 1] || s == k)),
                  "batch_set_learned: body starts of problem %d are not contiguous at point %d", p, k);
      ls[o + k] = s;
    }
    for (int k = 0; k < n;) {  // body lengths
      int e = k + 1;
      while (e < n && ls[o + e] == ls[o + k]) ++e;
      ILM_REQUIRE(e - k >= std::max(3, P), "batch_set_learned: body of %d points in problem %d (need >= %d)", e - k,
                  p, std::max(3, P));
      for (int q = k; q < e; ++q) {
        ll[o + q] = e - k;
        as[o + q] = o + k;
      }
      k = e;
    }
  }
  auto clk = std::chrono::steady_clock::now();
  auto phase = [&](const char* name) {
    const auto now = std::chrono::steady_clock::now();
    b->setup_ms.emplace_back(name, std::chrono::duration<double, std::milli>(now - clk).count());
    clk = now;
  };
  // the points of the problems of the selected kinds, compacted, with their
  // body segments in compacted indices
  std::vector<int> c2o, sst_c, sln_c;
  c2o.reserve(Ptot);
  if (b->band_k < 0) b->has_band.assign(b->nprob, 0);
  for (int p = 0; p < b->nprob; ++p) {
    if (!(kind_mask & (1 << b->probs[p].kind))) continue;
    b->has_band[p] = 1;
    const int o = (int)b->poff[p], base = (int)c2o.size();
    for (int k = 0; k < b->probs[p].npts; ++k) {
      c2o.push_back(o + k);
      sst_c.push_back(base + (as[o + k] - o));
      sln_c.push_back(ll[o + k]);
    }
  }
  const int Nsel = (int)c2o.size();
  // the set-up runs on its own stream, without host synchronisation: the CG
  // launches wait for band_ready, and the network's timeout flag is checked
  // before the first solve (check_band)
  if (!b->s_learn) ILM_CHECK_CUDA(cudaStreamCreateWithFlags(&b->s_learn, cudaStreamNonBlocking));
  if (!b->band_ready) ILM_CHECK_CUDA(cudaEventCreateWithFlags(&b->band_ready, cudaEventDisableTiming));
  cudaStream_t sl = b->s_learn;
  DevBuf d_c2o, d_sst, d_sln, dfeat, tmp;
  {
    // this call's temporaries, in an arena the batch keeps (freeing device
    // memory would wait for the whole device, the Schur build included)
    ArenaBuilder A;
    A.add(&d_c2o, c2o);
    A.add(&d_sst, sst_c);
    A.add(&d_sln, sln_c);
    A.add(&dfeat, (size_t)std::max(Nsel, 1) * 8 * sizeof(float));
    A.add(&tmp, (size_t)std::max(Nsel, 1) * P * sizeof(float));
    ILM_TRY(A.commit(b->arena_learned_tmp, sl));
    ArenaBuilder S;  // the body segments the CG reads (the same for every call)
    S.add(&b->lseg_start, ls);
    S.add(&b->lseg_len, ll);
    ILM_TRY(S.commit(b->arena_learned, sl));
    if (b->band_k < 0) ILM_TRY(b->band.alloc((size_t)std::max(Ptot, 1) * P * sizeof(float)));
  }
  phase("learned: segments (host) and upload");
  if (Nsel > 0) {
    k_batch_features<<<(Nsel + 255) / 256, 256, 0, sl>>>(Nsel, d_c2o.as<int>(), d_sst.as<int>(), d_sln.as<int>(),
                                                  b->px.as<double>(), b->py.as<double>(), b->nx64.as<double>(),
                                                  b->ny64.as<double>(), b->ds64.as<double>(), b->pt2prob.as<int>(),
                                                  b->ph.as<double>(), dfeat.as<float>());
    ILM_CHECK_LAUNCH();
    ILM_TRY(net_forward_packed(net, Nsel, dfeat.as<float>(), d_sst.as<int>(), d_sln.as<int>(), tmp.as<float>(),
                               sl));
    k_scatter_rows<<<std::min(4096, (Nsel * P + 255) / 256), 256, 0, sl>>>(Nsel, P, d_c2o.as<int>(), tmp.as<float>(),
                                                                            b->band.as<float>());
    ILM_CHECK_LAUNCH();
    if (int* flag = net_tc_flag(net)) {  // the timeout flag, moved into the batch
      ILM_TRY(b->band_err.alloc(sizeof(int)));
      ILM_CHECK_CUDA(cudaMemcpyAsync(b->band_err.p, flag, sizeof(int), cudaMemcpyDeviceToDevice, sl));
      ILM_CHECK_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), sl));
      b->band_check = true;
    }
  }
  ILM_CHECK_CUDA(cudaEventRecord(b->band_ready, sl));
  phase("learned: features and network inference (issued; device, selected problems)");
  b->band_k = K;
  b->precond = 2;
  b->params_dirty = true;
  return ILM_OK;
}

int ilm_batch_schur_apply(ilm_batch_t b, const double* x, double* y, ilm_stream_t stream) {
  ILM_REQUIRE(b && x && y, "batch_schur_apply: null argument");
  if (!b->dpoff.p) {
    ILM_TRY(up(b->dpoff, b->poff));
  }
  DevBuf dsoff;
  ILM_TRY(up(dsoff, b->soff));
  cudaStream_t st = as_stream(stream);
  ILM_TRY(wait_schur(b, st));
  k_batch_schur_apply<<<(b->Ptot * 32 + 255) / 256, 256, 0, st>>>(b->Ptot, b->pt2prob.as<int>(),
                                                                  b->dpoff.as<size_t>(), b->Shi.as<float>(),
                                                                  b->Slo.as<float>(), dsoff.as<size_t>(), x, y);
  ILM_CHECK_LAUNCH();
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  return ILM_OK;
}

int ilm_batch_schur_solve(ilm_batch_t b, const double* rhs, double* x, double tol, int maxiter,
                          ilm_stream_t stream) {
  ILM_REQUIRE(b && rhs && x, "batch_schur_solve: null argument");
  ILM_REQUIRE(tol > 0 && maxiter > 0, "batch_schur_solve: bad tolerance / iteration limit");
  cudaStream_t st = as_stream(stream);
  ILM_TRY(ensure_cg_params(b, tol, maxiter));
  ILM_CHECK_CUDA(cudaMemcpyAsync(b->rhs64.p, rhs, (size_t)b->Ptot * 8, cudaMemcpyDeviceToDevice, st));
  ILM_TRY(wait_schur(b, st));
  ILM_TRY(wait_precond(b, st));
  ILM_TRY(launch_cg_cluster(b->cgp.p, b->order.as<int>(), b->nprob, b->counter.as<int>(), b->maxN, b->nclusters, st,
                            b->cg_variant));
  ILM_CHECK_CUDA(cudaMemcpyAsync(x, b->x64.p, (size_t)b->Ptot * 8, cudaMemcpyDeviceToDevice, st));
  return ILM_OK;
}

}  // extern "C"
