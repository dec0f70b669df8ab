// Internal declarations shared by the libilm translation units.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ilm.h"

namespace ilm {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
void set_error(const char* fmt, ...);

#define ILM_CHECK_CUDA(expr)                                                     \
  do {                                                                           \
    cudaError_t _e = (expr);                                                     \
    if (_e != cudaSuccess) {                                                     \
      ::ilm::set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr,                \
                       cudaGetErrorString(_e));                                  \
      return ILM_ERR_CUDA;                                                       \
    }                                                                            \
  } while (0)

#define ILM_CHECK_LAUNCH() ILM_CHECK_CUDA(cudaGetLastError())

#define ILM_TRY(expr)                 \
  do {                                \
    int _s = (expr);                  \
    if (_s != ILM_OK) return _s;      \
  } while (0)

#define ILM_REQUIRE(cond, ...)                     \
  do {                                             \
    if (!(cond)) {                                 \
      ::ilm::set_error(__VA_ARGS__);               \
      return ILM_ERR_INVALID_ARG;                  \
    }                                              \
  } while (0)

inline cudaStream_t as_stream(ilm_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

// fn(i) for i in [0, n) on up to min(n, hardware threads, 16) host threads
// (contiguous chunks; fn must only touch data of its own i)
template <typename F>
void parallel_for(int n, F fn) {
  const int hw = (int)std::thread::hardware_concurrency();
  const int nt = std::max(1, std::min({n, hw > 0 ? hw : 1, 16}));
  if (nt <= 1) {
    for (int i = 0; i < n; ++i) fn(i);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      for (int i = (int)((long long)n * t / nt); i < (int)((long long)n * (t + 1) / nt); ++i) fn(i);
    });
  for (auto& x : th) x.join();
}

// ---------------------------------------------------------------------------
// device buffer (RAII)
// ---------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  bool own = true;  // false: a view into memory another DevBuf owns (an arena)
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p && own) cudaFree(p);
    p = nullptr;
    bytes = 0;
    own = true;
  }
  // point at [ptr, ptr + nbytes) of an arena (not freed by this buffer)
  void view(void* ptr, size_t nbytes) {
    release();
    p = ptr;
    bytes = nbytes;
    own = false;
  }
  int alloc(size_t nbytes) {
    if (nbytes <= bytes && p) return ILM_OK;
    release();
    if (nbytes == 0) return ILM_OK;
    cudaError_t e = cudaMalloc(&p, nbytes);
    if (e != cudaSuccess) {
      set_error("cudaMalloc(%zu) failed: %s", nbytes, cudaGetErrorString(e));
      p = nullptr;
      return ILM_ERR_NO_MEMORY;
    }
    bytes = nbytes;
    return ILM_OK;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

// ---------------------------------------------------------------------------
// grid and staggering
// ---------------------------------------------------------------------------
// Position classes (dual_x, dual_y): a dual direction is offset by h/2 and
// carries the ghost layer.
enum PosClass { PC_P = 0, PC_D = 1, PC_U = 2, PC_V = 3 };  // (0,0) (1,1) (1,0) (0,1)

inline int pc_dx(int pc) { return (pc == PC_D || pc == PC_U) ? 1 : 0; }
inline int pc_dy(int pc) { return (pc == PC_D || pc == PC_V) ? 1 : 0; }

struct Shape2 {
  int n1, n2;
  size_t numel() const { return (size_t)n1 * (size_t)n2; }
};

}  // namespace ilm

struct ilm_grid_s {
  int nx, ny;
  double h;
  int i0x, i0y;
  ilm::Shape2 shape(int pc) const {
    return {ilm::pc_dx(pc) ? nx : nx - 1, ilm::pc_dy(pc) ? ny : ny - 1};
  }
};

namespace ilm {

// number of components and their classes for a grid data kind
int gridkind_components(int kind, int* pcs);  // returns ncomp, fills pcs[]
size_t gridkind_numel(const ilm_grid_s* g, int kind);

// ---------------------------------------------------------------------------
// DDF point windows: 4 taps per direction and per 1-D offset class
// ---------------------------------------------------------------------------
constexpr int NTAP = 4;
constexpr int TILE_X = 32;
constexpr int TILE_Y = 8;

// coefficient codes for fused point-wise products
enum Coef { CF_ZERO = 0, CF_ONE = 1, CF_NX = 2, CF_NY = 3, CF_MNX = 4, CF_MNY = 5, CF_MONE = 6 };

// ---------------------------------------------------------------------------
// Deterministic tile scatter (regularize!): one 256-thread CTA per occupied
// TILE_X x TILE_Y tile, one thread per cell.  The tile's candidate points are
// staged in shared memory up to 256 at a time (the caller fills bx, by, amp
// = weight x data, wx, wy for staging slots [0, nc)).  A point's window
// starts at column bx, so it reaches the tile's column li only if bx lies in
// x0 + li - (NTAP - 1) .. x0 + li: the staged points are bucketed by
// key = bx - x0 + NTAP - 1 (TILE_X + NTAP - 1 keys) and each cell visits
// only its NTAP buckets, about NTAP / (TILE_X + NTAP - 1) of the points
// instead of all of them.  The buckets are ordered by key, then by staging
// slot (warp match groups and per-warp offsets, no atomics), so every cell
// sums its points in a fixed order.  Small chunks skip the bucketing.
// ---------------------------------------------------------------------------
constexpr int SCAT_NB = TILE_X * TILE_Y;
constexpr int SCAT_NKEY = TILE_X + NTAP - 1;

template <typename T>
struct ScatterSmem {
  int bx[SCAT_NB], by[SCAT_NB];
  T amp[SCAT_NB], wx[SCAT_NB * NTAP], wy[SCAT_NB * NTAP];
  int wcnt[SCAT_NB / 32][SCAT_NKEY];  // per-warp bucket counts, then offsets
  int start[SCAT_NKEY + 1];
  unsigned short perm[SCAT_NB];       // sorted position -> staging slot
};

// chunks of at most this many points are summed directly in staging order:
// for sparse tiles (points ds >= h apart: ~25 per tile) the bucketing's
// barriers and scan cost more than the loop they shorten
constexpr int SCAT_DIRECT_MAX = 64;
// points per pass of the direct sum's loop (the batched Poisson scatter:
// 62.6 us per launch with a loop over every slot, 58.8 / 57.9 / 58.3 us
// with 2 / 3 / 4 points per pass, 69.5 us with one)
constexpr int SCAT_PASS = 3;

// sum of the staged points' contributions to cell (i, j) of the tile whose
// first column is x0; all threads of the CTA call it (it synchronises the
// CTA; the caller synchronises again before restaging).  The CTA is
// TILE_X (= 32) x TILE_Y threads, so a warp is one row j of the tile.
template <typename T>
__device__ __forceinline__ T tile_sum_bucketed(ScatterSmem<T>& sm, int nc, int x0, int i, int j) {
  static_assert(TILE_X == 32, "one warp per tile row");
  if (nc <= SCAT_DIRECT_MAX) {  // block-uniform
    __syncthreads();
    // Direct sum in staging order.  Whether a point's window reaches row j
    // is the same for the whole warp: each lane tests one staged point's
    // rows, a ballot keeps the ~NTAP / (TILE_Y + NTAP - 1) that reach the
    // row, and the warp visits only those, lowest slot first -- the points
    // and the order of the sum of a loop over every slot, so the same result.
    // SCAT_PASS points per pass, their shared-memory loads issued together
    // (one point per pass is a chain of dependent loads).
    const int lane = threadIdx.x;
    T acc = (T)0;
    for (int e0 = 0; e0 < nc; e0 += 32) {
      const int e = e0 + lane;
      unsigned m = __ballot_sync(0xffffffffu, e < nc && (unsigned)(j - sm.by[e < nc ? e : 0]) < (unsigned)NTAP);
      while (m) {
        int f[SCAT_PASS];
        bool h[SCAT_PASS];
        T p[SCAT_PASS], q[SCAT_PASS];
#pragma unroll
        for (int u = 0; u < SCAT_PASS; ++u) {
          const bool ok = m != 0u;  // always true for u = 0
          f[u] = ok ? e0 + __ffs(m) - 1 : f[0];
          m &= m - 1u;
          const int di = i - sm.bx[f[u]], dj = j - sm.by[f[u]];
          h[u] = ok && (unsigned)di < (unsigned)NTAP;
          p[u] = sm.amp[f[u]] * sm.wx[f[u] * NTAP + (h[u] ? di : 0)];
          q[u] = sm.wy[f[u] * NTAP + dj];
        }
#pragma unroll
        for (int u = 0; u < SCAT_PASS; ++u)
          if (h[u]) acc += p[u] * q[u];
      }
    }
    return acc;
  }
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int q = tid; q < (SCAT_NB / 32) * SCAT_NKEY; q += SCAT_NB) (&sm.wcnt[0][0])[q] = 0;
  __syncthreads();  // staged points and zeroed counts visible
  int key = SCAT_NKEY;  // idle slot
  if (tid < nc) key = min(max(sm.bx[tid] - x0 + (NTAP - 1), 0), SCAT_NKEY - 1);
  const unsigned grp = __match_any_sync(0xffffffffu, key);
  const int rank = __popc(grp & ((1u << lane) - 1u));
  if (key < SCAT_NKEY && rank == 0) sm.wcnt[warp][key] = __popc(grp);
  __syncthreads();
  if (warp == 0) {  // exclusive scan of the bucket totals; per-warp offsets
    int t0 = 0, t1 = 0;
    for (int w = 0; w < SCAT_NB / 32; ++w) {
      t0 += lane < SCAT_NKEY ? sm.wcnt[w][lane] : 0;
      t1 += lane + 32 < SCAT_NKEY ? sm.wcnt[w][lane + 32] : 0;
    }
    int i0 = t0, i1 = t1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int a = __shfl_up_sync(0xffffffffu, i0, o), b = __shfl_up_sync(0xffffffffu, i1, o);
      if (lane >= o) {
        i0 += a;
        i1 += b;
      }
    }
    const int s0 = __shfl_sync(0xffffffffu, i0, 31);
    int e0 = i0 - t0, e1 = s0 + i1 - t1;
    if (lane < SCAT_NKEY) {
      sm.start[lane] = e0;
      for (int w = 0; w < SCAT_NB / 32; ++w) {
        const int c = sm.wcnt[w][lane];
        sm.wcnt[w][lane] = e0;
        e0 += c;
      }
    }
    if (lane + 32 < SCAT_NKEY) {
      sm.start[lane + 32] = e1;
      for (int w = 0; w < SCAT_NB / 32; ++w) {
        const int c = sm.wcnt[w][lane + 32];
        sm.wcnt[w][lane + 32] = e1;
        e1 += c;
      }
    }
    if (lane == 0) sm.start[SCAT_NKEY] = nc;
  }
  __syncthreads();
  if (key < SCAT_NKEY) sm.perm[sm.wcnt[warp][key] + rank] = (unsigned short)tid;
  __syncthreads();
  const int li = min(max(i - x0, 0), TILE_X - 1);
  T acc = (T)0;
  for (int q = sm.start[li], qe = sm.start[li + NTAP]; q < qe; ++q) {
    const int e = sm.perm[q];
    const int di = i - sm.bx[e];
    const int dj = j - sm.by[e];
    if ((unsigned)di < (unsigned)NTAP && (unsigned)dj < (unsigned)NTAP)
      acc += sm.amp[e] * sm.wx[e * NTAP + di] * sm.wy[e * NTAP + dj];
  }
  return acc;
}

template <typename T>
struct PointWin {
  // [npts] base indices and [npts*4] weights for x-primal, x-dual, y-primal, y-dual
  const int* bx[2];
  const int* by[2];
  const T* wx[2];
  const T* wy[2];
};

// tile candidate list for one position class
struct TileList {
  DevBuf ptr;     // int [ntiles+1]
  DevBuf pts;     // int [capacity >= 4 npts]
  DevBuf ne;      // int [ntiles]: the tiles with at least one candidate point (first ne_cnt)
  DevBuf ne_cnt;  // int: their number (device copy)
  int ntx = 0, nty = 0, nne = 0;
  int nne_launch = 0;  // scatter grid: nne, or an upper bound after a device re-binning
};
// out[0, n) = 0 (16-byte stores where aligned); the scatters fill their
// output with it and then visit only the tiles that hold points
int fill_zero(void* out, size_t bytes, cudaStream_t st);

// ---------------------------------------------------------------------------
// FFT convolution (inverse Laplacian)
// ---------------------------------------------------------------------------
struct ConvPlan {
  int n1 = 0, n2 = 0, P1 = 0, P2 = 0, dtype = ILM_F64;
  const void* spec = nullptr;   // (P1/2+1) x (P2/2+1) real, scaled, device (shared)
  const void* tw1 = nullptr;    // twiddles length P1 (device, shared)
  const void* tw2 = nullptr;    // twiddles length P2
  DevBuf work;                  // n2 x (P1/2+1) complex
};

struct ConvJobDev {
  const void* in;
  void* out;
  void* work;
  const void* spec;
  const void* tw1;   // length P1
  const void* tw2;   // length P2
  int n1, n2;        // valid input columns / rows
  int n2out;         // rows produced by the column pass
  int P1, P2;
  double scale;
  int row_off, col_off;
  int frow_off, frb;   // register-FFT path: first row CTA of this job, rows per CTA
  // Input box: only rows [ra, rb) and columns [ca, cb) of `in` are read (the
  // rest of the input is taken as zero and may hold anything).  has_box = 0:
  // the whole n1 x n2 input.
  int has_box, ra, rb, ca, cb;
  int irow_off;        // register-FFT path: first inverse-row CTA of this job
  int fcw;             // register-FFT path: spectral columns per column-pass CTA
  // optional field (n1 x n2) added to the result: out = add + scale * conv
  const void* add;
  // out_base != nullptr at launch: out = out_base + out_off bytes (lets a
  // prepared job table write into a caller's buffer)
  size_t out_off;
};
struct ConvLaunch {
  int rows = 0, cols = 0, CW = 1, maxP1 = 0, maxP2 = 0;
  int fast = 0, frows = 0, firows = 0;  // register four-step FFT path (FP32): forward / inverse row CTAs
  size_t fsm_rows = 0, fsm_cols = 0, fsm_irows = 0;  // its dynamic shared memory per CTA
  // register-FFT path: job of every CTA of the forward-row / column /
  // inverse-row launches (host copies from conv_jobs_finalize; the owner of
  // the job table uploads them and sets dmap, nullptr = binary search)
  std::vector<int> mrows, mcols, mirows;
  const int* dmap[3] = {nullptr, nullptr, nullptr};
};
// fill row/col offsets of a job table and the launch geometry
int conv_jobs_finalize(std::vector<ConvJobDev>& jobs, int dtype, ConvLaunch* L);
// launch a prepared (device-resident) job table; no host<->device traffic.
// out_base: see ConvJobDev::out_off (nullptr: each job's `out`)
int conv_jobs_launch(const ConvJobDev* jobs_dev, int njobs, const ConvLaunch& L, int dtype, cudaStream_t st,
                     void* out_base = nullptr);
// shared spectrum and twiddle tables for padded sizes P1 x P2
int conv_resources(int P1, int P2, int dtype, const void** spec, const void** tw1, const void** tw2, cudaStream_t st);

int good_fft_size(int n);
// G(m,n) table for 0<=m,n<=M (row-major (M+1)x(M+1), FP64, device; library-owned)
int lgf_table_device(int M, const double** tab, int* ld, cudaStream_t st);
int lgf_table_ff_device(int M, const float2** tab, int* ld, cudaStream_t st);  // (hi, lo) pairs
int conv_plan_init(ConvPlan* plan, int n1, int n2, int dtype, cudaStream_t st);
// out = (1/factor) * G * in (linear convolution), in/out n1 x n2 (x fastest)
int conv_apply(ConvPlan* plan, const void* in, void* out, double inv_factor, cudaStream_t st);

// ---------------------------------------------------------------------------
// kernels launchers (defined in the .cu files)
// ---------------------------------------------------------------------------
// float-float arithmetic on the FP32 pipes (value = hi + lo, ~2^-44 relative
// per operation): GB300 issues FP64 at a small fraction of its FP32 rate
// Programmatic dependent launch for chains of stream-ordered grid kernels:
// launched by launch_pdl, a kernel lets the next launch in its stream begin
// scheduling as soon as all of its CTAs have started
// (griddepcontrol.launch_dependents) and waits for the previous grid's
// completion and memory before its first load (griddepcontrol.wait; a no-op
// when the launch has no programmatic dependency), so launch latency and
// the ramp of one grid overlap the tail of the one before.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
template <typename... P, typename... A>
cudaError_t launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, cudaStream_t st, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<P>(args)...);
}

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

__device__ __forceinline__ FF ff_renorm(float hi, float lo) {
  const float s = hi + lo;
  return FF{s, lo - (s - hi)};
}

__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return ff_renorm(p, e);
}

// a - f b
__device__ __forceinline__ FF ff_sub_mul(FF a, FF f, FF b) {
  const float p = f.hi * b.hi;
  float pe = fmaf(f.hi, b.hi, -p);
  pe = fmaf(f.hi, b.lo, fmaf(f.lo, b.hi, pe));
  float s, e;
  two_sum(a.hi, -p, s, e);
  return ff_renorm(s, e + a.lo - pe);
}

struct GatherTerm {
  int pc;             // position class of the grid array
  const void* arr;    // grid array (cache dtype)
  int coef;           // Coef code
};

}  // namespace ilm

struct ilm_cache_s {
  ilm_grid_s grid;
  int kind, npts, ddf, scaling, dtype;
  double h;
  // host copies (double)
  std::vector<double> hx, hy, hnx, hny, hds;
  // device point data (cache dtype) and FP64 copies used by the Schur build
  ilm::DevBuf nx, ny, wscale;          // wscale = ds/h^2 (GridScaling) or 1
  ilm::DevBuf ds64, nx64, ny64;        // FP64
  ilm::DevBuf bx[2], by[2];            // int
  ilm::DevBuf wx[2], wy[2];            // cache dtype
  ilm::DevBuf wx64[2], wy64[2];        // FP64
  std::vector<int> hbx[2], hby[2];
  std::vector<double> hwx[2], hwy[2];  // host copies of the window weights
  ilm::TileList tiles[4];
  ilm::DevBuf x64, y64;                // FP64 point coordinates (device; set by a re-binning)
  ilm::DevBuf rebin_cnt, rebin_cur;    // re-binning scratch (int per tile)
  bool host_stale = false;             // host copies behind the device after ilm_cache_update_points
  // inverse Laplacian plans per position class
  ilm::ConvPlan conv[4];
  bool conv_ready[4] = {false, false, false, false};
  // scratch grid buffers (cache dtype)
  ilm::DevBuf g_scr[6];
  // scratch point buffers (FP64 and cache dtype)
  ilm::DevBuf p_scr[8];
  // cached Schur complements for the problem solves (FP64 and FP32 copies)
  ilm::DevBuf S_dir64, S_dir32, S_neu64, S_neu32;
  bool S_dir_ready = false, S_neu_ready = false;
  // surface filter: W = E R 1 (cache dtype) and a grid buffer of the cache's class
  ilm::DevBuf filt_diag, filt_grid;
  bool filt_ready = false;
  // Stokes preconditioner: inverse of the gauge-shifted Nodes{Primal} Schur
  // complement -E L^-1 E^T (FP64, N x N), built on first use
  ilm::DevBuf stokes_pc;
  bool stokes_pc_ready = false;
  ilm::DevBuf red;                     // reduction scratch (double)
  // FP64 iterative refinement (ilm_solve_*_refined): an FP64 cache of the same
  // points (FP32 caches only; built on first use, dropped when points move)
  // and FP64 vectors
  ilm_cache_s* twin = nullptr;
  ilm::DevBuf ref_in, ref_f, ref_s, ref_b, ref_x, ref_r, ref_y, ref_norm;
  ilm_cache_s() = default;
  ilm_cache_s(const ilm_cache_s&) = delete;
  ilm_cache_s& operator=(const ilm_cache_s&) = delete;
  ~ilm_cache_s() { delete twin; }

  template <typename T> ilm::PointWin<T> win() const {
    ilm::PointWin<T> w;
    for (int a = 0; a < 2; ++a) {
      w.bx[a] = bx[a].as<int>();
      w.by[a] = by[a].as<int>();
      w.wx[a] = wx[a].as<T>();
      w.wy[a] = wy[a].as<T>();
    }
    return w;
  }
};

namespace ilm {

// DDF / transfer launchers (ilm_ddf.cu)
struct HostWindows {
  std::vector<int> bx[2], by[2];         // [primal|dual] base index per point
  std::vector<double> wx[2], wy[2];      // [primal|dual] 4 weights per point
  std::vector<int> tptr[4], tpts[4];     // per position class: tile CSR
  int ntx[4], nty[4];
};
void host_windows(const ilm_grid_s& g, int ddf, int N, const double* x, const double* y, HostWindows* W);
int cache_build_windows(ilm_cache_s* c);
// Forward 1-D convolution layer of the learned preconditioner on the tcgen05
// tensor cores (ilm_tcconv.cu): out = relu?(bias + W * in) with W BF16
// (Cout x Cin x 5), activations FP32 (split into a BF16 hi / lo pair), FP32
// accumulation in tensor memory.  *err is set to 1 by a CTA whose MMA
// completion wait ran out (the layer's output is then incomplete).
bool conv_tc_supported(int Cin, int Cout);
int launch_conv_tc(int N, int Cin, int Cout, bool relu, const __nv_bfloat16* W, const float* bias, const float* in,
                   const int* sst, const int* sln, float* out, int* err, cudaStream_t st);
// after a completed forward: ILM_ERR_TIMEOUT if a tensor-core layer's wait ran out
int net_check_tc(ilm_net_t n);

// Geometry features of one surface point for the learned preconditioner: ds/h,
// 10 h x (turning angle over the local arc length), the normal, and sin/cos
// of the sub-cell position in x and y.  (p, m: the next and previous points
// of the point's body, circularly.)  Shared by the host entry point
// ilm_point_features and the batch's device set-up.
__host__ __device__ inline void point_feature(double xi, double yi, double nxi, double nyi, double dsi, double nxp,
                                              double nyp, double dsp, double nxm, double nym, double dsm, double h,
                                              float* f) {
  const double pi = 3.14159265358979323846, two_pi = 6.283185307179586476925286766559;
  double dth = atan2(nyp, nxp) - atan2(nym, nxm);
  dth = fmod(dth + 3.0 * pi, two_pi);
  if (dth < 0) dth += two_pi;
  dth -= pi;
  const double arc = 0.5 * dsm + dsi + 0.5 * dsp;
  const double fx = xi / h - floor(xi / h), fy = yi / h - floor(yi / h);
  f[0] = (float)(dsi / h);
  f[1] = (float)(10.0 * h * dth / arc);
  f[2] = (float)nxi;
  f[3] = (float)nyi;
  f[4] = (float)sin(two_pi * fx);
  f[5] = (float)cos(two_pi * fx);
  f[6] = (float)sin(two_pi * fy);
  f[7] = (float)cos(two_pi * fy);
}

// Batched DDF windows and tile candidate lists on the device (batch set-up).
// Per point k of problem p = pt2prob[k] (grid nx, ny, i0 of grid[4p..], h[p]):
// 4-tap windows on primal and dual lines (FP64 and `dtype` copies), the
// normals / weights in `dtype` and FP64.  Per problem and position class
// pc, a CSR list of the problem's points (local index, increasing) per
// TILE_X x TILE_Y tile: tptr[pc] holds nt + 1 entries per problem at
// tp_off[pc][p], tpts[pc] holds room for 4 npts entries per problem at
// ts_off[pc][p] (a 4 x 4 window touches at most 2 x 2 tiles).
struct BatchGeomDev {
  const double *x, *y, *nx, *ny, *ds;  // inputs, all points
  const int* pt2prob;
  const int* poff;                     // nprob + 1 point offsets
  const int* grid;                     // per problem: nx, ny, i0x, i0y
  const double* h;                     // per problem
  int* bx[2];
  int* by[2];
  double* wx64[2];
  double* wy64[2];
  void* wx[2];
  void* wy[2];
  void *nxo, *nyo, *wsc;               // dtype
  double *nx64, *ny64, *ds64;
  int* tptr[4];
  int* tpts[4];
  const int* tp_off[4];                // per problem
  const int* ts_off[4];
  int* cnt;                            // scratch: one int per entry of every tptr (4 classes), zeroed here
  int cnt_total;
  int cnt_off[4];                      // offset of class pc's counters in cnt (= tptr layout)
};
int batch_windows_and_tiles(int nprob, int Ptot, const BatchGeomDev& G, int ddf, int dtype, int grid_scaling,
                            cudaStream_t st);

// device re-binning of the cache's points (ilm_cache_update_points); the
// host copies are refreshed lazily by cache_sync_host
int cache_rebin_points(ilm_cache_s* c, const double* x, const double* y, const double* nx, const double* ny,
                       const double* ds, cudaStream_t st);
int cache_sync_host(ilm_cache_s* c);
// out_pc(cell) = sum_k w_k (a_k in1_k + b_k in2_k) phi phi ; in2 may be null
int launch_scatter(ilm_cache_s* c, int pc, const void* in1, int coef1, const void* in2, int coef2,
                   void* out, cudaStream_t st, bool accumulate = false);
// out_k (+)= sum_t coef_t * E_{pc_t} arr_t
int launch_gather(ilm_cache_s* c, const GatherTerm* terms, int nterms, void* out, bool accumulate,
                  double scale, cudaStream_t st);

// stencils (ilm_stencil.cu); scale multiplies the result
int st_mul_add(size_t n, int dtype, const void* a, const void* b, void* out, cudaStream_t st);  // out += a b
int st_div_edges(const ilm_grid_s* g, int dtype, const void* q, void* w, double scale, cudaStream_t st);
int st_grad_nodes(const ilm_grid_s* g, int dtype, const void* w, void* q, double scale, cudaStream_t st);
int st_curl_dual_to_edges(const ilm_grid_s* g, int dtype, const void* s, void* q, double scale, cudaStream_t st);
int st_curl_edges_to_dual(const ilm_grid_s* g, int dtype, const void* q, void* w, double scale, cudaStream_t st);
int st_grad_edges(const ilm_grid_s* g, int dtype, const void* q, void* t, double scale, cudaStream_t st);
int st_div_edgegrad(const ilm_grid_s* g, int dtype, const void* t, void* q, double scale, cudaStream_t st);
int st_laplacian(int n1, int n2, int dtype, const void* in, void* out, double scale, cudaStream_t st);
int st_axpby(size_t n, int dtype, double a, const void* x, double b, const void* y, void* out, cudaStream_t st);
int st_fill(size_t n, int dtype, double v, void* out, cudaStream_t st);
int st_affine(size_t n, int dtype, double a, const void* x, double b, void* out, cudaStream_t st);
int st_convert(size_t n, int dtype_in, const void* in, int dtype_out, void* out, cudaStream_t st);
int st_primal_to_dual(const ilm_grid_s* g, int dtype, const void* p, void* out, cudaStream_t st);
// Edges{Primal}.u interpolated to Nodes{Dual} / Nodes{Primal} (vector-cache masks)
int st_xedge_to_dual(const ilm_grid_s* g, int dtype, const void* u, void* out, cudaStream_t st);
int st_xedge_to_primal(const ilm_grid_s* g, int dtype, const void* u, void* out, cudaStream_t st);
int st_primal_to_edges(const ilm_grid_s* g, int dtype, const void* p, void* out, cudaStream_t st);
int st_mul(size_t n, int dtype, const void* a, void* inout, cudaStream_t st);
// convective derivatives and w x v (ilm_convective.cu); field_kind: the kind of q and out
int st_convective(const ilm_grid_s* g, int dtype, int field_kind, const void* v, const void* q, void* out,
                  double scale, cudaStream_t st);
int st_w_cross_v(const ilm_grid_s* g, int dtype, const void* w, const void* v, void* out, cudaStream_t st);
int st_weighted_dot(int n1, int n2, int dx, int dy, int dtype, const void* a, const void* b,
                    double* dres, cudaStream_t st);
int st_point_dot(int n, int dtype, const void* a, const void* b, const double* w, double* dres,
                 cudaStream_t st);

// Schur (ilm_schur.cu)
// any_cache: also on vector caches (their Nodes{Primal} / Nodes{Dual} windows)
int schur_build(ilm_cache_s* c, int which, double scale, double* A, cudaStream_t st, bool any_cache = false);
// an FP64 cache of the same points as c (c itself when it is FP64), built on
// first use and dropped when the points move
int ensure_twin(ilm_cache_s* c, ilm_cache_s** out);
struct CGParams {
  const double* A64;   // n x n column-major
  const float* A32;    // n x n column-major
  const double* b;     // rhs
  double* x;           // solution
  const double* w;     // inner-product weights (ds)
  int n;
  int maxiter;
  double tol;
  int* iters;          // device out
  double* relres;      // device out
};
int launch_cg_batched(const CGParams* probs_dev, int nprob, int max_n, cudaStream_t st);

// batched Schur builds (one launch over all problems of a batch)
// Row stride (floats) of a batched n x n Schur complement: n rounded up to a
// multiple of 4, so that every row starts on a 16-byte boundary (vector
// loads in the CG); the padding columns hold zeros.
__host__ __device__ inline int schur_ld(int n) { return (n + 3) & ~3; }

struct SchurProbDev {
  int kind;      // ILM_SCHUR_RTLINVR (Dirichlet) or ILM_SCHUR_CLINVCT (Neumann)
  int n;         // points of this problem
  int poff;      // first point in the packed point arrays
  int tile0;     // first 16x16 pair tile of this problem
  size_t soff;   // offset of this problem's n x n matrix
  double invh;   // derivative scale 1/h
};
struct BatchWin {
  const int* bx[2];
  const int* by[2];
  const double* wx64[2];
  const double* wy64[2];
  const double* nx64;
  const double* ny64;
};
struct Functional;
size_t functional_size();
// probs_dev: the nprob descriptors in problem order.  order != nullptr: the
// pair tiles in two launches, the descriptors order[0, nfirst) (tiles_first
// tiles, numbered from zero) then the rest (numbered from zero again), event
// mid recorded between them
int schur_build_batched(int nprob, const SchurProbDev* probs_dev, int total_tiles, int Ptot, const int* pt2prob,
                        const BatchWin& W, const double* w, Functional* F, float* Shi, float* Slo, int max_grid,
                        cudaStream_t st, const SchurProbDev* order = nullptr, int nfirst = 0, int tiles_first = 0,
                        cudaEvent_t mid = nullptr);
// right-hand-side operator of the batched solves (E L^-1 D_s / G_s L^-1 R),
// full n x n tiles numbered from probs_full_dev[p].tile0
int rhsop_build_batched(int nprob, const SchurProbDev* probs_full_dev, int total_tiles, int Ptot, const int* pt2prob,
                        const BatchWin& W, const double* w, Functional* FU, Functional* FD, float* Mhi, float* Mlo,
                        int max_grid, cudaStream_t st);

// cluster CG with float-float matvecs (ilm_cg.cu); S stored row-major as hi/lo FP32
size_t cgff_params_size();
void cgff_params_fill(void* dst, const float* Shi, const float* Slo, const double* b, double* x, const double* w,
                      int n, int maxiter, double tol, int* iters, double* relres, const int* blk,
                      const int* bstart, const int* bsize, const int* boff, const float* binv_hi,
                      const float* binv_lo);
int net_forward_packed(ilm_net_t n, int N, const float* feat, const int* sst, const int* sln, float* band,
                       cudaStream_t st);
int net_band(ilm_net_t n);
int* net_tc_flag(ilm_net_t n);
int net_nfeat(ilm_net_t n);
void cgff_params_set_deflation(void* dst, const double* sz, const double* inv_e);
// per-problem timing of the cluster CG (3 u64 per problem: start ns, end ns, SM), nullptr: off
void cgff_params_set_timing(void* dst, unsigned long long* tspan);
void cgff_params_set_band(void* dst, const float* band, int band_k, const int* seg_start, const int* seg_len);
// coarse correction of block-Jacobi on up to CG_COARSE_MAX bodies' constants:
// starts[0..nb] local body boundaries, Einv nb x CG_COARSE_MAX row-major
constexpr int CG_COARSE_MAX = 4;
void cgff_params_set_coarse(void* dst, int nb, const int* starts, const double* Einv);
// warm start from x0 (may be the output array itself: each CTA reads its rows first)
void cgff_params_set_x0(void* dst, const double* x0);
void cgff_params_fill_csr(void* dst, const float* vhi, const float* vlo, const int* rowptr, const int* colidx,
                          const double* b, double* x, const double* x0, const double* w, int n, int maxiter,
                          double tol, int* iters, double* relres);
struct BJBlockTask {
  const float* Shi;  // problem's S as float-float pairs (n x n row-major)
  const float* Slo;
  int n, s, sz;      // block = points [s, s + sz)
  float* out_hi;     // sz x sz inverse, row-major, float-float
  float* out_lo;
};
int launch_block_inverse(const BJBlockTask* tasks_dev, int ntasks, int max_sz, cudaStream_t st);
// variant: 0 auto, 1 row-distributed vectors, 2 replicated vectors (see ilm_cg.cu)
// single-CTA CG over the problems order[0 .. nprob) (CG variant 6's small problems)
int launch_cg_single(const void* params_dev, const int* order, int nprob, int* counter, int max_n, int nctas,
                     cudaStream_t st);
int cg_single_slots(int max_n);
int launch_cg_cluster(const void* params_dev, const int* order, int nprob, int* counter, int max_n, int nclusters,
                      cudaStream_t st, int variant = 0);
int cg_cluster_count(int nprob, int max_n, int variant = 0);
size_t cg_variant_smem(int max_n, int variant);  // dynamic shared memory of a CG variant
size_t cg_rep_smem(int max_n);  // shared memory of the replicated-vector CG per CTA

}  // namespace ilm
