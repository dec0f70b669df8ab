// DDF regularization (scatter) and interpolation (gather) between surface
// points and the staggered grid.
//
// Replaces the sparse RegularizationMatrix / InterpolationMatrix products of
// CartesianGrids used by regularize!/interpolate! (src/surface_operators.jl:
// 38-46, 80-88) and their normal/cross/dot variants (:98-343).
//
// Setup (host, once per cache): for every point and each 1-D offset class
// (x on primal/dual lines, y on primal/dual lines) the 4-tap window base index
// and the DDF weights phi((x_i - X_k)/h) are computed in FP64; for each grid
// position class the points are binned into 32x8 output tiles.
//
// Scatter: one thread per output cell, one CTA per tile.  Each thread sums the
// contributions of the tile's candidate points in index order, so the result
// is deterministic (no atomics) and every cell of the output is written (the
// reference's fill!(s,0) + mul! overwrite) in one coalesced pass.
// Gather: one thread per point, 16 taps per term, fixed order.
#include <math.h>

#include <algorithm>

#include "ilm_internal.cuh"

namespace ilm {

// ---------------------------------------------------------------------------
// DDF kernels (host, FP64) -- published formulas
// ---------------------------------------------------------------------------
__host__ __device__ inline double ddf_eval(int ddf, double r) {
  r = fabs(r);
  const double s3 = 1.7320508075688772935;
  switch (ddf) {
    case ILM_DDF_YANG3:  // Yang, Zhang, Li & Yang, JCP 228 (2009), smoothed 3-point
      if (r <= 1.0)
        return 17.0 / 48.0 + s3 * M_PI / 108.0 + r / 4.0 - r * r / 4.0 +
               (1.0 - 2.0 * r) / 16.0 * sqrt(fmax(-12.0 * r * r + 12.0 * r + 1.0, 0.0)) -
               s3 / 12.0 * asin(s3 / 2.0 * (2.0 * r - 1.0));
      if (r < 2.0)
        return 55.0 / 48.0 - s3 * M_PI / 108.0 - 13.0 * r / 12.0 + r * r / 4.0 +
               (2.0 * r - 3.0) / 48.0 * sqrt(fmax(-12.0 * r * r + 36.0 * r - 23.0, 0.0)) +
               s3 / 36.0 * asin(s3 / 2.0 * (2.0 * r - 3.0));
      return 0.0;
    case ILM_DDF_ROMA:  // Roma, Peskin & Berger, JCP 153 (1999)
      if (r <= 0.5) return (1.0 + sqrt(1.0 - 3.0 * r * r)) / 3.0;
      if (r < 1.5) return (5.0 - 3.0 * r - sqrt(fmax(1.0 - 3.0 * (1.0 - r) * (1.0 - r), 0.0))) / 6.0;
      return 0.0;
    case ILM_DDF_M4PRIME:  // Monaghan M4'
      if (r <= 1.0) return 1.0 - 2.5 * r * r + 1.5 * r * r * r;
      if (r < 2.0) return 0.5 * (2.0 - r) * (2.0 - r) * (1.0 - r);
      return 0.0;
    case ILM_DDF_WITCHHAT:
      return r < 1.0 ? 1.0 - r : 0.0;
    case ILM_DDF_M3:
      if (r <= 0.5) return 0.75 - r * r;
      if (r < 1.5) return 0.5 * (1.5 - r) * (1.5 - r);
      return 0.0;
  }
  return 0.0;
}

// window of 4 taps covering the support: base = floor(r) - 1 (r = fractional
// index of the point on that line), weights phi(base + t - r)
__host__ __device__ inline void ddf_window(int ddf, double r, int* base, double* w) {
  const int b = (int)floor(r) - 1;
  *base = b;
  for (int t = 0; t < NTAP; ++t) w[t] = ddf_eval(ddf, (double)(b + t) - r);
}

template <typename T>
static int upload(DevBuf& b, const T* h, size_t n) {
  ILM_TRY(b.alloc(std::max<size_t>(n, 1) * sizeof(T)));
  if (n) ILM_CHECK_CUDA(cudaMemcpy(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice));
  return ILM_OK;
}

static int upload_typed(DevBuf& b, const std::vector<double>& h, int dtype) {
  if (dtype == ILM_F64) return upload(b, h.data(), h.size());
  std::vector<float> f(h.begin(), h.end());
  return upload(b, f.data(), f.size());
}

void host_windows(const ilm_grid_s& g, int ddf, int N, const double* x, const double* y, HostWindows* W) {
  const double h = g.h;
  for (int dual = 0; dual < 2; ++dual) {
    W->bx[dual].resize(N);
    W->by[dual].resize(N);
    W->wx[dual].resize((size_t)N * NTAP);
    W->wy[dual].resize((size_t)N * NTAP);
  }
  // fractional 0-based index of a point on primal / dual lines:
  // primal i at x = (i + 1 - i0) h ; dual i at x = (i + 1/2 - i0) h
  for (int k = 0; k < N; ++k) {
    for (int dual = 0; dual < 2; ++dual) {
      const double off = dual ? 0.5 : 1.0;
      const double rx = x[k] / h + g.i0x - off;
      const double ry = y[k] / h + g.i0y - off;
      ddf_window(ddf, rx, &W->bx[dual][k], &W->wx[dual][(size_t)k * NTAP]);
      ddf_window(ddf, ry, &W->by[dual][k], &W->wy[dual][(size_t)k * NTAP]);
    }
  }
  // tile candidate lists per position class, each sorted by point index
  for (int pc = 0; pc < 4; ++pc) {
    const Shape2 sh = g.shape(pc);
    const int dx = pc_dx(pc), dy = pc_dy(pc);
    W->ntx[pc] = (sh.n1 + TILE_X - 1) / TILE_X;
    W->nty[pc] = (sh.n2 + TILE_Y - 1) / TILE_Y;
    const size_t nt = (size_t)W->ntx[pc] * W->nty[pc];
    std::vector<int>& cnt = W->tptr[pc];
    cnt.assign(nt + 1, 0);
    auto tiles_of = [&](int k, int* tx0, int* tx1, int* ty0, int* ty1) {
      int b0 = W->bx[dx][k], b1 = b0 + NTAP - 1;
      int e0 = W->by[dy][k], e1 = e0 + NTAP - 1;
      b0 = std::max(b0, 0);
      e0 = std::max(e0, 0);
      b1 = std::min(b1, sh.n1 - 1);
      e1 = std::min(e1, sh.n2 - 1);
      if (b0 > b1 || e0 > e1) return false;
      *tx0 = b0 / TILE_X;
      *tx1 = b1 / TILE_X;
      *ty0 = e0 / TILE_Y;
      *ty1 = e1 / TILE_Y;
      return true;
    };
    for (int k = 0; k < N; ++k) {
      int a0, a1, b0, b1;
      if (!tiles_of(k, &a0, &a1, &b0, &b1)) continue;
      for (int ty = b0; ty <= b1; ++ty)
        for (int tx = a0; tx <= a1; ++tx) cnt[(size_t)ty * W->ntx[pc] + tx + 1]++;
    }
    for (size_t t = 0; t < nt; ++t) cnt[t + 1] += cnt[t];
    std::vector<int>& pts = W->tpts[pc];
    pts.assign(std::max(cnt[nt], 1), 0);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int k = 0; k < N; ++k) {
      int a0, a1, b0, b1;
      if (!tiles_of(k, &a0, &a1, &b0, &b1)) continue;
      for (int ty = b0; ty <= b1; ++ty)
        for (int tx = a0; tx <= a1; ++tx) pts[fill[(size_t)ty * W->ntx[pc] + tx]++] = k;
    }
  }
}

int cache_build_windows(ilm_cache_s* c) {
  const int N = c->npts;
  HostWindows W;
  host_windows(c->grid, c->ddf, N, c->hx.data(), c->hy.data(), &W);
  for (int dual = 0; dual < 2; ++dual) {
    c->hbx[dual] = W.bx[dual];
    c->hby[dual] = W.by[dual];
    c->hwx[dual] = W.wx[dual];
    c->hwy[dual] = W.wy[dual];
    ILM_TRY(upload(c->bx[dual], W.bx[dual].data(), N));
    ILM_TRY(upload(c->by[dual], W.by[dual].data(), N));
    ILM_TRY(upload_typed(c->wx[dual], W.wx[dual], c->dtype));
    ILM_TRY(upload_typed(c->wy[dual], W.wy[dual], c->dtype));
    ILM_TRY(upload_typed(c->wx64[dual], W.wx[dual], ILM_F64));
    ILM_TRY(upload_typed(c->wy64[dual], W.wy[dual], ILM_F64));
  }
  for (int pc = 0; pc < 4; ++pc) {
    TileList& tl = c->tiles[pc];
    tl.ntx = W.ntx[pc];
    tl.nty = W.nty[pc];
    ILM_TRY(upload(tl.ptr, W.tptr[pc].data(), W.tptr[pc].size()));
    // candidate list with room for a re-binning (a point's window touches at
    // most 2 x 2 tiles)
    std::vector<int> pts = W.tpts[pc];
    pts.resize(std::max<size_t>(pts.size(), (size_t)4 * std::max(N, 1)), 0);
    ILM_TRY(upload(tl.pts, pts.data(), pts.size()));
    std::vector<int> ne;
    for (int t = 0; t < tl.ntx * tl.nty; ++t)
      if (W.tptr[pc][t + 1] > W.tptr[pc][t]) ne.push_back(t);
    tl.nne = (int)ne.size();
    tl.nne_launch = tl.nne;
    ne.resize(std::max<size_t>((size_t)tl.ntx * tl.nty, 1), 0);  // room for a re-binning
    ILM_TRY(upload(tl.ne, ne.data(), ne.size()));
    ILM_TRY(upload(tl.ne_cnt, &tl.nne, 1));
  }
  return ILM_OK;
}

// ---------------------------------------------------------------------------
// device kernels
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T coef_val(int code, const T* __restrict__ nx, const T* __restrict__ ny, int k) {
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

// Deterministic scatter over the tiles that hold candidate points (the rest
// of the output was zero-filled): one thread per cell of a 32 x 8 tile; the
// tile's candidates (index order) are staged in shared memory 256 at a time,
// one point per thread, and every cell sums the points of its window buckets
// (tile_sum_bucketed) in a fixed order.
template <typename T>
__device__ __forceinline__ void stage_point(ScatterSmem<T>& sm, int slot, int k, const int* __restrict__ bx,
                                            const int* __restrict__ by, const T* __restrict__ wx,
                                            const T* __restrict__ wy, const T* __restrict__ wsc,
                                            const T* __restrict__ nx, const T* __restrict__ ny,
                                            const T* __restrict__ in1, int c1, const T* __restrict__ in2, int c2) {
  T g = coef_val<T>(c1, nx, ny, k) * in1[k];
  if (in2) g += coef_val<T>(c2, nx, ny, k) * in2[k];
  sm.bx[slot] = bx[k];
  sm.by[slot] = by[k];
  sm.amp[slot] = wsc[k] * g;
#pragma unroll
  for (int q = 0; q < NTAP; ++q) {
    sm.wx[slot * NTAP + q] = wx[k * NTAP + q];
    sm.wy[slot * NTAP + q] = wy[k * NTAP + q];
  }
}

template <typename T>
__device__ __forceinline__ T occupied_tile_sum(ScatterSmem<T>& sm, int p0, int p1, int x0, int i, int j,
                                               const int* __restrict__ tpts, const int* __restrict__ bx,
                                               const int* __restrict__ by, const T* __restrict__ wx,
                                               const T* __restrict__ wy, const T* __restrict__ wsc,
                                               const T* __restrict__ nx, const T* __restrict__ ny,
                                               const T* __restrict__ in1, int c1, const T* __restrict__ in2, int c2) {
  const int tid = threadIdx.y * TILE_X + threadIdx.x;
  T acc = (T)0;
  for (int c0 = p0; c0 < p1; c0 += SCAT_NB) {
    const int nc = min(SCAT_NB, p1 - c0);
    if (tid < nc) stage_point<T>(sm, tid, tpts[c0 + tid], bx, by, wx, wy, wsc, nx, ny, in1, c1, in2, c2);
    acc += tile_sum_bucketed<T>(sm, nc, x0, i, j);
    __syncthreads();
  }
  return acc;
}

template <typename T>
__global__ void __launch_bounds__(TILE_X* TILE_Y, 6)
k_scatter(int n1, int n2, int ntx, const int* __restrict__ ne, const int* __restrict__ ne_cnt, const int* __restrict__ tptr,
          const int* __restrict__ tpts, const int* __restrict__ bx, const int* __restrict__ by,
          const T* __restrict__ wx, const T* __restrict__ wy, const T* __restrict__ wsc, const T* __restrict__ nx,
          const T* __restrict__ ny, const T* __restrict__ in1, int c1, const T* __restrict__ in2, int c2,
          T* __restrict__ out, int accumulate) {
  __shared__ ScatterSmem<T> sm;
  if ((int)blockIdx.x >= *ne_cnt) return;  // launched for an upper bound after a device re-binning
  const int t = ne[blockIdx.x];
  const int x0 = (t % ntx) * TILE_X, y0 = (t / ntx) * TILE_Y;
  const int i = x0 + threadIdx.x, j = y0 + threadIdx.y;
  const T acc = occupied_tile_sum<T>(sm, tptr[t], tptr[t + 1], x0, i, j, tpts, bx, by, wx, wy, wsc, nx, ny, in1, c1,
                                     in2, c2);
  if (i < n1 && j < n2) {
    T* o = out + (size_t)j * n1 + i;
    *o = accumulate ? *o + acc : acc;
  }
}

// Overwriting scatter in one launch over the whole output, two kinds of
// block: blocks [0, nocc) take one occupied tile each (from the list `ne`,
// the first *ne_cnt entries; summed as in k_scatter), the blocks after them
// write zeros into the empty tiles, SCAT_TPB consecutive tiles (row-major
// tile ids) each, skipping the occupied ones.  Every tile is written by
// exactly one block; the long occupied-tile blocks start first and the zero
// fill's bandwidth overlaps their load latency.
constexpr int SCAT_TPB = 32;
template <typename T>
__global__ void __launch_bounds__(TILE_X* TILE_Y, 6)
k_scatter_all(int n1, int n2, int ntx, int ntiles, int nocc, const int* __restrict__ ne,
              const int* __restrict__ ne_cnt, const int* __restrict__ tptr, const int* __restrict__ tpts,
              const int* __restrict__ bx, const int* __restrict__ by, const T* __restrict__ wx,
              const T* __restrict__ wy, const T* __restrict__ wsc, const T* __restrict__ nx,
              const T* __restrict__ ny, const T* __restrict__ in1, int c1, const T* __restrict__ in2, int c2,
              T* __restrict__ out) {
  __shared__ int s_ptr[SCAT_TPB + 1];
  __shared__ ScatterSmem<T> sm;
  pdl_begin();
  const int tid = threadIdx.y * TILE_X + threadIdx.x;
  if ((int)blockIdx.x >= nocc) {  // zero writer
    const int t0 = ((int)blockIdx.x - nocc) * SCAT_TPB;
    if (tid <= SCAT_TPB) s_ptr[tid] = tptr[min(t0 + tid, ntiles)];
    __syncthreads();
    const int nt = min(SCAT_TPB, ntiles - t0);
    int tx = t0 % ntx, ty = t0 / ntx;
    for (int q = 0; q < nt; ++q) {
      if (s_ptr[q + 1] == s_ptr[q]) {  // empty (an occupied-tile block writes the others)
        const int i = tx * TILE_X + threadIdx.x, j = ty * TILE_Y + threadIdx.y;
        if (i < n1 && j < n2) out[(size_t)j * n1 + i] = (T)0;
      }
      if (++tx == ntx) {
        tx = 0;
        ++ty;
      }
    }
    return;
  }
  if ((int)blockIdx.x >= *ne_cnt) return;  // launched for an upper bound after a device re-binning
  const int t = ne[blockIdx.x];
  const int x0 = (t % ntx) * TILE_X, y0 = (t / ntx) * TILE_Y;
  const int i = x0 + threadIdx.x, j = y0 + threadIdx.y;
  const T acc = occupied_tile_sum<T>(sm, tptr[t], tptr[t + 1], x0, i, j, tpts, bx, by, wx, wy, wsc, nx, ny, in1, c1,
                                     in2, c2);
  if (i < n1 && j < n2) out[(size_t)j * n1 + i] = acc;
}

__global__ void k_fill_zero(float4* __restrict__ p4, size_t n4, unsigned char* __restrict__ tail, int ntail) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n4; k += stride)
    p4[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (blockIdx.x == 0 && (int)threadIdx.x < ntail) tail[threadIdx.x] = 0;
}

struct GTermDev {
  const void* arr;
  int n1, n2;
  int xsel, ysel;  // 0 primal 1 dual
  int coef;
};

template <typename T>
__global__ void k_gather(int N, const GTermDev* __restrict__ terms_unused, GTermDev t0, GTermDev t1, GTermDev t2,
                         GTermDev t3, int nterms, const int* __restrict__ bx0, const int* __restrict__ bx1,
                         const int* __restrict__ by0, const int* __restrict__ by1, const T* __restrict__ wx0,
                         const T* __restrict__ wx1, const T* __restrict__ wy0, const T* __restrict__ wy1,
                         const T* __restrict__ nx, const T* __restrict__ ny, T* __restrict__ out, int accumulate,
                         T scale) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  T total = (T)0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if (q >= nterms) break;
    const GTermDev tt = q == 0 ? t0 : (q == 1 ? t1 : (q == 2 ? t2 : t3));
    const int* bx = tt.xsel ? bx1 : bx0;
    const int* by = tt.ysel ? by1 : by0;
    const T* wx = tt.xsel ? wx1 : wx0;
    const T* wy = tt.ysel ? wy1 : wy0;
    const T* __restrict__ a = static_cast<const T*>(tt.arr);
    const int b0 = bx[k], e0 = by[k];
    T acc = (T)0;
#pragma unroll
    for (int jj = 0; jj < NTAP; ++jj) {
      const int j = e0 + jj;
      if ((unsigned)j >= (unsigned)tt.n2) continue;
      T racc = (T)0;
#pragma unroll
      for (int ii = 0; ii < NTAP; ++ii) {
        const int i = b0 + ii;
        if ((unsigned)i >= (unsigned)tt.n1) continue;
        racc += wx[k * NTAP + ii] * a[(size_t)j * tt.n1 + i];
      }
      acc += wy[k * NTAP + jj] * racc;
    }
    total += coef_val<T>(tt.coef, nx, ny, k) * acc;
  }
  total *= scale;
  if (accumulate) out[k] += total;
  else out[k] = total;
}

int fill_zero(void* out, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return ILM_OK;
  // vector stores from the first 16-byte boundary, bytes before / after it by the tail path
  const uintptr_t a = reinterpret_cast<uintptr_t>(out);
  if (a % 16 != 0) {
    ILM_CHECK_CUDA(cudaMemsetAsync(out, 0, bytes, st));
    return ILM_OK;
  }
  const size_t n4 = bytes / 16;
  const int ntail = (int)(bytes - 16 * n4);
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const size_t want = (n4 + 255) / 256;
  const int grid = (int)std::max<size_t>(1, std::min<size_t>(want, (size_t)nsm * 8));
  k_fill_zero<<<grid, 256, 0, st>>>(static_cast<float4*>(out), n4, static_cast<unsigned char*>(out) + 16 * n4, ntail);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int launch_scatter(ilm_cache_s* c, int pc, const void* in1, int coef1, const void* in2, int coef2, void* out,
                   cudaStream_t st, bool accumulate) {
  const Shape2 sh = c->grid.shape(pc);
  const TileList& tl = c->tiles[pc];
  const int dx = pc_dx(pc), dy = pc_dy(pc);
  dim3 blk(TILE_X, TILE_Y);
  if (!accumulate) {
    // overwrite: one launch over every tile (zeros where no point reaches)
    const int ntiles = tl.ntx * tl.nty;
    if (ntiles == 0) return ILM_OK;
    const int nocc = tl.nne_launch;
    const int nb = nocc + (ntiles + SCAT_TPB - 1) / SCAT_TPB;
    if (c->dtype == ILM_F64)
      ILM_CHECK_CUDA(launch_pdl(k_scatter_all<double>, dim3(nb), blk, st, sh.n1, sh.n2, tl.ntx, ntiles, nocc,
                                tl.ne.as<int>(), tl.ne_cnt.as<int>(), tl.ptr.as<int>(), tl.pts.as<int>(),
                                c->bx[dx].as<int>(), c->by[dy].as<int>(), c->wx[dx].as<double>(),
                                c->wy[dy].as<double>(), c->wscale.as<double>(), c->nx.as<double>(),
                                c->ny.as<double>(), static_cast<const double*>(in1), coef1,
                                static_cast<const double*>(in2), coef2, static_cast<double*>(out)));
    else
      ILM_CHECK_CUDA(launch_pdl(k_scatter_all<float>, dim3(nb), blk, st, sh.n1, sh.n2, tl.ntx, ntiles, nocc,
                                tl.ne.as<int>(), tl.ne_cnt.as<int>(), tl.ptr.as<int>(), tl.pts.as<int>(),
                                c->bx[dx].as<int>(), c->by[dy].as<int>(), c->wx[dx].as<float>(),
                                c->wy[dy].as<float>(), c->wscale.as<float>(), c->nx.as<float>(),
                                c->ny.as<float>(), static_cast<const float*>(in1), coef1,
                                static_cast<const float*>(in2), coef2, static_cast<float*>(out)));
    return ILM_OK;
  }
  // accumulate: the occupied tiles only (the others add nothing)
  const int nb = tl.nne_launch;
  if (nb == 0) return ILM_OK;
  if (c->dtype == ILM_F64) {
    k_scatter<double><<<nb, blk, 0, st>>>(sh.n1, sh.n2, tl.ntx, tl.ne.as<int>(), tl.ne_cnt.as<int>(), tl.ptr.as<int>(), tl.pts.as<int>(), c->bx[dx].as<int>(),
                                          c->by[dy].as<int>(), c->wx[dx].as<double>(), c->wy[dy].as<double>(),
                                          c->wscale.as<double>(), c->nx.as<double>(), c->ny.as<double>(),
                                          static_cast<const double*>(in1), coef1, static_cast<const double*>(in2),
                                          coef2, static_cast<double*>(out), 1);
  } else {
    k_scatter<float><<<nb, blk, 0, st>>>(sh.n1, sh.n2, tl.ntx, tl.ne.as<int>(), tl.ne_cnt.as<int>(), tl.ptr.as<int>(), tl.pts.as<int>(), c->bx[dx].as<int>(),
                                         c->by[dy].as<int>(), c->wx[dx].as<float>(), c->wy[dy].as<float>(),
                                         c->wscale.as<float>(), c->nx.as<float>(), c->ny.as<float>(),
                                         static_cast<const float*>(in1), coef1, static_cast<const float*>(in2), coef2,
                                         static_cast<float*>(out), 1);
  }
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int launch_gather(ilm_cache_s* c, const GatherTerm* terms, int nterms, void* out, bool accumulate, double scale,
                  cudaStream_t st) {
  if (nterms < 1 || nterms > 4) {
    set_error("gather: 1..4 terms");
    return ILM_ERR_INVALID_ARG;
  }
  GTermDev td[4];
  for (int q = 0; q < 4; ++q) {
    td[q] = GTermDev{nullptr, 0, 0, 0, 0, CF_ZERO};
    if (q < nterms) {
      const Shape2 sh = c->grid.shape(terms[q].pc);
      td[q].arr = terms[q].arr;
      td[q].n1 = sh.n1;
      td[q].n2 = sh.n2;
      td[q].xsel = pc_dx(terms[q].pc);
      td[q].ysel = pc_dy(terms[q].pc);
      td[q].coef = terms[q].coef;
    }
  }
  const int N = c->npts;
  if (N == 0) return ILM_OK;
  const int bs = 128;
  const int nb = (N + bs - 1) / bs;
  if (c->dtype == ILM_F64) {
    k_gather<double><<<nb, bs, 0, st>>>(N, nullptr, td[0], td[1], td[2], td[3], nterms, c->bx[0].as<int>(),
                                        c->bx[1].as<int>(), c->by[0].as<int>(), c->by[1].as<int>(),
                                        c->wx[0].as<double>(), c->wx[1].as<double>(), c->wy[0].as<double>(),
                                        c->wy[1].as<double>(), c->nx.as<double>(), c->ny.as<double>(),
                                        static_cast<double*>(out), accumulate ? 1 : 0, scale);
  } else {
    k_gather<float><<<nb, bs, 0, st>>>(N, nullptr, td[0], td[1], td[2], td[3], nterms, c->bx[0].as<int>(),
                                       c->bx[1].as<int>(), c->by[0].as<int>(), c->by[1].as<int>(),
                                       c->wx[0].as<float>(), c->wx[1].as<float>(), c->wy[0].as<float>(),
                                       c->wy[1].as<float>(), c->nx.as<float>(), c->ny.as<float>(),
                                       static_cast<float*>(out), accumulate ? 1 : 0, (float)scale);
  }
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

}  // namespace ilm

// ---------------------------------------------------------------------------
// Device re-binning of a cache's points (moving bodies): windows, point
// arrays and tile candidate lists recomputed on the device from new point
// data, with the grid, FFT plans and scratch of the cache kept.
// ---------------------------------------------------------------------------
namespace ilm {

struct RebinPtrs {
  const double *x, *y, *nx, *ny, *ds;
  int* bx[2];
  int* by[2];
  double* wx64[2];
  double* wy64[2];
  void* wx[2];
  void* wy[2];
  void *nxo, *nyo, *wsc;  // cache dtype
  double *nx64, *ny64, *ds64, *x64, *y64;
};

template <typename T>
__global__ void k_rebin_points(int N, RebinPtrs P, double h, int i0x, int i0y, int ddf, int grid_scaling) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  const double xk = P.x[k], yk = P.y[k];
  for (int dual = 0; dual < 2; ++dual) {
    const double off = dual ? 0.5 : 1.0;
    const double rx = xk / h + i0x - off;
    const double ry = yk / h + i0y - off;
    double w[NTAP];
    int b;
    ddf_window(ddf, rx, &b, w);
    P.bx[dual][k] = b;
    for (int t = 0; t < NTAP; ++t) {
      P.wx64[dual][(size_t)k * NTAP + t] = w[t];
      static_cast<T*>(P.wx[dual])[(size_t)k * NTAP + t] = (T)w[t];
    }
    ddf_window(ddf, ry, &b, w);
    P.by[dual][k] = b;
    for (int t = 0; t < NTAP; ++t) {
      P.wy64[dual][(size_t)k * NTAP + t] = w[t];
      static_cast<T*>(P.wy[dual])[(size_t)k * NTAP + t] = (T)w[t];
    }
  }
  static_cast<T*>(P.nxo)[k] = (T)P.nx[k];
  static_cast<T*>(P.nyo)[k] = (T)P.ny[k];
  static_cast<T*>(P.wsc)[k] = (T)(grid_scaling ? P.ds[k] / (h * h) : 1.0);
  P.nx64[k] = P.nx[k];
  P.ny64[k] = P.ny[k];
  P.ds64[k] = P.ds[k];
  P.x64[k] = xk;
  P.y64[k] = yk;
}

// tiles of a position class touched by a point's 4 x 4 window (the host rule)
__device__ __forceinline__ bool window_tiles(int b0, int e0, int n1, int n2, int* tx0, int* tx1, int* ty0,
                                             int* ty1) {
  int b1 = b0 + NTAP - 1, e1 = e0 + NTAP - 1;
  b0 = max(b0, 0);
  e0 = max(e0, 0);
  b1 = min(b1, n1 - 1);
  e1 = min(e1, n2 - 1);
  if (b0 > b1 || e0 > e1) return false;
  *tx0 = b0 / TILE_X;
  *tx1 = b1 / TILE_X;
  *ty0 = e0 / TILE_Y;
  *ty1 = e1 / TILE_Y;
  return true;
}

__global__ void k_tile_count(int N, const int* __restrict__ bx, const int* __restrict__ by, int n1, int n2, int ntx,
                             int* __restrict__ cnt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  int a0, a1, b0, b1;
  if (!window_tiles(bx[k], by[k], n1, n2, &a0, &a1, &b0, &b1)) return;
  for (int ty = b0; ty <= b1; ++ty)
    for (int tx = a0; tx <= a1; ++tx) atomicAdd(&cnt[ty * ntx + tx], 1);
}

// one CTA (1024 threads): ptr = exclusive scan of cnt, cursor = ptr, the
// occupied tiles in tile order and their number
__global__ void __launch_bounds__(1024) k_tile_scan(int nt, const int* __restrict__ cnt, int* __restrict__ ptr,
                                                    int* __restrict__ cursor, int* __restrict__ ne,
                                                    int* __restrict__ ne_cnt) {
  __shared__ int s_sum[1024], s_occ[1024];
  const int T = blockDim.x, i = threadIdx.x;
  const int chunk = (nt + T - 1) / T;
  const int a = min(nt, i * chunk), b = min(nt, a + chunk);
  int sum = 0, occ = 0;
  for (int t = a; t < b; ++t) {
    sum += cnt[t];
    occ += cnt[t] > 0;
  }
  s_sum[i] = sum;
  s_occ[i] = occ;
  __syncthreads();
  if (i == 0) {  // exclusive scan of the per-thread totals (fixed order)
    int rs = 0, ro = 0;
    for (int j = 0; j < T; ++j) {
      const int vs = s_sum[j], vo = s_occ[j];
      s_sum[j] = rs;
      s_occ[j] = ro;
      rs += vs;
      ro += vo;
    }
    ptr[nt] = rs;
    *ne_cnt = ro;
  }
  __syncthreads();
  int run = s_sum[i], o = s_occ[i];
  for (int t = a; t < b; ++t) {
    ptr[t] = run;
    cursor[t] = run;
    run += cnt[t];
    if (cnt[t] > 0) ne[o++] = t;
  }
}

__global__ void k_tile_fill(int N, const int* __restrict__ bx, const int* __restrict__ by, int n1, int n2, int ntx,
                            int* __restrict__ cursor, int* __restrict__ pts) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  int a0, a1, b0, b1;
  if (!window_tiles(bx[k], by[k], n1, n2, &a0, &a1, &b0, &b1)) return;
  for (int ty = b0; ty <= b1; ++ty)
    for (int tx = a0; tx <= a1; ++tx) pts[atomicAdd(&cursor[ty * ntx + tx], 1)] = k;
}

// each tile's candidates in point order (the scatter sums them in list order)
__global__ void k_tile_sort(int nt, const int* __restrict__ ptr, int* __restrict__ pts) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const int a = ptr[t], b = ptr[t + 1];
  for (int i = a + 1; i < b; ++i) {
    const int v = pts[i];
    int j = i - 1;
    while (j >= a && pts[j] > v) {
      pts[j + 1] = pts[j];
      --j;
    }
    pts[j + 1] = v;
  }
}

// ---------------------------------------------------------------------------
// Batched windows and tile lists (ilm_batch_create): every point of every
// problem at once, the same rules as host_windows / k_rebin_points
// ---------------------------------------------------------------------------
struct BGrid {
  int nx, ny, i0x, i0y;
};

__device__ __forceinline__ BGrid bgrid(const BatchGeomDev& G, int p) {
  return BGrid{G.grid[4 * p], G.grid[4 * p + 1], G.grid[4 * p + 2], G.grid[4 * p + 3]};
}

__device__ __forceinline__ void bshape(const BGrid& g, int pc, int* n1, int* n2) {
  const int dx = (pc == PC_D || pc == PC_U) ? 1 : 0, dy = (pc == PC_D || pc == PC_V) ? 1 : 0;
  *n1 = dx ? g.nx : g.nx - 1;
  *n2 = dy ? g.ny : g.ny - 1;
}

template <typename T>
__global__ void k_bwindows(int Ptot, BatchGeomDev G, int ddf, int grid_scaling) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= Ptot) return;
  const int p = G.pt2prob[k];
  const BGrid g = bgrid(G, p);
  const double h = G.h[p];
  const double xk = G.x[k], yk = G.y[k];
  for (int dual = 0; dual < 2; ++dual) {
    const double off = dual ? 0.5 : 1.0;
    const double rx = xk / h + g.i0x - off;
    const double ry = yk / h + g.i0y - off;
    double w[NTAP];
    int b;
    ddf_window(ddf, rx, &b, w);
    G.bx[dual][k] = b;
    for (int t = 0; t < NTAP; ++t) {
      G.wx64[dual][(size_t)k * NTAP + t] = w[t];
      static_cast<T*>(G.wx[dual])[(size_t)k * NTAP + t] = (T)w[t];
    }
    ddf_window(ddf, ry, &b, w);
    G.by[dual][k] = b;
    for (int t = 0; t < NTAP; ++t) {
      G.wy64[dual][(size_t)k * NTAP + t] = w[t];
      static_cast<T*>(G.wy[dual])[(size_t)k * NTAP + t] = (T)w[t];
    }
  }
  static_cast<T*>(G.nxo)[k] = (T)G.nx[k];
  static_cast<T*>(G.nyo)[k] = (T)G.ny[k];
  static_cast<T*>(G.wsc)[k] = (T)(grid_scaling ? G.ds[k] / (h * h) : 1.0);
  G.nx64[k] = G.nx[k];
  G.ny64[k] = G.ny[k];
  G.ds64[k] = G.ds[k];
}

// one thread per (point, position class): count or place the point in the
// tiles its window touches
template <bool FILL>
__global__ void k_btile_place(int Ptot, BatchGeomDev G) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 4 * Ptot) return;
  const int k = idx >> 2, pc = idx & 3;
  const int p = G.pt2prob[k];
  const BGrid g = bgrid(G, p);
  int n1, n2;
  bshape(g, pc, &n1, &n2);
  const int ntx = (n1 + TILE_X - 1) / TILE_X;
  const int dx = (pc == PC_D || pc == PC_U) ? 1 : 0, dy = (pc == PC_D || pc == PC_V) ? 1 : 0;
  int a0, a1, b0, b1;
  if (!window_tiles(G.bx[dx][k], G.by[dy][k], n1, n2, &a0, &a1, &b0, &b1)) return;
  int* cnt = G.cnt + G.cnt_off[pc] + G.tp_off[pc][p];
  for (int ty = b0; ty <= b1; ++ty)
    for (int tx = a0; tx <= a1; ++tx) {
      const int pos = atomicAdd(&cnt[ty * ntx + tx], 1);
      if (FILL) G.tpts[pc][G.ts_off[pc][p] + pos] = k - G.poff[p];
    }
}

// one block per (problem, class): exclusive scan of the tile counts into
// tptr (nt + 1 entries, local to the problem's tpts region); the counters
// become the fill cursors
__global__ void __launch_bounds__(1024) k_btile_scan(BatchGeomDev G) {
  __shared__ int s_sum[1024];
  const int p = blockIdx.x, pc = blockIdx.y;
  const BGrid g = bgrid(G, p);
  int n1, n2;
  bshape(g, pc, &n1, &n2);
  const int nt = ((n1 + TILE_X - 1) / TILE_X) * ((n2 + TILE_Y - 1) / TILE_Y);
  int* cnt = G.cnt + G.cnt_off[pc] + G.tp_off[pc][p];
  int* ptr = G.tptr[pc] + G.tp_off[pc][p];
  const int T = blockDim.x, i = threadIdx.x;
  const int chunk = (nt + T - 1) / T;
  const int a = min(nt, i * chunk), b = min(nt, a + chunk);
  int sum = 0;
  for (int t = a; t < b; ++t) sum += cnt[t];
  s_sum[i] = sum;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {  // inclusive Hillis-Steele scan of the chunk sums
    const int v = i >= off ? s_sum[i - off] : 0;
    __syncthreads();
    s_sum[i] += v;
    __syncthreads();
  }
  int run = s_sum[i] - sum;
  for (int t = a; t < b; ++t) {
    const int c = cnt[t];
    ptr[t] = run;
    cnt[t] = run;
    run += c;
  }
  if (i == T - 1) ptr[nt] = s_sum[T - 1];
}

// per tile: its candidate list in increasing point order (insertion sort,
// lists are short), so the scatters' sums have a fixed order
__global__ void k_btile_sort(BatchGeomDev G) {
  const int p = blockIdx.x, pc = blockIdx.y;
  const BGrid g = bgrid(G, p);
  int n1, n2;
  bshape(g, pc, &n1, &n2);
  const int nt = ((n1 + TILE_X - 1) / TILE_X) * ((n2 + TILE_Y - 1) / TILE_Y);
  const int* ptr = G.tptr[pc] + G.tp_off[pc][p];
  int* pts = G.tpts[pc] + G.ts_off[pc][p];
  for (int t = threadIdx.x; t < nt; t += blockDim.x) {
    const int a = ptr[t], b = ptr[t + 1];
    for (int u = a + 1; u < b; ++u) {
      const int v = pts[u];
      int w = u - 1;
      while (w >= a && pts[w] > v) {
        pts[w + 1] = pts[w];
        --w;
      }
      pts[w + 1] = v;
    }
  }
}

int batch_windows_and_tiles(int nprob, int Ptot, const BatchGeomDev& G, int ddf, int dtype, int grid_scaling,
                            cudaStream_t st) {
  if (Ptot == 0 || nprob == 0) return ILM_OK;
  const int pb = (Ptot + 255) / 256;
  if (dtype == ILM_F64)
    k_bwindows<double><<<pb, 256, 0, st>>>(Ptot, G, ddf, grid_scaling);
  else
    k_bwindows<float><<<pb, 256, 0, st>>>(Ptot, G, ddf, grid_scaling);
  ILM_CHECK_LAUNCH();
  ILM_CHECK_CUDA(cudaMemsetAsync(G.cnt, 0, (size_t)G.cnt_total * sizeof(int), st));
  const int qb = (4 * Ptot + 255) / 256;
  k_btile_place<false><<<qb, 256, 0, st>>>(Ptot, G);
  ILM_CHECK_LAUNCH();
  k_btile_scan<<<dim3(nprob, 4), 1024, 0, st>>>(G);
  ILM_CHECK_LAUNCH();
  k_btile_place<true><<<qb, 256, 0, st>>>(Ptot, G);
  ILM_CHECK_LAUNCH();
  k_btile_sort<<<dim3(nprob, 4), 256, 0, st>>>(G);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int cache_rebin_points(ilm_cache_s* c, const double* x, const double* y, const double* nx, const double* ny,
                       const double* ds, cudaStream_t st) {
  const int N = c->npts;
  if (!c->x64.p) {
    ILM_TRY(c->x64.alloc((size_t)std::max(N, 1) * sizeof(double)));
    ILM_TRY(c->y64.alloc((size_t)std::max(N, 1) * sizeof(double)));
  }
  int ntmax = 1;
  for (int pc = 0; pc < 4; ++pc) ntmax = std::max(ntmax, c->tiles[pc].ntx * c->tiles[pc].nty);
  if (c->rebin_cnt.bytes < (size_t)ntmax * sizeof(int)) {
    ILM_TRY(c->rebin_cnt.alloc((size_t)ntmax * sizeof(int)));
    ILM_TRY(c->rebin_cur.alloc((size_t)ntmax * sizeof(int)));
  }
  if (N == 0) return ILM_OK;
  RebinPtrs P;
  P.x = x;
  P.y = y;
  P.nx = nx;
  P.ny = ny;
  P.ds = ds;
  for (int d = 0; d < 2; ++d) {
    P.bx[d] = c->bx[d].as<int>();
    P.by[d] = c->by[d].as<int>();
    P.wx64[d] = c->wx64[d].as<double>();
    P.wy64[d] = c->wy64[d].as<double>();
    P.wx[d] = c->wx[d].p;
    P.wy[d] = c->wy[d].p;
  }
  P.nxo = c->nx.p;
  P.nyo = c->ny.p;
  P.wsc = c->wscale.p;
  P.nx64 = c->nx64.as<double>();
  P.ny64 = c->ny64.as<double>();
  P.ds64 = c->ds64.as<double>();
  P.x64 = c->x64.as<double>();
  P.y64 = c->y64.as<double>();
  const int pb = (N + 255) / 256;
  if (c->dtype == ILM_F64)
    k_rebin_points<double><<<pb, 256, 0, st>>>(N, P, c->h, c->grid.i0x, c->grid.i0y, c->ddf,
                                                c->scaling == ILM_GRID_SCALING);
  else
    k_rebin_points<float><<<pb, 256, 0, st>>>(N, P, c->h, c->grid.i0x, c->grid.i0y, c->ddf,
                                               c->scaling == ILM_GRID_SCALING);
  ILM_CHECK_LAUNCH();
  for (int pc = 0; pc < 4; ++pc) {
    TileList& tl = c->tiles[pc];
    const Shape2 sh = c->grid.shape(pc);
    const int nt = tl.ntx * tl.nty, dx = pc_dx(pc), dy = pc_dy(pc);
    ILM_CHECK_CUDA(cudaMemsetAsync(c->rebin_cnt.p, 0, (size_t)nt * sizeof(int), st));
    k_tile_count<<<pb, 256, 0, st>>>(N, c->bx[dx].as<int>(), c->by[dy].as<int>(), sh.n1, sh.n2, tl.ntx,
                                     c->rebin_cnt.as<int>());
    ILM_CHECK_LAUNCH();
    k_tile_scan<<<1, 1024, 0, st>>>(nt, c->rebin_cnt.as<int>(), tl.ptr.as<int>(), c->rebin_cur.as<int>(),
                                    tl.ne.as<int>(), tl.ne_cnt.as<int>());
    ILM_CHECK_LAUNCH();
    k_tile_fill<<<pb, 256, 0, st>>>(N, c->bx[dx].as<int>(), c->by[dy].as<int>(), sh.n1, sh.n2, tl.ntx,
                                    c->rebin_cur.as<int>(), tl.pts.as<int>());
    ILM_CHECK_LAUNCH();
    k_tile_sort<<<(nt + 255) / 256, 256, 0, st>>>(nt, tl.ptr.as<int>(), tl.pts.as<int>());
    ILM_CHECK_LAUNCH();
    // the exact count is on the device; launches cover the largest possible
    tl.nne_launch = std::min(nt, 4 * N);
  }
  c->host_stale = true;
  c->S_dir_ready = false;
  c->S_neu_ready = false;
  c->filt_ready = false;
  c->stokes_pc_ready = false;
  return ILM_OK;
}

// host copies (points, windows) brought up to date after device re-binnings
int cache_sync_host(ilm_cache_s* c) {
  if (!c->host_stale) return ILM_OK;
  const size_t N = (size_t)c->npts;
  ILM_CHECK_CUDA(cudaDeviceSynchronize());
  c->hx.resize(N);
  c->hy.resize(N);
  c->hnx.resize(N);
  c->hny.resize(N);
  c->hds.resize(N);
  ILM_CHECK_CUDA(cudaMemcpy(c->hx.data(), c->x64.p, N * 8, cudaMemcpyDeviceToHost));
  ILM_CHECK_CUDA(cudaMemcpy(c->hy.data(), c->y64.p, N * 8, cudaMemcpyDeviceToHost));
  ILM_CHECK_CUDA(cudaMemcpy(c->hnx.data(), c->nx64.p, N * 8, cudaMemcpyDeviceToHost));
  ILM_CHECK_CUDA(cudaMemcpy(c->hny.data(), c->ny64.p, N * 8, cudaMemcpyDeviceToHost));
  ILM_CHECK_CUDA(cudaMemcpy(c->hds.data(), c->ds64.p, N * 8, cudaMemcpyDeviceToHost));
  HostWindows W;
  host_windows(c->grid, c->ddf, c->npts, c->hx.data(), c->hy.data(), &W);
  for (int d = 0; d < 2; ++d) {
    c->hbx[d] = W.bx[d];
    c->hby[d] = W.by[d];
    c->hwx[d] = W.wx[d];
    c->hwy[d] = W.wy[d];
  }
  c->host_stale = false;
  return ILM_OK;
}

}  // namespace ilm
