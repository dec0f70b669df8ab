// Staggered-grid stencils: divergence, gradient, curl (both directions),
// 5-point Laplacian, grid interpolation for masks, and small vector kernels.
//
// Replaces CartesianGrids' divergence!/grad!/curl!/laplacian! as called by
// src/grid_operators.jl:25-134 (with the 1/h GridScaling of :8-9 fused) and
// grid_interpolate! used by the masks (src/surface_operators.jl:880-923).
// All kernels are one thread per output cell, x fastest (coalesced), and write
// every output cell (boundary / ghost cells receive 0), so callers never need a
// separate fill.
#include "ilm_internal.cuh"

namespace ilm {

namespace {

constexpr int BX = 32, BY = 8;

inline dim3 grid2(int n1, int n2) { return dim3((n1 + BX - 1) / BX, (n2 + BY - 1) / BY); }

// Edges{Primal} (u: NX x (NY-1), v: (NX-1) x NY) -> Nodes{Primal} (NX-1)x(NY-1),
// RY rows per thread (rows j, j + BY, ...): every load of a thread is issued
// before its first subtraction, so a thread keeps 4 RY loads in flight (one
// row per thread left HBM idle between the loads of consecutive rows).
// RY consecutive rows per thread (jb .. jb+RY-1): the v value above a row is
// the next row's own, kept in a register; 32-bit indices (checked at
// launch); blocks wholly inside the grid take the path without bounds tests.
template <typename T, int RY, bool IN>
__device__ __forceinline__ void div_edges_rows(int NX, int NY, const T* __restrict__ u, const T* __restrict__ v,
                                               T* __restrict__ w, T sc) {
  const int m = NX - 1;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = (blockIdx.y * BY + threadIdx.y) * RY;
  if (!IN && (i >= m || jb >= NY - 1)) return;
  T u0[RY], u1[RY], vv[RY + 1];
#pragma unroll
  for (int k = 0; k < RY; ++k) {
    const int j = jb + k;
    const bool row = IN || j < NY - 1;
    u0[k] = row ? u[j * NX + i] : (T)0;
    u1[k] = row ? u[j * NX + i + 1] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < RY + 1; ++k) {  // v rows jb .. jb+RY (v is m x NY)
    const int j = jb + k;
    vv[k] = (IN || j < NY) ? v[j * m + i] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < RY; ++k) {
    const int j = jb + k;
    if (IN || j < NY - 1) w[j * m + i] = ((u1[k] - u0[k]) + (vv[k + 1] - vv[k])) * sc;
  }
}

template <typename T, int RY>
__global__ void __launch_bounds__(BX* BY) k_div_edges_r(int NX, int NY, const T* __restrict__ u,
                                                       const T* __restrict__ v, T* __restrict__ w, T sc) {
  pdl_begin();
  const int i0 = blockIdx.x * BX, j0 = blockIdx.y * BY * RY;
  if (i0 + BX - 1 <= NX - 2 && j0 + BY * RY - 1 <= NY - 2)
    div_edges_rows<T, RY, true>(NX, NY, u, v, w, sc);
  else
    div_edges_rows<T, RY, false>(NX, NY, u, v, w, sc);
}

// Nodes{Primal} -> Edges{Primal} (both components); faces adjacent to the
// ghost layer are 0.  RY consecutive rows per thread (jb .. jb+RY-1): a
// row's lower neighbour is the previous row's centre value, kept in a
// register; every load is issued before the arithmetic; 32-bit indices
// (checked at launch).  Blocks whose threads all lie inside the grid
// (1 <= i <= NX-2 and rows 1 .. NY-2, neighbours included) take the path
// with every bounds test constant (IN): the kernel was issue-bound.
template <typename T, int RY, bool IN>
__device__ __forceinline__ void grad_nodes_rows(int NX, int NY, const T* __restrict__ w, T* __restrict__ u,
                                                T* __restrict__ v, T sc) {
  const int m = NX - 1;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = (blockIdx.y * BY + threadIdx.y) * RY;
  if (!IN && (i >= NX || jb >= NY)) return;
  const bool ci = IN || i < m;                     // w (m columns) has column i
  const bool cu = IN || (i >= 1 && i <= NX - 2);  // u nonzero in this column
  T wc[RY + 1], wl[RY];  // wc: column i rows jb-1 .. jb+RY-1; wl: column i-1 rows jb .. jb+RY-1
#pragma unroll
  for (int k = 0; k < RY + 1; ++k) {
    const int j = jb - 1 + k;
    wc[k] = (ci && (IN || (j >= 0 && j < NY - 1))) ? w[j * m + i] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < RY; ++k) {
    const int j = jb + k;
    wl[k] = (cu && (IN || j < NY - 1)) ? w[j * m + i - 1] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < RY; ++k) {
    const int j = jb + k;
    if (!IN && j >= NY) break;
    if (IN || j < NY - 1) u[j * NX + i] = cu ? (wc[k + 1] - wl[k]) * sc : (T)0;
    if (ci) v[j * m + i] = (IN || (j >= 1 && j <= NY - 2)) ? (wc[k + 1] - wc[k]) * sc : (T)0;
  }
}

template <typename T, int RY>
__global__ void __launch_bounds__(BX* BY) k_grad_nodes_r(int NX, int NY, const T* __restrict__ w, T* __restrict__ u,
                                                        T* __restrict__ v, T sc) {
  pdl_begin();
  const int i0 = blockIdx.x * BX, j0 = blockIdx.y * BY * RY;
  if (i0 >= 1 && i0 + BX - 1 <= NX - 2 && j0 >= 1 && j0 + BY * RY - 1 <= NY - 2)
    grad_nodes_rows<T, RY, true>(NX, NY, w, u, v, sc);
  else
    grad_nodes_rows<T, RY, false>(NX, NY, w, u, v, sc);
}

// The curl and Laplacian kernels below take the layout of the divergence and
// gradient: RY consecutive rows per thread (jb .. jb+RY-1), vertical
// neighbours shared in registers, every load before the arithmetic, 32-bit
// indices (checked at launch), a path without bounds tests for the blocks
// inside the grid (IN), programmatic dependent launch.
constexpr int SRY = 4;
inline dim3 grid_rows(int n1, int n2) { return dim3((n1 + BX - 1) / BX, (n2 + BY * SRY - 1) / (BY * SRY)); }
// blockIdx inner: columns [lo, n1 - 1 - hi] and rows [lo, n2 - 1 - hi] hold
// every thread of the block
__device__ __forceinline__ bool block_within(int n1, int n2, int lo, int hi) {
  const int i0 = blockIdx.x * BX, j0 = blockIdx.y * BY * SRY;
  return i0 >= lo && i0 + BX - 1 <= n1 - 1 - hi && j0 >= lo && j0 + BY * SRY - 1 <= n2 - 1 - hi;
}

// Nodes{Dual} (NX x NY) -> Edges{Primal} in one pass: u = s[j+1]-s[j]
// (NX x NY-1), v = s[i]-s[i+1] ((NX-1) x NY)
template <typename T, bool IN>
__device__ __forceinline__ void curl_s_rows(int NX, int NY, const T* __restrict__ s, T* __restrict__ u,
                                            T* __restrict__ v, T sc) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = (blockIdx.y * BY + threadIdx.y) * SRY;
  if (!IN && (i >= NX || jb >= NY)) return;
  const bool vc = IN || i < NX - 1;  // v has column i
  T s0[SRY + 1], s1[SRY];  // s column i rows jb .. jb+SRY; column i+1 rows jb .. jb+SRY-1
#pragma unroll
  for (int k = 0; k < SRY + 1; ++k) {
    const int j = jb + k;
    s0[k] = (IN || j < NY) ? s[j * NX + i] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < SRY; ++k) {
    const int j = jb + k;
    s1[k] = (vc && (IN || j < NY)) ? s[j * NX + i + 1] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < SRY; ++k) {
    const int j = jb + k;
    if (!IN && j >= NY) break;
    if (IN || j < NY - 1) u[j * NX + i] = (s0[k + 1] - s0[k]) * sc;
    if (vc) v[j * (NX - 1) + i] = (s0[k] - s1[k]) * sc;
  }
}
template <typename T>
__global__ void __launch_bounds__(BX* BY) k_curl_s(int NX, int NY, const T* __restrict__ s, T* __restrict__ u,
                                                   T* __restrict__ v, T sc) {
  pdl_begin();
  if (block_within(NX, NY, 0, 1))
    curl_s_rows<T, true>(NX, NY, s, u, v, sc);
  else
    curl_s_rows<T, false>(NX, NY, s, u, v, sc);
}

// Edges{Primal} -> Nodes{Dual}: w = v[i]-v[i-1] - (u[j]-u[j-1]) on interior dual nodes
template <typename T, bool IN>
__device__ __forceinline__ void curl_q_rows(int NX, int NY, const T* __restrict__ u, const T* __restrict__ v,
                                            T* __restrict__ w, T sc) {
  const int m = NX - 1;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = (blockIdx.y * BY + threadIdx.y) * SRY;
  if (!IN && (i >= NX || jb >= NY)) return;
  const bool col = IN || (i >= 1 && i <= NX - 2);
  T uc[SRY + 1], vl[SRY], vr[SRY];  // u column i rows jb-1 .. jb+SRY-1; v columns i-1, i rows jb ..
#pragma unroll
  for (int k = 0; k < SRY + 1; ++k) {
    const int j = jb - 1 + k;
    uc[k] = (col && (IN || (j >= 0 && j <= NY - 2))) ? u[j * NX + i] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < SRY; ++k) {
    const int j = jb + k;
    const bool r = col && (IN || j < NY);
    vl[k] = r ? v[j * m + i - 1] : (T)0;
    vr[k] = r ? v[j * m + i] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < SRY; ++k) {
    const int j = jb + k;
    if (!IN && j >= NY) break;
    T r = (T)0;
    if (IN || (col && j >= 1 && j <= NY - 2)) {
      r = (vr[k] - vl[k]) - (uc[k + 1] - uc[k]);
      r *= sc;
    }
    w[j * NX + i] = r;
  }
}
template <typename T>
__global__ void __launch_bounds__(BX* BY) k_curl_q(int NX, int NY, const T* __restrict__ u, const T* __restrict__ v,
                                                   T* __restrict__ w, T sc) {
  pdl_begin();
  if (block_within(NX, NY, 1, 1))
    curl_q_rows<T, true>(NX, NY, u, v, w, sc);
  else
    curl_q_rows<T, false>(NX, NY, u, v, w, sc);
}

// Edges{Primal} -> EdgeGradient{Primal}: dudx, dvdy ((NX-1) x (NY-1)),
// dudy, dvdx (NX x NY, interior dual nodes only)
template <typename T, bool IN>
__device__ __forceinline__ void grad_edges_rows(int NX, int NY, const T* __restrict__ u, const T* __restrict__ v,
                                                T* __restrict__ dudx, T* __restrict__ dudy, T* __restrict__ dvdx,
                                                T* __restrict__ dvdy, T sc) {
  const int m = NX - 1;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = (blockIdx.y * BY + threadIdx.y) * SRY;
  if (!IN && (i >= NX || jb >= NY)) return;
  const bool cp = IN || i < NX - 1;                 // the (NX-1)-column arrays have column i
  const bool cd = IN || (i >= 1 && i <= NX - 2);    // dudy, dvdx nonzero in this column
  // uc: u column i rows jb-1 .. jb+SRY-1; ur: u column i+1 rows jb .. jb+SRY-1;
  // vc: v column i rows jb .. jb+SRY; vl: v column i-1 rows jb .. jb+SRY-1
  T uc[SRY + 1], ur[SRY], vc[SRY + 1], vl[SRY];
#pragma unroll
  for (int k = 0; k < SRY + 1; ++k) {
    const int j = jb - 1 + k;
    uc[k] = (IN || (j >= 0 && j <= NY - 2)) ? u[j * NX + i] : (T)0;
    const int jv = jb + k;
    vc[k] = (cp && (IN || jv < NY)) ? v[jv * m + i] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < SRY; ++k) {
    const int j = jb + k;
    ur[k] = (cp && (IN || j <= NY - 2)) ? u[j * NX + i + 1] : (T)0;
    vl[k] = (cd && (IN || j < NY)) ? v[j * m + i - 1] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < SRY; ++k) {
    const int j = jb + k;
    if (!IN && j >= NY) break;
    if (cp && (IN || j < NY - 1)) {
      dudx[j * m + i] = (ur[k] - uc[k + 1]) * sc;
      dvdy[j * m + i] = (vc[k + 1] - vc[k]) * sc;
    }
    T a = (T)0, b = (T)0;
    if (IN || (cd && j >= 1 && j <= NY - 2)) {
      a = (uc[k + 1] - uc[k]) * sc;
      b = (vc[k] - vl[k]) * sc;
    }
    dudy[j * NX + i] = a;
    dvdx[j * NX + i] = b;
  }
}
template <typename T>
__global__ void __launch_bounds__(BX* BY) k_grad_edges(int NX, int NY, const T* __restrict__ u, const T* __restrict__ v,
                                                       T* __restrict__ dudx, T* __restrict__ dudy, T* __restrict__ dvdx,
                                                       T* __restrict__ dvdy, T sc) {
  pdl_begin();
  if (block_within(NX, NY, 1, 1))
    grad_edges_rows<T, true>(NX, NY, u, v, dudx, dudy, dvdx, dvdy, sc);
  else
    grad_edges_rows<T, false>(NX, NY, u, v, dudx, dudy, dvdx, dvdy, sc);
}

// EdgeGradient{Primal} -> Edges{Primal}: u (NX x NY-1) from dudx, dudy on the
// interior columns, v ((NX-1) x NY) from dvdx, dvdy on the interior rows
template <typename T, bool IN>
__device__ __forceinline__ void div_edgegrad_rows(int NX, int NY, const T* __restrict__ dudx,
                                                  const T* __restrict__ dudy, const T* __restrict__ dvdx,
                                                  const T* __restrict__ dvdy, T* __restrict__ u, T* __restrict__ v,
                                                  T sc) {
  const int m = NX - 1;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = (blockIdx.y * BY + threadIdx.y) * SRY;
  if (!IN && (i >= NX || jb >= NY)) return;
  const bool cu = IN || (i >= 1 && i <= NX - 2);  // u nonzero in this column
  const bool cv = IN || i < NX - 1;               // v has this column
  // xl, xr: dudx columns i-1, i rows jb .. jb+SRY-1; yc: dudy column i rows
  // jb .. jb+SRY; vx0, vx1: dvdx columns i, i+1 rows jb .. jb+SRY-1; vy: dvdy
  // column i rows jb-1 .. jb+SRY-1
  T xl[SRY], xr[SRY], yc[SRY + 1], vx0[SRY], vx1[SRY], vy[SRY + 1];
#pragma unroll
  for (int k = 0; k < SRY + 1; ++k) {
    const int j = jb + k;
    yc[k] = (cu && (IN || j < NY)) ? dudy[j * NX + i] : (T)0;
    const int jy = jb - 1 + k;
    vy[k] = (cv && (IN || (jy >= 0 && jy <= NY - 2))) ? dvdy[jy * m + i] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < SRY; ++k) {
    const int j = jb + k;
    const bool ur = cu && (IN || j <= NY - 2);
    xl[k] = ur ? dudx[j * m + i - 1] : (T)0;
    xr[k] = ur ? dudx[j * m + i] : (T)0;
    const bool vr = cv && (IN || j < NY);
    vx0[k] = vr ? dvdx[j * NX + i] : (T)0;
    vx1[k] = vr ? dvdx[j * NX + i + 1] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < SRY; ++k) {
    const int j = jb + k;
    if (!IN && j >= NY) break;
    if (IN || j < NY - 1) u[j * NX + i] = cu ? ((xr[k] - xl[k]) + (yc[k + 1] - yc[k])) * sc : (T)0;
    if (cv) {
      T r = (T)0;
      if (IN || (j >= 1 && j <= NY - 2)) r = ((vx1[k] - vx0[k]) + (vy[k + 1] - vy[k])) * sc;
      v[j * m + i] = r;
    }
  }
}
template <typename T>
__global__ void __launch_bounds__(BX* BY) k_div_edgegrad(int NX, int NY, const T* __restrict__ dudx,
                                                         const T* __restrict__ dudy, const T* __restrict__ dvdx,
                                                         const T* __restrict__ dvdy, T* __restrict__ u,
                                                         T* __restrict__ v, T sc) {
  pdl_begin();
  if (block_within(NX, NY, 1, 1))
    div_edgegrad_rows<T, true>(NX, NY, dudx, dudy, dvdx, dvdy, u, v, sc);
  else
    div_edgegrad_rows<T, false>(NX, NY, dudx, dudy, dvdx, dvdy, u, v, sc);
}

// 5-point Laplacian on an n1 x n2 node grid (interior nodes; the outer ring
// is 0), times sc
template <typename T, bool IN>
__device__ __forceinline__ void laplacian_rows(int n1, int n2, const T* __restrict__ a, T* __restrict__ o, T sc) {
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = (blockIdx.y * BY + threadIdx.y) * SRY;
  if (!IN && (i >= n1 || jb >= n2)) return;
  const bool col = IN || (i >= 1 && i <= n1 - 2);
  T ac[SRY + 2], al[SRY], ar[SRY];  // column i rows jb-1 .. jb+SRY; columns i-1, i+1 rows jb .. jb+SRY-1
#pragma unroll
  for (int k = 0; k < SRY + 2; ++k) {
    const int j = jb - 1 + k;
    ac[k] = (col && (IN || (j >= 0 && j < n2))) ? a[j * n1 + i] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < SRY; ++k) {
    const int j = jb + k;
    const bool r = col && (IN || j < n2);
    al[k] = r ? a[j * n1 + i - 1] : (T)0;
    ar[k] = r ? a[j * n1 + i + 1] : (T)0;
  }
#pragma unroll
  for (int k = 0; k < SRY; ++k) {
    const int j = jb + k;
    if (!IN && j >= n2) break;
    T r = (T)0;
    if (IN || (col && j >= 1 && j <= n2 - 2)) r = (ar[k] + al[k] + ac[k + 2] + ac[k] - (T)4 * ac[k + 1]) * sc;
    o[j * n1 + i] = r;
  }
}
template <typename T>
__global__ void __launch_bounds__(BX* BY) k_laplacian(int n1, int n2, const T* __restrict__ a, T* __restrict__ o,
                                                      T sc) {
  pdl_begin();
  if (block_within(n1, n2, 1, 1))
    laplacian_rows<T, true>(n1, n2, a, o, sc);
  else
    laplacian_rows<T, false>(n1, n2, a, o, sc);
}

// Nodes{Primal} -> Nodes{Dual} (4-point average on interior dual nodes)
// Edges{Primal}.u (NX x NY-1) -> Nodes{Dual}: mean over y onto the
// non-ghost dual rows (ghost rows 0), the vector-cache mask interpolation
template <typename T>
__global__ void k_xe2d(int NX, int NY, const T* __restrict__ u, T* __restrict__ o) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i >= NX || j >= NY) return;
  o[(size_t)j * NX + i] = (j >= 1 && j <= NY - 2) ? (T)0.5 * (u[(size_t)(j - 1) * NX + i] + u[(size_t)j * NX + i]) : (T)0;
}
// Edges{Primal}.u -> Nodes{Primal} ((NX-1) x (NY-1)): mean over x
template <typename T>
__global__ void k_xe2p(int NX, int NY, const T* __restrict__ u, T* __restrict__ o) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i >= NX - 1 || j >= NY - 1) return;
  o[(size_t)j * (NX - 1) + i] = (T)0.5 * (u[(size_t)j * NX + i] + u[(size_t)j * NX + i + 1]);
}

template <typename T>
__global__ void k_p2d(int NX, int NY, const T* __restrict__ p, T* __restrict__ o) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i >= NX || j >= NY) return;
  T r = (T)0;
  if (i >= 1 && i <= NX - 2 && j >= 1 && j <= NY - 2) {
    const int m = NX - 1;
    r = (T)0.25 * (p[(size_t)(j - 1) * m + i - 1] + p[(size_t)(j - 1) * m + i] + p[(size_t)j * m + i - 1] +
                   p[(size_t)j * m + i]);
  }
  o[(size_t)j * NX + i] = r;
}

// Nodes{Primal} -> Edges{Primal} (2-point averages)
template <typename T>
__global__ void k_p2e(int NX, int NY, const T* __restrict__ p, T* __restrict__ u, T* __restrict__ v) {
  const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i >= NX || j >= NY) return;
  const int m = NX - 1;
  if (j < NY - 1) {
    T r = (T)0;
    if (i >= 1 && i <= NX - 2) r = (T)0.5 * (p[(size_t)j * m + i - 1] + p[(size_t)j * m + i]);
    u[(size_t)j * NX + i] = r;
  }
  if (i < NX - 1) {
    T r = (T)0;
    if (j >= 1 && j <= NY - 2) r = (T)0.5 * (p[(size_t)(j - 1) * m + i] + p[(size_t)j * m + i]);
    v[(size_t)j * m + i] = r;
  }
}

// out += a * b (elementwise)
template <typename T>
__global__ void k_mul_add(size_t n, const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] += a[i] * b[i];
}

template <typename T>
__global__ void k_axpby(size_t n, T a, const T* __restrict__ x, T b, const T* __restrict__ y, T* __restrict__ o) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    T r = a * x[i];
    if (y) r += b * y[i];
    o[i] = r;
  }
}

template <typename T>
__global__ void k_affine(size_t n, T a, const T* __restrict__ x, T b, T* __restrict__ o) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    o[i] = a * x[i] + b;
}

template <typename T>
__global__ void k_fill(size_t n, T v, T* __restrict__ o) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) o[i] = v;
}

template <typename T>
__global__ void k_mul(size_t n, const T* __restrict__ a, T* __restrict__ o) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) o[i] *= a[i];
}

template <typename A, typename B>
__global__ void k_convert(size_t n, const A* __restrict__ in, B* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (B)in[i];
}

// weighted grid dot: dual direction interior only, primal trapezoid.  One
// block per row, fixed-order tree reduction -> per-row partials, then a
// single block sums the rows in order (deterministic).
template <typename T>
__global__ void k_wdot_rows(int n1, int n2, int dx, int dy, const T* __restrict__ a, const T* __restrict__ b,
                            double* __restrict__ part) {
  __shared__ double sh[256];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int i = threadIdx.x; i < n1; i += blockDim.x) {
    double wx = 1.0;
    if (i == 0 || i == n1 - 1) wx = dx ? 0.0 : 0.5;
    s += wx * (double)a[(size_t)j * n1 + i] * (double)b[(size_t)j * n1 + i];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double wy = 1.0;
    if (j == 0 || j == n2 - 1) wy = dy ? 0.0 : 0.5;
    part[j] = wy * sh[0];
  }
}

__global__ void k_sum_ordered(int n, const double* __restrict__ part, double* __restrict__ out, double scale) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0] * scale;
}

template <typename T>
__global__ void k_pdot(int n, const T* __restrict__ a, const T* __restrict__ b, const double* __restrict__ w,
                       double* __restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += (w ? w[i] : 1.0) * (double)a[i] * (double)b[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

inline int nblocks(size_t n) {
  size_t b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

#define DISPATCH(dtype, ...)                      \
  do {                                            \
    if ((dtype) == ILM_F64) {                     \
      using T = double;                           \
      __VA_ARGS__;                                \
    } else {                                      \
      using T = float;                            \
      __VA_ARGS__;                                \
    }                                             \
  } while (0)

int st_div_edges(const ilm_grid_s* g, int dtype, const void* q, void* w, double scale, cudaStream_t st) {
  const int NX = g->nx, NY = g->ny;
  ILM_REQUIRE((long long)NX * NY < (1LL << 31), "divergence: grid of %d x %d exceeds 32-bit indexing", NX, NY);
  DISPATCH(dtype, {
    const T* u = static_cast<const T*>(q);
    const T* v = u + (size_t)NX * (NY - 1);
    constexpr int RY = 4;
    const dim3 grid((NX - 1 + BX - 1) / BX, (NY - 1 + BY * RY - 1) / (BY * RY));
    ILM_CHECK_CUDA(launch_pdl(k_div_edges_r<T, RY>, grid, dim3(BX, BY), st, NX, NY, u, v, static_cast<T*>(w),
                              (T)scale));
  });
  return ILM_OK;
}

int st_grad_nodes(const ilm_grid_s* g, int dtype, const void* w, void* q, double scale, cudaStream_t st) {
  const int NX = g->nx, NY = g->ny;
  ILM_REQUIRE((long long)NX * NY < (1LL << 31), "grad: grid of %d x %d exceeds 32-bit indexing", NX, NY);
  DISPATCH(dtype, {
    T* u = static_cast<T*>(q);
    T* v = u + (size_t)NX * (NY - 1);
    constexpr int RY = 4;
    const dim3 grid((NX + BX - 1) / BX, (NY + BY * RY - 1) / (BY * RY));
    ILM_CHECK_CUDA(launch_pdl(k_grad_nodes_r<T, RY>, grid, dim3(BX, BY), st, NX, NY, static_cast<const T*>(w), u, v,
                              (T)scale));
  });
  return ILM_OK;
}

int st_curl_dual_to_edges(const ilm_grid_s* g, int dtype, const void* s, void* q, double scale, cudaStream_t st) {
  const int NX = g->nx, NY = g->ny;
  ILM_REQUIRE((long long)NX * NY < (1LL << 31), "curl: grid of %d x %d exceeds 32-bit indexing", NX, NY);
  DISPATCH(dtype, {
    T* u = static_cast<T*>(q);
    T* v = u + (size_t)NX * (NY - 1);
    ILM_CHECK_CUDA(launch_pdl(k_curl_s<T>, grid_rows(NX, NY), dim3(BX, BY), st, NX, NY, static_cast<const T*>(s), u,
                              v, (T)scale));
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_curl_edges_to_dual(const ilm_grid_s* g, int dtype, const void* q, void* w, double scale, cudaStream_t st) {
  const int NX = g->nx, NY = g->ny;
  ILM_REQUIRE((long long)NX * NY < (1LL << 31), "curl: grid of %d x %d exceeds 32-bit indexing", NX, NY);
  DISPATCH(dtype, {
    const T* u = static_cast<const T*>(q);
    const T* v = u + (size_t)NX * (NY - 1);
    ILM_CHECK_CUDA(launch_pdl(k_curl_q<T>, grid_rows(NX, NY), dim3(BX, BY), st, NX, NY, u, v, static_cast<T*>(w),
                              (T)scale));
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_grad_edges(const ilm_grid_s* g, int dtype, const void* q, void* t, double scale, cudaStream_t st) {
  const int NX = g->nx, NY = g->ny;
  ILM_REQUIRE((long long)NX * NY < (1LL << 31), "vector gradient: grid of %d x %d exceeds 32-bit indexing", NX, NY);
  const size_t np = (size_t)(NX - 1) * (NY - 1), nd = (size_t)NX * NY;
  DISPATCH(dtype, {
    const T* u = static_cast<const T*>(q);
    const T* v = u + (size_t)NX * (NY - 1);
    T* dudx = static_cast<T*>(t);
    T* dudy = dudx + np;
    T* dvdx = dudy + nd;
    T* dvdy = dvdx + nd;
    ILM_CHECK_CUDA(launch_pdl(k_grad_edges<T>, grid_rows(NX, NY), dim3(BX, BY), st, NX, NY, u, v, dudx, dudy, dvdx,
                              dvdy, (T)scale));
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_div_edgegrad(const ilm_grid_s* g, int dtype, const void* t, void* q, double scale, cudaStream_t st) {
  const int NX = g->nx, NY = g->ny;
  ILM_REQUIRE((long long)NX * NY < (1LL << 31), "vector gradient: grid of %d x %d exceeds 32-bit indexing", NX, NY);
  const size_t np = (size_t)(NX - 1) * (NY - 1), nd = (size_t)NX * NY;
  DISPATCH(dtype, {
    const T* dudx = static_cast<const T*>(t);
    const T* dudy = dudx + np;
    const T* dvdx = dudy + nd;
    const T* dvdy = dvdx + nd;
    T* u = static_cast<T*>(q);
    T* v = u + (size_t)NX * (NY - 1);
    ILM_CHECK_CUDA(launch_pdl(k_div_edgegrad<T>, grid_rows(NX, NY), dim3(BX, BY), st, NX, NY, dudx, dudy, dvdx,
                              dvdy, u, v, (T)scale));
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_laplacian(int n1, int n2, int dtype, const void* in, void* out, double scale, cudaStream_t st) {
  ILM_REQUIRE((long long)n1 * n2 < (1LL << 31), "laplacian: grid of %d x %d exceeds 32-bit indexing", n1, n2);
  DISPATCH(dtype, {
    ILM_CHECK_CUDA(launch_pdl(k_laplacian<T>, grid_rows(n1, n2), dim3(BX, BY), st, n1, n2, static_cast<const T*>(in),
                              static_cast<T*>(out), (T)scale));
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_primal_to_dual(const ilm_grid_s* g, int dtype, const void* p, void* out, cudaStream_t st) {
  DISPATCH(dtype, {
    k_p2d<T><<<grid2(g->nx, g->ny), dim3(BX, BY), 0, st>>>(g->nx, g->ny, static_cast<const T*>(p),
                                                           static_cast<T*>(out));
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_xedge_to_dual(const ilm_grid_s* g, int dtype, const void* u, void* out, cudaStream_t st) {
  DISPATCH(dtype, {
    k_xe2d<T><<<grid2(g->nx, g->ny), dim3(BX, BY), 0, st>>>(g->nx, g->ny, static_cast<const T*>(u),
                                                            static_cast<T*>(out));
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_xedge_to_primal(const ilm_grid_s* g, int dtype, const void* u, void* out, cudaStream_t st) {
  DISPATCH(dtype, {
    k_xe2p<T><<<grid2(g->nx, g->ny), dim3(BX, BY), 0, st>>>(g->nx, g->ny, static_cast<const T*>(u),
                                                            static_cast<T*>(out));
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_primal_to_edges(const ilm_grid_s* g, int dtype, const void* p, void* out, cudaStream_t st) {
  DISPATCH(dtype, {
    T* u = static_cast<T*>(out);
    T* v = u + (size_t)g->nx * (g->ny - 1);
    k_p2e<T><<<grid2(g->nx, g->ny), dim3(BX, BY), 0, st>>>(g->nx, g->ny, static_cast<const T*>(p), u, v);
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_axpby(size_t n, int dtype, double a, const void* x, double b, const void* y, void* out, cudaStream_t st) {
  if (n == 0) return ILM_OK;
  DISPATCH(dtype, {
    k_axpby<T><<<nblocks(n), 256, 0, st>>>(n, (T)a, static_cast<const T*>(x), (T)b, static_cast<const T*>(y),
                                           static_cast<T*>(out));
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_mul_add(size_t n, int dtype, const void* a, const void* b, void* out, cudaStream_t st) {
  if (n == 0) return ILM_OK;
  DISPATCH(dtype, {
    k_mul_add<T><<<nblocks(n), 256, 0, st>>>(n, static_cast<const T*>(a), static_cast<const T*>(b),
                                             static_cast<T*>(out));
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_fill(size_t n, int dtype, double v, void* out, cudaStream_t st) {
  if (n == 0) return ILM_OK;
  DISPATCH(dtype, { k_fill<T><<<nblocks(n), 256, 0, st>>>(n, (T)v, static_cast<T*>(out)); });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_affine(size_t n, int dtype, double a, const void* x, double b, void* out, cudaStream_t st) {
  if (n == 0) return ILM_OK;
  DISPATCH(dtype, {
    k_affine<T><<<nblocks(n), 256, 0, st>>>(n, (T)a, static_cast<const T*>(x), (T)b, static_cast<T*>(out));
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_mul(size_t n, int dtype, const void* a, void* inout, cudaStream_t st) {
  if (n == 0) return ILM_OK;
  DISPATCH(dtype, { k_mul<T><<<nblocks(n), 256, 0, st>>>(n, static_cast<const T*>(a), static_cast<T*>(inout)); });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_convert(size_t n, int dtype_in, const void* in, int dtype_out, void* out, cudaStream_t st) {
  if (n == 0) return ILM_OK;
  if (dtype_in == ILM_F64 && dtype_out == ILM_F32)
    k_convert<double, float><<<nblocks(n), 256, 0, st>>>(n, static_cast<const double*>(in), static_cast<float*>(out));
  else if (dtype_in == ILM_F32 && dtype_out == ILM_F64)
    k_convert<float, double><<<nblocks(n), 256, 0, st>>>(n, static_cast<const float*>(in), static_cast<double*>(out));
  else if (dtype_in == ILM_F64)
    k_convert<double, double><<<nblocks(n), 256, 0, st>>>(n, static_cast<const double*>(in), static_cast<double*>(out));
  else
    k_convert<float, float><<<nblocks(n), 256, 0, st>>>(n, static_cast<const float*>(in), static_cast<float*>(out));
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_weighted_dot(int n1, int n2, int dx, int dy, int dtype, const void* a, const void* b, double* dres,
                    cudaStream_t st) {
  // dres: device buffer of at least n2 + 1 doubles; result in dres[n2]
  DISPATCH(dtype, {
    k_wdot_rows<T><<<n2, 256, 0, st>>>(n1, n2, dx, dy, static_cast<const T*>(a), static_cast<const T*>(b), dres);
  });
  ILM_CHECK_LAUNCH();
  k_sum_ordered<<<1, 256, 0, st>>>(n2, dres, dres + n2, 1.0);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_point_dot(int n, int dtype, const void* a, const void* b, const double* w, double* dres, cudaStream_t st) {
  DISPATCH(dtype, {
    k_pdot<T><<<1, 256, 0, st>>>(n, static_cast<const T*>(a), static_cast<const T*>(b), w, dres);
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

}  // namespace ilm
