// Convective derivatives and the rotational term w x v on the staggered grid
// (src/grid_operators.jl:186-434), each fused into one stencil pass.
//
// The reference forms them in steps through a ConvectiveDerivativeCache:
// grad! into an EdgeGradient (or Edges) temporary, CartesianGrids'
// grid_interpolate! of the velocity into a second one, transpose!, a
// pointwise product into a third, and grid_interpolate! back -- four to six
// full-grid passes and three temporaries.  Here every output value gathers
// its few neighbours of v and q, forms the differences, the averages and the
// products in registers and is written once: each kernel reads v and q and
// writes the result (HBM traffic = inputs + output), and no temporary grid
// exists.
//
// grid_interpolate! (CartesianGrids, un-vendored) is the staggered-grid
// average: onto a primal position from the two dual neighbours everywhere;
// onto a dual position from the two primal neighbours only at the non-ghost
// dual positions 1..n-2 (the ghost layers stay zero), the same boundary rule
// as grad!/curl! onto dual positions.  Layout: x fastest; Edges{Primal} =
// [u (NX x NY-1); v (NX-1 x NY)]; Nodes{Primal} (NX-1)x(NY-1); Nodes{Dual}
// NX x NY.  Indices are 32-bit (grids below 2^31 values; checked at launch):
// the kernels issue more instructions than they move bytes, and 64-bit index
// arithmetic was a large part of them.
#include "ilm_internal.cuh"

namespace ilm {

namespace {

constexpr int BX = 32, BY = 8, RY = 4;

inline dim3 grid2(int n1, int n2) { return dim3((n1 + BX - 1) / BX, (n2 + BY * RY - 1) / (BY * RY)); }

template <typename T>
__device__ __forceinline__ T ld(const T* p, int k) {
  return __ldg(p + k);
}

// A block is inner when every thread's columns i-1 .. i+2 and rows jb-1 ..
// jb+RY+1 lie inside the grid with the ghost layers excluded: columns
// 1 <= i <= NX-3 and rows 1 <= jb, jb+RY <= NY-2 for all of its threads.
// The kernels below then take a path with every bounds test constant (IN =
// true); the blocks along the edges take the general one.
__device__ __forceinline__ bool inner_block(int NX, int NY) {
  const int i0 = blockIdx.x * BX, j0 = blockIdx.y * BY * RY;
  return i0 >= 1 && i0 + BX - 1 <= NX - 3 && j0 >= 1 && j0 + BY * RY <= NY - 2;
}

// v . grad p, p on Nodes{Primal} (m = NX-1 by NY-1), v on Edges{Primal}
// (:318-328).  gx at dual x k: p[k]-p[k-1] for 1 <= k <= NX-2, else 0.
// RY consecutive output rows per thread (jb .. jb+RY-1): the rows share
// their vertical neighbours in registers, and every load of the RY rows is
// issued before the arithmetic.
template <typename T, bool IN>
__device__ __forceinline__ void vdp_np_rows(int NX, int NY, const T* __restrict__ vu, const T* __restrict__ vv,
    const T* __restrict__ p, T* __restrict__ out, T sc) {
  const int m = NX - 1, n = NY - 1;  // p is m x n
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = (blockIdx.y * BY + threadIdx.y) * RY;
  if (!IN && (i >= m || jb >= n)) return;
  const bool has_l = IN || i >= 1, has_r = IN || i + 1 <= NX - 2;
  T pc[RY + 2], pl[RY], pr[RY], u0[RY], u1[RY], vd[RY + 1];
#pragma unroll
  for (int k = 0; k < RY + 2; ++k) {  // p column i, rows jb-1 .. jb+RY
    const int j = jb - 1 + k;
    pc[k] = (IN || (j >= 0 && j < n)) ? ld(p, j * m + i) : (T)0;
  }
#pragma unroll
  for (int k = 0; k < RY; ++k) {
    const int j = jb + k;
    const bool ok = IN || j < n;
    pl[k] = (ok && has_l) ? ld(p, j * m + i - 1) : (T)0;
    pr[k] = (ok && has_r) ? ld(p, j * m + i + 1) : (T)0;
    u0[k] = ok ? ld(vu, j * NX + i) : (T)0;
    u1[k] = ok ? ld(vu, j * NX + i + 1) : (T)0;
  }
#pragma unroll
  for (int k = 0; k < RY + 1; ++k) {  // vv column i, rows jb .. jb+RY (vv is m x NY)
    const int j = jb + k;
    vd[k] = (IN || j < NY) ? ld(vv, j * m + i) : (T)0;
  }
#pragma unroll
  for (int k = 0; k < RY; ++k) {
    const int j = jb + k;
    if (IN || j < n) {
      const T c = pc[k + 1];
      const T gxl = has_l ? c - pl[k] : (T)0;
      const T gxr = has_r ? pr[k] - c : (T)0;
      const T gyd = (IN || j >= 1) ? c - pc[k] : (T)0;
      const T gyu = (IN || j + 1 <= NY - 2) ? pc[k + 2] - c : (T)0;
      const T tx = u0[k] * gxl + u1[k] * gxr;
      const T ty = vd[k] * gyd + vd[k + 1] * gyu;
      out[j * m + i] = (T)0.5 * (tx + ty) * sc;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(BX* BY) k_vdp_np(int NX, int NY, const T* __restrict__ vu, const T* __restrict__ vv,
    const T* __restrict__ p, T* __restrict__ out, T sc) {
  pdl_begin();
  if (inner_block(NX, NY))
    vdp_np_rows<T, true>(NX, NY, vu, vv, p, out, sc);
  else
    vdp_np_rows<T, false>(NX, NY, vu, vv, p, out, sc);
}

// v . grad w, w on Nodes{Dual} (NX x NY), v on Edges{Primal} (:330-342):
// v averaged onto the Edges{Dual} positions (four-point means), times the
// Edges{Dual} gradient of w, averaged onto the non-ghost dual nodes.
// RY consecutive output rows per thread (jb .. jb+RY-1), vertical
// neighbours shared in registers, every load issued before the arithmetic.
// Interior cells only (1 <= i <= NX-2, 1 <= j <= NY-2); the ghost layer is 0.
template <typename T, bool IN>
__device__ __forceinline__ void vdw_nd_rows(int NX, int NY, const T* __restrict__ vu, const T* __restrict__ vv,
    const T* __restrict__ w, T* __restrict__ out, T sc) {
  const int m = NX - 1;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = (blockIdx.y * BY + threadIdx.y) * RY;
  if (!IN && (i >= NX || jb >= NY)) return;
  const bool col = IN || (i >= 1 && i <= NX - 2);
  // wc: w column i rows jb-1 .. jb+RY; wl, wr: columns i-1, i+1 rows jb ..
  // jb+RY-1; a0..a2: vu columns i-1, i, i+1 rows jb-1 .. jb+RY-1 (vu is
  // NX x NY-1); e0, e1: vv columns i-1, i rows jb-1 .. jb+RY (vv is m x NY)
  T wc[RY + 2], wl[RY], wr[RY], a0[RY + 1], a1[RY + 1], a2[RY + 1], e0[RY + 2], e1[RY + 2];
#pragma unroll
  for (int k = 0; k < RY + 2; ++k) {
    const int j = jb - 1 + k;
    const bool row = IN || (col && j >= 0 && j < NY);
    wc[k] = row ? ld(w, j * NX + i) : (T)0;
    e0[k] = row ? ld(vv, j * m + i - 1) : (T)0;
    e1[k] = row ? ld(vv, j * m + i) : (T)0;
    if (k < RY + 1) {
      const bool urow = IN || (col && j >= 0 && j <= NY - 2);
      a0[k] = urow ? ld(vu, j * NX + i - 1) : (T)0;
      a1[k] = urow ? ld(vu, j * NX + i) : (T)0;
      a2[k] = urow ? ld(vu, j * NX + i + 1) : (T)0;
    }
    if (k >= 1 && k <= RY) {
      wl[k - 1] = row ? ld(w, j * NX + i - 1) : (T)0;
      wr[k - 1] = row ? ld(w, j * NX + i + 1) : (T)0;
    }
  }
#pragma unroll
  for (int k = 0; k < RY; ++k) {
    const int j = jb + k;
    if (!IN && j >= NY) break;
    T r = (T)0;
    if (IN || (col && j >= 1 && j <= NY - 2)) {
      const T c = wc[k + 1];
      // Edges{Dual}.u at (primal x i-1 / i, dual y j): mean of vu over
      // dual x and primal y j-1, j
      const T udl = (T)0.25 * (a0[k] + a1[k] + a0[k + 1] + a1[k + 1]);
      const T udr = (T)0.25 * (a1[k] + a2[k] + a1[k + 1] + a2[k + 1]);
      const T tx = udl * (c - wl[k]) + udr * (wr[k] - c);
      // Edges{Dual}.v at (dual x i, primal y j-1 / j): mean of vv over
      // primal x i-1, i and dual y
      const T s0 = e0[k] + e1[k], s1 = e0[k + 1] + e1[k + 1], s2 = e0[k + 2] + e1[k + 2];
      const T vdd = (T)0.25 * (s0 + s1), vdu = (T)0.25 * (s1 + s2);
      const T ty = vdd * (c - wc[k]) + vdu * (wc[k + 2] - c);
      r = (T)0.5 * (tx + ty) * sc;
    }
    out[j * NX + i] = r;
  }
}

template <typename T>
__global__ void __launch_bounds__(BX* BY) k_vdw_nd(int NX, int NY, const T* __restrict__ vu, const T* __restrict__ vv,
    const T* __restrict__ w, T* __restrict__ out, T sc) {
  pdl_begin();
  if (inner_block(NX, NY))
    vdw_nd_rows<T, true>(NX, NY, vu, vv, w, out, sc);
  else
    vdw_nd_rows<T, false>(NX, NY, vu, vv, w, out, sc);
}

// v . grad u for Edges{Primal} v and u (:344-371; u . grad u with v = u).
// Thread (i, j) writes out.u(i, j) (j <= NY-2) and out.v(i, j) (i <= NX-2):
// both components in one CTA, so the inputs a CTA needs come from DRAM once.
// The EdgeGradient slots after transpose!:
//   dudx (primal x, primal y): mean_x(v.u) * (u.u[k+1]-u.u[k])
//   dudy (dual, dual):         mean_x(v.v) * (u.u[l]-u.u[l-1])   (non-ghost only)
//   dvdx (dual, dual):         mean_y(v.u) * (u.v[k]-u.v[k-1])   (non-ghost only)
//   dvdy (primal, primal):     mean_y(v.v) * (u.v[l+1]-u.v[l])
// and the result is their average back onto the edges.
// RY consecutive rows per thread (jb .. jb+RY-1), the vertical neighbours
// shared in registers (53 loads for four rows of both components instead of
// 96) and every load issued before the arithmetic.
template <typename T, bool IN>
__device__ __forceinline__ void vdu_edges_rows(int NX, int NY, const T* __restrict__ vu,
    const T* __restrict__ vv, const T* __restrict__ uu, const T* __restrict__ uv, T* __restrict__ ou,
    T* __restrict__ ov, T sc) {
  const int m = NX - 1;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = (blockIdx.y * BY + threadIdx.y) * RY;
  if (!IN && (i >= NX || jb >= NY)) return;
  const bool u_in = IN || (i >= 1 && i <= NX - 2);  // out.u nonzero in this column
  const bool v_col = IN || i <= NX - 2;             // out.v has this column
  const bool v_rt = IN || i + 1 <= NX - 2;          // out.v's dvdx slot at dual x i+1
  // Columns of the u components (NX x NY-1): uuc = uu column i rows jb-1 ..
  // jb+RY, uul / uur columns i-1 / i+1 rows jb .. jb+RY-1; vuc / vur = vu
  // columns i / i+1 rows jb-1 .. jb+RY-1, vul column i-1 rows jb ..
  // jb+RY-1.  Columns of the v components (NX-1 x NY): vvc / uvc = column i
  // rows jb-1 .. jb+RY, vvl column i-1 rows jb .. jb+RY, uvl / uvr columns
  // i-1 / i+1 rows jb .. jb+RY-1.
  T uuc[RY + 2], uul[RY], uur[RY], vuc[RY + 1], vur[RY + 1], vul[RY];
  T vvc[RY + 2], uvc[RY + 2], vvl[RY + 1], uvl[RY], uvr[RY];
#pragma unroll
  for (int k = 0; k < RY + 2; ++k) {
    const int j = jb - 1 + k;  // row of index k in the jb-1 based arrays
    const bool urow = IN || (j >= 0 && j <= NY - 2), vrow = IN || (j >= 0 && j < NY);
    uuc[k] = (u_in && urow) ? ld(uu, j * NX + i) : (T)0;
    vvc[k] = (v_col && vrow) ? ld(vv, j * m + i) : (T)0;
    uvc[k] = (v_col && vrow) ? ld(uv, j * m + i) : (T)0;
    if (k < RY + 1) {
      vuc[k] = (u_in && urow) ? ld(vu, j * NX + i) : (T)0;
      vur[k] = ((u_in || v_rt) && urow) ? ld(vu, j * NX + i + 1) : (T)0;
    }
    if (k >= 1) {  // rows jb .. jb+RY
      vvl[k - 1] = (u_in && vrow) ? ld(vv, j * m + i - 1) : (T)0;
      if (k <= RY) {  // rows jb .. jb+RY-1
        uul[k - 1] = (u_in && urow) ? ld(uu, j * NX + i - 1) : (T)0;
        uur[k - 1] = (u_in && urow) ? ld(uu, j * NX + i + 1) : (T)0;
        vul[k - 1] = (u_in && urow) ? ld(vu, j * NX + i - 1) : (T)0;
        uvl[k - 1] = (u_in && vrow) ? ld(uv, j * m + i - 1) : (T)0;
        uvr[k - 1] = (v_rt && vrow) ? ld(uv, j * m + i + 1) : (T)0;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < RY; ++k) {
    const int j = jb + k;
    if (!IN && j >= NY) break;
    if (IN || j <= NY - 2) {
      T r = (T)0;
      if (u_in) {
        // x part: dudx slots at primal x i-1, i (row j)
        const T u0 = uul[k], u1 = uuc[k + 1], u2 = uur[k];
        const T v0 = vul[k], v1 = vuc[k + 1], v2 = vur[k + 1];
        const T tx = (T)0.5 * (v0 + v1) * (u1 - u0) + (T)0.5 * (v1 + v2) * (u2 - u1);
        // y part: dudy slots at dual (i, l), l = j, j+1, nonzero for 1 <= l <= NY-2
        T ty = (T)0;
        if (IN || j >= 1) {
          const T a = (T)0.5 * (vvl[k] + vvc[k + 1]);
          ty += a * (u1 - uuc[k]);
        }
        if (IN || j + 1 <= NY - 2) {
          const T a = (T)0.5 * (vvl[k + 1] + vvc[k + 2]);
          ty += a * (uuc[k + 2] - u1);
        }
        r = (T)0.5 * (tx + ty) * sc;
      }
      ou[j * NX + i] = r;
    }
    if (v_col) {
      T r = (T)0;
      if (IN || (j >= 1 && j <= NY - 2)) {
        // y part: dvdy slots at primal y j-1, j (column i)
        const T u0 = uvc[k], u1 = uvc[k + 1], u2 = uvc[k + 2];
        const T v0 = vvc[k], v1 = vvc[k + 1], v2 = vvc[k + 2];
        const T ty = (T)0.5 * (v0 + v1) * (u1 - u0) + (T)0.5 * (v1 + v2) * (u2 - u1);
        // x part: dvdx slots at dual (k, j), k = i, i+1, nonzero for 1 <= k <= NX-2
        T tx = (T)0;
        if (IN || i >= 1) {
          const T a = (T)0.5 * (vuc[k] + vuc[k + 1]);
          tx += a * (u1 - uvl[k]);
        }
        if (v_rt) {
          const T a = (T)0.5 * (vur[k] + vur[k + 1]);
          tx += a * (uvr[k] - u1);
        }
        r = (T)0.5 * (tx + ty) * sc;
      }
      ov[j * m + i] = r;
    }
  }
}

// FP32: at most 64 registers, four CTAs per SM (32 bytes of spills; the
// kernel is issue-limited, and 80 registers left three CTAs per SM: 53% ->
// 55% of HBM on 4096^2); FP64 keeps its 128 registers
template <typename T>
__global__ void __launch_bounds__(BX* BY, sizeof(T) == 4 ? 4 : 2) k_vdu_edges(int NX, int NY, const T* __restrict__ vu,
    const T* __restrict__ vv, const T* __restrict__ uu, const T* __restrict__ uv, T* __restrict__ ou,
    T* __restrict__ ov, T sc) {
  pdl_begin();
  if (inner_block(NX, NY))
    vdu_edges_rows<T, true>(NX, NY, vu, vv, uu, uv, ou, ov, sc);
  else
    vdu_edges_rows<T, false>(NX, NY, vu, vv, uu, uv, ou, ov, sc);
}

// w x v (:419-434): out.u = mean_y(-mean_x(v.v) w), out.v = mean_x(mean_y(v.u) w),
// the inner means onto the non-ghost dual nodes only.  Thread (i, j) writes
// out.u(i, j) (j <= NY-2) and out.v(i, j) (i <= NX-2).
// RY consecutive rows per thread (jb .. jb+RY-1), vertical neighbours shared
// in registers, every load issued before the arithmetic.
template <typename T, bool IN>
__device__ __forceinline__ void w_cross_v_rows(int NX, int NY, const T* __restrict__ w,
    const T* __restrict__ vu, const T* __restrict__ vv, T* __restrict__ ou, T* __restrict__ ov) {
  const int m = NX - 1;
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = (blockIdx.y * BY + threadIdx.y) * RY;
  if (!IN && (i >= NX || jb >= NY)) return;
  const bool u_in = IN || (i >= 1 && i <= NX - 2);  // out.u nonzero in this column
  const bool v_col = IN || i <= NX - 2;             // out.v has this column
  // wc: w column i rows jb .. jb+RY; wr: w column i+1 rows jb .. jb+RY-1;
  // vl, vr: vv columns i-1, i rows jb .. jb+RY; ua, ub: vu columns i, i+1
  // rows jb-1 .. jb+RY-1
  T wc[RY + 1], wr[RY], vl[RY + 1], vr[RY + 1], ua[RY + 1], ub[RY + 1];
#pragma unroll
  for (int k = 0; k < RY + 1; ++k) {
    const int j = jb + k;
    const bool row = IN || j < NY;
    wc[k] = row ? ld(w, j * NX + i) : (T)0;
    vl[k] = (row && u_in) ? ld(vv, j * m + i - 1) : (T)0;
    vr[k] = (row && u_in) ? ld(vv, j * m + i) : (T)0;
    const int jv = j - 1;
    const bool vrow = IN || (v_col && jv >= 0 && jv <= NY - 2);
    ua[k] = vrow ? ld(vu, jv * NX + i) : (T)0;
    ub[k] = vrow ? ld(vu, jv * NX + i + 1) : (T)0;
    if (k < RY) wr[k] = (row && v_col) ? ld(w, j * NX + i + 1) : (T)0;
  }
#pragma unroll
  for (int k = 0; k < RY; ++k) {
    const int j = jb + k;
    if (IN || j <= NY - 2) {
      T r = (T)0;
      if (u_in) {
        const T vd0 = (T)0.5 * (vl[k] + vr[k]);
        const T vd1 = (T)0.5 * (vl[k + 1] + vr[k + 1]);
        r = (T)-0.5 * (vd0 * wc[k] + vd1 * wc[k + 1]);
      }
      ou[j * NX + i] = r;
    }
    if (IN || (v_col && j < NY)) {
      T r = (T)0;
      if (IN || (j >= 1 && j <= NY - 2)) {
        const T ud0 = (T)0.5 * (ua[k] + ua[k + 1]);
        const T ud1 = (T)0.5 * (ub[k] + ub[k + 1]);
        r = (T)0.5 * (ud0 * wc[k] + ud1 * wr[k]);
      }
      ov[j * m + i] = r;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(BX* BY) k_w_cross_v(int NX, int NY, const T* __restrict__ w,
    const T* __restrict__ vu, const T* __restrict__ vv, T* __restrict__ ou, T* __restrict__ ov) {
  pdl_begin();
  if (inner_block(NX, NY))
    w_cross_v_rows<T, true>(NX, NY, w, vu, vv, ou, ov);
  else
    w_cross_v_rows<T, false>(NX, NY, w, vu, vv, ou, ov);
}

}  // namespace

#define CV_DISPATCH(dtype, ...)                   \
  do {                                            \
    if ((dtype) == ILM_F64) {                     \
      using T = double;                           \
      __VA_ARGS__;                                \
    } else {                                      \
      using T = float;                            \
      __VA_ARGS__;                                \
    }                                             \
  } while (0)

int st_convective(const ilm_grid_s* g, int dtype, int field_kind, const void* v, const void* q, void* out,
                  double scale, cudaStream_t st) {
  const int NX = g->nx, NY = g->ny;
  ILM_REQUIRE((long long)NX * NY < (1LL << 31), "convective_derivative: grid of %d x %d exceeds 32-bit indexing", NX, NY);
  const size_t ne_u = (size_t)NX * (NY - 1);
  CV_DISPATCH(dtype, {
    const T* vu = static_cast<const T*>(v);
    const T* vv = vu + ne_u;
    switch (field_kind) {
      case ILM_NODES_PRIMAL:
        ILM_CHECK_CUDA(launch_pdl(k_vdp_np<T>, grid2(NX - 1, NY - 1), dim3(BX, BY), st, NX, NY, vu, vv,
                                  static_cast<const T*>(q), static_cast<T*>(out), (T)scale));
        break;
      case ILM_NODES_DUAL:
        ILM_CHECK_CUDA(launch_pdl(k_vdw_nd<T>, grid2(NX, NY), dim3(BX, BY), st, NX, NY, vu, vv,
                                  static_cast<const T*>(q), static_cast<T*>(out), (T)scale));
        break;
      case ILM_EDGES_PRIMAL: {
        const T* uu = static_cast<const T*>(q);
        T* ou = static_cast<T*>(out);
        ILM_CHECK_CUDA(launch_pdl(k_vdu_edges<T>, grid2(NX, NY), dim3(BX, BY), st, NX, NY, vu, vv, uu, uu + ne_u,
                                  ou, ou + ne_u, (T)scale));
        break;
      }
      default:
        set_error("convective_derivative: unsupported field kind %d", field_kind);
        return ILM_ERR_INVALID_ARG;
    }
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int st_w_cross_v(const ilm_grid_s* g, int dtype, const void* w, const void* v, void* out, cudaStream_t st) {
  const int NX = g->nx, NY = g->ny;
  ILM_REQUIRE((long long)NX * NY < (1LL << 31), "w_cross_v: grid of %d x %d exceeds 32-bit indexing", NX, NY);
  const size_t ne_u = (size_t)NX * (NY - 1);
  CV_DISPATCH(dtype, {
    const T* vu = static_cast<const T*>(v);
    T* ou = static_cast<T*>(out);
    ILM_CHECK_CUDA(launch_pdl(k_w_cross_v<T>, grid2(NX, NY), dim3(BX, BY), st, NX, NY, static_cast<const T*>(w), vu,
                              vu + ne_u, ou, ou + ne_u));
  });
  return ILM_OK;
}

}  // namespace ilm
