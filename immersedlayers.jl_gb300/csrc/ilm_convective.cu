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

// v . grad p, p on Nodes{Primal} (m = NX-1 by NY-1), v on Edges{Primal}
// (:318-328).  gx at dual x k: p[k]-p[k-1] for 1 <= k <= NX-2, else 0.
template <typename T>
__device__ __forceinline__ void vdp_np_at(int i, int j, int NX, int NY, const T* __restrict__ vu,
    const T* __restrict__ vv, const T* __restrict__ p, T* __restrict__ out, T sc) {
  const int m = NX - 1;
  if (i >= m || j >= NY - 1) return;
  const int c = j * m + i;
  const T pc = ld(p, c);
  const T gxl = (i >= 1) ? pc - ld(p, c - 1) : (T)0;            // dual x = i
  const T gxr = (i + 1 <= NX - 2) ? ld(p, c + 1) - pc : (T)0;  // dual x = i+1
  const T gyd = (j >= 1) ? pc - ld(p, c - m) : (T)0;           // dual y = j
  const T gyu = (j + 1 <= NY - 2) ? ld(p, c + m) - pc : (T)0;  // dual y = j+1
  const T tx = ld(vu, j * NX + i) * gxl + ld(vu, j * NX + i + 1) * gxr;
  const T ty = ld(vv, j * m + i) * gyd + ld(vv, (j + 1) * m + i) * gyu;
  out[c] = (T)0.5 * (tx + ty) * sc;
}

template <typename T>
__global__ void __launch_bounds__(BX* BY) k_vdp_np(int NX, int NY, const T* __restrict__ vu, const T* __restrict__ vv,
    const T* __restrict__ p, T* __restrict__ out, T sc) {
  // RY output rows per thread (j, j + BY, ...), all independent, so their
  // loads are in flight together
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = blockIdx.y * BY * RY + threadIdx.y;
#pragma unroll
  for (int r = 0; r < RY; ++r) vdp_np_at(i, jb + r * BY, NX, NY, vu, vv, p, out, sc);
}

// v . grad w, w on Nodes{Dual} (NX x NY), v on Edges{Primal} (:330-342):
// v averaged onto the Edges{Dual} positions (four-point means), times the
// Edges{Dual} gradient of w, averaged onto the non-ghost dual nodes.
template <typename T>
__device__ __forceinline__ void vdw_nd_at(int i, int j, int NX, int NY, const T* __restrict__ vu,
    const T* __restrict__ vv, const T* __restrict__ w, T* __restrict__ out, T sc) {
  if (i >= NX || j >= NY) return;
  const int c = j * NX + i;
  if (i < 1 || i > NX - 2 || j < 1 || j > NY - 2) {
    out[c] = (T)0;
    return;
  }
  const int m = NX - 1;
  const T wc = ld(w, c);
  // Edges{Dual}.u at (primal x k, dual y j), k = i-1, i: mean of vu over
  // dual x k, k+1 and primal y j-1, j
  const int r0 = (j - 1) * NX, r1 = j * NX;
  const T a0 = ld(vu, r0 + i - 1), a1 = ld(vu, r0 + i), a2 = ld(vu, r0 + i + 1);
  const T b0 = ld(vu, r1 + i - 1), b1 = ld(vu, r1 + i), b2 = ld(vu, r1 + i + 1);
  const T udl = (T)0.25 * (a0 + a1 + b0 + b1), udr = (T)0.25 * (a1 + a2 + b1 + b2);
  const T tx = udl * (wc - ld(w, c - 1)) + udr * (ld(w, c + 1) - wc);
  // Edges{Dual}.v at (dual x i, primal y l), l = j-1, j: mean of vv over
  // primal x i-1, i and dual y l, l+1
  const int s0 = (j - 1) * m, s1 = j * m, s2 = (j + 1) * m;
  const T e0 = ld(vv, s0 + i - 1) + ld(vv, s0 + i), e1 = ld(vv, s1 + i - 1) + ld(vv, s1 + i);
  const T e2 = ld(vv, s2 + i - 1) + ld(vv, s2 + i);
  const T vdd = (T)0.25 * (e0 + e1), vdu = (T)0.25 * (e1 + e2);
  const T ty = vdd * (wc - ld(w, c - NX)) + vdu * (ld(w, c + NX) - wc);
  out[c] = (T)0.5 * (tx + ty) * sc;
}

template <typename T>
__global__ void __launch_bounds__(BX* BY) k_vdw_nd(int NX, int NY, const T* __restrict__ vu, const T* __restrict__ vv,
    const T* __restrict__ w, T* __restrict__ out, T sc) {
  // RY output rows per thread (j, j + BY, ...), all independent, so their
  // loads are in flight together
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = blockIdx.y * BY * RY + threadIdx.y;
#pragma unroll
  for (int r = 0; r < RY; ++r) vdw_nd_at(i, jb + r * BY, NX, NY, vu, vv, w, out, sc);
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
template <typename T>
__device__ __forceinline__ void vdu_edges_at(int i, int j, int NX, int NY, const T* __restrict__ vu,
    const T* __restrict__ vv, const T* __restrict__ uu, const T* __restrict__ uv, T* __restrict__ ou,
    T* __restrict__ ov, T sc) {
  const int m = NX - 1;
  if (i >= NX || j >= NY) return;
  if (j <= NY - 2) {
    const int c = j * NX + i;
    T r = (T)0;
    if (i >= 1 && i <= NX - 2) {
      // x part: dudx slots at primal x i-1, i (row j)
      const T u0 = ld(uu, c - 1), u1 = ld(uu, c), u2 = ld(uu, c + 1);
      const T v0 = ld(vu, c - 1), v1 = ld(vu, c), v2 = ld(vu, c + 1);
      const T tx = (T)0.5 * (v0 + v1) * (u1 - u0) + (T)0.5 * (v1 + v2) * (u2 - u1);
      // y part: dudy slots at dual (i, l), l = j, j+1, nonzero for 1 <= l <= NY-2
      T ty = (T)0;
      if (j >= 1) {
        const T a = (T)0.5 * (ld(vv, j * m + i - 1) + ld(vv, j * m + i));
        ty += a * (u1 - ld(uu, c - NX));
      }
      if (j + 1 <= NY - 2) {
        const T a = (T)0.5 * (ld(vv, (j + 1) * m + i - 1) + ld(vv, (j + 1) * m + i));
        ty += a * (ld(uu, c + NX) - u1);
      }
      r = (T)0.5 * (tx + ty) * sc;
    }
    ou[c] = r;
  }
  if (i <= NX - 2) {
    const int c = j * m + i;
    T r = (T)0;
    if (j >= 1 && j <= NY - 2) {
      // y part: dvdy slots at primal y j-1, j (column i)
      const T u0 = ld(uv, c - m), u1 = ld(uv, c), u2 = ld(uv, c + m);
      const T v0 = ld(vv, c - m), v1 = ld(vv, c), v2 = ld(vv, c + m);
      const T ty = (T)0.5 * (v0 + v1) * (u1 - u0) + (T)0.5 * (v1 + v2) * (u2 - u1);
      // x part: dvdx slots at dual (k, j), k = i, i+1, nonzero for 1 <= k <= NX-2
      T tx = (T)0;
      if (i >= 1) {
        const T a = (T)0.5 * (ld(vu, (j - 1) * NX + i) + ld(vu, j * NX + i));
        tx += a * (u1 - ld(uv, c - 1));
      }
      if (i + 1 <= NX - 2) {
        const T a = (T)0.5 * (ld(vu, (j - 1) * NX + i + 1) + ld(vu, j * NX + i + 1));
        tx += a * (ld(uv, c + 1) - u1);
      }
      r = (T)0.5 * (tx + ty) * sc;
    }
    ov[c] = r;
  }
}

template <typename T>
__global__ void __launch_bounds__(BX* BY) k_vdu_edges(int NX, int NY, const T* __restrict__ vu,
    const T* __restrict__ vv, const T* __restrict__ uu, const T* __restrict__ uv, T* __restrict__ ou,
    T* __restrict__ ov, T sc) {
  // RY output rows per thread (j, j + BY, ...), all independent, so their
  // loads are in flight together
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = blockIdx.y * BY * RY + threadIdx.y;
#pragma unroll
  for (int r = 0; r < RY; ++r) vdu_edges_at(i, jb + r * BY, NX, NY, vu, vv, uu, uv, ou, ov, sc);
}

// w x v (:419-434): out.u = mean_y(-mean_x(v.v) w), out.v = mean_x(mean_y(v.u) w),
// the inner means onto the non-ghost dual nodes only.  Thread (i, j) writes
// out.u(i, j) (j <= NY-2) and out.v(i, j) (i <= NX-2).
template <typename T>
__device__ __forceinline__ void w_cross_v_at(int i, int j, int NX, int NY, const T* __restrict__ w,
    const T* __restrict__ vu, const T* __restrict__ vv, T* __restrict__ ou, T* __restrict__ ov) {
  const int m = NX - 1;
  if (i >= NX || j >= NY) return;
  const T w0 = ld(w, j * NX + i);
  if (j <= NY - 2) {
    T r = (T)0;
    if (i >= 1 && i <= NX - 2) {
      const T vd0 = (T)0.5 * (ld(vv, j * m + i - 1) + ld(vv, j * m + i));
      const T vd1 = (T)0.5 * (ld(vv, (j + 1) * m + i - 1) + ld(vv, (j + 1) * m + i));
      r = (T)-0.5 * (vd0 * w0 + vd1 * ld(w, (j + 1) * NX + i));
    }
    ou[j * NX + i] = r;
  }
  if (i <= NX - 2) {
    T r = (T)0;
    if (j >= 1 && j <= NY - 2) {
      const T ud0 = (T)0.5 * (ld(vu, (j - 1) * NX + i) + ld(vu, j * NX + i));
      const T ud1 = (T)0.5 * (ld(vu, (j - 1) * NX + i + 1) + ld(vu, j * NX + i + 1));
      r = (T)0.5 * (ud0 * w0 + ud1 * ld(w, j * NX + i + 1));
    }
    ov[j * m + i] = r;
  }
}

template <typename T>
__global__ void __launch_bounds__(BX* BY) k_w_cross_v(int NX, int NY, const T* __restrict__ w,
    const T* __restrict__ vu, const T* __restrict__ vv, T* __restrict__ ou, T* __restrict__ ov) {
  // RY output rows per thread (j, j + BY, ...), all independent, so their
  // loads are in flight together
  const int i = blockIdx.x * BX + threadIdx.x;
  const int jb = blockIdx.y * BY * RY + threadIdx.y;
#pragma unroll
  for (int r = 0; r < RY; ++r) w_cross_v_at(i, jb + r * BY, NX, NY, w, vu, vv, ou, ov);
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
        k_vdp_np<T><<<grid2(NX - 1, NY - 1), dim3(BX, BY), 0, st>>>(NX, NY, vu, vv, static_cast<const T*>(q),
                                                                     static_cast<T*>(out), (T)scale);
        break;
      case ILM_NODES_DUAL:
        k_vdw_nd<T><<<grid2(NX, NY), dim3(BX, BY), 0, st>>>(NX, NY, vu, vv, static_cast<const T*>(q),
                                                             static_cast<T*>(out), (T)scale);
        break;
      case ILM_EDGES_PRIMAL: {
        const T* uu = static_cast<const T*>(q);
        T* ou = static_cast<T*>(out);
        k_vdu_edges<T><<<grid2(NX, NY), dim3(BX, BY), 0, st>>>(NX, NY, vu, vv, uu, uu + ne_u, ou, ou + ne_u,
                                                                   (T)scale);
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
    k_w_cross_v<T><<<grid2(NX, NY), dim3(BX, BY), 0, st>>>(NX, NY, static_cast<const T*>(w), vu, vu + ne_u, ou,
                                                               ou + ne_u);
  });
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

}  // namespace ilm
