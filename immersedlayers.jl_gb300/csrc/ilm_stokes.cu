// Stokes flow with no-slip surfaces on a vector cache: the reference's
// StokesFlowProblem `solve` (test/literate/stokes.jl:101-166) on the device.
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
// closed form; here both Schur systems are solved matrix-free by CG in the
// ds-weighted inner product (W S symmetric, S negative definite, Ss positive
// semi-definite), each iteration one surface curl, one or two LGF FFT
// convolutions and one surface curl back -- no N x N matrix is formed.
//
// The filter F = W^-1 E R, W = diag(E R 1): the filtered interpolation of
// CartesianGrids' Regularize(filter = true) (un-vendored) restated from
// Goza, Liska, Morley & Colonius (2016).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <functional>

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

struct Work {
  DevBuf e1, e2, d1, d2, p1, v1, v2, v3, v4, v5, s1, s2, s3, s4, s5, diag;
};

using Apply = std::function<int(const void*, void*)>;

// CG on A x = b in the ds-weighted inner product (dots through
// ilm_dot_surface: FP64, host-synchronised).  x starts at 0.
int cg_matfree(ilm_cache_t c, int ncomp, const Apply& A, const void* b, void* x, void* r, void* p, void* q,
               double tol, int maxiter, int* iters, double* relres, cudaStream_t st) {
  const size_t n = (size_t)ncomp * c->npts;
  const int dt = c->dtype;
  ILM_TRY(st_fill(n, dt, 0.0, x, st));
  ILM_TRY(st_affine(n, dt, 1.0, b, 0.0, r, st));
  ILM_TRY(st_affine(n, dt, 1.0, b, 0.0, p, st));
  double bb = 0.0, rz = 0.0;
  // unweighted norm of b for the residual test: weights are ds, so use the
  // weighted dot for CG and an unweighted norm through a unit-weight pass
  auto unweighted = [&](const void* a, double* out) -> int {
    double tot = 0.0;
    for (int i = 0; i < ncomp; ++i) {
      ILM_TRY(st_point_dot(c->npts, dt, elem_ptr(a, (size_t)i * c->npts, dt), elem_ptr(a, (size_t)i * c->npts, dt),
                           nullptr, c->red.as<double>(), st));
      double v = 0.0;
      ILM_CHECK_CUDA(cudaMemcpyAsync(&v, c->red.as<double>(), sizeof(double), cudaMemcpyDeviceToHost, st));
      ILM_CHECK_CUDA(cudaStreamSynchronize(st));
      tot += v;
    }
    *out = tot;
    return ILM_OK;
  };
  ILM_TRY(unweighted(b, &bb));
  ILM_TRY(ilm_dot_surface(c, ncomp, r, r, &rz, st));
  const double bn = sqrt(bb);
  int it = 0;
  double rel = bn > 0 ? 1.0 : 0.0;
  if (bn == 0.0) {
    *iters = 0;
    *relres = 0.0;
    return ILM_OK;
  }
  while (it < maxiter) {
    ILM_TRY(A(p, q));
    double pq = 0.0;
    ILM_TRY(ilm_dot_surface(c, ncomp, p, q, &pq, st));
    if (pq == 0.0) break;
    const double alpha = rz / pq;
    ILM_TRY(st_axpby(n, dt, alpha, p, 1.0, x, x, st));
    ILM_TRY(st_axpby(n, dt, -alpha, q, 1.0, r, r, st));
    ++it;
    double rr = 0.0;
    ILM_TRY(unweighted(r, &rr));
    rel = sqrt(rr) / bn;
    if (rel <= tol || it % 50 == 0) {  // true residual
      ILM_TRY(A(x, q));
      ILM_TRY(st_axpby(n, dt, 1.0, b, -1.0, q, r, st));
      ILM_TRY(unweighted(r, &rr));
      rel = sqrt(rr) / bn;
      if (rel <= tol) break;
    }
    double rzn = 0.0;
    ILM_TRY(ilm_dot_surface(c, ncomp, r, r, &rzn, st));
    ILM_TRY(st_axpby(n, dt, 1.0, r, rzn / rz, p, p, st));
    rz = rzn;
  }
  *iters = it;
  *relres = rel;
  return ILM_OK;
}

}  // namespace
}  // namespace ilm

using namespace ilm;

extern "C" {

int ilm_solve_stokes(ilm_cache_t c, const void* vplus, const void* vminus, void* v_out, void* s_out, void* sigma_out,
                     double tol, int maxiter, ilm_solve_info_t* info, ilm_stream_t stream) {
  ILM_REQUIRE(c, "null cache");
  ILM_REQUIRE(vplus && vminus && v_out && s_out && sigma_out, "solve_stokes: null argument");
  ILM_REQUIRE(c->kind == ILM_CACHE_VECTOR, "solve_stokes: vector cache required");
  ILM_REQUIRE(c->scaling == ILM_GRID_SCALING, "solve_stokes: GridScaling cache required");
  ILM_REQUIRE(tol > 0 && maxiter > 0, "solve_stokes: bad tolerance / iteration limit");
  cudaStream_t st = as_stream(stream);
  const int N = c->npts, dt = c->dtype;
  const size_t es = dt == ILM_F64 ? 8 : 4;
  const size_t ne = c->grid.shape(PC_U).numel() + c->grid.shape(PC_V).numel();
  const size_t nd = c->grid.shape(PC_D).numel();
  const size_t np = c->grid.shape(PC_P).numel();
  Work w;
  ILM_TRY(w.e1.alloc(ne * es));
  ILM_TRY(w.e2.alloc(ne * es));
  ILM_TRY(w.d1.alloc(nd * es));
  ILM_TRY(w.d2.alloc(nd * es));
  ILM_TRY(w.p1.alloc(np * es));
  for (DevBuf* b : {&w.v1, &w.v2, &w.v3, &w.v4, &w.v5, &w.diag}) ILM_TRY(b->alloc((size_t)std::max(2 * N, 1) * es));
  for (DevBuf* b : {&w.s1, &w.s2, &w.s3, &w.s4, &w.s5}) ILM_TRY(b->alloc((size_t)std::max(N, 1) * es));
  const size_t n2 = 2 * (size_t)N;
  void* dv = w.v1.p;   // [v]
  void* vb = w.v2.p;   // avg
  void* vp = w.v3.p;   // v'
  // jump and average
  ILM_TRY(st_axpby(n2, dt, 1.0, vplus, -1.0, vminus, dv, st));
  ILM_TRY(st_axpby(n2, dt, 0.5, vplus, 0.5, vminus, vb, st));
  // psi* = L^-2 (-C D_s^symm [v])
  ILM_TRY(ilm_surface_divergence_symm(c, dv, w.e1.p, stream));
  ILM_TRY(ilm_curl(c, ILM_EDGES_PRIMAL, w.e1.p, w.d1.p, stream));
  ILM_TRY(st_affine(nd, dt, -1.0, w.d1.p, 0.0, w.d1.p, st));
  ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, w.d1.p, w.d2.p, stream));
  ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, w.d2.p, s_out, stream));  // s_out holds psi*
  // phi = L^-1 R (n . [v]),  v_phi = G phi  (kept in v_out)
  if (N > 0) {
    if (dt == ILM_F64)
      k_ndot<double><<<(N + 255) / 256, 256, 0, st>>>(N, c->nx.as<double>(), c->ny.as<double>(),
                                                      static_cast<const double*>(dv), w.s1.as<double>());
    else
      k_ndot<float><<<(N + 255) / 256, 256, 0, st>>>(N, c->nx.as<float>(), c->ny.as<float>(),
                                                     static_cast<const float*>(dv), w.s1.as<float>());
    ILM_CHECK_LAUNCH();
  }
  ILM_TRY(ilm_regularize(c, ILM_NODES_PRIMAL, w.s1.p, w.p1.p, stream));
  void* phi = w.p1.p;
  {
    DevBuf tmp;
    ILM_TRY(tmp.alloc(np * es));
    ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_PRIMAL, phi, tmp.p, stream));
    ILM_CHECK_CUDA(cudaMemcpyAsync(phi, tmp.p, np * es, cudaMemcpyDeviceToDevice, st));
    ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  ILM_TRY(ilm_grad(c, ILM_NODES_PRIMAL, phi, v_out, stream));
  // v' = avg - E v_phi - E C psi*
  ILM_TRY(ilm_interpolate(c, ILM_EDGES_PRIMAL, v_out, w.v4.p, stream));
  ILM_TRY(st_axpby(n2, dt, 1.0, vb, -1.0, w.v4.p, vp, st));
  ILM_TRY(ilm_curl(c, ILM_NODES_DUAL, s_out, w.e1.p, stream));
  ILM_TRY(ilm_interpolate(c, ILM_EDGES_PRIMAL, w.e1.p, w.v4.p, stream));
  ILM_TRY(st_axpby(n2, dt, 1.0, vp, -1.0, w.v4.p, vp, st));
  // S sigma = v'  (matrix-free CG)
  Apply applyS = [&](const void* x, void* y) -> int {
    ILM_TRY(ilm_surface_curl(c, 0, ILM_VECTOR_DATA, x, w.d1.p, stream));
    ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, w.d1.p, w.d2.p, stream));
    ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, w.d2.p, w.d1.p, stream));
    ILM_TRY(ilm_surface_curl(c, 1, ILM_VECTOR_DATA, w.d1.p, y, stream));
    return st_affine(n2, dt, -1.0, y, 0.0, y, st);
  };
  int it1 = 0, it2 = 0;
  double rr1 = 0.0, rr2 = 0.0;
  ILM_TRY(cg_matfree(c, 2, applyS, vp, sigma_out, w.v4.p, w.v5.p, w.diag.p, tol, maxiter, &it1, &rr1, st));
  // psi = psi* + L^-2 (-C_s^T sigma)
  ILM_TRY(ilm_surface_curl(c, 0, ILM_VECTOR_DATA, sigma_out, w.d1.p, stream));
  ILM_TRY(st_affine(nd, dt, -1.0, w.d1.p, 0.0, w.d1.p, st));
  ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, w.d1.p, w.d2.p, stream));
  ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, w.d2.p, w.d1.p, stream));
  ILM_TRY(st_axpby(nd, dt, 1.0, w.d1.p, 1.0, s_out, s_out, st));
  // v = C psi + v_phi
  ILM_TRY(ilm_curl(c, ILM_NODES_DUAL, s_out, w.e1.p, stream));
  ILM_TRY(st_axpby(ne, dt, 1.0, w.e1.p, 1.0, v_out, v_out, st));
  // streamfunction equivalent of the scalar potential: Ss d = G^x_s phi
  ILM_TRY(ilm_surface_grad_cross(c, phi, w.s1.p, stream));
  Apply applySs = [&](const void* x, void* y) -> int {
    ILM_TRY(ilm_surface_curl(c, 0, ILM_SCALAR_DATA, x, w.d1.p, stream));
    ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, w.d1.p, w.d2.p, stream));
    ILM_TRY(ilm_surface_curl(c, 1, ILM_SCALAR_DATA, w.d2.p, y, stream));
    return st_affine(N, dt, -1.0, y, 0.0, y, st);
  };
  ILM_TRY(cg_matfree(c, 1, applySs, w.s1.p, w.s2.p, w.s3.p, w.s4.p, w.s5.p, tol, maxiter, &it2, &rr2, st));
  ILM_TRY(ilm_surface_curl_cross(c, 0, w.s2.p, w.d1.p, stream));
  ILM_TRY(st_affine(nd, dt, -1.0, w.d1.p, 0.0, w.d1.p, st));
  ILM_TRY(ilm_inverse_laplacian(c, ILM_NODES_DUAL, w.d1.p, w.d2.p, stream));
  ILM_TRY(st_axpby(nd, dt, 1.0, w.d2.p, 1.0, s_out, s_out, st));
  // sigma <- F^2 sigma,  F = W^-1 E R,  W = E R 1
  ILM_TRY(ilm_surface_filter(c, 2, sigma_out, sigma_out, stream));
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  if (info) {
    info->iterations = it1 + it2;
    info->converged = (rr1 <= tol && rr2 <= tol) ? 1 : 0;
    info->rel_residual = std::max(rr1, rr2);
  }
  return (rr1 <= tol && rr2 <= tol) ? ILM_OK : ILM_ERR_NOT_CONVERGED;
}

}  // extern "C"
