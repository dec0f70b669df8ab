# ImmersedLayersGPU.jl -- the Julia side of the drop-in boundary.
#
# ImmersedLayers.jl has no FFI for its hot path: its operators are generic
# functions `op!(out, in, cache)` (src/surface_operators.jl,
# src/grid_operators.jl) forwarded from `ILMSystem` by `@eval` loops
# (src/system.jl:184-227).  This module adds methods to those generic
# functions for device-resident data, each forwarding to one entry point of
# libilm.so (include/ilm.h) through `ccall`.
#
#  * `LibILM`: one Julia function per `ILM_API` declaration of include/ilm.h,
#    same name, same argument order, `ccall` argument types matching the C
#    types (int -> Cint, double -> Cdouble, size_t -> Csize_t, device arrays
#    -> CuPtr, host arrays -> Ptr, out-parameters -> Ref, opaque handles and
#    streams -> Ptr{Cvoid}).  tests/test_julia_shim.py checks every `ccall`
#    below against the header.
#  * `GPUILMCache`: the device counterpart of BasicILMCache (src/cache.jl:16-88),
#    built from a body list and a PhysicalGrid; the operator methods take
#    CuArrays in CartesianGrids' memory layout (column-major, x first; Edges
#    u then v; VectorData u then v), so no copies are made at the boundary.
#  * `GPUILMSystem`: ILMSystem's forwarding of operators, inner products and
#    Schur builders to its base cache (src/system.jl:198-227), plus the
#    problem solves (test/literate/problems.jl:259-298, neumann.jl:101-142,
#    stokes.jl:101-166) and heat time marching (heatconduction.jl:87-189).
#
# Julia is not installed where this library is built and tested; the same
# entry points are exercised through the Python ctypes mirror
# (immersedlayers/_lib.py) by the test suite.
module ImmersedLayersGPU

using CUDA
using CartesianGrids
using RigidBodyTools
import ImmersedLayers
import ImmersedLayers: regularize!, interpolate!, regularize_normal!, normal_interpolate!,
                       regularize_normal_cross!, normal_cross_interpolate!, regularize_normal_dot!,
                       normal_dot_interpolate!, regularize_normal_symm!, normal_interpolate_symm!,
                       surface_divergence!, surface_grad!, surface_curl!, surface_divergence_symm!,
                       surface_grad_symm!, surface_curl_cross!, surface_divergence_cross!,
                       surface_grad_cross!, mask, complementary_mask, create_RTLinvR, create_CLinvCT,
                       create_GLinvD, create_nRTRn, create_CL2invCT, create_GLinvD_symm, create_GLinvD_cross,
                       create_CLinvCT_scalar
import CartesianGrids: divergence!, grad!, curl!, laplacian!, inverse_laplacian!
import LinearAlgebra: dot, norm

export GPUILMCache, GPUILMSystem, GPUBatch, GPUHeatIntegrator, solve_dirichlet!, solve_neumann!,
       solve_neumann_refined!, solve_stokes!, update_points!, surface_filter!, batch_solve!

const libilm = get(ENV, "ILM_LIB", joinpath(@__DIR__, "..", "immersedlayers.jl_gb300", "immersedlayers", "libilm.so"))

# ---------------------------------------------------------------------------
# enums and structs of include/ilm.h
# ---------------------------------------------------------------------------
const ILM_OK, ILM_ERR_NOT_CONVERGED = Cint(0), Cint(4)
const ILM_F64, ILM_F32 = Cint(0), Cint(1)
const ILM_GRID_SCALING, ILM_INDEX_SCALING = Cint(0), Cint(1)
const ILM_CACHE_SCALAR, ILM_CACHE_VECTOR = Cint(0), Cint(1)
const ILM_NODES_PRIMAL, ILM_NODES_DUAL, ILM_EDGES_PRIMAL, ILM_EDGES_DUAL, ILM_EDGEGRAD_PRIMAL =
    Cint(0), Cint(1), Cint(2), Cint(3), Cint(4)
const ILM_SCALAR_DATA, ILM_VECTOR_DATA, ILM_TENSOR_DATA = Cint(0), Cint(1), Cint(2)
const ILM_DDF = Dict(:Yang3 => Cint(0), :Roma => Cint(1), :M4prime => Cint(2), :Witchhat => Cint(3), :M3 => Cint(4))
# Schur builders (ilm_schur_kind_t)
const ILM_SCHUR_RTLINVR, ILM_SCHUR_CLINVCT, ILM_SCHUR_GLINVD, ILM_SCHUR_NRTRN = Cint(0), Cint(1), Cint(2), Cint(3)
const ILM_SCHUR_CLINVCT_SCALAR, ILM_SCHUR_CL2INVCT, ILM_SCHUR_GLINVD_SYMM, ILM_SCHUR_GLINVD_CROSS =
    Cint(4), Cint(5), Cint(6), Cint(7)

# ilm_solve_info_t
struct SolveInfo
    iterations::Cint
    converged::Cint
    rel_residual::Cdouble
end

# ilm_batch_problem_t
struct BatchProblem
    nx::Cint
    ny::Cint
    h::Cdouble
    i0x::Cint
    i0y::Cint
    npts::Cint
    kind::Cint
end

# ---------------------------------------------------------------------------
# LibILM: one wrapper per ILM_API entry point (same names and order as the header)
# ---------------------------------------------------------------------------
module LibILM
using CUDA
import ..libilm, ..SolveInfo, ..BatchProblem
const H = Ptr{Cvoid}      # opaque handle (ilm_grid_t, ilm_cache_t, ilm_batch_t, ilm_net_t, ilm_heat_t)
const S = Ptr{Cvoid}      # ilm_stream_t (a CUstream)
const D = CuPtr{Cvoid}    # device array of the cache dtype

ilm_version() = ccall((:ilm_version, libilm), Cint, ())
ilm_status_string(status) = ccall((:ilm_status_string, libilm), Cstring, (Cint,), status)
ilm_last_error() = ccall((:ilm_last_error, libilm), Cstring, ())

ilm_grid_create(nx, ny, h, i0x, i0y, out) =
    ccall((:ilm_grid_create, libilm), Cint, (Cint, Cint, Cdouble, Cint, Cint, Ref{Ptr{Cvoid}}), nx, ny, h, i0x, i0y, out)
ilm_grid_destroy(g) = ccall((:ilm_grid_destroy, libilm), Cint, (Ptr{Cvoid},), g)
ilm_grid_numel(g, kind, numel) =
    ccall((:ilm_grid_numel, libilm), Cint, (Ptr{Cvoid}, Cint, Ref{Csize_t}), g, kind, numel)
ilm_alloc(nbytes, out) = ccall((:ilm_alloc, libilm), Cint, (Csize_t, Ref{Ptr{Cvoid}}), nbytes, out)
ilm_free(p) = ccall((:ilm_free, libilm), Cint, (Ptr{Cvoid},), p)
ilm_copy_h2d(dst, src, nbytes, stream) =
    ccall((:ilm_copy_h2d, libilm), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t, Ptr{Cvoid}), dst, src, nbytes, stream)
ilm_copy_d2h(dst, src, nbytes, stream) =
    ccall((:ilm_copy_d2h, libilm), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t, Ptr{Cvoid}), dst, src, nbytes, stream)

ilm_cache_create(g, kind, npts, x, y, nrmx, nrmy, ds, ddf, scaling, dtype, out) =
    ccall((:ilm_cache_create, libilm), Cint,
          (Ptr{Cvoid}, Cint, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Cint, Cint,
           Cint, Ref{Ptr{Cvoid}}),
          g, kind, npts, x, y, nrmx, nrmy, ds, ddf, scaling, dtype, out)
ilm_cache_update_points(c, x, y, nrmx, nrmy, ds, stream) =
    ccall((:ilm_cache_update_points, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Ptr{Cvoid}),
          c, x, y, nrmx, nrmy, ds, stream)
ilm_cache_destroy(c) = ccall((:ilm_cache_destroy, libilm), Cint, (Ptr{Cvoid},), c)
ilm_cache_npts(c, npts) = ccall((:ilm_cache_npts, libilm), Cint, (Ptr{Cvoid}, Ref{Cint}), c, npts)

# point <-> grid transfers (src/surface_operators.jl:13-343)
ilm_regularize(c, out_kind, f, out, stream) =
    ccall((:ilm_regularize, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, out_kind, f, out, stream)
ilm_regularize_add(c, out_kind, f, out, stream) =
    ccall((:ilm_regularize_add, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, out_kind, f, out, stream)
ilm_grid_mul_add(n, dtype, a, b, out, stream) =
    ccall((:ilm_grid_mul_add, libilm), Cint, (Csize_t, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          n, dtype, a, b, out, stream)
ilm_surface_filter(c, power, s_in, s_out, stream) =
    ccall((:ilm_surface_filter, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, power, s_in, s_out, stream)
ilm_interpolate(c, in_kind, grid_in, f_out, stream) =
    ccall((:ilm_interpolate, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, in_kind, grid_in, f_out, stream)
ilm_regularize_normal(c, f, out, stream) =
    ccall((:ilm_regularize_normal, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}), c, f, out, stream)
ilm_regularize_normal_symm(c, v, out, stream) =
    ccall((:ilm_regularize_normal_symm, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, v, out, stream)
ilm_regularize_normal_cross(c, out_kind, in, out, stream) =
    ccall((:ilm_regularize_normal_cross, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, out_kind, in, out, stream)
ilm_regularize_normal_dot(c, out_kind, in, out, stream) =
    ccall((:ilm_regularize_normal_dot, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, out_kind, in, out, stream)
ilm_normal_interpolate(c, grid_in, out, stream) =
    ccall((:ilm_normal_interpolate, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, grid_in, out, stream)
ilm_normal_interpolate_symm(c, grid_in, out, stream) =
    ccall((:ilm_normal_interpolate_symm, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, grid_in, out, stream)
ilm_normal_cross_interpolate(c, in_kind, grid_in, out, stream) =
    ccall((:ilm_normal_cross_interpolate, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, in_kind, grid_in, out, stream)
ilm_normal_dot_interpolate(c, in_kind, grid_in, out, stream) =
    ccall((:ilm_normal_dot_interpolate, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, in_kind, grid_in, out, stream)

# composite layer operators (src/surface_operators.jl:357-725)
ilm_surface_divergence(c, in, out, stream) =
    ccall((:ilm_surface_divergence, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}), c, in, out, stream)
ilm_surface_divergence_symm(c, in, out, stream) =
    ccall((:ilm_surface_divergence_symm, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, in, out, stream)
ilm_surface_grad(c, in, out, stream) =
    ccall((:ilm_surface_grad, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}), c, in, out, stream)
ilm_surface_grad_symm(c, in, out, stream) =
    ccall((:ilm_surface_grad_symm, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}), c, in, out, stream)
ilm_surface_curl(c, direction, point_kind, in, out, stream) =
    ccall((:ilm_surface_curl, libilm), Cint, (Ptr{Cvoid}, Cint, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, direction, point_kind, in, out, stream)
ilm_surface_curl_cross(c, direction, in, out, stream) =
    ccall((:ilm_surface_curl_cross, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, direction, in, out, stream)
ilm_surface_divergence_cross(c, in, out, stream) =
    ccall((:ilm_surface_divergence_cross, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, in, out, stream)
ilm_surface_grad_cross(c, in, out, stream) =
    ccall((:ilm_surface_grad_cross, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, in, out, stream)

# staggered stencils and the LGF inverse Laplacian (src/grid_operators.jl:25-434)
ilm_divergence(c, in_kind, in, out, stream) =
    ccall((:ilm_divergence, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, in_kind, in, out, stream)
ilm_grad(c, in_kind, in, out, stream) =
    ccall((:ilm_grad, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}), c, in_kind, in, out, stream)
ilm_curl(c, in_kind, in, out, stream) =
    ccall((:ilm_curl, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}), c, in_kind, in, out, stream)
ilm_convective_derivative(c, field_kind, v, q, out, stream) =
    ccall((:ilm_convective_derivative, libilm), Cint,
          (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}), c, field_kind, v, q, out, stream)
ilm_w_cross_v(c, w, v, out, stream) =
    ccall((:ilm_w_cross_v, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, w, v, out, stream)
ilm_vecfield_helmholtz(c, curlv, divv, dv, vp, uniform, v_out, stream) =
    ccall((:ilm_vecfield_helmholtz, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cdouble}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, curlv, divv, dv, vp, uniform, v_out, stream)
ilm_laplacian(c, kind, in, out, stream) =
    ccall((:ilm_laplacian, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}), c, kind, in, out, stream)
ilm_inverse_laplacian(c, kind, in, out, stream) =
    ccall((:ilm_inverse_laplacian, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ptr{Cvoid}),
          c, kind, in, out, stream)
ilm_mask(c, kind, complementary, out, stream) =
    ccall((:ilm_mask, libilm), Cint, (Ptr{Cvoid}, Cint, Cint, CuPtr{Cvoid}, Ptr{Cvoid}), c, kind, complementary, out, stream)

# inner products (src/tools.jl:101-236)
ilm_dot_grid(c, kind, a, b, result, stream) =
    ccall((:ilm_dot_grid, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ref{Cdouble}, Ptr{Cvoid}),
          c, kind, a, b, result, stream)
ilm_dot_surface(c, ncomp, a, b, result, stream) =
    ccall((:ilm_dot_surface, libilm), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ref{Cdouble}, Ptr{Cvoid}),
          c, ncomp, a, b, result, stream)
ilm_dot_grid_noalloc(nx, ny, h, scaling, kind, dtype, a, b, result, stream) =
    ccall((:ilm_dot_grid_noalloc, libilm), Cint,
          (Cint, Cint, Cdouble, Cint, Cint, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, Ref{Cdouble}, Ptr{Cvoid}),
          nx, ny, h, scaling, kind, dtype, a, b, result, stream)

# Schur complements and problem solves
ilm_schur_build(c, which, scale, A_dev, stream) =
    ccall((:ilm_schur_build, libilm), Cint, (Ptr{Cvoid}, Cint, Cdouble, CuPtr{Cdouble}, Ptr{Cvoid}),
          c, which, scale, A_dev, stream)
ilm_solve_dirichlet(c, fplus, fminus, f_out, s_out, tol, maxiter, info, stream) =
    ccall((:ilm_solve_dirichlet, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Cdouble, Cint, Ref{SolveInfo}, Ptr{Cvoid}),
          c, fplus, fminus, f_out, s_out, tol, maxiter, info, stream)
ilm_solve_dirichlet_refined(c, fplus, fminus, f_out, s_out, tol, maxiter, max_refine, info, stream) =
    ccall((:ilm_solve_dirichlet_refined, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cint, Cint, Ref{SolveInfo},
           Ptr{Cvoid}),
          c, fplus, fminus, f_out, s_out, tol, maxiter, max_refine, info, stream)
ilm_solve_neumann_refined(c, vplus, vminus, f_out, df_out, tol, maxiter, max_refine, info, stream) =
    ccall((:ilm_solve_neumann_refined, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cint, Cint, Ref{SolveInfo},
           Ptr{Cvoid}),
          c, vplus, vminus, f_out, df_out, tol, maxiter, max_refine, info, stream)
ilm_solve_neumann(c, vplus, vminus, f_out, df_out, tol, maxiter, info, stream) =
    ccall((:ilm_solve_neumann, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Cdouble, Cint, Ref{SolveInfo}, Ptr{Cvoid}),
          c, vplus, vminus, f_out, df_out, tol, maxiter, info, stream)
ilm_solve_neumann_full(c, vplus, vminus, f_out, df_out, s_out, ds_out, tol, maxiter, info, stream) =
    ccall((:ilm_solve_neumann_full, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Cdouble, Cint,
           Ref{SolveInfo}, Ptr{Cvoid}),
          c, vplus, vminus, f_out, df_out, s_out, ds_out, tol, maxiter, info, stream)
ilm_solve_stokes(c, vplus, vminus, v_out, s_out, sigma_out, tol, maxiter, info, stream) =
    ccall((:ilm_solve_stokes, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Cdouble, Cint, Ref{SolveInfo},
           Ptr{Cvoid}),
          c, vplus, vminus, v_out, s_out, sigma_out, tol, maxiter, info, stream)
ilm_solve_stokes_multi(c, nrhs, vplus, vminus, v_out, s_out, sigma_out, tol, maxiter, precond, info, stream) =
    ccall((:ilm_solve_stokes_multi, libilm), Cint,
          (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Cdouble, Cint, Cint,
           Ptr{SolveInfo}, Ptr{Cvoid}),
          c, nrhs, vplus, vminus, v_out, s_out, sigma_out, tol, maxiter, precond, info, stream)
ilm_solve_stokes_multi_refined(c, nrhs, vplus, vminus, v_out, s_out, sigma_out, tol, maxiter, max_refine, info,
                               stream) =
    ccall((:ilm_solve_stokes_multi_refined, libilm), Cint,
          (Ptr{Cvoid}, Cint, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble,
           Cint, Cint, Ptr{SolveInfo}, Ptr{Cvoid}),
          c, nrhs, vplus, vminus, v_out, s_out, sigma_out, tol, maxiter, max_refine, info, stream)

# batched solves
ilm_batch_create(nprob, probs, x, y, nrmx, nrmy, ds, ddf, dtype, out) =
    ccall((:ilm_batch_create, libilm), Cint,
          (Cint, Ptr{BatchProblem}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Cint, Cint,
           Ref{Ptr{Cvoid}}),
          nprob, probs, x, y, nrmx, nrmy, ds, ddf, dtype, out)
ilm_batch_destroy(b) = ccall((:ilm_batch_destroy, libilm), Cint, (Ptr{Cvoid},), b)
ilm_batch_layout(b, field_offsets, point_offsets) =
    ccall((:ilm_batch_layout, libilm), Cint, (Ptr{Cvoid}, Ptr{Csize_t}, Ptr{Csize_t}), b, field_offsets, point_offsets)
ilm_batch_solve(b, fplus, fminus, f_out, s_out, tol, maxiter, stream) =
    ccall((:ilm_batch_solve, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Cdouble, Cint, Ptr{Cvoid}),
          b, fplus, fminus, f_out, s_out, tol, maxiter, stream)
ilm_batch_solve_graph(b, fplus, fminus, f_out, s_out, tol, maxiter, stream) =
    ccall((:ilm_batch_solve_graph, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Cdouble, Cint, Ptr{Cvoid}),
          b, fplus, fminus, f_out, s_out, tol, maxiter, stream)
ilm_batch_solve_refined(b, fplus, fminus, f_out, s_out, tol, maxiter, max_refine, stream) =
    ccall((:ilm_batch_solve_refined, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cint, Cint, Ptr{Cvoid}),
          b, fplus, fminus, f_out, s_out, tol, maxiter, max_refine, stream)
ilm_batch_set_precond(b, mode, block_size) =
    ccall((:ilm_batch_set_precond, libilm), Cint, (Ptr{Cvoid}, Cint, Cint), b, mode, block_size)
ilm_batch_set_profiling(b, enable) = ccall((:ilm_batch_set_profiling, libilm), Cint, (Ptr{Cvoid}, Cint), b, enable)
ilm_batch_stage_times(b, ms, nstages, launches) =
    ccall((:ilm_batch_stage_times, libilm), Cint, (Ptr{Cvoid}, Ptr{Cfloat}, Ref{Cint}, Ref{Cint}), b, ms, nstages, launches)
ilm_batch_stats(b, stats) = ccall((:ilm_batch_stats, libilm), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), b, stats)
ilm_batch_setup_times(b, ms, max_phases, nphases, names) =
    ccall((:ilm_batch_setup_times, libilm), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ref{Cint}, Ptr{Cstring}),
          b, ms, max_phases, nphases, names)
ilm_batch_cg_times(b, start_us, end_us, sm) =
    ccall((:ilm_batch_cg_times, libilm), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cint}), b, start_us, end_us, sm)
ilm_batch_set_rhs_operator(b, enable) =
    ccall((:ilm_batch_set_rhs_operator, libilm), Cint, (Ptr{Cvoid}, Cint), b, enable)
ilm_batch_set_cg_variant(b, variant) = ccall((:ilm_batch_set_cg_variant, libilm), Cint, (Ptr{Cvoid}, Cint), b, variant)
ilm_batch_get_cg_variant(b, variant, nclusters) =
    ccall((:ilm_batch_get_cg_variant, libilm), Cint, (Ptr{Cvoid}, Ref{Cint}, Ref{Cint}), b, variant, nclusters)
ilm_batch_autotune(b, fplus, fminus, f_out, s_out, tol, maxiter, reps, stream, chosen, ms_per_variant) =
    ccall((:ilm_batch_autotune, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Cdouble, Cint, Cint, Ptr{Cvoid}, Ref{Cint},
           Ptr{Cfloat}),
          b, fplus, fminus, f_out, s_out, tol, maxiter, reps, stream, chosen, ms_per_variant)
ilm_batch_info(b, iterations, rel_residual) =
    ccall((:ilm_batch_info, libilm), Cint, (Ptr{Cvoid}, Ptr{Cint}, Ptr{Cdouble}), b, iterations, rel_residual)

# learned preconditioner
ilm_net_create(nfeat, width, nlayers, band, out) =
    ccall((:ilm_net_create, libilm), Cint, (Cint, Cint, Cint, Cint, Ref{Ptr{Cvoid}}), nfeat, width, nlayers, band, out)
ilm_net_destroy(n) = ccall((:ilm_net_destroy, libilm), Cint, (Ptr{Cvoid},), n)
ilm_net_set_tensor_cores(n, enable) = ccall((:ilm_net_set_tensor_cores, libilm), Cint, (Ptr{Cvoid}, Cint), n, enable)
ilm_net_nparams(n, count) = ccall((:ilm_net_nparams, libilm), Cint, (Ptr{Cvoid}, Ref{Csize_t}), n, count)
ilm_net_set_params(n, host) = ccall((:ilm_net_set_params, libilm), Cint, (Ptr{Cvoid}, Ptr{Cfloat}), n, host)
ilm_net_get_params(n, host) = ccall((:ilm_net_get_params, libilm), Cint, (Ptr{Cvoid}, Ptr{Cfloat}), n, host)
ilm_net_forward(n, npts, feat, seg_start, seg_len, band_out, stream) =
    ccall((:ilm_net_forward, libilm), Cint,
          (Ptr{Cvoid}, Cint, CuPtr{Cfloat}, CuPtr{Cint}, CuPtr{Cint}, CuPtr{Cfloat}, Ptr{Cvoid}),
          n, npts, feat, seg_start, seg_len, band_out, stream)
ilm_net_loss_grad(n, npts, npairs, pair_off, feat, seg_start, seg_len, w, b, x, loss_out, grad_out, stream) =
    ccall((:ilm_net_loss_grad, libilm), Cint,
          (Ptr{Cvoid}, Cint, Cint, CuPtr{Cint}, CuPtr{Cfloat}, CuPtr{Cint}, CuPtr{Cint}, CuPtr{Cfloat}, CuPtr{Cfloat},
           CuPtr{Cfloat}, Ref{Cdouble}, Ptr{Cfloat}, Ptr{Cvoid}),
          n, npts, npairs, pair_off, feat, seg_start, seg_len, w, b, x, loss_out, grad_out, stream)
ilm_net_train_step(n, npts, npairs, pair_off, feat, seg_start, seg_len, w, b, x, lr, loss_dev, stream) =
    ccall((:ilm_net_train_step, libilm), Cint,
          (Ptr{Cvoid}, Cint, Cint, CuPtr{Cint}, CuPtr{Cfloat}, CuPtr{Cint}, CuPtr{Cint}, CuPtr{Cfloat}, CuPtr{Cfloat},
           CuPtr{Cfloat}, Cdouble, CuPtr{Cdouble}, Ptr{Cvoid}),
          n, npts, npairs, pair_off, feat, seg_start, seg_len, w, b, x, lr, loss_dev, stream)
ilm_point_features(npts, x, y, nx, ny, ds, seg_start, seg_len, h, out) =
    ccall((:ilm_point_features, libilm), Cint,
          (Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cint}, Ptr{Cint}, Cdouble,
           Ptr{Cfloat}),
          npts, x, y, nx, ny, ds, seg_start, seg_len, h, out)
ilm_batch_set_learned(b, net, kind_mask, body_start) =
    ccall((:ilm_batch_set_learned, libilm), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cint}), b, net, kind_mask, body_start)
ilm_batch_set_coarse(b, kind_mask, body_start) =
    ccall((:ilm_batch_set_coarse, libilm), Cint, (Ptr{Cvoid}, Cint, Ptr{Cint}), b, kind_mask, body_start)
ilm_batch_schur_apply(b, x, y, stream) =
    ccall((:ilm_batch_schur_apply, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Ptr{Cvoid}), b, x, y, stream)
ilm_batch_schur_solve(b, rhs, x, tol, maxiter, stream) =
    ccall((:ilm_batch_schur_solve, libilm), Cint,
          (Ptr{Cvoid}, CuPtr{Cdouble}, CuPtr{Cdouble}, Cdouble, Cint, Ptr{Cvoid}), b, rhs, x, tol, maxiter, stream)

# heat conduction time marching (test/literate/heatconduction.jl:87-189)
ilm_heat_create(c, kappa, dt, tb_plus, tb_minus, tol, maxiter, out) =
    ccall((:ilm_heat_create, libilm), Cint,
          (Ptr{Cvoid}, Cdouble, Cdouble, Ptr{Cdouble}, Ptr{Cdouble}, Cdouble, Cint, Ref{Ptr{Cvoid}}),
          c, kappa, dt, tb_plus, tb_minus, tol, maxiter, out)
ilm_heat_destroy(h) = ccall((:ilm_heat_destroy, libilm), Cint, (Ptr{Cvoid},), h)
ilm_heat_advance(h, T, sigma_out, nsteps, stream) =
    ccall((:ilm_heat_advance, libilm), Cint, (Ptr{Cvoid}, CuPtr{Cvoid}, CuPtr{Cvoid}, Cint, Ptr{Cvoid}),
          h, T, sigma_out, nsteps, stream)
ilm_heat_info(h, last_iters, last_relres, nnz) =
    ccall((:ilm_heat_info, libilm), Cint, (Ptr{Cvoid}, Ptr{Cint}, Ptr{Cdouble}, Ref{Csize_t}), h, last_iters, last_relres, nnz)
end # module LibILM

using .LibILM

# Status check: every entry point returns an ilm_status_t; a failure raises
# with the library's message, as the reference raises Julia exceptions.
function check(st::Cint)
    st == ILM_OK && return nothing
    msg = unsafe_string(LibILM.ilm_last_error())
    code = unsafe_string(LibILM.ilm_status_string(st))
    st == Cint(1) && throw(ArgumentError("libilm ($code): $msg"))
    st == Cint(7) && throw(DimensionMismatch("libilm ($code): $msg"))
    error("libilm ($code): $msg")
end

cur_stream() = CUDA.stream().handle

# ---------------------------------------------------------------------------
# GPUILMCache: the device BasicILMCache (src/cache.jl:16-88, 164-316)
# ---------------------------------------------------------------------------
mutable struct GPUILMCache{T<:Union{Float32,Float64}}
    handle::Ptr{Cvoid}
    grid::Ptr{Cvoid}
    g::PhysicalGrid
    npts::Int
    vector::Bool
    scaling::Symbol
end

_dtype(::Type{Float64}) = ILM_F64
_dtype(::Type{Float32}) = ILM_F32

"""
    GPUILMCache(body, g::PhysicalGrid; vector=false, ddftype=:Yang3, scaling=:GridScaling, T=Float64)

Device counterpart of `SurfaceScalarCache(body, g; ddftype, scaling)`
(`vector=false`) and `SurfaceVectorCache` (`vector=true`), src/cache.jl:209-261.
Points, normals and areas come from RigidBodyTools as in `BasicILMCache`.
"""
function GPUILMCache(body, g::PhysicalGrid; vector::Bool=false, ddftype::Symbol=:Yang3,
                     scaling::Symbol=:GridScaling, T::Type=Float64)
    X = collect(points(body))
    nrm = collect(normals(body))
    ds = collect(areas(body))
    n = length(ds)
    x, y = Float64.(X.u), Float64.(X.v)
    nx, ny = Float64.(nrm.u), Float64.(nrm.v)
    gh = Ref{Ptr{Cvoid}}(C_NULL)
    check(LibILM.ilm_grid_create(size(g, 1), size(g, 2), cellsize(g), origin(g)[1], origin(g)[2], gh))
    ch = Ref{Ptr{Cvoid}}(C_NULL)
    check(LibILM.ilm_cache_create(gh[], vector ? ILM_CACHE_VECTOR : ILM_CACHE_SCALAR, n, x, y, nx, ny,
                                  Float64.(ds.data), ILM_DDF[ddftype],
                                  scaling == :GridScaling ? ILM_GRID_SCALING : ILM_INDEX_SCALING, _dtype(T), ch))
    c = GPUILMCache{T}(ch[], gh[], g, n, vector, scaling)
    finalizer(c) do c
        LibILM.ilm_cache_destroy(c.handle)
        LibILM.ilm_grid_destroy(c.grid)
    end
    return c
end

"""
    update_points!(c, x, y, nrmx, nrmy, ds)

Moving bodies (src/system.jl:26-50, `update_system!`): new point data
(device FP64 arrays) re-binned on the device without rebuilding the cache.
"""
update_points!(c::GPUILMCache, x::CuArray{Float64}, y::CuArray{Float64}, nrmx::CuArray{Float64},
               nrmy::CuArray{Float64}, ds::CuArray{Float64}) =
    check(LibILM.ilm_cache_update_points(c.handle, x, y, nrmx, nrmy, ds, cur_stream()))

const Dev{T} = CuArray{T}

# -- regularize! / interpolate! (src/surface_operators.jl:13-88) ------------
# The grid kind of the output selects the staggering: Nodes{Primal} (cell
# centres, scalar caches), Nodes{Dual}, Edges{Primal} (faces, vector caches).
regularize!(s::Dev{T}, f::Dev{T}, c::GPUILMCache{T}; kind=c.vector ? ILM_EDGES_PRIMAL : ILM_NODES_PRIMAL) where {T} =
    check(LibILM.ilm_regularize(c.handle, kind, f, s, cur_stream()))
interpolate!(f::Dev{T}, s::Dev{T}, c::GPUILMCache{T}; kind=c.vector ? ILM_EDGES_PRIMAL : ILM_NODES_PRIMAL) where {T} =
    check(LibILM.ilm_interpolate(c.handle, kind, s, f, cur_stream()))

# -- normal / cross / dot / symm transfers (:98-343) ------------------------
regularize_normal!(q::Dev{T}, f::Dev{T}, c::GPUILMCache{T}) where {T} =
    check(LibILM.ilm_regularize_normal(c.handle, f, q, cur_stream()))
normal_interpolate!(f::Dev{T}, q::Dev{T}, c::GPUILMCache{T}) where {T} =
    check(LibILM.ilm_normal_interpolate(c.handle, q, f, cur_stream()))
regularize_normal_symm!(q::Dev{T}, v::Dev{T}, c::GPUILMCache{T}) where {T} =
    check(LibILM.ilm_regularize_normal_symm(c.handle, v, q, cur_stream()))
normal_interpolate_symm!(v::Dev{T}, q::Dev{T}, c::GPUILMCache{T}) where {T} =
    check(LibILM.ilm_normal_interpolate_symm(c.handle, q, v, cur_stream()))
regularize_normal_cross!(q::Dev{T}, f::Dev{T}, c::GPUILMCache{T}; kind=c.vector ? ILM_NODES_DUAL : ILM_EDGES_PRIMAL) where {T} =
    check(LibILM.ilm_regularize_normal_cross(c.handle, kind, f, q, cur_stream()))
normal_cross_interpolate!(f::Dev{T}, q::Dev{T}, c::GPUILMCache{T}; kind=c.vector ? ILM_NODES_DUAL : ILM_EDGES_PRIMAL) where {T} =
    check(LibILM.ilm_normal_cross_interpolate(c.handle, kind, q, f, cur_stream()))
regularize_normal_dot!(q::Dev{T}, v::Dev{T}, c::GPUILMCache{T}; kind=ILM_NODES_PRIMAL) where {T} =
    check(LibILM.ilm_regularize_normal_dot(c.handle, kind, v, q, cur_stream()))
normal_dot_interpolate!(v::Dev{T}, q::Dev{T}, c::GPUILMCache{T}; kind=ILM_NODES_PRIMAL) where {T} =
    check(LibILM.ilm_normal_dot_interpolate(c.handle, kind, q, v, cur_stream()))

# -- composite layer operators (:357-725) -----------------------------------
surface_divergence!(θ::Dev{T}, f::Dev{T}, c::GPUILMCache{T}) where {T} =
    check(LibILM.ilm_surface_divergence(c.handle, f, θ, cur_stream()))
surface_grad!(f::Dev{T}, θ::Dev{T}, c::GPUILMCache{T}) where {T} =
    check(LibILM.ilm_surface_grad(c.handle, θ, f, cur_stream()))
surface_divergence_symm!(θ::Dev{T}, v::Dev{T}, c::GPUILMCache{T}) where {T} =
    check(LibILM.ilm_surface_divergence_symm(c.handle, v, θ, cur_stream()))
surface_grad_symm!(v::Dev{T}, q::Dev{T}, c::GPUILMCache{T}) where {T} =
    check(LibILM.ilm_surface_grad_symm(c.handle, q, v, cur_stream()))
# surface_curl!(ψ, f, cache) (point -> grid, C_s^T) and surface_curl!(f, ψ, cache)
# (grid -> point, C_s) share a name in the reference; `direction` selects them
surface_curl!(out::Dev{T}, in::Dev{T}, c::GPUILMCache{T}; to_grid::Bool=true,
              point_kind=c.vector ? ILM_VECTOR_DATA : ILM_SCALAR_DATA) where {T} =
    check(LibILM.ilm_surface_curl(c.handle, to_grid ? Cint(0) : Cint(1), point_kind, in, out, cur_stream()))
surface_curl_cross!(out::Dev{T}, in::Dev{T}, c::GPUILMCache{T}; to_grid::Bool=true) where {T} =
    check(LibILM.ilm_surface_curl_cross(c.handle, to_grid ? Cint(0) : Cint(1), in, out, cur_stream()))
surface_divergence_cross!(θ::Dev{T}, f::Dev{T}, c::GPUILMCache{T}) where {T} =
    check(LibILM.ilm_surface_divergence_cross(c.handle, f, θ, cur_stream()))
surface_grad_cross!(f::Dev{T}, θ::Dev{T}, c::GPUILMCache{T}) where {T} =
    check(LibILM.ilm_surface_grad_cross(c.handle, θ, f, cur_stream()))

# -- stencils and the LGF inverse Laplacian (src/grid_operators.jl) ---------
divergence!(out::Dev{T}, q::Dev{T}, c::GPUILMCache{T}; kind=ILM_EDGES_PRIMAL) where {T} =
    check(LibILM.ilm_divergence(c.handle, kind, q, out, cur_stream()))
grad!(out::Dev{T}, w::Dev{T}, c::GPUILMCache{T}; kind=ILM_NODES_PRIMAL) where {T} =
    check(LibILM.ilm_grad(c.handle, kind, w, out, cur_stream()))
curl!(out::Dev{T}, w::Dev{T}, c::GPUILMCache{T}; kind=ILM_NODES_DUAL) where {T} =
    check(LibILM.ilm_curl(c.handle, kind, w, out, cur_stream()))
laplacian!(out::Dev{T}, w::Dev{T}, c::GPUILMCache{T}; kind=ILM_NODES_PRIMAL) where {T} =
    check(LibILM.ilm_laplacian(c.handle, kind, w, out, cur_stream()))
inverse_laplacian!(w::Dev{T}, c::GPUILMCache{T}; kind=ILM_NODES_PRIMAL) where {T} =
    check(LibILM.ilm_inverse_laplacian(c.handle, kind, w, w, cur_stream()))

# -- masks (src/surface_operators.jl:737-923) -------------------------------
function mask!(out::Dev{T}, c::GPUILMCache{T}; kind=ILM_NODES_PRIMAL, complementary::Bool=false) where {T}
    check(LibILM.ilm_mask(c.handle, kind, complementary ? Cint(1) : Cint(0), out, cur_stream()))
    return out
end
mask(c::GPUILMCache{T}, out::Dev{T}) where {T} = mask!(out, c)
complementary_mask(c::GPUILMCache{T}, out::Dev{T}) where {T} = mask!(out, c; complementary=true)

# -- inner products (src/tools.jl:101-236) ----------------------------------
function dot(a::Dev{T}, b::Dev{T}, c::GPUILMCache{T}; kind=ILM_NODES_PRIMAL, surface::Bool=false, ncomp=1) where {T}
    r = Ref{Cdouble}(0.0)
    if surface
        check(LibILM.ilm_dot_surface(c.handle, ncomp, a, b, r, cur_stream()))
    else
        check(LibILM.ilm_dot_grid(c.handle, kind, a, b, r, cur_stream()))
    end
    return r[]
end
norm(a::Dev{T}, c::GPUILMCache{T}; kwargs...) where {T} = sqrt(dot(a, a, c; kwargs...))

# -- Schur complements (src/matrix_operators.jl:9-244) ----------------------
function _schur(c::GPUILMCache{T}, which::Cint, n::Int; scale=1.0) where {T}
    A = CUDA.zeros(Float64, n, n)
    check(LibILM.ilm_schur_build(c.handle, which, scale, A, cur_stream()))
    return A
end
_nsurf(c) = c.vector ? 2c.npts : c.npts
create_RTLinvR(c::GPUILMCache; scale=1.0) = _schur(c, ILM_SCHUR_RTLINVR, _nsurf(c); scale)
create_CLinvCT(c::GPUILMCache; scale=1.0) = _schur(c, ILM_SCHUR_CLINVCT, _nsurf(c); scale)
create_GLinvD(c::GPUILMCache; scale=1.0) = _schur(c, ILM_SCHUR_GLINVD, _nsurf(c); scale)
create_nRTRn(c::GPUILMCache; scale=1.0) = _schur(c, ILM_SCHUR_NRTRN, _nsurf(c); scale)
create_CLinvCT_scalar(c::GPUILMCache; scale=1.0) = _schur(c, ILM_SCHUR_CLINVCT_SCALAR, c.npts; scale)
create_CL2invCT(c::GPUILMCache; scale=1.0) = _schur(c, ILM_SCHUR_CL2INVCT, _nsurf(c); scale)
create_GLinvD_symm(c::GPUILMCache; scale=1.0) = _schur(c, ILM_SCHUR_GLINVD_SYMM, _nsurf(c); scale)
create_GLinvD_cross(c::GPUILMCache; scale=1.0) = _schur(c, ILM_SCHUR_GLINVD_CROSS, _nsurf(c); scale)

"""
    surface_filter!(s_out, s_in, c; power=1)

`C^power s` with the surface filter `C = Ẽᵀ R` (src/matrix_operators.jl:254-268),
applied matrix-free.
"""
surface_filter!(s_out::Dev{T}, s_in::Dev{T}, c::GPUILMCache{T}; power::Integer=1) where {T} =
    check(LibILM.ilm_surface_filter(c.handle, power, s_in, s_out, cur_stream()))

# ---------------------------------------------------------------------------
# GPUILMSystem: ILMSystem's forwarding (src/system.jl:184-227) and solves
# ---------------------------------------------------------------------------
struct GPUILMSystem{T,P}
    base_cache::GPUILMCache{T}
    phys_params::P
    bc::Dict{String,Any}
end
GPUILMSystem(c::GPUILMCache; phys_params=nothing, bc=Dict{String,Any}()) = GPUILMSystem(c, phys_params, bc)

for f in [:regularize!, :interpolate!, :regularize_normal!, :normal_interpolate!,
          :regularize_normal_cross!, :normal_cross_interpolate!,
          :regularize_normal_dot!, :normal_dot_interpolate!,
          :regularize_normal_symm!, :normal_interpolate_symm!,
          :surface_curl!, :surface_divergence!, :surface_grad!,
          :surface_divergence_symm!, :surface_grad_symm!,
          :surface_curl_cross!, :surface_divergence_cross!, :surface_grad_cross!,
          :divergence!, :grad!, :curl!, :laplacian!]
    @eval $f(a, b, sys::GPUILMSystem; kwargs...) = $f(a, b, sys.base_cache; kwargs...)
end
for f in [:create_nRTRn, :create_GLinvD, :create_CLinvCT, :create_CL2invCT, :create_RTLinvR,
          :create_GLinvD_symm, :create_GLinvD_cross, :create_CLinvCT_scalar]
    @eval $f(sys::GPUILMSystem; kwargs...) = $f(sys.base_cache; kwargs...)
end
dot(a, b, sys::GPUILMSystem; kwargs...) = dot(a, b, sys.base_cache; kwargs...)
norm(a, sys::GPUILMSystem; kwargs...) = norm(a, sys.base_cache; kwargs...)
inverse_laplacian!(w, sys::GPUILMSystem; kwargs...) = inverse_laplacian!(w, sys.base_cache; kwargs...)

function _solved(st::Cint, info::Ref{SolveInfo})
    st == ILM_ERR_NOT_CONVERGED && @warn "libilm: Schur CG not converged" info[]
    st == ILM_ERR_NOT_CONVERGED || check(st)
    return info[]
end

"""
    solve_dirichlet!(f, s, fplus, fminus, sys; tol=1e-8, maxiter=5000, refine=0)

`solve(prob::DirichletPoissonProblem, sys)` (test/literate/problems.jl:259-298)
with the dense `S\\s` replaced by the device CG.  `refine > 0` runs FP64
iterative refinement (f and s are then FP64 device arrays).
"""
function solve_dirichlet!(f::CuArray, s::CuArray, fplus::Dev{T}, fminus::Dev{T}, sys::GPUILMSystem{T};
                          tol=1e-8, maxiter=5000, refine::Integer=0) where {T}
    info = Ref{SolveInfo}()
    c = sys.base_cache
    st = refine > 0 ?
        LibILM.ilm_solve_dirichlet_refined(c.handle, fplus, fminus, f, s, tol, maxiter, refine, info, cur_stream()) :
        LibILM.ilm_solve_dirichlet(c.handle, fplus, fminus, f, s, tol, maxiter, info, cur_stream())
    return f, s, _solved(st, info)
end

"""
    solve_neumann!(f, df, s, ds, vplus, vminus, sys; tol=1e-8, maxiter=5000)

`solve(prob::NeumannPoissonProblem, sys)` (test/literate/neumann.jl:101-142):
potential f and [φ], streamfunction s and [ψ].
"""
function solve_neumann!(f::Dev{T}, df::Dev{T}, s::Dev{T}, ds::Dev{T}, vplus::Dev{T}, vminus::Dev{T},
                        sys::GPUILMSystem{T}; tol=1e-8, maxiter=5000) where {T}
    info = Ref{SolveInfo}()
    st = LibILM.ilm_solve_neumann_full(sys.base_cache.handle, vplus, vminus, f, df, s, ds, tol, maxiter, info,
                                       cur_stream())
    return f, df, s, ds, _solved(st, info)
end

"""
    solve_neumann_refined!(f, df, vplus, vminus, sys; tol=1e-12, maxiter=20000, max_refine=8)

Potential f and [φ] of the Neumann problem with FP64 iterative refinement
(FP64 device arrays in and out, any cache dtype).
"""
function solve_neumann_refined!(f::CuArray{Float64}, df::CuArray{Float64}, vplus::CuArray{Float64},
                                vminus::CuArray{Float64}, sys::GPUILMSystem; tol=1e-12, maxiter=20000, max_refine=8)
    info = Ref{SolveInfo}()
    st = LibILM.ilm_solve_neumann_refined(sys.base_cache.handle, vplus, vminus, f, df, tol, maxiter, max_refine, info,
                                          cur_stream())
    return f, df, _solved(st, info)
end

"""
    solve_stokes!(v, s, σ, vplus, vminus, sys; tol=1e-8, maxiter=5000)

`solve(prob::StokesFlowProblem, sys)` (test/literate/stokes.jl:101-166) on a
vector cache: velocity on faces, streamfunction, filtered traction.
"""
function solve_stokes!(v::Dev{T}, s::Dev{T}, σ::Dev{T}, vplus::Dev{T}, vminus::Dev{T}, sys::GPUILMSystem{T};
                       tol=1e-8, maxiter=5000) where {T}
    info = Ref{SolveInfo}()
    st = LibILM.ilm_solve_stokes(sys.base_cache.handle, vplus, vminus, v, s, σ, tol, maxiter, info, cur_stream())
    return v, s, σ, _solved(st, info)
end

# ---------------------------------------------------------------------------
# Batched solves: many independent problems per launch
# ---------------------------------------------------------------------------
mutable struct GPUBatch
    handle::Ptr{Cvoid}
    field_offsets::Vector{Csize_t}
    point_offsets::Vector{Csize_t}
end

"""
    GPUBatch(problems::Vector{BatchProblem}, x, y, nrmx, nrmy, ds; ddftype=:Yang3, T=Float32)

Set up many independent Dirichlet (kind 0) / Neumann (kind 1) problems; the
point arrays hold all problems' points, concatenated in problem order.
"""
function GPUBatch(probs::Vector{BatchProblem}, x::Vector{Float64}, y::Vector{Float64}, nrmx::Vector{Float64},
                  nrmy::Vector{Float64}, ds::Vector{Float64}; ddftype::Symbol=:Yang3, T::Type=Float32)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(LibILM.ilm_batch_create(length(probs), probs, x, y, nrmx, nrmy, ds, ILM_DDF[ddftype], _dtype(T), h))
    fo = zeros(Csize_t, length(probs) + 1)
    po = zeros(Csize_t, length(probs) + 1)
    check(LibILM.ilm_batch_layout(h[], fo, po))
    b = GPUBatch(h[], fo, po)
    finalizer(b -> LibILM.ilm_batch_destroy(b.handle), b)
    return b
end

"""
    batch_solve!(f, s, b, fplus, fminus; tol=1e-8, maxiter=5000, graph=false)

Solve every problem of the batch; `graph=true` replays a captured CUDA graph
of the launch sequence.  Returns per-problem CG iterations and residuals.
"""
function batch_solve!(f::CuArray, s::CuArray, b::GPUBatch, fplus::CuArray, fminus::CuArray; tol=1e-8,
                      maxiter=5000, graph::Bool=false, refine::Integer=0)
    if refine > 0   # FP64 iterative refinement: FP64 arrays in and out
        check(LibILM.ilm_batch_solve_refined(b.handle, fplus, fminus, f, s, tol, maxiter, refine, cur_stream()))
    else
        fn = graph ? LibILM.ilm_batch_solve_graph : LibILM.ilm_batch_solve
        check(fn(b.handle, fplus, fminus, f, s, tol, maxiter, cur_stream()))
    end
    n = length(b.field_offsets) - 1
    its = zeros(Cint, n)
    rr = zeros(Cdouble, n)
    check(LibILM.ilm_batch_info(b.handle, its, rr))
    return its, rr
end

# ---------------------------------------------------------------------------
# Heat conduction: init / step! of ConstrainedSystems, on the device
# (test/literate/heatconduction.jl:87-189, src/timemarching.jl:254-277)
# ---------------------------------------------------------------------------
mutable struct GPUHeatIntegrator
    handle::Ptr{Cvoid}
    T::CuArray
    t::Float64
    dt::Float64
end

function GPUHeatIntegrator(c::GPUILMCache, T0::CuArray, κ, Δt, Tb_plus::Vector{Float64}, Tb_minus::Vector{Float64};
                           tol=1e-10, maxiter=2000)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(LibILM.ilm_heat_create(c.handle, κ, Δt, Tb_plus, Tb_minus, tol, maxiter, h))
    integ = GPUHeatIntegrator(h[], copy(T0), 0.0, Δt)
    finalizer(i -> LibILM.ilm_heat_destroy(i.handle), integ)
    return integ
end

function step!(integ::GPUHeatIntegrator, nsteps::Integer=1)
    check(LibILM.ilm_heat_advance(integ.handle, integ.T, CU_NULL, nsteps, cur_stream()))
    integ.t += nsteps * integ.dt
    return integ
end

end # module
