/*
 * ilm.h -- C ABI of the GB300 (sm_103a) immersed-layer library (libilm.so).
 *
 * Drop-in boundary for the hot path of ImmersedLayers.jl v0.5.6.  The reference
 * has no FFI of its own: its operators are Julia generic functions of the form
 * `op!(out, in, cache)` that mutate `out` (src/surface_operators.jl,
 * src/grid_operators.jl).  Each entry point below replaces one such method; the
 * citation beside it names the reference method it stands in for.  A Julia
 * `ccall` shim (and the Python ctypes mirror shipped with this library) binds
 * these symbols one-to-one.
 *
 * Conventions
 *  - Every function returns an int status (ilm_status_t); ILM_OK == 0.  The
 *    message of the last failure on the calling thread is ilm_last_error().
 *  - Grid and surface arrays passed to operators are DEVICE pointers of the
 *    cache's dtype (ILM_F64 -> double, ILM_F32 -> float).  Setup functions take
 *    HOST arrays of double.
 *  - Memory layout follows the reference (column-major, first index x):
 *      Nodes{Primal}      (NX-1) x (NY-1), x fastest
 *      Nodes{Dual}        NX x NY
 *      Edges{Primal}      u block NX x (NY-1), then v block (NX-1) x NY
 *      Edges{Dual}        u block (NX-1) x NY, then v block NX x (NY-1)
 *      EdgeGradient{Primal} dudx (NX-1)x(NY-1), dudy NXxNY, dvdx NXxNY,
 *                         dvdy (NX-1)x(NY-1), concatenated
 *      ScalarData N, VectorData [u;v] 2N, TensorData [dudx;dudy;dvdx;dvdy] 4N
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls on one
 *    cache must be serialised by the caller (the cache owns scratch buffers,
 *    like the reference's non-reentrant BasicILMCache).
 */
#ifndef ILM_H
#define ILM_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define ILM_API __attribute__((visibility("default")))
#else
#define ILM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  ILM_OK = 0,
  ILM_ERR_INVALID_ARG = 1,
  ILM_ERR_CUDA = 2,
  ILM_ERR_NO_MEMORY = 3,
  ILM_ERR_NOT_CONVERGED = 4,
  ILM_ERR_TIMEOUT = 5,
  ILM_ERR_UNSUPPORTED = 6,
  ILM_ERR_SIZE_LIMIT = 7
} ilm_status_t;

typedef enum { ILM_F64 = 0, ILM_F32 = 1 } ilm_dtype_t;

/* Discrete delta functions (CartesianGrids Yang3 / Roma / M4prime / Witchhat / M3). */
typedef enum {
  ILM_DDF_YANG3 = 0, ILM_DDF_ROMA = 1, ILM_DDF_M4PRIME = 2, ILM_DDF_WITCHHAT = 3, ILM_DDF_M3 = 4
} ilm_ddf_t;

/* src/ImmersedLayers.jl:81-83 (GridScaling default for problems) */
typedef enum { ILM_GRID_SCALING = 0, ILM_INDEX_SCALING = 1 } ilm_scaling_t;

/* SurfaceScalarCache / SurfaceVectorCache (src/cache.jl:164-202) */
typedef enum { ILM_CACHE_SCALAR = 0, ILM_CACHE_VECTOR = 1 } ilm_cache_kind_t;

/* CartesianGrids grid data types */
typedef enum {
  ILM_NODES_PRIMAL = 0, ILM_NODES_DUAL = 1, ILM_EDGES_PRIMAL = 2, ILM_EDGES_DUAL = 3,
  ILM_EDGEGRAD_PRIMAL = 4
} ilm_gridkind_t;

/* Surface point data types */
typedef enum { ILM_SCALAR_DATA = 0, ILM_VECTOR_DATA = 1, ILM_TENSOR_DATA = 2 } ilm_pointkind_t;

/* Dense Schur-complement builders (src/matrix_operators.jl) */
typedef enum {
  ILM_SCHUR_RTLINVR = 0,   /* create_RTLinvR        :9-30    -R^T L^-1 R        */
  ILM_SCHUR_CLINVCT = 1,   /* create_CLinvCT        :40-61   -C_s L^-1 C_s^T    */
  ILM_SCHUR_GLINVD = 2,    /* create_GLinvD         :135-155 -G_s L^-1 D_s      */
  ILM_SCHUR_NRTRN = 3,     /* create_nRTRn          :225-244  n.R_f^T R_f n o   */
  ILM_SCHUR_CLINVCT_SCALAR = 4, /* create_CLinvCT_scalar :71-93 (vector cache, ScalarData) */
  ILM_SCHUR_CL2INVCT = 5,  /* create_CL2invCT       :102-125 -C_s L^-2 C_s^T (vector cache) */
  ILM_SCHUR_GLINVD_SYMM = 6, /* create_GLinvD_symm  :165-185 (vector cache)     */
  ILM_SCHUR_GLINVD_CROSS = 7 /* create_GLinvD_cross :195-215 (scalar cache)     */
} ilm_schur_kind_t;

typedef struct ilm_grid_s* ilm_grid_t;
typedef struct ilm_cache_s* ilm_cache_t;
typedef void* ilm_stream_t; /* cudaStream_t */

/* Result of an iterative Schur solve. */
typedef struct {
  int iterations;          /* Krylov iterations taken                          */
  int converged;           /* 1 if rel. residual <= tol                        */
  double rel_residual;     /* ||b - S s||_2 / ||b||_2, evaluated in FP64       */
} ilm_solve_info_t;

/* ---- library ----------------------------------------------------------- */
ILM_API int ilm_version(void);
ILM_API const char* ilm_status_string(int status);
ILM_API const char* ilm_last_error(void);

/* ---- grid: PhysicalGrid (CartesianGrids; printed in examples/caches.ipynb) */
/* nx, ny: number of dual nodes (ghosts included); i0x, i0y: 1-based index of
 * the origin (primal node i sits at x = (i - i0x) h).                       */
ILM_API int ilm_grid_create(int nx, int ny, double h, int i0x, int i0y, ilm_grid_t* out);
ILM_API int ilm_grid_destroy(ilm_grid_t g);
/* Number of elements of one grid data kind (all components). */
ILM_API int ilm_grid_numel(ilm_grid_t g, int kind, size_t* numel);

/* ---- device buffers -------------------------------------------------------
 * For callers without their own device allocator (the Julia shim passes
 * CuArray pointers instead): nbytes of device memory on the current device,
 * freed by ilm_free; host <-> device copies in `stream` order (host memory
 * may be pageable; ilm_copy_d2h returns after the copy has completed).     */
ILM_API int ilm_alloc(size_t nbytes, void** out);
ILM_API int ilm_free(void* p);
ILM_API int ilm_copy_h2d(void* dst_dev, const void* src_host, size_t nbytes, ilm_stream_t stream);
ILM_API int ilm_copy_d2h(void* dst_host, const void* src_dev, size_t nbytes, ilm_stream_t stream);

/* ---- cache: SurfaceScalarCache/SurfaceVectorCache (src/cache.jl:209-261) */
/* x, y: point coordinates; nrmx, nrmy: outward normals; ds: panel areas
 * (src/tools.jl:16-38).  All host arrays of length npts.                    */
ILM_API int ilm_cache_create(ilm_grid_t g, int kind, int npts,
                     const double* x, const double* y,
                     const double* nrmx, const double* nrmy, const double* ds,
                     int ddf, int scaling, int dtype, ilm_cache_t* out);
/* Moving bodies: replace the cache's points by new positions, normals and
 * areas (same number of points; DEVICE FP64 arrays of npts each) and redo
 * the DDF windows, the point arrays and the tile candidate lists on the
 * device, in stream order, keeping the grid, the FFT plans and the scratch.
 * Replaces the cache rebuild of update_system / update_system!
 * (src/system.jl:26-49, regenerate_problem src/problem.jl:95-105), which
 * constructs new regularization matrices for the new body configuration.
 * Cached Schur complements are invalidated; no host synchronisation.      */
ILM_API int ilm_cache_update_points(ilm_cache_t c, const double* x, const double* y, const double* nrmx,
                                    const double* nrmy, const double* ds, ilm_stream_t stream);
ILM_API int ilm_cache_destroy(ilm_cache_t c);
ILM_API int ilm_cache_npts(ilm_cache_t c, int* npts);

/* ---- point <-> grid transfers (src/surface_operators.jl:13-88) --------- */
/* regularize!(s::Nodes{Primal|Dual}, f::ScalarData) (:13,:25) and
 * regularize!(v::Edges{Primal}, vb::VectorData) (:36); output overwritten.  */
ILM_API int ilm_regularize(ilm_cache_t c, int out_kind, const void* f, void* out, ilm_stream_t stream);
/* Forcing (src/forcing.jl:451-515): out += R f without clearing `out` --
 * the accumulation of line and point forcing (_apply_forcing! does
 * fill!(gdata,0); regularize!(gdata,str,cache); dy .+= gdata); only the
 * tiles that hold points are visited.  ilm_grid_mul_add: out += a .* b
 * over n grid values (area forcing, dy .+= str .* mask).                   */
ILM_API int ilm_regularize_add(ilm_cache_t c, int out_kind, const void* f, void* out, ilm_stream_t stream);
ILM_API int ilm_grid_mul_add(size_t n, int dtype, const void* a, const void* b, void* out, ilm_stream_t stream);
/* Surface filter C = E~ R (create_surface_filter, src/matrix_operators.jl:
 * 254-268) applied `power` times: s_out = C^power s_in (the C^6 s of
 * test/literate/problems.jl:107,297).  E~ is the filtered interpolation of
 * CartesianGrids' Regularize(filter = true): E~ = W^-1 E, W = diag(E R 1),
 * so constant surface data pass unchanged.  Scalar caches filter
 * ScalarData through Nodes{Primal}, vector caches VectorData through
 * Edges{Primal}.  W is formed on the first call and kept until the points
 * move (ilm_cache_update_points).  s_in may equal s_out; power 0 copies.
 * No N x N matrix is formed: each power is one regularize, one
 * interpolation and one scaling.                                          */
ILM_API int ilm_surface_filter(ilm_cache_t c, int power, const void* s_in, void* s_out, ilm_stream_t stream);
/* interpolate!(f, s::Nodes{Primal|Dual}) (:56,:67), interpolate!(vb, v::Edges{Primal}) (:78) */
ILM_API int ilm_interpolate(ilm_cache_t c, int in_kind, const void* grid_in, void* f_out, ilm_stream_t stream);

/* regularize_normal!(q::Edges{Primal}, f::ScalarData) (:98-103) and
 * regularize_normal!(qt::EdgeGradient{Primal}, v::VectorData) (:113-123)    */
ILM_API int ilm_regularize_normal(ilm_cache_t c, const void* f, void* out, ilm_stream_t stream);
/* regularize_normal_symm!(qt::EdgeGradient{Primal}, v::VectorData) (:125-133) */
ILM_API int ilm_regularize_normal_symm(ilm_cache_t c, const void* v, void* out, ilm_stream_t stream);
/* regularize_normal_cross!(q::Edges{Primal}, f::ScalarData) (:150-165) and
 * regularize_normal_cross!(w::Nodes{Dual}, vs::VectorData) (:167-178)       */
ILM_API int ilm_regularize_normal_cross(ilm_cache_t c, int out_kind, const void* in, void* out, ilm_stream_t stream);
/* regularize_normal_dot!(f::Nodes{Primal}, vs::VectorData) (:188-203) and
 * regularize_normal_dot!(v::Edges{Primal}, taus::TensorData) (:205-215)     */
ILM_API int ilm_regularize_normal_dot(ilm_cache_t c, int out_kind, const void* in, void* out, ilm_stream_t stream);
/* normal_interpolate!(vn, q::Edges{Primal}) (:228-240),
 * normal_interpolate!(tau::VectorData, A::EdgeGradient{Primal}) (:242-250)  */
ILM_API int ilm_normal_interpolate(ilm_cache_t c, const void* grid_in, void* out, ilm_stream_t stream);
/* normal_interpolate_symm!(tau, A::EdgeGradient{Primal}) (:252-283)        */
ILM_API int ilm_normal_interpolate_symm(ilm_cache_t c, const void* grid_in, void* out, ilm_stream_t stream);
/* normal_cross_interpolate!(wn, v::Edges{Primal}) (:277-295),
 * normal_cross_interpolate!(vs::VectorData, s::Nodes{Dual}) (:298-307)      */
ILM_API int ilm_normal_cross_interpolate(ilm_cache_t c, int in_kind, const void* grid_in, void* out, ilm_stream_t stream);
/* normal_dot_interpolate!(vs, f::Nodes{Primal}) (:316-330),
 * normal_dot_interpolate!(taus::TensorData, v::Edges{Primal}) (:332-343)   */
ILM_API int ilm_normal_dot_interpolate(ilm_cache_t c, int in_kind, const void* grid_in, void* out, ilm_stream_t stream);

/* ---- composite layer operators (src/surface_operators.jl:357-725) ------- */
/* direction: 0 = surface -> grid (e.g. surface_divergence!(theta, f)),
 *            1 = grid -> surface (e.g. surface_grad!(vn, phi)).             */
ILM_API int ilm_surface_divergence(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream);      /* :530-591 */
ILM_API int ilm_surface_divergence_symm(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream); /* :574-591 */
ILM_API int ilm_surface_grad(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream);            /* :604-664 */
ILM_API int ilm_surface_grad_symm(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream);       /* :650-664 */
ILM_API int ilm_surface_curl(ilm_cache_t c, int direction, int point_kind, const void* in, void* out, ilm_stream_t stream); /* :357-452 */
ILM_API int ilm_surface_curl_cross(ilm_cache_t c, int direction, const void* in, void* out, ilm_stream_t stream);          /* :467-515 */
ILM_API int ilm_surface_divergence_cross(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream);/* :679-690 */
ILM_API int ilm_surface_grad_cross(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream);      /* :704-725 */

/* ---- grid operators (src/grid_operators.jl:17-179) ---------------------- */
/* divergence!(p::Nodes{Primal}, v::Edges{Primal}) (:25-31) and
 * divergence!(v::Edges{Primal}, A::EdgeGradient{Primal}); scaled by 1/h
 * under GridScaling.  in_kind names the input type.                        */
ILM_API int ilm_divergence(ilm_cache_t c, int in_kind, const void* in, void* out, ilm_stream_t stream);
/* grad!(v::Edges{Primal}, p::Nodes{Primal}) (:45-52), grad!(A::EdgeGradient{Primal}, v::Edges{Primal}) (:61-67) */
ILM_API int ilm_grad(ilm_cache_t c, int in_kind, const void* in, void* out, ilm_stream_t stream);
/* curl!(v::Edges{Primal}, s::Nodes{Dual}) (:79-85), curl!(w::Nodes{Dual}, v::Edges{Primal}) (:97-103) */
ILM_API int ilm_curl(ilm_cache_t c, int in_kind, const void* in, void* out, ilm_stream_t stream);
/* convective_derivative!(out, v, q, base_cache, extra_cache)
 * (src/grid_operators.jl:258-315, steps :318-371): v . grad q with v on
 * Edges{Primal} and q of field_kind -- Nodes{Primal} (v . grad p),
 * Nodes{Dual} (v . grad w) or Edges{Primal} (v . grad u; u . grad u is
 * q = v) -- scaled by 1/h under GridScaling; out has field_kind and must
 * not alias v or q.  One fused stencil pass; the reference's
 * ConvectiveDerivativeCache temporaries are not needed.  (The reference's
 * 5-argument Edges method v . grad u refers to an undefined variable at
 * :368 and raises; here it computes v . grad u.)                           */
ILM_API int ilm_convective_derivative(ilm_cache_t c, int field_kind, const void* v, const void* q, void* out,
                                      ilm_stream_t stream);
/* w_cross_v!(out::Edges{Primal}, w::Nodes{Dual}, v::Edges{Primal}) (:401-434):
 * the rotational convective term w x v (no derivative scaling).           */
ILM_API int ilm_w_cross_v(ilm_cache_t c, const void* w, const void* v, void* out, ilm_stream_t stream);
/* vecfield_helmholtz!(v, curlv, divv, dv, vp, base_cache, veccache)
 * (src/helmholtz.jl:327-347; vector caches): v = curl psi + grad phi + vp
 * with L psi = -(curlv + R_n n x dv) and L phi = divv + R_c n . dv (:85-120,
 * :196-231).  curlv: Nodes{Dual} masked curl; divv: Nodes{Primal} masked
 * divergence; dv: VectorData surface jump (may be null without points);
 * vp: Edges{Primal} or null; uniform: (Vx, Vy) added to every u / v value
 * (the tuple method, :346-347) or null.                                    */
ILM_API int ilm_vecfield_helmholtz(ilm_cache_t c, const void* curlv, const void* divv, const void* dv,
                                   const void* vp, const double* uniform, void* v_out, ilm_stream_t stream);
/* laplacian!(w, s) (:123-134): 5-point Laplacian, interior points, x 1/h^2 */
ILM_API int ilm_laplacian(ilm_cache_t c, int kind, const void* in, void* out, ilm_stream_t stream);
/* inverse_laplacian!(sol, rhs) (:153-179): unbounded-domain L^-1 via the
 * lattice Green's function (FFT convolution).  in may equal out.           */
ILM_API int ilm_inverse_laplacian(ilm_cache_t c, int kind, const void* in, void* out, ilm_stream_t stream);
/* mask(cache) / complementary_mask(cache) (:737-760, :856-877) evaluated on
 * grid data of `kind`, GridScaling caches.  Scalar caches: H on
 * Nodes{Primal}, Nodes{Dual} / Edges{Primal} by the grid interpolation of
 * mask! (:880-905).  Vector caches: H on Edges{Primal} from the all-ones
 * VectorData, Nodes{Dual} / Nodes{Primal} / EdgeGradient{Primal} from its u
 * component (:907-923).                                                   */
ILM_API int ilm_mask(ilm_cache_t c, int kind, int complementary, void* out, ilm_stream_t stream);

/* ---- inner products (src/tools.jl:101-236, src/cache.jl:815-909) -------- */
/* dot(u1, u2, cache) for grid data of kind `kind` (cell-volume weighted). */
ILM_API int ilm_dot_grid(ilm_cache_t c, int kind, const void* a, const void* b, double* result, ilm_stream_t stream);
/* dot(u1, u2, cache) for point data with `ncomp` components (ds weighted). */
ILM_API int ilm_dot_surface(ilm_cache_t c, int ncomp, const void* a, const void* b, double* result, ilm_stream_t stream);

/* Allocation-free weighted grid inner product.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory when
 * they need an inner product (services whose memory pool owns the device,
 * latency-critical loops that must not call cudaMalloc or cudaFree, which can
 * synchronise the whole device).  Same result as ilm_dot_grid on grid data of
 * `kind` for an nx x ny grid with cell size h and `scaling`, without a cache;
 * it calls no allocating routine.  Its scratch is a fixed 128 KiB device array
 * held by every GPU that loads the library: one FP64 partial sum per grid row,
 * so grids are limited to ny <= 16384 dual nodes (taller ones fail with
 * ILM_ERR_SIZE_LIMIT; nx is not limited).  `stream` must belong to the
 * current device (else ILM_ERR_INVALID_ARG).  The first call on a device
 * looks up that array's address (cudaGetSymbolAddress).  Calls share the
 * array: calls that may overlap on the GPU race and must be
 * serialised by the caller.  Waits for `stream` and copies the result to
 * host memory before it returns.                                             */
ILM_API int ilm_dot_grid_noalloc(int nx, int ny, double h, int scaling, int kind, int dtype, const void* a,
                                 const void* b, double* result, ilm_stream_t stream);

/* ---- Schur complements (src/matrix_operators.jl:9-244) ------------------ */
/* Dense n x n (column-major, FP64, device) Schur complement; n = N for
 * ScalarData kinds, 2N for the VectorData of vector caches.  Scalar caches,
 * kinds 0-3: built directly from lattice-Green's-function point-point sums
 * instead of the reference's N operator applications.  Vector caches and
 * kinds 4-7: the reference's column-by-column build, on the device (one unit
 * vector per column through the operator chain).  create_GLinvD_cross
 * raises in the reference (surface_divergence_cross! refers to an undefined
 * variable, src/surface_operators.jl:680); kind 7 builds the operator its
 * documentation states.  A_dev must hold n*n doubles.                      */
ILM_API int ilm_schur_build(ilm_cache_t c, int which, double scale, double* A_dev, ilm_stream_t stream);

/* ---- problem solves (test/literate/problems.jl:259-298, neumann.jl:101-142) */
/* Dirichlet Poisson: inputs fplus/fminus (ScalarData, device, cache dtype);
 * outputs f (Nodes{Primal}) and s (ScalarData).  The Schur system is solved
 * by CG on the device to rel. residual `tol` (FP64).                        */
ILM_API int ilm_solve_dirichlet(ilm_cache_t c, const void* fplus, const void* fminus,
                        void* f_out, void* s_out, double tol, int maxiter,
                        ilm_solve_info_t* info, ilm_stream_t stream);
/* Neumann Poisson: outputs f (Nodes{Primal}) and df = [phi] (ScalarData). */
ILM_API int ilm_solve_neumann(ilm_cache_t c, const void* vplus, const void* vminus,
                      void* f_out, void* df_out, double tol, int maxiter,
                      ilm_solve_info_t* info, ilm_stream_t stream);
/* FP64 iterative refinement of the Dirichlet / Neumann solves (the
 * reference solves S s = rhs by FP64 dense LU, test/literate/problems.jl:291,
 * neumann.jl:123).  Inputs fplus/fminus (or vplus/vminus) and outputs f_out
 * (Nodes{Primal}) and s_out / df_out (ScalarData) are FP64 device arrays for
 * every cache dtype.  An FP32 cache first solves in FP32; an FP64 cache of
 * the same points (built on the first call, dropped by
 * ilm_cache_update_points) forms the Schur right-hand side in FP64; each
 * refinement step forms the FP64 Schur residual, solves for the correction by
 * CG and adds it in FP64, until ||b - S s||_2 / ||b||_2 <= tol or
 * `max_refine` steps (then ILM_ERR_NOT_CONVERGED); f is assembled in FP64.
 * info: CG iterations of all solves and the final FP64 residual.           */
ILM_API int ilm_solve_dirichlet_refined(ilm_cache_t c, const double* fplus, const double* fminus, double* f_out,
                                        double* s_out, double tol, int maxiter, int max_refine,
                                        ilm_solve_info_t* info, ilm_stream_t stream);
ILM_API int ilm_solve_neumann_refined(ilm_cache_t c, const double* vplus, const double* vminus, double* f_out,
                                      double* df_out, double tol, int maxiter, int max_refine,
                                      ilm_solve_info_t* info, ilm_stream_t stream);
/* The whole NeumannPoissonProblem solve of test/literate/neumann.jl:101-142:
 * the potential f (Nodes{Primal}) and df = [phi], then the streamfunction
 * s (Nodes{Dual}) and ds = [psi] (ScalarData): s* = C_s^T df, S ds =
 * G^x_s f* with the same S = -C_s L^-1 C_s^T, s = L^-1 (s* - C^x_s^T ds)
 * (:129-138).  s_out and ds_out both null: the potential part only (=
 * ilm_solve_neumann).  info sums the two CG solves' iterations and reports
 * the worse residual.                                                      */
ILM_API int ilm_solve_neumann_full(ilm_cache_t c, const void* vplus, const void* vminus, void* f_out, void* df_out,
                                   void* s_out, void* ds_out, double tol, int maxiter, ilm_solve_info_t* info,
                                   ilm_stream_t stream);
/* Stokes flow with no-slip surfaces (vector GridScaling cache): the
 * StokesFlowProblem solve of test/literate/stokes.jl:101-166.  vplus/vminus:
 * VectorData (2N) surface velocities outside/inside; v_out: Edges{Primal}
 * velocity, s_out: Nodes{Dual} streamfunction, sigma_out: VectorData
 * traction (filtered twice, :165).  The Schur systems -C_s L^-2 C_s^T
 * (create_CL2invCT, src/matrix_operators.jl:102) and -C_s L^-1 C_s^T on
 * scalars (create_CLinvCT_scalar, :71) are solved matrix-free by
 * (preconditioned) CG in place of the reference's dense LU; info reports
 * both solves (iterations summed, worst relative residual).               */
ILM_API int ilm_solve_stokes(ilm_cache_t c, const void* vplus, const void* vminus, void* v_out, void* s_out,
                             void* sigma_out, double tol, int maxiter, ilm_solve_info_t* info,
                             ilm_stream_t stream);
/* The same solve for `nrhs` (1..ILM_STOKES_MAX_RHS) velocity right-hand
 * sides at once (stokes.jl:138,156 solved for several surface velocities
 * with one S).  vplus/vminus: nrhs x 2N (right-hand side r at offset 2N r);
 * v_out: nrhs Edges{Primal} fields, s_out: nrhs Nodes{Dual} fields,
 * sigma_out: nrhs x 2N, each contiguous in the cache dtype.  Both Schur
 * systems are solved by block CG over all right-hand sides (maxiter block
 * iterations each, Krylov vectors FP64); precond = 1 preconditions S with
 * the inverse of the gauge-shifted point-point Schur complement -E L^-1 E^T
 * on each velocity component (N <= 4096; built once per cache and kept
 * until the points move), 0 runs plain block CG.  info: nrhs entries
 * (iterations = block iterations of both solves).  ilm_solve_stokes is this
 * call with nrhs = 1 and precond = 1.                                      */
#define ILM_STOKES_MAX_RHS 32
ILM_API int ilm_solve_stokes_multi(ilm_cache_t c, int nrhs, const void* vplus, const void* vminus, void* v_out,
                                   void* s_out, void* sigma_out, double tol, int maxiter, int precond,
                                   ilm_solve_info_t* info, ilm_stream_t stream);
/* FP64-refined Stokes solves for `nrhs` right-hand sides: FP64 inputs and
 * outputs (layouts as ilm_solve_stokes_multi).  The pre-step (psi*, v_phi,
 * v'), every Schur residual b - S sigma and the field assembly run in FP64
 * on an FP64 cache of the same points (built on first use, dropped when the
 * points move); the corrections S d = r are block CG with the cache's own
 * operator (FP32 for an FP32 cache; S preconditioned as in
 * ilm_solve_stokes_multi), each to 1e-4 of its residual or until it stops
 * improving, for at most max_refine steps per Schur system, and until a step
 * no longer reduces the FP64 residual (refinement converges while the
 * corrections' operator resolves every mode of S: cond(S) x its rounding
 * < 1).  info: FP64 relative residuals; iterations = block iterations of all
 * corrections.                                                             */
ILM_API int ilm_solve_stokes_multi_refined(ilm_cache_t c, int nrhs, const double* vplus, const double* vminus,
                                           double* v_out, double* s_out, double* sigma_out, double tol, int maxiter,
                                           int max_refine, ilm_solve_info_t* info, ilm_stream_t stream);

/* ---- batched problem solves (configs of many independent problems) ------ */
/* Many independent Dirichlet/Neumann Poisson problems (each its own grid and
 * bodies) set up and solved together: every stage of the block-LU solve of
 * test/literate/problems.jl:259-298 / neumann.jl:101-127 is one launch for the
 * whole batch, and the dense LU per problem is replaced by device CG on the
 * LGF-assembled Schur complement.  GridScaling.                             */
typedef struct ilm_batch_s* ilm_batch_t;
typedef struct {
  int nx, ny;      /* dual nodes of this problem's grid                    */
  double h;        /* cell size                                            */
  int i0x, i0y;    /* 1-based origin index                                 */
  int npts;        /* surface points of this problem                       */
  int kind;        /* 0 = Dirichlet, 1 = Neumann                           */
} ilm_batch_problem_t;
/* x, y, nrmx, nrmy, ds: host arrays of all problems' points, concatenated in
 * problem order.  dtype: precision of the grid-side work (the Schur CG is
 * always FP64).  Builds DDF windows, tile lists and the Schur complements.
 * Returns while the Schur build still runs on the device (its own stream):
 * every later call that reads the Schur complements orders its device work
 * after that build, so the caller's host work (the preconditioner set-up)
 * overlaps it.  With both kinds in the batch the Neumann problems' matrices
 * are built first, and the set-up work that reads only those (their block
 * inverses, the coarse correction) starts before the Dirichlet ones are
 * done.                                                                     */
ILM_API int ilm_batch_create(int nprob, const ilm_batch_problem_t* probs, const double* x, const double* y,
                             const double* nrmx, const double* nrmy, const double* ds, int ddf, int dtype,
                             ilm_batch_t* out);
ILM_API int ilm_batch_destroy(ilm_batch_t b);
/* Offsets (nprob+1 each, in elements) of each problem's Nodes{Primal} field
 * in the packed field array and of its points in the packed point arrays.  */
ILM_API int ilm_batch_layout(ilm_batch_t b, size_t* field_offsets, size_t* point_offsets);
/* fplus/fminus: packed surface data (device, batch dtype).  f_out: packed
 * Nodes{Primal} fields; s_out: packed surface strengths.  Issues no
 * host<->device copies (capturable in a CUDA graph once tol/maxiter are set). */
ILM_API int ilm_batch_solve(ilm_batch_t b, const void* fplus, const void* fminus, void* f_out, void* s_out,
                            double tol, int maxiter, ilm_stream_t stream);
/* FP64 iterative refinement of the batched solve (the reference's solves are
 * FP64 dense LU, test/literate/problems.jl:291, neumann.jl:123).  fplus /
 * fminus: packed surface data in FP64 (device); f_out / s_out: FP64 packed
 * fields and surface strengths.  The batch's pipeline (FP32 grid work for an
 * FP32 batch) gives the first strengths; an FP64 copy of the pipeline
 * (built on the first call) forms the Schur right-hand side; each
 * refinement step forms the FP64 Schur residual of every problem, solves for
 * the correction with the batch's preconditioned CG and adds it in FP64,
 * until every ||b - S s||_2 / ||b||_2 <= tol or `max_refine` steps; the field
 * is then assembled in FP64.  ilm_batch_info reports the CG iterations of
 * all solves and the final FP64 residual per problem.  Synchronises `stream`. */
ILM_API int ilm_batch_solve_refined(ilm_batch_t b, const double* fplus, const double* fminus, double* f_out,
                                    double* s_out, double tol, int maxiter, int max_refine, ilm_stream_t stream);
/* The same solve as one CUDA graph launch on `stream` (a created stream,
 * not the legacy default stream): the first call for a set of buffers,
 * tolerance, limit and CG configuration captures the launch sequence of
 * ilm_batch_solve, later calls with the same arguments replay it.  A
 * GB300-side launch path with no counterpart in the reference.             */
ILM_API int ilm_batch_solve_graph(ilm_batch_t b, const void* fplus, const void* fminus, void* f_out, void* s_out,
                                  double tol, int maxiter, ilm_stream_t stream);
/* Preconditioner of the Schur CG for the following solves: mode 0 = none
 * (plain CG), 1 = block-Jacobi (inverses of the diagonal blocks of ~block_size
 * consecutive surface points, eliminated and applied in float-float
 * arithmetic inside flexible CG), 2 = the learned band set by
 * ilm_batch_set_learned, block-Jacobi for the problems without a network.
 * The block inverses are formed on the device on a stream of the batch,
 * issued by this call in mode 2 and by the first solve in mode 1; the
 * call does not wait for them, and the solves order their CG after them.   */
ILM_API int ilm_batch_set_precond(ilm_batch_t b, int mode, int block_size);
/* Coarse correction of the block-Jacobi preconditioner on the bodies'
 * constant vectors (the near-null space of the Neumann Schur complement
 * -C_s L^-1 C_s^T, neumann.jl:123, one small eigenvalue per closed body):
 * z = M_bj r + Z E^-1 Z^T W r, Z the bodies' indicator vectors, E = Z^T W S Z
 * (E and E^-1 formed on the device on a stream of the batch after the Schur
 * build; the call does not wait for them, the solves order their CG after
 * them; a singular E leaves the correction out).  kind_mask 2: the
 * Neumann problems with at most 4 bodies; 0: off.  body_start: as
 * ilm_batch_set_learned.  Applies wherever block-Jacobi runs (mode 1, and
 * mode 2 for the problems without a network); no counterpart in the
 * reference (its Schur systems are LU-solved).                             */
ILM_API int ilm_batch_set_coarse(ilm_batch_t b, int kind_mask, const int* body_start);
/* Stage timing: when enabled, ilm_batch_solve records a CUDA event on its
 * stream at each stage boundary; ilm_batch_stage_times returns the elapsed
 * ms per stage (up to 31), the number of stages and the number of kernel
 * launches the last solve issued.  ilm_batch_stats returns 6 doubles: total
 * points, total Nodes{Primal} cells, sum of npts^2, sum of padded FFT sizes
 * P1*P2, number of problems, total cells of the problems' source boxes (the
 * part of each grid the surface operators can reach, the only cells the
 * scatters write and the FFT row pass reads).                               */
ILM_API int ilm_batch_set_profiling(ilm_batch_t b, int enable);
ILM_API int ilm_batch_stage_times(ilm_batch_t b, float* ms, int* nstages, int* launches);
ILM_API int ilm_batch_stats(ilm_batch_t b, double* stats);
/* Host wall-clock (ms) of the phases of this batch's set-up
 * (ilm_batch_create): up to max_phases times into ms[] and static phase
 * names into names[] (either may be null); *nphases = the number of phases.
 * No counterpart in the reference (its caches have no set-up profile).     */
ILM_API int ilm_batch_setup_times(ilm_batch_t b, double* ms, int max_phases, int* nphases, const char** names);
/* Per-problem Schur CG timing of the last solve issued with profiling
 * enabled: start and end (us, relative to the first problem taken) and the
 * SM of the first CTA of the cluster that solved it.  A profiling helper
 * with no counterpart in the reference.                                     */
ILM_API int ilm_batch_cg_times(ilm_batch_t b, double* start_us, double* end_us, int* sm);
/* Schur CG kernel of the batch: 0 default (= 6, which is 1 when no problem
 * is at or below the size split), 1 row-distributed
 * vectors over 8-CTA clusters with 256-thread CTAs (two or three cluster
 * barriers per iteration, FP64 work on the owned rows only), 2 replicated
 * vectors (one cluster barrier per iteration, every vector operation in
 * every CTA), 3 row-distributed with 128-thread CTAs (twice the resident
 * clusters), 4 256-thread CTAs at most two per SM, 5 512-thread CTAs one
 * per SM, 6 size split: problems above 192 points on variant 1's clusters,
 * the smaller ones one CTA each (no cluster barriers) on a second stream in
 * the CTA slots the clusters leave free, joined by events (the Schur-only
 * entry points run every problem on variant 1).  ilm_batch_autotune solves the given
 * data with every variant (one untimed and `reps` timed solves each, each
 * between CUDA events on `stream`), keeps the fastest and returns it in
 * *chosen and the least ms per solve of variants 1..ILM_CG_VARIANTS in
 * ms_per_variant[ILM_CG_VARIANTS] (-1: skipped; the least of the reps, so
 * that one solve delayed by the host does not decide); the outputs hold the
 * last solve.
 * Tuning helpers with no counterpart in the reference (the reference
 * solves one problem at a time with a dense LU).                           */
/* Precomputed right-hand-side operator, for batches solved more than once
 * (no counterpart in the reference, which forms the right-hand side with a
 * full-grid convolution each solve): enable != 0 builds, once, per problem
 * M = E L^-1 D_s (Dirichlet) / G_s L^-1 R (Neumann) from the same LGF
 * point-point sums as S (float-float, as much memory as S), after which a
 * solve forms the Schur right-hand side as M [jump] - avg and the field with
 * one LGF convolution of the combined source instead of two.  The results
 * agree with the default path to the FP32 rounding of the convolution.  A
 * set-up call: the build runs on a stream of its own (no legacy-stream or
 * device-wide synchronisation) and the call returns when it is done.       */
ILM_API int ilm_batch_set_rhs_operator(ilm_batch_t b, int enable);
#define ILM_CG_VARIANTS 6
ILM_API int ilm_batch_set_cg_variant(ilm_batch_t b, int variant);
ILM_API int ilm_batch_get_cg_variant(ilm_batch_t b, int* variant, int* nclusters);
ILM_API int ilm_batch_autotune(ilm_batch_t b, const void* fplus, const void* fminus, void* f_out, void* s_out,
                               double tol, int maxiter, int reps, ilm_stream_t stream, int* chosen,
                               float* ms_per_variant);
/* Per-problem CG iterations and FP64 relative residuals of the last solve. */
ILM_API int ilm_batch_info(ilm_batch_t b, int* iterations, double* rel_residual);

/* ---- learned Schur-complement preconditioner ------------------------------
 * No counterpart in the reference (its Schur solve is the dense LU of
 * test/literate/problems.jl:291); it accelerates the device CG that replaces
 * that LU.  A 1-D convolutional network over arc length (circular within each
 * body, kernel 5, ReLU, `nlayers` layers of `width` channels) maps 8 point
 * features (ilm_point_features) to a band of 2*band+1 coefficients per point,
 * C; the preconditioner is M r = W^-1 C^T C r with W = diag(ds), self-adjoint
 * in the ds-weighted inner product in which W S is symmetric.  FP32 master
 * weights, BF16 copies read by every pass, FP32 accumulation.
 * Point arrays below are packed over problems/bodies; seg_start/seg_len give
 * each point's body as [seg_start, seg_start + seg_len) in packed indices.  */
typedef struct ilm_net_s* ilm_net_t;
ILM_API int ilm_net_create(int nfeat, int width, int nlayers, int band, ilm_net_t* out);
ILM_API int ilm_net_destroy(ilm_net_t n);
/* Forward convolutions on the tcgen05 tensor cores (enable != 0, the
 * default: BF16 weights, FP32 activations as a BF16 hi / lo pair, FP32
 * accumulation in tensor memory) or by FP32 FMA (0).  GB300-specific: no
 * counterpart in the reference.  With the tensor cores ilm_net_forward waits
 * for its stream and returns ILM_ERR_TIMEOUT if a layer did not complete.  */
ILM_API int ilm_net_set_tensor_cores(ilm_net_t n, int enable);
ILM_API int ilm_net_nparams(ilm_net_t n, size_t* count);
/* host FP32 parameters, per layer W[out][in][5] then bias[out]; set resets Adam */
ILM_API int ilm_net_set_params(ilm_net_t n, const float* host);
ILM_API int ilm_net_get_params(ilm_net_t n, float* host);
/* band_out (device, npts x (2 band + 1)): coefficients of C, identity included */
ILM_API int ilm_net_forward(ilm_net_t n, int npts, const float* feat, const int* seg_start, const int* seg_len,
                            float* band_out, ilm_stream_t stream);
/* Loss mean_p |M b - x|^2 / |x|^2 over pairs p (points pair_off[p] ..
 * pair_off[p+1], device int array) and its gradient w.r.t. the FP32
 * parameters; loss_out / grad_out are host pointers (either may be NULL). */
ILM_API int ilm_net_loss_grad(ilm_net_t n, int npts, int npairs, const int* pair_off, const float* feat,
                              const int* seg_start, const int* seg_len, const float* w, const float* b,
                              const float* x, double* loss_out, float* grad_out, ilm_stream_t stream);
/* One Adam step (lr) on the same loss; loss_dev (device double, optional)
 * receives the loss before the step.  Issues no host synchronisation.   */
ILM_API int ilm_net_train_step(ilm_net_t n, int npts, int npairs, const int* pair_off, const float* feat,
                               const int* seg_start, const int* seg_len, const float* w, const float* b,
                               const float* x, double lr, double* loss_dev, ilm_stream_t stream);
/* Host: features of npts points (out: npts x 8 floats) -- ds/h,
 * 10 h curvature, n_x, n_y, sin/cos(2 pi frac(x/h)), sin/cos(2 pi frac(y/h)). */
ILM_API int ilm_point_features(int npts, const double* x, const double* y, const double* nx, const double* ny,
                               const double* ds, const int* seg_start, const int* seg_len, double h, float* out);
/* Batch: run the network over the batch's points (body_start: host, per
 * packed point, the local index of its body's first point within its
 * problem) and use its band for the problems whose kind is in kind_mask
 * (bit 0 Dirichlet, bit 1 Neumann); call once per network.  Switches the
 * Schur CG to the learned preconditioner (mode 2 of ilm_batch_set_precond);
 * problems of a kind no network was set for run plain CG.  The features
 * and the network run on a stream of the batch; the call does not wait for
 * them (the first solve that reads the band orders its CG after them and
 * reports a tensor-core timeout of the network).  A network may serve
 * several batches: its forwards are ordered among themselves.              */
ILM_API int ilm_batch_set_learned(ilm_batch_t b, ilm_net_t net, int kind_mask, const int* body_start);
/* Batch Schur products / solves on device FP64 packed vectors (training data
 * and checks): y = S x;  S x = rhs by the batch's CG (current preconditioner). */
ILM_API int ilm_batch_schur_apply(ilm_batch_t b, const double* x, double* y, ilm_stream_t stream);
ILM_API int ilm_batch_schur_solve(ilm_batch_t b, const double* rhs, double* x, double tol, int maxiter,
                                  ilm_stream_t stream);

/* ---- heat conduction with Dirichlet surfaces (time marching) -------------
 * dT/dt = kappa L T + R sigma - kappa D_s[T_b+ - T_b-],  E T = (T_b+ + T_b-)/2
 * on Nodes{Primal}, advanced by IF-HERK (Liska-Colonius scheme A) with the
 * exact lattice integrating factor.  Replaces the DirichletHeatConduction
 * problem of test/literate/heatconduction.jl:87-189 driven by
 * ConstrainedSystems' LiskaIFHERK (src/timemarching.jl:4,254-277).
 * The cache must be a scalar GridScaling cache; bodies must stay at least
 * the heat-kernel radius plus two cells away from the grid edge.  The stage
 * Schur complements E exp(tau kappa L) R are assembled once here as sparse
 * matrices; each step warm-starts the stage CG solves from the last step.  */
typedef struct ilm_heat_s* ilm_heat_t;
ILM_API int ilm_heat_create(ilm_cache_t c, double kappa, double dt, const double* tb_plus, const double* tb_minus,
                            double tol, int maxiter, ilm_heat_t* out);
ILM_API int ilm_heat_destroy(ilm_heat_t h);
/* T: device Nodes{Primal} field (cache dtype), advanced in place by nsteps
 * steps of dt.  sigma_out (optional, device, cache dtype, npts): the last
 * stage's constraint force.  Returns after the work is queued on `stream`
 * and the iteration counts of the last step were read back.               */
ILM_API int ilm_heat_advance(ilm_heat_t h, void* T, void* sigma_out, int nsteps, ilm_stream_t stream);
/* CG iterations and relative residuals of the three stage solves of the last
 * step, and the nonzeros of the sparse S(tau) for tau = dt/3, 2dt/3, dt, 0. */
ILM_API int ilm_heat_info(ilm_heat_t h, int* last_iters, double* last_relres, size_t* nnz);

#ifdef __cplusplus
}
#endif

#endif /* ILM_H */
