// C ABI of libilm: grids, caches, operators and problem solves.
// Each entry point stands in for one method of ImmersedLayers.jl's operator
// API (see include/ilm.h for the citation of each).
#include <stdarg.h>
#include <string.h>

#include <algorithm>
#include <new>

#include "ilm_internal.cuh"

namespace ilm {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int gridkind_components(int kind, int* pcs) {
  switch (kind) {
    case ILM_NODES_PRIMAL: pcs[0] = PC_P; return 1;
    case ILM_NODES_DUAL: pcs[0] = PC_D; return 1;
    case ILM_EDGES_PRIMAL: pcs[0] = PC_U; pcs[1] = PC_V; return 2;
    case ILM_EDGES_DUAL: pcs[0] = PC_V; pcs[1] = PC_U; return 2;
    case ILM_EDGEGRAD_PRIMAL: pcs[0] = PC_P; pcs[1] = PC_D; pcs[2] = PC_D; pcs[3] = PC_P; return 4;
  }
  return 0;
}

size_t gridkind_numel(const ilm_grid_s* g, int kind) {
  int pcs[4];
  int n = gridkind_components(kind, pcs);
  size_t t = 0;
  for (int i = 0; i < n; ++i) t += g->shape(pcs[i]).numel();
  return t;
}

static size_t esize(int dtype) { return dtype == ILM_F64 ? 8 : 4; }

// pointer to component `comp` of a grid array of `kind`
static void* comp_ptr(const ilm_grid_s* g, int kind, int dtype, const void* base, int comp) {
  int pcs[4];
  int n = gridkind_components(kind, pcs);
  size_t off = 0;
  for (int i = 0; i < comp && i < n; ++i) off += g->shape(pcs[i]).numel();
  return (void*)((const unsigned char*)base + off * esize(dtype));
}

static void* ptr_off(const void* base, size_t elems, int dtype) {
  return (void*)((const unsigned char*)base + elems * esize(dtype));
}

static int gscr(ilm_cache_s* c, int i, void** out) {
  const size_t n = gridkind_numel(&c->grid, ILM_EDGEGRAD_PRIMAL);
  ILM_TRY(c->g_scr[i].alloc(n * esize(c->dtype)));
  *out = c->g_scr[i].p;
  return ILM_OK;
}

static int pscr(ilm_cache_s* c, int i, void** out) {
  ILM_TRY(c->p_scr[i].alloc((size_t)std::max(c->npts, 1) * 4 * sizeof(double)));
  *out = c->p_scr[i].p;
  return ILM_OK;
}

static double dscale(const ilm_cache_s* c) { return c->scaling == ILM_GRID_SCALING ? 1.0 / c->h : 1.0; }
static double lfactor(const ilm_cache_s* c) { return c->scaling == ILM_GRID_SCALING ? 1.0 / (c->h * c->h) : 1.0; }

#define CHECK_CACHE(c)                                   \
  do {                                                   \
    if (!(c)) {                                          \
      ::ilm::set_error("null cache");                    \
      return ILM_ERR_INVALID_ARG;                        \
    }                                                    \
  } while (0)

// ---- transfer building blocks ---------------------------------------------
static int scatter_scalar(ilm_cache_s* c, int pc, const void* f, int coef, void* out, cudaStream_t st) {
  return launch_scatter(c, pc, f, coef, nullptr, CF_ZERO, out, st);
}

// Edges{Primal} <- (a_u in1u + b_u in2u, a_v in1v + b_v in2v)
static int scatter_edges(ilm_cache_s* c, const void* u1, int cu1, const void* u2, int cu2, const void* v1, int cv1,
                         const void* v2, int cv2, void* out, cudaStream_t st) {
  ILM_TRY(launch_scatter(c, PC_U, u1, cu1, u2, cu2, out, st));
  void* vout = comp_ptr(&c->grid, ILM_EDGES_PRIMAL, c->dtype, out, 1);
  return launch_scatter(c, PC_V, v1, cv1, v2, cv2, vout, st);
}

static int normal_scatter_edges(ilm_cache_s* c, const void* f, void* out, cudaStream_t st) {
  return scatter_edges(c, f, CF_NX, nullptr, CF_ZERO, f, CF_NY, nullptr, CF_ZERO, out, st);
}

static int normal_cross_scatter_edges(ilm_cache_s* c, const void* f, void* out, cudaStream_t st) {
  return scatter_edges(c, f, CF_NY, nullptr, CF_ZERO, f, CF_MNX, nullptr, CF_ZERO, out, st);
}

// VectorData -> EdgeGradient with tensor n o v (symm = 0) or symmetric form (symm = 1)
static int tensor_scatter(ilm_cache_s* c, const void* v, int symm, void* out, cudaStream_t st) {
  const void* vx = v;
  const void* vy = ptr_off(v, c->npts, c->dtype);
  const ilm_grid_s* g = &c->grid;
  void* o0 = comp_ptr(g, ILM_EDGEGRAD_PRIMAL, c->dtype, out, 0);
  void* o1 = comp_ptr(g, ILM_EDGEGRAD_PRIMAL, c->dtype, out, 1);
  void* o2 = comp_ptr(g, ILM_EDGEGRAD_PRIMAL, c->dtype, out, 2);
  void* o3 = comp_ptr(g, ILM_EDGEGRAD_PRIMAL, c->dtype, out, 3);
  if (!symm) {  // dudx = n_x v_x, dudy = n_y v_x, dvdx = n_x v_y, dvdy = n_y v_y
    ILM_TRY(launch_scatter(c, PC_P, vx, CF_NX, nullptr, CF_ZERO, o0, st));
    ILM_TRY(launch_scatter(c, PC_D, vx, CF_NY, nullptr, CF_ZERO, o1, st));
    ILM_TRY(launch_scatter(c, PC_D, vy, CF_NX, nullptr, CF_ZERO, o2, st));
    ILM_TRY(launch_scatter(c, PC_P, vy, CF_NY, nullptr, CF_ZERO, o3, st));
  } else {
    ILM_TRY(launch_scatter(c, PC_P, vx, CF_NX, vy, CF_MNY, o0, st));
    ILM_TRY(launch_scatter(c, PC_D, vx, CF_NY, vy, CF_NX, o1, st));
    ILM_TRY(launch_scatter(c, PC_D, vx, CF_NY, vy, CF_NX, o2, st));
    ILM_TRY(launch_scatter(c, PC_P, vx, CF_MNX, vy, CF_NY, o3, st));
  }
  return ILM_OK;
}

// n . E(q) for q Edges{Primal}  -> scalar
static int normal_gather_edges(ilm_cache_s* c, const void* q, void* out, double scale, cudaStream_t st) {
  GatherTerm t[2] = {{PC_U, q, CF_NX}, {PC_V, comp_ptr(&c->grid, ILM_EDGES_PRIMAL, c->dtype, q, 1), CF_NY}};
  return launch_gather(c, t, 2, out, false, scale, st);
}

static int normal_cross_gather_edges(ilm_cache_s* c, const void* q, void* out, double scale, cudaStream_t st) {
  GatherTerm t[2] = {{PC_V, comp_ptr(&c->grid, ILM_EDGES_PRIMAL, c->dtype, q, 1), CF_NX}, {PC_U, q, CF_MNY}};
  return launch_gather(c, t, 2, out, false, scale, st);
}

// n . E_t(A) (symm = 0) or n . E_t(A + A^T - tr A I) (symm = 1) -> VectorData
static int tensor_gather(ilm_cache_s* c, const void* A, int symm, void* out, double scale, cudaStream_t st) {
  const ilm_grid_s* g = &c->grid;
  const void* dudx = comp_ptr(g, ILM_EDGEGRAD_PRIMAL, c->dtype, A, 0);
  const void* dudy = comp_ptr(g, ILM_EDGEGRAD_PRIMAL, c->dtype, A, 1);
  const void* dvdx = comp_ptr(g, ILM_EDGEGRAD_PRIMAL, c->dtype, A, 2);
  const void* dvdy = comp_ptr(g, ILM_EDGEGRAD_PRIMAL, c->dtype, A, 3);
  void* ox = out;
  void* oy = ptr_off(out, c->npts, c->dtype);
  if (!symm) {  // (n_x dudx + n_y dudy, n_x dvdx + n_y dvdy)
    GatherTerm tx[2] = {{PC_P, dudx, CF_NX}, {PC_D, dudy, CF_NY}};
    GatherTerm ty[2] = {{PC_D, dvdx, CF_NX}, {PC_P, dvdy, CF_NY}};
    ILM_TRY(launch_gather(c, tx, 2, ox, false, scale, st));
    return launch_gather(c, ty, 2, oy, false, scale, st);
  }
  GatherTerm tx[4] = {{PC_P, dudx, CF_NX}, {PC_P, dvdy, CF_MNX}, {PC_D, dudy, CF_NY}, {PC_D, dvdx, CF_NY}};
  GatherTerm ty[4] = {{PC_D, dudy, CF_NX}, {PC_D, dvdx, CF_NX}, {PC_P, dvdy, CF_NY}, {PC_P, dudx, CF_MNY}};
  ILM_TRY(launch_gather(c, tx, 4, ox, false, scale, st));
  return launch_gather(c, ty, 4, oy, false, scale, st);
}

static int conv_for(ilm_cache_s* c, int pc, ConvPlan** plan, cudaStream_t st) {
  if (!c->conv_ready[pc]) {
    const Shape2 sh = c->grid.shape(pc);
    ILM_TRY(conv_plan_init(&c->conv[pc], sh.n1, sh.n2, c->dtype, st));
    c->conv_ready[pc] = true;
  }
  *plan = &c->conv[pc];
  return ILM_OK;
}

static int inverse_laplacian_kind(ilm_cache_s* c, int kind, const void* in, void* out, cudaStream_t st) {
  int pcs[4];
  const int n = gridkind_components(kind, pcs);
  if (n == 0) {
    set_error("inverse_laplacian: bad grid kind %d", kind);
    return ILM_ERR_INVALID_ARG;
  }
  for (int i = 0; i < n; ++i) {
    ConvPlan* plan = nullptr;
    ILM_TRY(conv_for(c, pcs[i], &plan, st));
    ILM_TRY(conv_apply(plan, comp_ptr(&c->grid, kind, c->dtype, in, i), comp_ptr(&c->grid, kind, c->dtype, out, i),
                       1.0 / lfactor(c), st));
  }
  return ILM_OK;
}

}  // namespace ilm

namespace ilm {
// x <- x / d (0 where d = 0): the W^-1 of the surface filter
template <typename T>
__global__ void k_div_rows(int n, const T* __restrict__ d, const T* x, T* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = d[k] != (T)0 ? x[k] / d[k] : (T)0;
}
// Schur builds by columns: e = unit vector, y = the operator chain of e
template <typename T>
__global__ void k_unit_col(int n, int col, T* __restrict__ e) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) e[k] = k == col ? (T)1 : (T)0;
}
template <typename T>
__global__ void k_store_col(int n, const T* __restrict__ y, double s, double* __restrict__ A) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) A[k] = s * (double)y[k];
}
}  // namespace ilm

using namespace ilm;

extern "C" {

int ilm_version(void) { return 10000; }

const char* ilm_status_string(int s) {
  switch (s) {
    case ILM_OK: return "ok";
    case ILM_ERR_INVALID_ARG: return "invalid argument";
    case ILM_ERR_CUDA: return "CUDA error";
    case ILM_ERR_NO_MEMORY: return "out of device memory";
    case ILM_ERR_NOT_CONVERGED: return "iterative solve did not converge";
    case ILM_ERR_TIMEOUT: return "timeout";
    case ILM_ERR_UNSUPPORTED: return "unsupported";
    case ILM_ERR_SIZE_LIMIT: return "size limit exceeded";
  }
  return "unknown status";
}

const char* ilm_last_error(void) { return g_err; }

int ilm_grid_create(int nx, int ny, double h, int i0x, int i0y, ilm_grid_t* out) {
  ILM_REQUIRE(out, "null output");
  ILM_REQUIRE(nx >= 4 && ny >= 4, "grid needs at least 4x4 dual nodes (got %d x %d)", nx, ny);
  ILM_REQUIRE(nx <= 16384 && ny <= 16384, "grid too large (%d x %d)", nx, ny);
  ILM_REQUIRE(h > 0.0, "cell size must be positive");
  auto* g = new (std::nothrow) ilm_grid_s{nx, ny, h, i0x, i0y};
  if (!g) return ILM_ERR_NO_MEMORY;
  *out = g;
  return ILM_OK;
}

int ilm_grid_destroy(ilm_grid_t g) {
  delete g;
  return ILM_OK;
}

int ilm_grid_numel(ilm_grid_t g, int kind, size_t* numel) {
  ILM_REQUIRE(g && numel, "null argument");
  size_t n = gridkind_numel(g, kind);
  ILM_REQUIRE(n > 0, "bad grid kind %d", kind);
  *numel = n;
  return ILM_OK;
}

int ilm_alloc(size_t nbytes, void** out) {
  ILM_REQUIRE(out, "alloc: null argument");
  *out = nullptr;
  if (nbytes == 0) return ILM_OK;
  const cudaError_t e = cudaMalloc(out, nbytes);
  if (e != cudaSuccess) {
    *out = nullptr;
    set_error("alloc: cudaMalloc(%zu) failed: %s", nbytes, cudaGetErrorString(e));
    return ILM_ERR_NO_MEMORY;
  }
  return ILM_OK;
}

int ilm_free(void* p) {
  if (p) ILM_CHECK_CUDA(cudaFree(p));
  return ILM_OK;
}

int ilm_copy_h2d(void* dst_dev, const void* src_host, size_t nbytes, ilm_stream_t stream) {
  ILM_REQUIRE(nbytes == 0 || (dst_dev && src_host), "copy_h2d: null argument");
  if (nbytes) ILM_CHECK_CUDA(cudaMemcpyAsync(dst_dev, src_host, nbytes, cudaMemcpyHostToDevice, as_stream(stream)));
  return ILM_OK;
}

int ilm_copy_d2h(void* dst_host, const void* src_dev, size_t nbytes, ilm_stream_t stream) {
  ILM_REQUIRE(nbytes == 0 || (dst_host && src_dev), "copy_d2h: null argument");
  if (!nbytes) return ILM_OK;
  ILM_CHECK_CUDA(cudaMemcpyAsync(dst_host, src_dev, nbytes, cudaMemcpyDeviceToHost, as_stream(stream)));
  ILM_CHECK_CUDA(cudaStreamSynchronize(as_stream(stream)));
  return ILM_OK;
}

int ilm_cache_create(ilm_grid_t g, int kind, int npts, const double* x, const double* y, const double* nrmx,
                     const double* nrmy, const double* ds, int ddf, int scaling, int dtype, ilm_cache_t* out) {
  ILM_REQUIRE(g && out, "null argument");
  ILM_REQUIRE(kind == ILM_CACHE_SCALAR || kind == ILM_CACHE_VECTOR, "bad cache kind %d", kind);
  ILM_REQUIRE(npts >= 0, "negative number of points");
  ILM_REQUIRE(npts == 0 || (x && y && nrmx && nrmy && ds), "null point arrays");
  ILM_REQUIRE(ddf >= ILM_DDF_YANG3 && ddf <= ILM_DDF_M3, "bad ddf %d", ddf);
  ILM_REQUIRE(scaling == ILM_GRID_SCALING || scaling == ILM_INDEX_SCALING, "bad scaling %d", scaling);
  ILM_REQUIRE(dtype == ILM_F64 || dtype == ILM_F32, "bad dtype %d", dtype);
  for (int k = 0; k < npts; ++k) {
    ILM_REQUIRE(isfinite(x[k]) && isfinite(y[k]) && isfinite(nrmx[k]) && isfinite(nrmy[k]) && isfinite(ds[k]),
                "non-finite point data at index %d", k);
  }
  auto* c = new (std::nothrow) ilm_cache_s();
  if (!c) return ILM_ERR_NO_MEMORY;
  c->grid = *g;
  c->kind = kind;
  c->npts = npts;
  c->ddf = ddf;
  c->scaling = scaling;
  c->dtype = dtype;
  c->h = g->h;
  c->hx.assign(x, x + npts);
  c->hy.assign(y, y + npts);
  c->hnx.assign(nrmx, nrmx + npts);
  c->hny.assign(nrmy, nrmy + npts);
  c->hds.assign(ds, ds + npts);
  int st = ILM_OK;
  auto up = [&](DevBuf& b, const std::vector<double>& v, int dt) -> int {
    ILM_TRY(b.alloc(std::max<size_t>(v.size(), 1) * esize(dt)));
    if (v.empty()) return ILM_OK;
    if (dt == ILM_F64) {
      ILM_CHECK_CUDA(cudaMemcpy(b.p, v.data(), v.size() * 8, cudaMemcpyHostToDevice));
    } else {
      std::vector<float> f(v.begin(), v.end());
      ILM_CHECK_CUDA(cudaMemcpy(b.p, f.data(), f.size() * 4, cudaMemcpyHostToDevice));
    }
    return ILM_OK;
  };
  std::vector<double> wsc(npts);
  for (int k = 0; k < npts; ++k) wsc[k] = scaling == ILM_GRID_SCALING ? ds[k] / (g->h * g->h) : 1.0;
  if ((st = up(c->nx, c->hnx, dtype)) || (st = up(c->ny, c->hny, dtype)) || (st = up(c->wscale, wsc, dtype)) ||
      (st = up(c->ds64, c->hds, ILM_F64)) || (st = up(c->nx64, c->hnx, ILM_F64)) ||
      (st = up(c->ny64, c->hny, ILM_F64)) || (st = cache_build_windows(c)) ||
      (st = c->red.alloc((size_t)(std::max(g->nx, g->ny) + 8) * sizeof(double)))) {
    delete c;
    return st;
  }
  *out = c;
  return ILM_OK;
}

int ilm_cache_update_points(ilm_cache_t c, const double* x, const double* y, const double* nrmx, const double* nrmy,
                            const double* ds, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(c->npts == 0 || (x && y && nrmx && nrmy && ds), "cache_update_points: null point array");
  delete c->twin;  // the FP64 refinement cache holds the old points
  c->twin = nullptr;
  return cache_rebin_points(c, x, y, nrmx, nrmy, ds, as_stream(stream));
}

int ilm_cache_destroy(ilm_cache_t c) {
  delete c;
  return ILM_OK;
}

int ilm_cache_npts(ilm_cache_t c, int* npts) {
  ILM_REQUIRE(c && npts, "null argument");
  *npts = c->npts;
  return ILM_OK;
}

// ---- transfers -----------------------------------------------------------
int ilm_regularize(ilm_cache_t c, int out_kind, const void* f, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  switch (out_kind) {
    case ILM_NODES_PRIMAL: return scatter_scalar(c, PC_P, f, CF_ONE, out, st);
    case ILM_NODES_DUAL: return scatter_scalar(c, PC_D, f, CF_ONE, out, st);
    case ILM_EDGES_PRIMAL:
      return scatter_edges(c, f, CF_ONE, nullptr, CF_ZERO, ptr_off(f, c->npts, c->dtype), CF_ONE, nullptr, CF_ZERO,
                           out, st);
  }
  set_error("regularize: unsupported output kind %d", out_kind);
  return ILM_ERR_INVALID_ARG;
}

int ilm_regularize_add(ilm_cache_t c, int out_kind, const void* f, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  switch (out_kind) {
    case ILM_NODES_PRIMAL: return launch_scatter(c, PC_P, f, CF_ONE, nullptr, CF_ZERO, out, st, true);
    case ILM_NODES_DUAL: return launch_scatter(c, PC_D, f, CF_ONE, nullptr, CF_ZERO, out, st, true);
    case ILM_EDGES_PRIMAL: {
      ILM_TRY(launch_scatter(c, PC_U, f, CF_ONE, nullptr, CF_ZERO, out, st, true));
      void* vout = comp_ptr(&c->grid, ILM_EDGES_PRIMAL, c->dtype, out, 1);
      return launch_scatter(c, PC_V, ptr_off(f, c->npts, c->dtype), CF_ONE, nullptr, CF_ZERO, vout, st, true);
    }
  }
  set_error("regularize_add: unsupported output kind %d", out_kind);
  return ILM_ERR_INVALID_ARG;
}

int ilm_grid_mul_add(size_t n, int dtype, const void* a, const void* b, void* out, ilm_stream_t stream) {
  ILM_REQUIRE(dtype == ILM_F64 || dtype == ILM_F32, "grid_mul_add: bad dtype %d", dtype);
  ILM_REQUIRE(n == 0 || (a && b && out), "grid_mul_add: null argument");
  return st_mul_add(n, dtype, a, b, out, as_stream(stream));
}

int ilm_interpolate(ilm_cache_t c, int in_kind, const void* s, void* f, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  switch (in_kind) {
    case ILM_NODES_PRIMAL: {
      GatherTerm t{PC_P, s, CF_ONE};
      return launch_gather(c, &t, 1, f, false, 1.0, st);
    }
    case ILM_NODES_DUAL: {
      GatherTerm t{PC_D, s, CF_ONE};
      return launch_gather(c, &t, 1, f, false, 1.0, st);
    }
    case ILM_EDGES_PRIMAL: {
      GatherTerm tu{PC_U, s, CF_ONE};
      GatherTerm tv{PC_V, comp_ptr(&c->grid, ILM_EDGES_PRIMAL, c->dtype, s, 1), CF_ONE};
      ILM_TRY(launch_gather(c, &tu, 1, f, false, 1.0, st));
      return launch_gather(c, &tv, 1, ptr_off(f, c->npts, c->dtype), false, 1.0, st);
    }
  }
  set_error("interpolate: unsupported input kind %d", in_kind);
  return ILM_ERR_INVALID_ARG;
}

int ilm_surface_filter(ilm_cache_t c, int power, const void* s_in, void* s_out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(power >= 0, "surface_filter: negative power %d", power);
  ILM_REQUIRE(c->npts == 0 || (s_in && s_out), "surface_filter: null argument");
  cudaStream_t st = as_stream(stream);
  const int gk = c->kind == ILM_CACHE_SCALAR ? ILM_NODES_PRIMAL : ILM_EDGES_PRIMAL;
  const size_t n = (size_t)c->npts * (c->kind == ILM_CACHE_SCALAR ? 1 : 2);
  const size_t es = esize(c->dtype);
  if (n == 0) return ILM_OK;
  if (power == 0) {
    if (s_out != s_in) ILM_CHECK_CUDA(cudaMemcpyAsync(s_out, s_in, n * es, cudaMemcpyDeviceToDevice, st));
    return ILM_OK;
  }
  ILM_TRY(c->filt_grid.alloc(gridkind_numel(&c->grid, gk) * es));
  if (!c->filt_ready) {
    // W = E R 1
    ILM_TRY(c->filt_diag.alloc(n * es));
    ILM_TRY(st_fill(n, c->dtype, 1.0, c->filt_diag.p, st));
    ILM_TRY(ilm_regularize(c, gk, c->filt_diag.p, c->filt_grid.p, stream));
    ILM_TRY(ilm_interpolate(c, gk, c->filt_grid.p, c->filt_diag.p, stream));
    c->filt_ready = true;
  }
  const void* src = s_in;
  for (int k = 0; k < power; ++k) {
    ILM_TRY(ilm_regularize(c, gk, src, c->filt_grid.p, stream));
    ILM_TRY(ilm_interpolate(c, gk, c->filt_grid.p, s_out, stream));
    const int nb = (int)((n + 255) / 256);
    if (c->dtype == ILM_F64)
      k_div_rows<double><<<nb, 256, 0, st>>>((int)n, c->filt_diag.as<double>(), static_cast<const double*>(s_out),
                                            static_cast<double*>(s_out));
    else
      k_div_rows<float><<<nb, 256, 0, st>>>((int)n, c->filt_diag.as<float>(), static_cast<const float*>(s_out),
                                           static_cast<float*>(s_out));
    ILM_CHECK_LAUNCH();
    src = s_out;
  }
  return ILM_OK;
}

int ilm_regularize_normal(ilm_cache_t c, const void* f, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  if (c->kind == ILM_CACHE_SCALAR) return normal_scatter_edges(c, f, out, as_stream(stream));
  return tensor_scatter(c, f, 0, out, as_stream(stream));
}

int ilm_regularize_normal_symm(ilm_cache_t c, const void* v, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(c->kind == ILM_CACHE_VECTOR, "regularize_normal_symm needs a vector cache");
  return tensor_scatter(c, v, 1, out, as_stream(stream));
}

int ilm_regularize_normal_cross(ilm_cache_t c, int out_kind, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  if (out_kind == ILM_EDGES_PRIMAL) return normal_cross_scatter_edges(c, in, out, st);
  if (out_kind == ILM_NODES_DUAL)
    return launch_scatter(c, PC_D, in, CF_MNY, ptr_off(in, c->npts, c->dtype), CF_NX, out, st);
  set_error("regularize_normal_cross: unsupported output kind %d", out_kind);
  return ILM_ERR_INVALID_ARG;
}

int ilm_regularize_normal_dot(ilm_cache_t c, int out_kind, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  const int N = c->npts;
  if (out_kind == ILM_NODES_PRIMAL)
    return launch_scatter(c, PC_P, in, CF_NX, ptr_off(in, N, c->dtype), CF_NY, out, st);
  if (out_kind == ILM_EDGES_PRIMAL) {
    const void* t11 = in;
    const void* t12 = ptr_off(in, N, c->dtype);
    const void* t21 = ptr_off(in, 2 * (size_t)N, c->dtype);
    const void* t22 = ptr_off(in, 3 * (size_t)N, c->dtype);
    // u = n_x dudx + n_y dudy, v = n_x dvdx + n_y dvdy
    return scatter_edges(c, t11, CF_NX, t12, CF_NY, t21, CF_NX, t22, CF_NY, out, st);
  }
  set_error("regularize_normal_dot: unsupported output kind %d", out_kind);
  return ILM_ERR_INVALID_ARG;
}

int ilm_normal_interpolate(ilm_cache_t c, const void* q, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  if (c->kind == ILM_CACHE_SCALAR) return normal_gather_edges(c, q, out, 1.0, as_stream(stream));
  return tensor_gather(c, q, 0, out, 1.0, as_stream(stream));
}

int ilm_normal_interpolate_symm(ilm_cache_t c, const void* q, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(c->kind == ILM_CACHE_VECTOR, "normal_interpolate_symm needs a vector cache");
  return tensor_gather(c, q, 1, out, 1.0, as_stream(stream));
}

int ilm_normal_cross_interpolate(ilm_cache_t c, int in_kind, const void* q, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  if (in_kind == ILM_EDGES_PRIMAL) return normal_cross_gather_edges(c, q, out, 1.0, st);
  if (in_kind == ILM_NODES_DUAL) {
    GatherTerm tx{PC_D, q, CF_NY};
    GatherTerm ty{PC_D, q, CF_MNX};
    ILM_TRY(launch_gather(c, &tx, 1, out, false, 1.0, st));
    return launch_gather(c, &ty, 1, ptr_off(out, c->npts, c->dtype), false, 1.0, st);
  }
  set_error("normal_cross_interpolate: unsupported input kind %d", in_kind);
  return ILM_ERR_INVALID_ARG;
}

int ilm_normal_dot_interpolate(ilm_cache_t c, int in_kind, const void* q, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  const int N = c->npts;
  if (in_kind == ILM_NODES_PRIMAL) {
    GatherTerm tx{PC_P, q, CF_NX};
    GatherTerm ty{PC_P, q, CF_NY};
    ILM_TRY(launch_gather(c, &tx, 1, out, false, 1.0, st));
    return launch_gather(c, &ty, 1, ptr_off(out, N, c->dtype), false, 1.0, st);
  }
  if (in_kind == ILM_EDGES_PRIMAL) {
    const void* u = q;
    const void* v = comp_ptr(&c->grid, ILM_EDGES_PRIMAL, c->dtype, q, 1);
    // (dudx, dudy, dvdx, dvdy) = (n_x s_x, n_y s_x, n_x s_y, n_y s_y), s = E v
    GatherTerm t[4] = {{PC_U, u, CF_NX}, {PC_U, u, CF_NY}, {PC_V, v, CF_NX}, {PC_V, v, CF_NY}};
    for (int i = 0; i < 4; ++i) ILM_TRY(launch_gather(c, &t[i], 1, ptr_off(out, (size_t)i * N, c->dtype), false, 1.0, st));
    return ILM_OK;
  }
  set_error("normal_dot_interpolate: unsupported input kind %d", in_kind);
  return ILM_ERR_INVALID_ARG;
}

// ---- composite layer operators --------------------------------------------
int ilm_surface_divergence(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  void* q;
  ILM_TRY(gscr(c, 0, &q));
  if (c->kind == ILM_CACHE_SCALAR) {
    ILM_TRY(normal_scatter_edges(c, in, q, st));
    return st_div_edges(&c->grid, c->dtype, q, out, dscale(c), st);
  }
  ILM_TRY(tensor_scatter(c, in, 0, q, st));
  return st_div_edgegrad(&c->grid, c->dtype, q, out, dscale(c), st);
}

int ilm_surface_divergence_symm(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(c->kind == ILM_CACHE_VECTOR, "surface_divergence_symm needs a vector cache");
  cudaStream_t st = as_stream(stream);
  void* q;
  ILM_TRY(gscr(c, 0, &q));
  ILM_TRY(tensor_scatter(c, in, 1, q, st));
  return st_div_edgegrad(&c->grid, c->dtype, q, out, dscale(c), st);
}

int ilm_surface_grad(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  void* q;
  ILM_TRY(gscr(c, 0, &q));
  if (c->kind == ILM_CACHE_SCALAR) {
    ILM_TRY(st_grad_nodes(&c->grid, c->dtype, in, q, 1.0, st));
    return normal_gather_edges(c, q, out, dscale(c), st);
  }
  ILM_TRY(st_grad_edges(&c->grid, c->dtype, in, q, 1.0, st));
  return tensor_gather(c, q, 0, out, dscale(c), st);
}

int ilm_surface_grad_symm(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(c->kind == ILM_CACHE_VECTOR, "surface_grad_symm needs a vector cache");
  cudaStream_t st = as_stream(stream);
  void* q;
  ILM_TRY(gscr(c, 0, &q));
  ILM_TRY(st_grad_edges(&c->grid, c->dtype, in, q, 1.0, st));
  return tensor_gather(c, q, 1, out, dscale(c), st);
}

int ilm_surface_curl(ilm_cache_t c, int direction, int point_kind, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  void* q;
  ILM_TRY(gscr(c, 0, &q));
  if (direction == 0) {
    if (point_kind == ILM_SCALAR_DATA) ILM_TRY(normal_scatter_edges(c, in, q, st));
    else if (point_kind == ILM_VECTOR_DATA)
      ILM_TRY(scatter_edges(c, in, CF_ONE, nullptr, CF_ZERO, ptr_off(in, c->npts, c->dtype), CF_ONE, nullptr,
                            CF_ZERO, q, st));
    else {
      set_error("surface_curl: bad point kind %d", point_kind);
      return ILM_ERR_INVALID_ARG;
    }
    return st_curl_edges_to_dual(&c->grid, c->dtype, q, out, dscale(c), st);
  }
  ILM_TRY(st_curl_dual_to_edges(&c->grid, c->dtype, in, q, 1.0, st));
  if (point_kind == ILM_SCALAR_DATA) return normal_gather_edges(c, q, out, dscale(c), st);
  if (point_kind == ILM_VECTOR_DATA) {
    GatherTerm tu{PC_U, q, CF_ONE};
    GatherTerm tv{PC_V, comp_ptr(&c->grid, ILM_EDGES_PRIMAL, c->dtype, q, 1), CF_ONE};
    ILM_TRY(launch_gather(c, &tu, 1, out, false, dscale(c), st));
    return launch_gather(c, &tv, 1, ptr_off(out, c->npts, c->dtype), false, dscale(c), st);
  }
  set_error("surface_curl: bad point kind %d", point_kind);
  return ILM_ERR_INVALID_ARG;
}

int ilm_surface_curl_cross(ilm_cache_t c, int direction, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  void* q;
  ILM_TRY(gscr(c, 0, &q));
  if (direction == 0) {
    ILM_TRY(normal_cross_scatter_edges(c, in, q, st));
    return st_curl_edges_to_dual(&c->grid, c->dtype, q, out, dscale(c), st);
  }
  ILM_TRY(st_curl_dual_to_edges(&c->grid, c->dtype, in, q, 1.0, st));
  return normal_cross_gather_edges(c, q, out, dscale(c), st);
}

int ilm_surface_divergence_cross(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  void* q;
  ILM_TRY(gscr(c, 0, &q));
  ILM_TRY(normal_cross_scatter_edges(c, in, q, st));
  return st_div_edges(&c->grid, c->dtype, q, out, dscale(c), st);
}

int ilm_surface_grad_cross(ilm_cache_t c, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  cudaStream_t st = as_stream(stream);
  void* q;
  ILM_TRY(gscr(c, 0, &q));
  ILM_TRY(st_grad_nodes(&c->grid, c->dtype, in, q, 1.0, st));
  return normal_cross_gather_edges(c, q, out, dscale(c), st);
}

// ---- grid operators -------------------------------------------------------
int ilm_divergence(ilm_cache_t c, int in_kind, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  if (in_kind == ILM_EDGES_PRIMAL) return st_div_edges(&c->grid, c->dtype, in, out, dscale(c), as_stream(stream));
  if (in_kind == ILM_EDGEGRAD_PRIMAL)
    return st_div_edgegrad(&c->grid, c->dtype, in, out, dscale(c), as_stream(stream));
  set_error("divergence: unsupported input kind %d", in_kind);
  return ILM_ERR_INVALID_ARG;
}

int ilm_grad(ilm_cache_t c, int in_kind, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  if (in_kind == ILM_NODES_PRIMAL) return st_grad_nodes(&c->grid, c->dtype, in, out, dscale(c), as_stream(stream));
  if (in_kind == ILM_EDGES_PRIMAL) return st_grad_edges(&c->grid, c->dtype, in, out, dscale(c), as_stream(stream));
  set_error("grad: unsupported input kind %d", in_kind);
  return ILM_ERR_INVALID_ARG;
}

int ilm_curl(ilm_cache_t c, int in_kind, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  if (in_kind == ILM_NODES_DUAL)
    return st_curl_dual_to_edges(&c->grid, c->dtype, in, out, dscale(c), as_stream(stream));
  if (in_kind == ILM_EDGES_PRIMAL)
    return st_curl_edges_to_dual(&c->grid, c->dtype, in, out, dscale(c), as_stream(stream));
  set_error("curl: unsupported input kind %d", in_kind);
  return ILM_ERR_INVALID_ARG;
}

int ilm_convective_derivative(ilm_cache_t c, int field_kind, const void* v, const void* q, void* out,
                              ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(v && q && out, "convective_derivative: null argument");
  ILM_REQUIRE(field_kind == ILM_NODES_PRIMAL || field_kind == ILM_NODES_DUAL || field_kind == ILM_EDGES_PRIMAL,
              "convective_derivative: unsupported field kind %d", field_kind);
  ILM_REQUIRE(out != v && out != q, "convective_derivative: out must not alias an input");
  return st_convective(&c->grid, c->dtype, field_kind, v, q, out, dscale(c), as_stream(stream));
}

int ilm_w_cross_v(ilm_cache_t c, const void* w, const void* v, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(w && v && out, "w_cross_v: null argument");
  ILM_REQUIRE(out != v, "w_cross_v: out must not alias v");
  return st_w_cross_v(&c->grid, c->dtype, w, v, out, as_stream(stream));
}

int ilm_vecfield_helmholtz(ilm_cache_t c, const void* curlv, const void* divv, const void* dv, const void* vp,
                           const double* uniform, void* v_out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(c->kind == ILM_CACHE_VECTOR, "vecfield_helmholtz needs a vector cache");
  ILM_REQUIRE(curlv && divv && v_out, "vecfield_helmholtz: null argument");
  ILM_REQUIRE(c->npts == 0 || dv, "vecfield_helmholtz: null surface jump");
  cudaStream_t st = as_stream(stream);
  const int dt = c->dtype;
  const size_t nd = c->grid.shape(PC_D).numel(), np = c->grid.shape(PC_P).numel();
  const size_t ne = gridkind_numel(&c->grid, ILM_EDGES_PRIMAL), neu = c->grid.shape(PC_U).numel();
  void *bd, *bp, *ge;
  ILM_TRY(gscr(c, 2, &bd));
  ILM_TRY(gscr(c, 5, &bp));
  ILM_TRY(gscr(c, 0, &ge));
  void* psi = ptr_off(bd, nd, dt);
  void* phi = ptr_off(bp, np, dt);
  // L psi' = curlv + R_n n x [v];  psi = -psi'  (src/helmholtz.jl:85-100,117-120)
  if (c->npts > 0) {
    ILM_TRY(ilm_regularize_normal_cross(c, ILM_NODES_DUAL, dv, bd, stream));
    ILM_TRY(st_axpby(nd, dt, 1.0, curlv, 1.0, bd, bd, st));
  } else {
    ILM_CHECK_CUDA(cudaMemcpyAsync(bd, curlv, nd * esize(dt), cudaMemcpyDeviceToDevice, st));
  }
  ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_DUAL, bd, psi, st));
  // L phi = divv + R_c n . [v]  (:196-207,227-231)
  if (c->npts > 0) {
    ILM_TRY(ilm_regularize_normal_dot(c, ILM_NODES_PRIMAL, dv, bp, stream));
    ILM_TRY(st_axpby(np, dt, 1.0, divv, 1.0, bp, bp, st));
  } else {
    ILM_CHECK_CUDA(cudaMemcpyAsync(bp, divv, np * esize(dt), cudaMemcpyDeviceToDevice, st));
  }
  ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_PRIMAL, bp, phi, st));
  // v = curl psi + grad phi + v_p  (:327-344)
  ILM_TRY(st_curl_dual_to_edges(&c->grid, dt, psi, v_out, dscale(c), st));
  ILM_TRY(st_grad_nodes(&c->grid, dt, phi, ge, dscale(c), st));
  ILM_TRY(st_axpby(ne, dt, -1.0, v_out, 1.0, ge, v_out, st));
  if (vp) ILM_TRY(st_axpby(ne, dt, 1.0, vp, 1.0, v_out, v_out, st));
  if (uniform) {
    if (uniform[0] != 0.0) ILM_TRY(st_affine(neu, dt, 1.0, v_out, uniform[0], v_out, st));
    if (uniform[1] != 0.0) ILM_TRY(st_affine(ne - neu, dt, 1.0, ptr_off(v_out, neu, dt), uniform[1],
                                             ptr_off(v_out, neu, dt), st));
  }
  return ILM_OK;
}

int ilm_laplacian(ilm_cache_t c, int kind, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  int pcs[4];
  const int n = gridkind_components(kind, pcs);
  ILM_REQUIRE(n > 0, "laplacian: bad grid kind %d", kind);
  for (int i = 0; i < n; ++i) {
    const Shape2 sh = c->grid.shape(pcs[i]);
    ILM_TRY(st_laplacian(sh.n1, sh.n2, c->dtype, comp_ptr(&c->grid, kind, c->dtype, in, i),
                         comp_ptr(&c->grid, kind, c->dtype, out, i), lfactor(c), as_stream(stream)));
  }
  return ILM_OK;
}

int ilm_inverse_laplacian(ilm_cache_t c, int kind, const void* in, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  return inverse_laplacian_kind(c, kind, in, out, as_stream(stream));
}

// Vector caches (src/surface_operators.jl:872-877, :912-923): the mask on
// Edges{Primal} from the all-ones VectorData, H = -L^{-1} D_s 1, and for the
// other grid types its u component interpolated (Nodes{Dual}: mean over y;
// Nodes{Primal}: mean over x; EdgeGradient per component).
static int mask_vector(ilm_cache_s* c, int kind, int complementary, void* out, cudaStream_t st) {
  ILM_REQUIRE(kind == ILM_NODES_PRIMAL || kind == ILM_NODES_DUAL || kind == ILM_EDGES_PRIMAL ||
                  kind == ILM_EDGEGRAD_PRIMAL,
              "mask: unsupported grid kind %d", kind);
  const size_t ne = gridkind_numel(&c->grid, ILM_EDGES_PRIMAL);
  void* m;
  ILM_TRY(gscr(c, 1, &m));
  if (c->npts == 0) {
    ILM_TRY(st_fill(ne, c->dtype, 1.0, m, st));
  } else {
    void* ones;
    ILM_TRY(pscr(c, 0, &ones));
    ILM_TRY(st_fill(2 * (size_t)c->npts, c->dtype, 1.0, ones, st));
    ILM_TRY(ilm_surface_divergence(c, ones, m, (void*)st));
    ILM_TRY(inverse_laplacian_kind(c, ILM_EDGES_PRIMAL, m, m, st));
    ILM_TRY(st_affine(ne, c->dtype, -1.0, m, 0.0, m, st));
  }
  if (complementary) ILM_TRY(st_affine(ne, c->dtype, -1.0, m, 1.0, m, st));
  switch (kind) {
    case ILM_EDGES_PRIMAL: return st_convert(ne, c->dtype, m, c->dtype, out, st);
    case ILM_NODES_DUAL: return st_xedge_to_dual(&c->grid, c->dtype, m, out, st);
    case ILM_NODES_PRIMAL: return st_xedge_to_primal(&c->grid, c->dtype, m, out, st);
    default:  // EdgeGradient: dudx, dvdy on Nodes{Primal}, dudy, dvdx on Nodes{Dual}
      for (int k = 0; k < 4; ++k) {
        void* o = comp_ptr(&c->grid, ILM_EDGEGRAD_PRIMAL, c->dtype, out, k);
        if (k == 0 || k == 3) ILM_TRY(st_xedge_to_primal(&c->grid, c->dtype, m, o, st));
        else ILM_TRY(st_xedge_to_dual(&c->grid, c->dtype, m, o, st));
      }
      return ILM_OK;
  }
}

int ilm_mask(ilm_cache_t c, int kind, int complementary, void* out, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(c->scaling == ILM_GRID_SCALING, "mask: GridScaling caches only (src/surface_operators.jl:737)");
  if (c->kind == ILM_CACHE_VECTOR) return mask_vector(c, kind, complementary, out, as_stream(stream));
  ILM_REQUIRE(kind == ILM_NODES_PRIMAL || kind == ILM_NODES_DUAL || kind == ILM_EDGES_PRIMAL,
              "mask: unsupported grid kind %d", kind);
  cudaStream_t st = as_stream(stream);
  const size_t np = c->grid.shape(PC_P).numel();
  void* m;
  ILM_TRY(gscr(c, 1, &m));
  if (c->npts == 0) {
    // no surface: all inside (src/surface_operators.jl:873-876)
    ILM_TRY(st_fill(np, c->dtype, 1.0, m, st));
  } else {
    // H = -L^{-1} D_s 1   (src/surface_operators.jl:865-871)
    void* ones;
    ILM_TRY(pscr(c, 0, &ones));
    ILM_TRY(st_fill(c->npts, c->dtype, 1.0, ones, st));
    ILM_TRY(ilm_surface_divergence(c, ones, m, stream));
    ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_PRIMAL, m, m, st));
    ILM_TRY(st_affine(np, c->dtype, -1.0, m, 0.0, m, st));
  }
  if (complementary) ILM_TRY(st_affine(np, c->dtype, -1.0, m, 1.0, m, st));
  if (kind == ILM_NODES_PRIMAL) return st_convert(np, c->dtype, m, c->dtype, out, st);
  if (kind == ILM_NODES_DUAL) return st_primal_to_dual(&c->grid, c->dtype, m, out, st);
  return st_primal_to_edges(&c->grid, c->dtype, m, out, st);
}

// ---- inner products ------------------------------------------------------
int ilm_dot_grid(ilm_cache_t c, int kind, const void* a, const void* b, double* result, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(result, "null result");
  cudaStream_t st = as_stream(stream);
  int pcs[4];
  const int n = gridkind_components(kind, pcs);
  ILM_REQUIRE(n > 0, "dot: bad grid kind %d", kind);
  double total = 0.0;
  for (int i = 0; i < n; ++i) {
    const Shape2 sh = c->grid.shape(pcs[i]);
    ILM_TRY(st_weighted_dot(sh.n1, sh.n2, pc_dx(pcs[i]), pc_dy(pcs[i]), c->dtype,
                            comp_ptr(&c->grid, kind, c->dtype, a, i), comp_ptr(&c->grid, kind, c->dtype, b, i),
                            c->red.as<double>(), st));
    double v = 0.0;
    ILM_CHECK_CUDA(cudaMemcpyAsync(&v, c->red.as<double>() + sh.n2, sizeof(double), cudaMemcpyDeviceToHost, st));
    ILM_CHECK_CUDA(cudaStreamSynchronize(st));
    total += v;
  }
  // GridScaling: weighted by the cell volume h^2 (src/tools.jl:101-105)
  *result = c->scaling == ILM_GRID_SCALING ? total * c->h * c->h : total;
  return ILM_OK;
}

int ilm_dot_surface(ilm_cache_t c, int ncomp, const void* a, const void* b, double* result, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(result && ncomp >= 1 && ncomp <= 4, "dot_surface: bad arguments");
  cudaStream_t st = as_stream(stream);
  double total = 0.0;
  const double* w = c->scaling == ILM_GRID_SCALING ? c->ds64.as<double>() : nullptr;
  for (int i = 0; i < ncomp; ++i) {
    ILM_TRY(st_point_dot(c->npts, c->dtype, ptr_off(a, (size_t)i * c->npts, c->dtype),
                         ptr_off(b, (size_t)i * c->npts, c->dtype), w, c->red.as<double>(), st));
    double v = 0.0;
    ILM_CHECK_CUDA(cudaMemcpyAsync(&v, c->red.as<double>(), sizeof(double), cudaMemcpyDeviceToHost, st));
    ILM_CHECK_CUDA(cudaStreamSynchronize(st));
    total += v;
  }
  *result = total;
  return ILM_OK;
}

// ---- Schur complements ----------------------------------------------------
// The reference's column-by-column build (src/matrix_operators.jl:9-244) on
// the device: one unit vector per column through the operator chain, for the
// kinds and caches the point-pair sums do not cover.
static int schur_build_columns(ilm_cache_s* c, int which, double scale, double* A, cudaStream_t st) {
  const bool vec = c->kind == ILM_CACHE_VECTOR;
  const bool scalar_data = !vec || which == ILM_SCHUR_CLINVCT_SCALAR;
  const int n = c->npts * (scalar_data ? 1 : 2);
  if (n == 0) return ILM_OK;
  void *e, *y, *g1, *g2;
  ILM_TRY(pscr(c, 1, &e));
  ILM_TRY(pscr(c, 2, &y));
  ILM_TRY(gscr(c, 2, &g1));
  ILM_TRY(gscr(c, 5, &g2));
  void* const s_ = (void*)st;
  const int gk = vec ? ILM_EDGES_PRIMAL : ILM_NODES_PRIMAL;  // the cache's grid data
  const int nb = (n + 255) / 256;
  double sign = -1.0;
  for (int col = 0; col < n; ++col) {
    if (c->dtype == ILM_F64) k_unit_col<double><<<nb, 256, 0, st>>>(n, col, static_cast<double*>(e));
    else k_unit_col<float><<<nb, 256, 0, st>>>(n, col, static_cast<float*>(e));
    ILM_CHECK_LAUNCH();
    switch (which) {
      case ILM_SCHUR_RTLINVR:  // -R^T L^-1 R
        ILM_TRY(ilm_regularize(c, gk, e, g1, s_));
        ILM_TRY(inverse_laplacian_kind(c, gk, g1, g2, st));
        ILM_TRY(ilm_interpolate(c, gk, g2, y, s_));
        break;
      case ILM_SCHUR_CLINVCT:  // -C_s L^-1 C_s^T (point data of the cache)
      case ILM_SCHUR_CLINVCT_SCALAR: {
        const int pk = scalar_data ? ILM_SCALAR_DATA : ILM_VECTOR_DATA;
        ILM_TRY(ilm_surface_curl(c, 0, pk, e, g1, s_));
        ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_DUAL, g1, g2, st));
        ILM_TRY(ilm_surface_curl(c, 1, pk, g2, y, s_));
        break;
      }
      case ILM_SCHUR_CL2INVCT:  // -C_s L^-2 C_s^T
        ILM_TRY(ilm_surface_curl(c, 0, ILM_VECTOR_DATA, e, g1, s_));
        ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_DUAL, g1, g2, st));
        ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_DUAL, g2, g1, st));
        ILM_TRY(ilm_surface_curl(c, 1, ILM_VECTOR_DATA, g1, y, s_));
        break;
      case ILM_SCHUR_GLINVD:  // -G_s L^-1 D_s
        ILM_TRY(ilm_surface_divergence(c, e, g1, s_));
        ILM_TRY(inverse_laplacian_kind(c, gk, g1, g2, st));
        ILM_TRY(ilm_surface_grad(c, g2, y, s_));
        break;
      case ILM_SCHUR_GLINVD_SYMM:
        ILM_TRY(ilm_surface_divergence_symm(c, e, g1, s_));
        ILM_TRY(inverse_laplacian_kind(c, gk, g1, g2, st));
        ILM_TRY(ilm_surface_grad_symm(c, g2, y, s_));
        break;
      case ILM_SCHUR_GLINVD_CROSS:  // -G^x_s L^-1 D^x_s (scalar caches)
        ILM_TRY(ilm_surface_divergence_cross(c, e, g1, s_));
        ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_PRIMAL, g1, g2, st));
        ILM_TRY(ilm_surface_grad_cross(c, g2, y, s_));
        break;
      case ILM_SCHUR_NRTRN:  // + n.R_f^T R_f n o (no inverse Laplacian)
        ILM_TRY(ilm_regularize_normal(c, e, g1, s_));
        ILM_TRY(ilm_normal_interpolate(c, g1, y, s_));
        sign = 1.0;
        break;
    }
    if (c->dtype == ILM_F64)
      k_store_col<double><<<nb, 256, 0, st>>>(n, static_cast<const double*>(y), sign * scale, A + (size_t)col * n);
    else
      k_store_col<float><<<nb, 256, 0, st>>>(n, static_cast<const float*>(y), sign * scale, A + (size_t)col * n);
    ILM_CHECK_LAUNCH();
  }
  return ILM_OK;
}

int ilm_schur_build(ilm_cache_t c, int which, double scale, double* A_dev, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(A_dev || c->npts == 0, "null matrix");
  ILM_REQUIRE(which >= ILM_SCHUR_RTLINVR && which <= ILM_SCHUR_GLINVD_CROSS, "bad Schur kind %d", which);
  const bool vec = c->kind == ILM_CACHE_VECTOR;
  ILM_REQUIRE(vec || (which != ILM_SCHUR_CLINVCT_SCALAR && which != ILM_SCHUR_CL2INVCT &&
                      which != ILM_SCHUR_GLINVD_SYMM),
              "Schur kind %d needs a vector cache", which);
  ILM_REQUIRE(!vec || which != ILM_SCHUR_GLINVD_CROSS, "Schur kind %d needs a scalar cache", which);
  cudaStream_t st = as_stream(stream);
  if (!vec && which <= ILM_SCHUR_NRTRN) return schur_build(c, which, scale, A_dev, st);
  return schur_build_columns(c, which, scale, A_dev, st);
}

}  // extern "C"

namespace ilm {

// S (FP64 and FP32 copies) cached in the cache
static int cached_schur(ilm_cache_s* c, int which, DevBuf& S64, DevBuf& S32, bool& ready, cudaStream_t st) {
  if (ready) return ILM_OK;
  const size_t nn = (size_t)c->npts * c->npts;
  (void)S32;
  ILM_TRY(S64.alloc(std::max<size_t>(nn, 1) * sizeof(double)));
  ILM_TRY(schur_build(c, which, 1.0, S64.as<double>(), st));
  ready = true;
  return ILM_OK;
}

// Solve S x = rhs (rhs, x FP64 device) by CG on the device.
static int schur_cg(ilm_cache_s* c, const DevBuf& S64, const DevBuf& S32, const double* rhs, double* x, double tol,
                    int maxiter, ilm_solve_info_t* info, cudaStream_t st) {
  const int N = c->npts;
  void* pb;
  ILM_TRY(pscr(c, 7, &pb));
  // layout in scratch 7: CGParams | iters (int) | relres (double)
  unsigned char* base = static_cast<unsigned char*>(pb);
  int* d_it = reinterpret_cast<int*>(base + 256);
  double* d_rr = reinterpret_cast<double*>(base + 264);
  if ((size_t)N * 4 * sizeof(double) < 512) {
    ILM_TRY(c->p_scr[7].alloc(512));
    base = static_cast<unsigned char*>(c->p_scr[7].p);
    d_it = reinterpret_cast<int*>(base + 256);
    d_rr = reinterpret_cast<double*>(base + 264);
  }
  CGParams P;
  P.A64 = S64.as<double>();
  P.A32 = nullptr;
  (void)S32;
  P.b = rhs;
  P.x = x;
  P.w = c->ds64.as<double>();
  P.n = N;
  P.maxiter = maxiter;
  P.tol = tol;
  P.iters = d_it;
  P.relres = d_rr;
  ILM_CHECK_CUDA(cudaMemcpyAsync(base, &P, sizeof(P), cudaMemcpyHostToDevice, st));
  ILM_TRY(launch_cg_batched(reinterpret_cast<CGParams*>(base), 1, N, st));
  int it = 0;
  double rr = 0.0;
  ILM_CHECK_CUDA(cudaMemcpyAsync(&it, d_it, sizeof(int), cudaMemcpyDeviceToHost, st));
  ILM_CHECK_CUDA(cudaMemcpyAsync(&rr, d_rr, sizeof(double), cudaMemcpyDeviceToHost, st));
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  if (info) {
    info->iterations = it;
    info->rel_residual = rr;
    info->converged = rr <= tol ? 1 : 0;
  }
  if (rr > tol) {
    set_error("Schur CG did not reach rel. residual %g in %d iterations (%g)", tol, it, rr);
    return ILM_ERR_NOT_CONVERGED;
  }
  return ILM_OK;
}

}  // namespace ilm

extern "C" {

// Dirichlet Poisson solve (test/literate/problems.jl:259-298 without the C^6
// filter; algebra in test/literate/dirichlet.jl:28-44):
//   f* = L^{-1} D_s [f];  S s = E f* - avg(f)  with S = create_RTLinvR;
//   f = f* + L^{-1} R s.
int ilm_solve_dirichlet(ilm_cache_t c, const void* fplus, const void* fminus, void* f_out, void* s_out, double tol,
                        int maxiter, ilm_solve_info_t* info, ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(c->kind == ILM_CACHE_SCALAR, "solve_dirichlet needs a scalar cache");
  ILM_REQUIRE(fplus && fminus && f_out && s_out, "null argument");
  ILM_REQUIRE(tol > 0.0 && maxiter > 0, "bad tolerance / iteration limit");
  cudaStream_t st = as_stream(stream);
  const int N = c->npts;
  const size_t np = c->grid.shape(PC_P).numel();
  if (N == 0) {
    if (info) *info = ilm_solve_info_t{0, 1, 0.0};
    return st_fill(np, c->dtype, 0.0, f_out, st);
  }
  void *jump, *avg, *g, *rhs64, *x64, *fstar, *corr;
  ILM_TRY(pscr(c, 1, &jump));
  ILM_TRY(pscr(c, 2, &avg));
  ILM_TRY(pscr(c, 3, &g));
  ILM_TRY(pscr(c, 4, &rhs64));
  ILM_TRY(pscr(c, 5, &x64));
  ILM_TRY(gscr(c, 3, &fstar));
  ILM_TRY(gscr(c, 4, &corr));
  ILM_TRY(st_axpby(N, c->dtype, 1.0, fplus, -1.0, fminus, jump, st));
  ILM_TRY(st_axpby(N, c->dtype, 0.5, fplus, 0.5, fminus, avg, st));
  ILM_TRY(ilm_surface_divergence(c, jump, fstar, stream));
  ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_PRIMAL, fstar, fstar, st));
  GatherTerm t{PC_P, fstar, CF_ONE};
  ILM_TRY(launch_gather(c, &t, 1, g, false, 1.0, st));
  ILM_TRY(st_axpby(N, c->dtype, 1.0, g, -1.0, avg, g, st));
  ILM_TRY(st_convert(N, c->dtype, g, ILM_F64, rhs64, st));
  ILM_TRY(cached_schur(c, ILM_SCHUR_RTLINVR, c->S_dir64, c->S_dir32, c->S_dir_ready, st));
  const int cg = schur_cg(c, c->S_dir64, c->S_dir32, static_cast<double*>(rhs64), static_cast<double*>(x64), tol,
                          maxiter, info, st);
  if (cg != ILM_OK && cg != ILM_ERR_NOT_CONVERGED) return cg;
  ILM_TRY(st_convert(N, ILM_F64, x64, c->dtype, s_out, st));
  ILM_TRY(scatter_scalar(c, PC_P, s_out, CF_ONE, corr, st));
  ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_PRIMAL, corr, corr, st));
  ILM_TRY(st_axpby(np, c->dtype, 1.0, corr, 1.0, fstar, f_out, st));
  return cg;
}

// Neumann Poisson solve (test/literate/neumann.jl:101-127):
//   f* = L^{-1} R [vn];  S [phi] = G_s f* - avg(vn)  with S = create_CLinvCT;
//   f = f* + L^{-1} D_s [phi].
int ilm_solve_neumann(ilm_cache_t c, const void* vplus, const void* vminus, void* f_out, void* df_out, double tol,
                      int maxiter, ilm_solve_info_t* info, ilm_stream_t stream) {
  return ilm_solve_neumann_full(c, vplus, vminus, f_out, df_out, nullptr, nullptr, tol, maxiter, info, stream);
}

int ilm_solve_neumann_full(ilm_cache_t c, const void* vplus, const void* vminus, void* f_out, void* df_out,
                           void* s_out, void* ds_out, double tol, int maxiter, ilm_solve_info_t* info,
                           ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(c->kind == ILM_CACHE_SCALAR, "solve_neumann needs a scalar cache");
  ILM_REQUIRE(vplus && vminus && f_out && df_out, "null argument");
  ILM_REQUIRE((s_out == nullptr) == (ds_out == nullptr), "solve_neumann: s_out and ds_out go together");
  ILM_REQUIRE(tol > 0.0 && maxiter > 0, "bad tolerance / iteration limit");
  cudaStream_t st = as_stream(stream);
  const int N = c->npts;
  const size_t np = c->grid.shape(PC_P).numel();
  const size_t nd = c->grid.shape(PC_D).numel();
  if (N == 0) {
    if (info) *info = ilm_solve_info_t{0, 1, 0.0};
    if (s_out) ILM_TRY(st_fill(nd, c->dtype, 0.0, s_out, st));
    return st_fill(np, c->dtype, 0.0, f_out, st);
  }
  void *jump, *avg, *g, *rhs64, *x64, *fstar, *corr;
  ILM_TRY(pscr(c, 1, &jump));
  ILM_TRY(pscr(c, 2, &avg));
  ILM_TRY(pscr(c, 3, &g));
  ILM_TRY(pscr(c, 4, &rhs64));
  ILM_TRY(pscr(c, 5, &x64));
  ILM_TRY(gscr(c, 3, &fstar));
  ILM_TRY(gscr(c, 4, &corr));
  ILM_TRY(st_axpby(N, c->dtype, 1.0, vplus, -1.0, vminus, jump, st));
  ILM_TRY(st_axpby(N, c->dtype, 0.5, vplus, 0.5, vminus, avg, st));
  ILM_TRY(scatter_scalar(c, PC_P, jump, CF_ONE, fstar, st));
  ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_PRIMAL, fstar, fstar, st));
  ILM_TRY(ilm_surface_grad(c, fstar, g, stream));
  ILM_TRY(st_axpby(N, c->dtype, 1.0, g, -1.0, avg, g, st));
  ILM_TRY(st_convert(N, c->dtype, g, ILM_F64, rhs64, st));
  ILM_TRY(cached_schur(c, ILM_SCHUR_CLINVCT, c->S_neu64, c->S_neu32, c->S_neu_ready, st));
  const int cg = schur_cg(c, c->S_neu64, c->S_neu32, static_cast<double*>(rhs64), static_cast<double*>(x64), tol,
                          maxiter, info, st);
  if (cg != ILM_OK && cg != ILM_ERR_NOT_CONVERGED) return cg;
  ILM_TRY(st_convert(N, ILM_F64, x64, c->dtype, df_out, st));
  ILM_TRY(ilm_surface_divergence(c, df_out, corr, stream));
  ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_PRIMAL, corr, corr, st));
  ILM_TRY(st_axpby(np, c->dtype, 1.0, corr, 1.0, fstar, f_out, st));
  if (!s_out) return cg;
  // streamfunction (test/literate/neumann.jl:129-138): s* = C_s^T [phi];
  // S ds = G^x_s f*;  s = L^-1 (s* - C^x_s^T ds)
  ilm_solve_info_t info2{0, 1, 0.0};
  ILM_TRY(ilm_surface_grad_cross(c, fstar, g, stream));
  ILM_TRY(st_convert(N, c->dtype, g, ILM_F64, rhs64, st));
  const int cg2 = schur_cg(c, c->S_neu64, c->S_neu32, static_cast<double*>(rhs64), static_cast<double*>(x64), tol,
                           maxiter, &info2, st);
  if (cg2 != ILM_OK && cg2 != ILM_ERR_NOT_CONVERGED) return cg2;
  ILM_TRY(st_convert(N, ILM_F64, x64, c->dtype, ds_out, st));
  ILM_TRY(ilm_surface_curl(c, 0, ILM_SCALAR_DATA, df_out, s_out, stream));   // s*
  ILM_TRY(ilm_surface_curl_cross(c, 0, ds_out, corr, stream));               // C^x_s^T ds (Nodes{Dual})
  ILM_TRY(st_axpby(nd, c->dtype, 1.0, s_out, -1.0, corr, corr, st));
  ILM_TRY(inverse_laplacian_kind(c, ILM_NODES_DUAL, corr, s_out, st));
  if (info) {
    info->iterations += info2.iterations;
    info->converged = info->converged && info2.converged;
    info->rel_residual = std::max(info->rel_residual, info2.rel_residual);
  }
  return cg != ILM_OK ? cg : cg2;
}

}  // extern "C"

namespace ilm {

// y = S x for a dense column-major FP64 n x n matrix, one thread per row
__global__ void k_dense_matvec64(int n, const double* __restrict__ S, const double* __restrict__ x,
                                 double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a0 = 0.0, a1 = 0.0;
  int j = 0;
  for (; j + 1 < n; j += 2) {
    a0 = fma(S[i + (size_t)j * n], x[j], a0);
    a1 = fma(S[i + (size_t)(j + 1) * n], x[j + 1], a1);
  }
  if (j < n) a0 = fma(S[i + (size_t)j * n], x[j], a0);
  y[i] = a0 + a1;
}

// r = b - y and (|r|^2, |b|^2), one block, fixed reduction order
__global__ void __launch_bounds__(256) k_residual64(int n, const double* __restrict__ bv, const double* __restrict__ y,
                                                   double* __restrict__ r, double* __restrict__ norms) {
  __shared__ double sr[256], sb[256];
  double rr = 0.0, bb = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double bi = bv[i];
    const double ri = bi - y[i];
    r[i] = ri;
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
    norms[0] = sr[0];
    norms[1] = sb[0];
  }
}

// FP64 cache of the same points for the refinement of an FP32 cache's solves
int ensure_twin(ilm_cache_s* c, ilm_cache_s** out) {
  if (c->dtype == ILM_F64) {
    *out = c;
    return ILM_OK;
  }
  if (!c->twin) {
    if (c->host_stale) ILM_TRY(cache_sync_host(c));
    ilm_cache_t t = nullptr;
    ILM_TRY(ilm_cache_create(&c->grid, c->kind, c->npts, c->hx.data(), c->hy.data(), c->hnx.data(), c->hny.data(),
                             c->hds.data(), c->ddf, c->scaling, ILM_F64, &t));
    c->twin = t;
  }
  *out = c->twin;
  return ILM_OK;
}

// Refined Dirichlet (neumann = false) or Neumann (true) Poisson solve; see
// ilm_solve_dirichlet_refined in ilm.h.
static int solve_refined(ilm_cache_s* c, bool neumann, const double* fplus, const double* fminus, double* f_out,
                         double* s_out, double tol, int maxiter, int max_refine, ilm_solve_info_t* info,
                         cudaStream_t st) {
  constexpr double kRefineFirstTol = 1e-8;  // first (bulk-precision) solve
  constexpr double kRefineInnerTol = 1e-6;  // each correction solve, relative to its residual
  const int N = c->npts;
  const size_t np = c->grid.shape(PC_P).numel();
  if (N == 0) {
    if (info) *info = ilm_solve_info_t{0, 1, 0.0};
    return st_fill(np, ILM_F64, 0.0, f_out, st);
  }
  ilm_cache_s* c64 = nullptr;
  ILM_TRY(ensure_twin(c, &c64));
  const size_t pv = (size_t)N * sizeof(double);
  ILM_TRY(c->ref_b.alloc(pv));
  ILM_TRY(c->ref_x.alloc(pv));
  ILM_TRY(c->ref_r.alloc(pv));
  ILM_TRY(c->ref_y.alloc(pv));
  ILM_TRY(c->ref_norm.alloc(2 * sizeof(double)));
  int total_its = 0;
  ilm_solve_info_t inf{0, 0, 0.0};
  // first solve in the cache's precision: its strengths start the refinement
  if (c->dtype != ILM_F64) {
    ILM_TRY(c->ref_in.alloc((size_t)2 * N * esize(c->dtype)));
    ILM_TRY(c->ref_f.alloc(np * esize(c->dtype)));
    ILM_TRY(c->ref_s.alloc((size_t)N * esize(c->dtype)));
    void* in_p = c->ref_in.p;
    void* in_m = ptr_off(c->ref_in.p, N, c->dtype);
    ILM_TRY(st_convert(N, ILM_F64, fplus, c->dtype, in_p, st));
    ILM_TRY(st_convert(N, ILM_F64, fminus, c->dtype, in_m, st));
    const int r0 = neumann ? ilm_solve_neumann(c, in_p, in_m, c->ref_f.p, c->ref_s.p, std::max(tol, kRefineFirstTol),
                                               maxiter, &inf, st)
                           : ilm_solve_dirichlet(c, in_p, in_m, c->ref_f.p, c->ref_s.p,
                                                 std::max(tol, kRefineFirstTol), maxiter, &inf, st);
    if (r0 != ILM_OK && r0 != ILM_ERR_NOT_CONVERGED) return r0;
    total_its += inf.iterations;
    void* x64;
    ILM_TRY(pscr(c, 5, &x64));  // the CG solution of the solve above (FP64)
    ILM_CHECK_CUDA(cudaMemcpyAsync(c->ref_x.p, x64, pv, cudaMemcpyDeviceToDevice, st));
  } else {
    ILM_CHECK_CUDA(cudaMemsetAsync(c->ref_x.p, 0, pv, st));
  }
  // FP64 Schur right-hand side: Dirichlet E f* - avg with f* = L^-1 D_s [f];
  // Neumann G_s f* - avg with f* = L^-1 R [vn]
  void *jump, *avg, *g, *fstar, *corr;
  ILM_TRY(pscr(c64, 1, &jump));
  ILM_TRY(pscr(c64, 2, &avg));
  ILM_TRY(pscr(c64, 3, &g));
  ILM_TRY(gscr(c64, 3, &fstar));
  ILM_TRY(gscr(c64, 4, &corr));
  ILM_TRY(st_axpby(N, ILM_F64, 1.0, fplus, -1.0, fminus, jump, st));
  ILM_TRY(st_axpby(N, ILM_F64, 0.5, fplus, 0.5, fminus, avg, st));
  if (neumann) {
    ILM_TRY(scatter_scalar(c64, PC_P, jump, CF_ONE, fstar, st));
    ILM_TRY(inverse_laplacian_kind(c64, ILM_NODES_PRIMAL, fstar, fstar, st));
    ILM_TRY(ilm_surface_grad(c64, fstar, g, st));
  } else {
    ILM_TRY(ilm_surface_divergence(c64, jump, fstar, st));
    ILM_TRY(inverse_laplacian_kind(c64, ILM_NODES_PRIMAL, fstar, fstar, st));
    GatherTerm t{PC_P, fstar, CF_ONE};
    ILM_TRY(launch_gather(c64, &t, 1, g, false, 1.0, st));
  }
  ILM_TRY(st_axpby(N, ILM_F64, 1.0, g, -1.0, avg, c->ref_b.p, st));
  // the FP64 Schur complement (the same pair sums for every dtype)
  DevBuf& S64 = neumann ? c->S_neu64 : c->S_dir64;
  if (neumann)
    ILM_TRY(cached_schur(c, ILM_SCHUR_CLINVCT, c->S_neu64, c->S_neu32, c->S_neu_ready, st));
  else
    ILM_TRY(cached_schur(c, ILM_SCHUR_RTLINVR, c->S_dir64, c->S_dir32, c->S_dir_ready, st));
  double rel = 0.0;
  for (int k = 0;; ++k) {
    k_dense_matvec64<<<(N + 127) / 128, 128, 0, st>>>(N, S64.as<double>(), c->ref_x.as<double>(),
                                                       c->ref_y.as<double>());
    ILM_CHECK_LAUNCH();
    k_residual64<<<1, 256, 0, st>>>(N, c->ref_b.as<double>(), c->ref_y.as<double>(), c->ref_r.as<double>(),
                                    c->ref_norm.as<double>());
    ILM_CHECK_LAUNCH();
    double nrm[2];
    ILM_CHECK_CUDA(cudaMemcpyAsync(nrm, c->ref_norm.p, sizeof(nrm), cudaMemcpyDeviceToHost, st));
    ILM_CHECK_CUDA(cudaStreamSynchronize(st));
    rel = nrm[1] > 0.0 ? std::sqrt(nrm[0] / nrm[1]) : 0.0;
    if (rel <= tol || k >= max_refine) break;
    // correction: S d = r by the FP64 CG, x += d
    ilm_solve_info_t ci{0, 0, 0.0};
    const int rc = schur_cg(c, S64, S64, c->ref_r.as<double>(), c->ref_y.as<double>(), kRefineInnerTol, maxiter, &ci,
                            st);
    if (rc != ILM_OK && rc != ILM_ERR_NOT_CONVERGED) return rc;
    total_its += ci.iterations;
    ILM_TRY(st_axpby(N, ILM_F64, 1.0, c->ref_x.p, 1.0, c->ref_y.p, c->ref_x.p, st));
  }
  // outputs: refined strengths, FP64 field f = f* + L^-1 (R s | D_s [phi])
  ILM_CHECK_CUDA(cudaMemcpyAsync(s_out, c->ref_x.p, pv, cudaMemcpyDeviceToDevice, st));
  if (neumann)
    ILM_TRY(ilm_surface_divergence(c64, s_out, corr, st));
  else
    ILM_TRY(scatter_scalar(c64, PC_P, s_out, CF_ONE, corr, st));
  ILM_TRY(inverse_laplacian_kind(c64, ILM_NODES_PRIMAL, corr, corr, st));
  ILM_TRY(st_axpby(np, ILM_F64, 1.0, corr, 1.0, fstar, f_out, st));
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  if (info) *info = ilm_solve_info_t{total_its, rel <= tol ? 1 : 0, rel};
  if (rel > tol) {
    set_error("refined solve: FP64 Schur residual %g after %d refinement steps (target %g)", rel, max_refine, tol);
    return ILM_ERR_NOT_CONVERGED;
  }
  return ILM_OK;
}

}  // namespace ilm

extern "C" {

int ilm_solve_dirichlet_refined(ilm_cache_t c, const double* fplus, const double* fminus, double* f_out,
                                double* s_out, double tol, int maxiter, int max_refine, ilm_solve_info_t* info,
                                ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(c->kind == ILM_CACHE_SCALAR, "solve_dirichlet_refined needs a scalar cache");
  ILM_REQUIRE(fplus && fminus && f_out && s_out, "null argument");
  ILM_REQUIRE(tol > 0.0 && maxiter > 0 && max_refine >= 0 && max_refine <= 100,
              "bad tolerance / iteration limit / refinement steps");
  return solve_refined(c, false, fplus, fminus, f_out, s_out, tol, maxiter, max_refine, info, as_stream(stream));
}

int ilm_solve_neumann_refined(ilm_cache_t c, const double* vplus, const double* vminus, double* f_out,
                              double* df_out, double tol, int maxiter, int max_refine, ilm_solve_info_t* info,
                              ilm_stream_t stream) {
  CHECK_CACHE(c);
  ILM_REQUIRE(c->kind == ILM_CACHE_SCALAR, "solve_neumann_refined needs a scalar cache");
  ILM_REQUIRE(vplus && vminus && f_out && df_out, "null argument");
  ILM_REQUIRE(tol > 0.0 && maxiter > 0 && max_refine >= 0 && max_refine <= 100,
              "bad tolerance / iteration limit / refinement steps");
  return solve_refined(c, true, vplus, vminus, f_out, df_out, tol, maxiter, max_refine, info, as_stream(stream));
}

}  // extern "C"
