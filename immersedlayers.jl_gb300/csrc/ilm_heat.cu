// Heat conduction with Dirichlet surfaces, marched by IF-HERK on the device.
//
// The reference's DirichletHeatConduction problem (test/literate/
// heatconduction.jl:87-189) is the constrained ODE
//     dT/dt = kappa L T + R sigma - kappa D_s[T],     E T = (T_b+ + T_b-)/2
// advanced by ConstrainedSystems' LiskaIFHERK (src/timemarching.jl:4,262-277):
// an integrating factor exp(tau kappa L) for the Laplacian and a half-explicit
// Runge-Kutta scheme for the constraint, one Schur solve per stage.
//
// Restatement used here (Liska & Colonius IF-HERK, scheme A: c = (0,1/3,1),
// a21 = 1/3, a31 = -1, a32 = 2, b = (0,3/4,1/4)):
//  * exp(a L5) on the unbounded lattice is the separable discrete heat kernel
//    e^{-2a} I_m(2a) per direction (a = kappa tau / h^2), applied as two short
//    1-D stencils (radius <= ~16 for the step sizes used);
//  * every stage needs the constraint only at the surface points, so the
//    stage right-hand sides are point-local gathers (E exp(aL) T is a gather
//    with the DDF window smeared by the heat kernel) and the stage Schur
//    complements S_a = E exp(aL) R are short-range: they are assembled once as
//    sparse matrices (float-float values) and solved by the cluster CG with a
//    warm start from the previous step;
//  * the grid is touched once per step: T <- exp(dt kappa L) T +
//    b2 dt exp(2/3 dt kappa L) R sigma_2 + b3 dt R sigma_3 + (constant field).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <new>
#include <unordered_map>

#include "ilm_internal.cuh"

namespace ilm {

namespace {

// e^{-2a} I_m(2a), m = 0..R, by the power series of I_m (a <= ~4)
std::vector<double> heat_kernel_taps(double a, double tol = 1e-17, int rmax = 40) {
  std::vector<double> k;
  if (a <= 0.0) return {1.0};
  const double x = a;  // I_m(2a) = sum_j a^(2j+m) / (j! (j+m)!)
  for (int m = 0; m <= rmax; ++m) {
    double term = exp(-2.0 * a);
    for (int i = 1; i <= m; ++i) term *= x / i;  // e^{-2a} a^m / m!
    double s = 0.0, t = term;
    for (int j = 0; j < 200; ++j) {
      s += t;
      t *= x * x / ((j + 1.0) * (j + 1.0 + m));
      if (t < 1e-30 * s) break;
    }
    if (m > 0 && s < tol) break;
    k.push_back(s);
  }
  return k;  // one side, k[0] at the centre
}

// one thread per output; x pass: out[j][i] = sum_m k[|m|] in[j][i+m] (zero outside)
template <typename T>
__global__ void k_if_x(int n1, int n2, const double* __restrict__ k, int R, const T* __restrict__ in,
                       T* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= n1) return;
  const T* row = in + (size_t)j * n1;
  double acc = k[0] * (double)row[i];
  for (int m = 1; m <= R; ++m) {
    const double km = k[m];
    if (i - m >= 0) acc += km * (double)row[i - m];
    if (i + m < n1) acc += km * (double)row[i + m];
  }
  out[(size_t)j * n1 + i] = (T)acc;
}

template <typename T>
__global__ void k_if_y(int n1, int n2, const double* __restrict__ k, int R, const T* __restrict__ in,
                       T* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= n1) return;
  double acc = k[0] * (double)in[(size_t)j * n1 + i];
  for (int m = 1; m <= R; ++m) {
    const double km = k[m];
    if (j - m >= 0) acc += km * (double)in[(size_t)(j - m) * n1 + i];
    if (j + m < n2) acc += km * (double)in[(size_t)(j + m) * n1 + i];
  }
  out[(size_t)j * n1 + i] = (T)acc;
}

// smeared-window gather: out_k = sum_{jj,ii} wy[k][jj] wx[k][ii] T[by+jj][bx+ii]
// one warp per point; two window sets (two integrating-factor arguments)
template <typename T>
__global__ void k_conv_gather2(int N, int n1, int n2, const T* __restrict__ f, int L0, const int* __restrict__ bx0,
                               const int* __restrict__ by0, const double* __restrict__ wx0,
                               const double* __restrict__ wy0, double* __restrict__ out0, int L1,
                               const int* __restrict__ bx1, const int* __restrict__ by1,
                               const double* __restrict__ wx1, const double* __restrict__ wy1,
                               double* __restrict__ out1) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= 2 * N) return;
  const int set = warp >= N ? 1 : 0;
  const int k = warp - set * N;
  const int L = set ? L1 : L0;
  const int b0 = set ? bx1[k] : bx0[k];
  const int e0 = set ? by1[k] : by0[k];
  const double* wx = (set ? wx1 : wx0) + (size_t)k * L;
  const double* wy = (set ? wy1 : wy0) + (size_t)k * L;
  double acc = 0.0;
  for (int jj = 0; jj < L; ++jj) {
    const int j = e0 + jj;
    if ((unsigned)j >= (unsigned)n2) continue;
    double racc = 0.0;
    for (int ii = lane; ii < L; ii += 32) {
      const int i = b0 + ii;
      if ((unsigned)i < (unsigned)n1) racc += wx[ii] * (double)f[(size_t)j * n1 + i];
    }
    acc += wy[jj] * racc;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) (set ? out1 : out0)[k] = acc;
}

// y = S x for a CSR float-float matrix (FP64 accumulation), one warp per row
__global__ void k_spmv_ff(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                          const float* __restrict__ vhi, const float* __restrict__ vlo, const double* __restrict__ x,
                          double* __restrict__ y) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  double acc = 0.0;
  for (int e = rowptr[warp] + lane; e < rowptr[warp + 1]; e += 32)
    acc += ((double)vhi[e] + (double)vlo[e]) * x[col[e]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) y[warp] = acc;
}

// stage right-hand sides.  rhs = (avg - (g + sum_t c_t v_t)) / denom
__global__ void k_stage_rhs(int n, const double* __restrict__ avg, const double* __restrict__ g, double c0,
                            const double* __restrict__ v0, double c1, const double* __restrict__ v1, double c2,
                            const double* __restrict__ v2, double c3, const double* __restrict__ v3, double inv_denom,
                            double* __restrict__ rhs) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double s = g[k];
  if (v0) s += c0 * v0[k];
  if (v1) s += c1 * v1[k];
  if (v2) s += c2 * v2[k];
  if (v3) s += c3 * v3[k];
  rhs[k] = (avg[k] - s) * inv_denom;
}

template <typename T>
__global__ void k_heat_combine(size_t n, const T* __restrict__ a, double cb, const T* __restrict__ b, double cc,
                               const T* __restrict__ c, const T* __restrict__ d, T* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (T)((double)a[i] + cb * (double)b[i] + cc * (double)c[i] + (double)d[i]);
}

}  // namespace

}  // namespace ilm

using namespace ilm;

struct ilm_heat_s {
  ilm_cache_s* c = nullptr;
  double kappa = 1.0, dt = 0.0;
  double a21 = 1.0 / 3.0, a31 = -1.0, a32 = 2.0, b1 = 0.0, b2 = 0.75, b3 = 0.25;
  double tol = 1e-10;
  int maxiter = 2000;
  int n1 = 0, n2 = 0;
  // integrating-factor taps for a * (1/3, 2/3, 1)
  int R[3] = {0, 0, 0};
  DevBuf kt[3];
  // smeared gather windows for a/3 (set 0) and a (set 1)
  int L[2] = {0, 0};
  DevBuf gbx[2], gby[2], gwx[2], gwy[2];
  // sparse stage Schur complements: 0 -> a/3, 1 -> 2a/3, 2 -> a, 3 -> 0
  DevBuf rowptr[4], colidx[4], vhi[4], vlo[4];
  size_t nnz[4] = {0, 0, 0, 0};
  DevBuf e[4], avg64, cfield;
  DevBuf g1, g3, rhs, q1, q2, sig[3], sig_t;
  DevBuf tmp[4];
  DevBuf cgp, order, counter, iters, relres;
  long long total_iters = 0;
  int last_iters[3] = {0, 0, 0};
};

namespace {

int upd(DevBuf& b, const void* h, size_t bytes) {
  ILM_TRY(b.alloc(std::max<size_t>(bytes, 8)));
  if (bytes) ILM_CHECK_CUDA(cudaMemcpy(b.p, h, bytes, cudaMemcpyHostToDevice));
  return ILM_OK;
}

int apply_if_dev(ilm_heat_s* H, int which, const void* in, void* tmp, void* out, cudaStream_t st) {
  const int R = H->R[which];
  const double* k = H->kt[which].as<double>();
  dim3 blk(256), grd((H->n1 + 255) / 256, H->n2);
  if (H->c->dtype == ILM_F64) {
    k_if_x<double><<<grd, blk, 0, st>>>(H->n1, H->n2, k, R, static_cast<const double*>(in), static_cast<double*>(tmp));
    k_if_y<double><<<grd, blk, 0, st>>>(H->n1, H->n2, k, R, static_cast<const double*>(tmp), static_cast<double*>(out));
  } else {
    k_if_x<float><<<grd, blk, 0, st>>>(H->n1, H->n2, k, R, static_cast<const float*>(in), static_cast<float*>(tmp));
    k_if_y<float><<<grd, blk, 0, st>>>(H->n1, H->n2, k, R, static_cast<const float*>(tmp), static_cast<float*>(out));
  }
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

// sparse S_a = E exp(aL) R on Nodes{Primal}: S_kl = (ds_l/h^2) X_kl Y_kl with X_kl the
// x-window of k smeared by the heat kernel, correlated with l's x-window.
int build_sparse_schur(ilm_heat_s* H, const std::vector<double>& taps, int slot) {
  ilm_cache_s* c = H->c;
  const int N = c->npts;
  const int R = (int)taps.size() - 1;
  const int reach = 2 * R + NTAP;  // |bx_k - bx_l| < reach for a nonzero X_kl
  const std::vector<int>& bx = c->hbx[0];
  const std::vector<int>& by = c->hby[0];
  const std::vector<double>& wx = c->hwx[0];
  const std::vector<double>& wy = c->hwy[0];
  auto kval = [&](int m) { m = m < 0 ? -m : m; return m <= R ? taps[m] : 0.0; };
  // smeared windows (length NTAP + 2R, base bx - R)
  const int Ls = NTAP + 2 * R;
  std::vector<double> sx((size_t)N * Ls, 0.0), sy((size_t)N * Ls, 0.0);
  for (int k = 0; k < N; ++k)
    for (int t = 0; t < NTAP; ++t)
      for (int m = -R; m <= R; ++m) {
        sx[(size_t)k * Ls + t + m + R] += wx[(size_t)k * NTAP + t] * kval(m);
        sy[(size_t)k * Ls + t + m + R] += wy[(size_t)k * NTAP + t] * kval(m);
      }
  // spatial hash of points by window base
  const int B = std::max(reach, 1);
  std::unordered_map<long long, std::vector<int>> cells;
  auto key = [](int a, int b) { return ((long long)a << 32) ^ (unsigned int)b; };
  auto fdiv = [](int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); };
  for (int k = 0; k < N; ++k) cells[key(fdiv(bx[k], B), fdiv(by[k], B))].push_back(k);
  std::vector<int> rp(N + 1, 0), ci;
  std::vector<float> vh, vl;
  const double ih2 = 1.0 / (c->h * c->h);
  std::vector<int> nb;
  for (int k = 0; k < N; ++k) {
    nb.clear();
    const int cx = fdiv(bx[k], B), cy = fdiv(by[k], B);
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        auto it = cells.find(key(cx + dx, cy + dy));
        if (it == cells.end()) continue;
        for (int l : it->second)
          if (std::abs(bx[k] - bx[l]) < reach && std::abs(by[k] - by[l]) < reach) nb.push_back(l);
      }
    std::sort(nb.begin(), nb.end());
    for (int l : nb) {
      // X_kl = sum_u wx_l[u] * sx_k[(bx_l + u) - (bx_k - R)]
      double X = 0.0, Y = 0.0;
      for (int u = 0; u < NTAP; ++u) {
        const int ix = bx[l] + u - (bx[k] - R);
        if (ix >= 0 && ix < Ls) X += wx[(size_t)l * NTAP + u] * sx[(size_t)k * Ls + ix];
        const int iy = by[l] + u - (by[k] - R);
        if (iy >= 0 && iy < Ls) Y += wy[(size_t)l * NTAP + u] * sy[(size_t)k * Ls + iy];
      }
      const double v = c->hds[l] * ih2 * X * Y;
      if (v == 0.0) continue;
      ci.push_back(l);
      const float h = (float)v;
      vh.push_back(h);
      vl.push_back((float)(v - (double)h));
    }
    rp[k + 1] = (int)ci.size();
  }
  H->nnz[slot] = ci.size();
  ILM_TRY(upd(H->rowptr[slot], rp.data(), rp.size() * sizeof(int)));
  ILM_TRY(upd(H->colidx[slot], ci.data(), ci.size() * sizeof(int)));
  ILM_TRY(upd(H->vhi[slot], vh.data(), vh.size() * sizeof(float)));
  ILM_TRY(upd(H->vlo[slot], vl.data(), vl.size() * sizeof(float)));
  return ILM_OK;
}

// smeared gather windows on Nodes{Primal} for one integrating-factor argument
int build_gather_windows(ilm_heat_s* H, const std::vector<double>& taps, int set) {
  ilm_cache_s* c = H->c;
  const int N = c->npts;
  const int R = (int)taps.size() - 1;
  const int Ls = NTAP + 2 * R;
  std::vector<int> bx(N), by(N);
  std::vector<double> sx((size_t)N * Ls, 0.0), sy((size_t)N * Ls, 0.0);
  for (int k = 0; k < N; ++k) {
    bx[k] = c->hbx[0][k] - R;
    by[k] = c->hby[0][k] - R;
    for (int t = 0; t < NTAP; ++t)
      for (int m = -R; m <= R; ++m) {
        const double km = taps[std::abs(m)];
        sx[(size_t)k * Ls + t + m + R] += c->hwx[0][(size_t)k * NTAP + t] * km;
        sy[(size_t)k * Ls + t + m + R] += c->hwy[0][(size_t)k * NTAP + t] * km;
      }
  }
  H->L[set] = Ls;
  ILM_TRY(upd(H->gbx[set], bx.data(), N * sizeof(int)));
  ILM_TRY(upd(H->gby[set], by.data(), N * sizeof(int)));
  ILM_TRY(upd(H->gwx[set], sx.data(), sx.size() * sizeof(double)));
  ILM_TRY(upd(H->gwy[set], sy.data(), sy.size() * sizeof(double)));
  return ILM_OK;
}

int run_cg(ilm_heat_s* H, int which_params, cudaStream_t st) {
  ILM_TRY(launch_cg_cluster(static_cast<unsigned char*>(H->cgp.p) + (size_t)which_params * cgff_params_size(),
                            H->order.as<int>(), 1, H->counter.as<int>() + which_params, H->c->npts, 1, st));
  return ILM_OK;
}

}  // namespace

extern "C" {

int ilm_heat_create(ilm_cache_t c, double kappa, double dt, const double* tb_plus, const double* tb_minus,
                    double tol, int maxiter, ilm_heat_t* out) {
  if (c) ILM_TRY(cache_sync_host(c));  // host windows used below
  ILM_REQUIRE(c && out && tb_plus && tb_minus, "heat: null argument");
  ILM_REQUIRE(c->kind == ILM_CACHE_SCALAR, "heat: scalar cache required");
  ILM_REQUIRE(c->scaling == ILM_GRID_SCALING, "heat: GridScaling cache required");
  ILM_REQUIRE(c->npts > 0, "heat: the cache has no surface points");
  ILM_REQUIRE(kappa > 0 && dt > 0 && tol > 0 && maxiter > 0, "heat: bad kappa / dt / tol / maxiter");
  const double af = kappa * dt / (c->h * c->h);
  ILM_REQUIRE(af <= 4.0, "heat: kappa dt / h^2 = %g too large for the integrating-factor stencil", af);
  auto* H = new (std::nothrow) ilm_heat_s();
  if (!H) return ILM_ERR_NO_MEMORY;
  std::unique_ptr<ilm_heat_s> guard(H);
  H->c = c;
  H->kappa = kappa;
  H->dt = dt;
  H->tol = tol;
  H->maxiter = maxiter;
  const ilm::Shape2 sh = c->grid.shape(PC_P);
  H->n1 = sh.n1;
  H->n2 = sh.n2;
  const int N = c->npts;
  const size_t np = sh.numel();
  const size_t es = c->dtype == ILM_F64 ? 8 : 4;
  const double frac[3] = {1.0 / 3.0, 2.0 / 3.0, 1.0};
  std::vector<double> taps[3];
  for (int w = 0; w < 3; ++w) {
    taps[w] = heat_kernel_taps(af * frac[w]);
    H->R[w] = (int)taps[w].size() - 1;
    ILM_TRY(upd(H->kt[w], taps[w].data(), taps[w].size() * sizeof(double)));
  }
  ILM_TRY(build_gather_windows(H, taps[0], 0));
  ILM_TRY(build_gather_windows(H, taps[2], 1));
  const std::vector<double> delta{1.0};
  ILM_TRY(build_sparse_schur(H, taps[0], 0));
  ILM_TRY(build_sparse_schur(H, taps[1], 1));
  ILM_TRY(build_sparse_schur(H, taps[2], 2));
  ILM_TRY(build_sparse_schur(H, delta, 3));
  // surface data, r1 = -kappa D_s[T] and its point images e_a = E exp(aL) r1
  std::vector<double> avg(N), jump(N);
  for (int k = 0; k < N; ++k) {
    avg[k] = 0.5 * (tb_plus[k] + tb_minus[k]);
    jump[k] = -kappa * (tb_plus[k] - tb_minus[k]);
  }
  ILM_TRY(upd(H->avg64, avg.data(), N * sizeof(double)));
  for (int t = 0; t < 4; ++t) ILM_TRY(H->tmp[t].alloc(np * es));
  DevBuf jd, pt;
  ILM_TRY(jd.alloc((size_t)N * es));
  ILM_TRY(pt.alloc((size_t)N * es));
  if (c->dtype == ILM_F64) {
    ILM_CHECK_CUDA(cudaMemcpy(jd.p, jump.data(), N * 8, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> jf(jump.begin(), jump.end());
    ILM_CHECK_CUDA(cudaMemcpy(jd.p, jf.data(), N * 4, cudaMemcpyHostToDevice));
  }
  void* r1 = H->tmp[0].p;
  ILM_TRY(ilm_surface_divergence(c, jd.p, r1, nullptr));
  ILM_TRY(H->cfield.alloc(np * es));
  for (int t = 0; t < 4; ++t) ILM_TRY(H->e[t].alloc((size_t)N * 8));
  for (int w = 0; w < 3; ++w) {
    ILM_TRY(apply_if_dev(H, w, r1, H->tmp[1].p, H->tmp[2].p, nullptr));
    ILM_TRY(ilm_interpolate(c, ILM_NODES_PRIMAL, H->tmp[2].p, pt.p, nullptr));
    ILM_TRY(st_convert(N, c->dtype, pt.p, ILM_F64, H->e[w].p, nullptr));
    if (w == 1) {  // cfield = dt b2 exp(2a/3 L) r1 + dt b3 r1   (b1 = 0)
      ILM_TRY(st_axpby(np, c->dtype, dt * H->b2, H->tmp[2].p, dt * H->b3, r1, H->cfield.p, nullptr));
    }
  }
  ILM_TRY(ilm_interpolate(c, ILM_NODES_PRIMAL, r1, pt.p, nullptr));
  ILM_TRY(st_convert(N, c->dtype, pt.p, ILM_F64, H->e[3].p, nullptr));
  // work vectors and CG parameter records (stage 2: S_{a/3}; stage 3: S_{2a/3}; final: S_0)
  ILM_TRY(H->g1.alloc((size_t)N * 8));
  ILM_TRY(H->g3.alloc((size_t)N * 8));
  ILM_TRY(H->rhs.alloc((size_t)N * 8 * 3));
  ILM_TRY(H->q1.alloc((size_t)N * 8));
  ILM_TRY(H->q2.alloc((size_t)N * 8));
  for (int s = 0; s < 3; ++s) {
    ILM_TRY(H->sig[s].alloc((size_t)N * 8));
    ILM_CHECK_CUDA(cudaMemset(H->sig[s].p, 0, (size_t)N * 8));
  }
  ILM_TRY(H->sig_t.alloc((size_t)N * es));
  ILM_TRY(H->iters.alloc(3 * sizeof(int)));
  ILM_TRY(H->relres.alloc(3 * sizeof(double)));
  ILM_TRY(H->counter.alloc(3 * sizeof(int)));
  int zero = 0;
  ILM_TRY(upd(H->order, &zero, sizeof(int)));
  std::vector<unsigned char> prm(3 * cgff_params_size());
  const int mslot[3] = {0, 1, 3};
  for (int s = 0; s < 3; ++s) {
    cgff_params_fill_csr(prm.data() + s * cgff_params_size(), H->vhi[mslot[s]].as<float>(),
                         H->vlo[mslot[s]].as<float>(), H->rowptr[mslot[s]].as<int>(), H->colidx[mslot[s]].as<int>(),
                         H->rhs.as<double>() + (size_t)s * N, H->sig[s].as<double>(), H->sig[s].as<double>(),
                         c->ds64.as<double>(), N, maxiter, tol, H->iters.as<int>() + s,
                         H->relres.as<double>() + s);
  }
  ILM_TRY(upd(H->cgp, prm.data(), prm.size()));
  ILM_CHECK_CUDA(cudaDeviceSynchronize());
  *out = guard.release();
  return ILM_OK;
}

int ilm_heat_destroy(ilm_heat_t h) {
  delete h;
  return ILM_OK;
}

int ilm_heat_advance(ilm_heat_t H, void* T, void* sigma_out, int nsteps, ilm_stream_t stream) {
  ILM_REQUIRE(H && T && nsteps >= 0, "heat_advance: bad arguments");
  ilm_cache_s* c = H->c;
  cudaStream_t st = as_stream(stream);
  const int N = c->npts;
  const size_t np = (size_t)H->n1 * H->n2;
  const double dt = H->dt;
  const int wb = (2 * N * 32 + 255) / 256;
  const int pb = (N + 255) / 256;
  const int sb = (N * 32 + 255) / 256;
  double* rhs = H->rhs.as<double>();
  for (int step = 0; step < nsteps; ++step) {
    // point images of the current field: g1 = E exp(a/3 L) T, g3 = E exp(a L) T
    if (c->dtype == ILM_F64)
      k_conv_gather2<double><<<wb, 256, 0, st>>>(N, H->n1, H->n2, static_cast<const double*>(T), H->L[0],
                                                  H->gbx[0].as<int>(), H->gby[0].as<int>(), H->gwx[0].as<double>(),
                                                  H->gwy[0].as<double>(), H->g1.as<double>(), H->L[1],
                                                  H->gbx[1].as<int>(), H->gby[1].as<int>(), H->gwx[1].as<double>(),
                                                  H->gwy[1].as<double>(), H->g3.as<double>());
    else
      k_conv_gather2<float><<<wb, 256, 0, st>>>(N, H->n1, H->n2, static_cast<const float*>(T), H->L[0],
                                                 H->gbx[0].as<int>(), H->gby[0].as<int>(), H->gwx[0].as<double>(),
                                                 H->gwy[0].as<double>(), H->g1.as<double>(), H->L[1],
                                                 H->gbx[1].as<int>(), H->gby[1].as<int>(), H->gwx[1].as<double>(),
                                                 H->gwy[1].as<double>(), H->g3.as<double>());
    ILM_CHECK_LAUNCH();
    // stage 2: S_{a/3} sigma1 = (avg - g1 - dt a21 e_{a/3}) / (dt a21)
    k_stage_rhs<<<pb, 256, 0, st>>>(N, H->avg64.as<double>(), H->g1.as<double>(), dt * H->a21, H->e[0].as<double>(),
                                     0.0, nullptr, 0.0, nullptr, 0.0, nullptr, 1.0 / (dt * H->a21), rhs);
    ILM_CHECK_LAUNCH();
    ILM_TRY(run_cg(H, 0, st));
    // stage 3: S_{2a/3} sigma2 = (avg - [g3 + dt a31 (e_a + S_a sigma1) + dt a32 e_{2a/3}]) / (dt a32)
    k_spmv_ff<<<sb, 256, 0, st>>>(N, H->rowptr[2].as<int>(), H->colidx[2].as<int>(), H->vhi[2].as<float>(),
                                  H->vlo[2].as<float>(), H->sig[0].as<double>(), H->q1.as<double>());
    ILM_CHECK_LAUNCH();
    k_stage_rhs<<<pb, 256, 0, st>>>(N, H->avg64.as<double>(), H->g3.as<double>(), dt * H->a31, H->e[2].as<double>(),
                                     dt * H->a31, H->q1.as<double>(), dt * H->a32, H->e[1].as<double>(), 0.0, nullptr,
                                     1.0 / (dt * H->a32), rhs + N);
    ILM_CHECK_LAUNCH();
    ILM_TRY(run_cg(H, 1, st));
    // final: S_0 sigma3 = (avg - [g3 + dt b2 (e_{2a/3} + S_{2a/3} sigma2) + dt b3 e_0]) / (dt b3)   (b1 = 0)
    k_spmv_ff<<<sb, 256, 0, st>>>(N, H->rowptr[1].as<int>(), H->colidx[1].as<int>(), H->vhi[1].as<float>(),
                                  H->vlo[1].as<float>(), H->sig[1].as<double>(), H->q2.as<double>());
    ILM_CHECK_LAUNCH();
    k_stage_rhs<<<pb, 256, 0, st>>>(N, H->avg64.as<double>(), H->g3.as<double>(), dt * H->b2, H->e[1].as<double>(),
                                     dt * H->b2, H->q2.as<double>(), dt * H->b3, H->e[3].as<double>(), 0.0, nullptr,
                                     1.0 / (dt * H->b3), rhs + 2 * N);
    ILM_CHECK_LAUNCH();
    ILM_TRY(run_cg(H, 2, st));
    // grid: T <- exp(aL) T + dt b2 exp(2a/3 L) R sigma2 + dt b3 R sigma3 + cfield
    ILM_TRY(apply_if_dev(H, 2, T, H->tmp[0].p, H->tmp[1].p, st));
    ILM_TRY(st_convert(N, ILM_F64, H->sig[1].p, c->dtype, H->sig_t.p, st));
    ILM_TRY(ilm_regularize(c, ILM_NODES_PRIMAL, H->sig_t.p, H->tmp[2].p, st));
    ILM_TRY(apply_if_dev(H, 1, H->tmp[2].p, H->tmp[0].p, H->tmp[3].p, st));
    ILM_TRY(st_convert(N, ILM_F64, H->sig[2].p, c->dtype, H->sig_t.p, st));
    ILM_TRY(ilm_regularize(c, ILM_NODES_PRIMAL, H->sig_t.p, H->tmp[2].p, st));
    if (c->dtype == ILM_F64)
      k_heat_combine<double><<<1024, 256, 0, st>>>(np, H->tmp[1].as<double>(), dt * H->b2, H->tmp[3].as<double>(),
                                                    dt * H->b3, H->tmp[2].as<double>(), H->cfield.as<double>(),
                                                    static_cast<double*>(T));
    else
      k_heat_combine<float><<<1024, 256, 0, st>>>(np, H->tmp[1].as<float>(), dt * H->b2, H->tmp[3].as<float>(),
                                                   dt * H->b3, H->tmp[2].as<float>(), H->cfield.as<float>(),
                                                   static_cast<float*>(T));
    ILM_CHECK_LAUNCH();
  }
  if (sigma_out) {  // the reference's constraint force enters as -R sigma
    ILM_TRY(st_convert(N, ILM_F64, H->sig[2].p, c->dtype, sigma_out, st));
    ILM_TRY(st_affine(N, c->dtype, -1.0, sigma_out, 0.0, sigma_out, st));
  }
  if (nsteps > 0) {
    int it[3];
    ILM_CHECK_CUDA(cudaMemcpyAsync(it, H->iters.p, 3 * sizeof(int), cudaMemcpyDeviceToHost, st));
    ILM_CHECK_CUDA(cudaStreamSynchronize(st));
    for (int s = 0; s < 3; ++s) H->last_iters[s] = it[s];
  }
  return ILM_OK;
}

int ilm_heat_info(ilm_heat_t H, int* last_iters, double* last_relres, size_t* nnz) {
  ILM_REQUIRE(H, "null heat integrator");
  if (last_iters) ILM_CHECK_CUDA(cudaMemcpy(last_iters, H->iters.p, 3 * sizeof(int), cudaMemcpyDeviceToHost));
  if (last_relres) ILM_CHECK_CUDA(cudaMemcpy(last_relres, H->relres.p, 3 * sizeof(double), cudaMemcpyDeviceToHost));
  if (nnz)
    for (int s = 0; s < 4; ++s) nnz[s] = H->nnz[s];
  return ILM_OK;
}

}  // extern "C"
