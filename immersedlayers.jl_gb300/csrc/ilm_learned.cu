// Learned preconditioner for the Schur-complement CG.
//
// A 1-D convolutional network over arc length (circular per body) reads
// dimensionless geometry features of each surface point and emits a banded
// factor C (2K+1 coefficients per point); the preconditioner is
// M r = W^-1 C^T C r with W = diag(ds), self-adjoint and semi-definite in
// the ds-weighted inner product in which the reference's Schur operator
// S = R^T L^-1 R (src/matrix_operators.jl:9-27, GridScaling) is symmetric.
// Inference runs once per problem at set-up; the CG applies the band.
//
// Weights are stored as FP32 masters with a BF16 copy that every forward and
// backward pass reads (FP32 accumulation); training is Adam on the relative
// error |M b - x|^2 / |x|^2 over (b, x = S^-1 b) pairs.  All kernels are
// deterministic (fixed reduction orders, no atomics).
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <memory>
#include <new>
#include <vector>

#include "ilm_internal.cuh"

namespace ilm {
namespace {

constexpr int NK = 5;    // taps per convolution
constexpr int NR = 2;    // tap radius
constexpr int TP = 32;   // points per block (convolution)
constexpr int CT = 256;  // threads per block (convolution)
constexpr int MAXC = 64;
constexpr int WCH = 256;  // points per block (weight gradient)
constexpr int WSUB = 32;
constexpr int WKS = 16;   // input channels per block (weight gradient)

// t-th neighbour of point i along its body [s, s + L), circular; any
// segment data give an index inside [s, s + max(L, 1))
__device__ __forceinline__ int nbr(int i, int s, int L, int t) {
  if (L < 1) return i;
  int q = (i - s + t) % L;
  q += q < 0 ? L : 0;
  return s + q;
}

// out[i][o] = bias[o] + sum_{t,k} Ws[t][k][o] in[nb(i, t-2)][k]  (optional relu)
// mode 0: Ws[t][k][o] = W[o][k][t]           (forward, W is Cout x Cin x 5)
// mode 1: Ws[t][k][o] = W[k][o][4 - t]       (data gradient, W is Cin x Cout x 5)
template <bool RELU>
__global__ void __launch_bounds__(CT) k_conv(int N, int Cin, int Cout, int mode, const __nv_bfloat16* __restrict__ W,
                                             const float* __restrict__ bias, const float* __restrict__ in,
                                             const int* __restrict__ sst, const int* __restrict__ sln,
                                             float* __restrict__ out) {
  extern __shared__ float sm[];
  float* ws = sm;                         // [5][Cin][Cout]
  float* xs = ws + NK * Cin * Cout;       // [5][TP][Cin]
  const int p0 = blockIdx.x * TP;
  for (int e = threadIdx.x; e < NK * Cin * Cout; e += CT) {
    const int o = e % Cout, k = (e / Cout) % Cin, t = e / (Cout * Cin);
    const int gi = mode == 0 ? (o * Cin + k) * NK + t : (k * Cout + o) * NK + (NK - 1 - t);
    ws[e] = __bfloat162float(W[gi]);
  }
  for (int e = threadIdx.x; e < NK * TP * Cin; e += CT) {
    const int k = e % Cin, p = (e / Cin) % TP, t = e / (Cin * TP);
    const int i = p0 + p;
    float v = 0.f;
    if (i < N) v = in[(size_t)nbr(i, sst[i], sln[i], t - NR) * Cin + k];
    xs[e] = v;
  }
  __syncthreads();
  const int o = threadIdx.x % MAXC, pg = threadIdx.x / MAXC;  // 4 groups of 8 points
  if (o >= Cout) return;
  float acc[8];
  const float b0 = bias ? bias[o] : 0.f;
#pragma unroll
  for (int p = 0; p < 8; ++p) acc[p] = b0;
  for (int t = 0; t < NK; ++t) {
    const float* xt = xs + ((size_t)t * TP + pg * 8) * Cin;
    const float* wt = ws + (size_t)t * Cin * Cout + o;
    for (int k = 0; k < Cin; ++k) {
      const float w = wt[(size_t)k * Cout];
#pragma unroll
      for (int p = 0; p < 8; ++p) acc[p] = fmaf(w, xt[p * Cin + k], acc[p]);
    }
  }
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    const int i = p0 + pg * 8 + p;
    if (i < N) out[(size_t)i * Cout + o] = RELU ? fmaxf(acc[p], 0.f) : acc[p];
  }
}

// partial[bx][o][k][t] = sum_{i in block's points} g[i][o] a[nb(i,t-2)][k], k in this block's slice
__global__ void __launch_bounds__(CT) k_conv_wgrad(int N, int Cin, int Cout, const float* __restrict__ g,
                                                   const float* __restrict__ a, const int* __restrict__ sst,
                                                   const int* __restrict__ sln, float* __restrict__ partW,
                                                   float* __restrict__ partB) {
  __shared__ float gs[WSUB][MAXC];
  __shared__ float as_[NK][WSUB][WKS];
  const int o = threadIdx.x % MAXC, kq = threadIdx.x / MAXC;
  const int k0 = blockIdx.y * WKS;
  float acc[4][NK];
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int t = 0; t < NK; ++t) acc[q][t] = 0.f;
  float accb = 0.f;
  for (int sub = 0; sub < WCH; sub += WSUB) {
    const int pb = blockIdx.x * WCH + sub;
    for (int e = threadIdx.x; e < WSUB * MAXC; e += CT) {
      const int p = e / MAXC, oo = e % MAXC, i = pb + p;
      gs[p][oo] = (i < N && oo < Cout) ? g[(size_t)i * Cout + oo] : 0.f;
    }
    for (int e = threadIdx.x; e < NK * WSUB * WKS; e += CT) {
      const int kk = e % WKS, p = (e / WKS) % WSUB, t = e / (WKS * WSUB);
      const int i = pb + p, k = k0 + kk;
      float v = 0.f;
      if (i < N && k < Cin) v = a[(size_t)nbr(i, sst[i], sln[i], t - NR) * Cin + k];
      as_[t][p][kk] = v;
    }
    __syncthreads();
    if (o < Cout) {
      for (int p = 0; p < WSUB; ++p) {
        const float gv = gs[p][o];
        accb += gv;
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int t = 0; t < NK; ++t) acc[q][t] = fmaf(gv, as_[t][p][kq * 4 + q], acc[q][t]);
      }
    }
    __syncthreads();
  }
  if (o >= Cout) return;
  for (int q = 0; q < 4; ++q) {
    const int k = k0 + kq * 4 + q;
    if (k >= Cin) continue;
    for (int t = 0; t < NK; ++t) partW[((size_t)blockIdx.x * Cout + o) * Cin * NK + (size_t)k * NK + t] = acc[q][t];
  }
  if (blockIdx.y == 0 && kq == 0) partB[(size_t)blockIdx.x * Cout + o] = accb;
}

// out[e] = sum_b part[b][e] in block order (deterministic)
__global__ void k_reduce_parts(int nparts, int n, const float* __restrict__ part, float* __restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double s = 0.0;
  for (int b = 0; b < nparts; ++b) s += part[(size_t)b * n + e];
  out[e] = (float)s;
}

__global__ void k_relu_mask(size_t n, const float* __restrict__ act, float* __restrict__ g) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (!(act[i] > 0.f)) g[i] = 0.f;
}

// c = out + e_K (identity on the band's centre)
__global__ void k_band_c(int N, int K, const float* __restrict__ out, float* __restrict__ c) {
  const int P = 2 * K + 1;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N * P; e += gridDim.x * blockDim.x)
    c[e] = out[e] + ((e % P) == K ? 1.f : 0.f);
}

// u_j = sum_t c[j][t+K] r[nb(j,t)]
__global__ void k_band_fwd(int N, int K, const float* __restrict__ c, const float* __restrict__ r,
                           const int* __restrict__ sst, const int* __restrict__ sln, float* __restrict__ u) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const int s = sst[j], L = sln[j], P = 2 * K + 1;
  float acc = 0.f;
  for (int t = -K; t <= K; ++t) acc = fmaf(c[(size_t)j * P + t + K], r[nbr(j, s, L, t)], acc);
  u[j] = acc;
}

// z_i = (1/w_i) sum_t c[nb(i,-t)][t+K] u[nb(i,-t)];  e_i = z_i - x_i
__global__ void k_band_z(int N, int K, const float* __restrict__ c, const float* __restrict__ u,
                         const float* __restrict__ w, const float* __restrict__ x, const int* __restrict__ sst,
                         const int* __restrict__ sln, float* __restrict__ e) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int s = sst[i], L = sln[i], P = 2 * K + 1;
  float acc = 0.f;
  for (int t = -K; t <= K; ++t) {
    const int j = nbr(i, s, L, -t);
    acc = fmaf(c[(size_t)j * P + t + K], u[j], acc);
  }
  e[i] = acc / w[i] - x[i];
}

// per pair: ee = |e|^2, xx = |x|^2 (block per pair, fixed tree)
__global__ void k_pair_sums(const int* __restrict__ off, const float* __restrict__ e, const float* __restrict__ x,
                            double* __restrict__ sums) {
  __shared__ double s1[256], s2[256];
  const int p = blockIdx.x;
  double a = 0.0, b = 0.0;
  for (int i = off[p] + threadIdx.x; i < off[p + 1]; i += blockDim.x) {
    a += (double)e[i] * e[i];
    b += (double)x[i] * x[i];
  }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      s1[threadIdx.x] += s1[threadIdx.x + h];
      s2[threadIdx.x] += s2[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    sums[2 * p] = s1[0];
    sums[2 * p + 1] = s2[0];
  }
}

__global__ void k_loss_total(int npair, const double* __restrict__ sums, double* __restrict__ loss) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double L = 0.0;
  for (int p = 0; p < npair; ++p) L += sums[2 * p] / sums[2 * p + 1];
  *loss = L / npair;
}

// y_i = 2 e_i / (xx_p npair w_i)
__global__ void k_band_gy(int N, int npair, const int* __restrict__ off, const float* __restrict__ e,
                          const float* __restrict__ w, const double* __restrict__ sums, float* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int lo = 0, hi = npair - 1;  // pair of point i: off[p] <= i < off[p+1]
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (off[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  y[i] = (float)(2.0 * e[i] / (sums[2 * lo + 1] * npair) / w[i]);
}

// gc[j][t+K] = y[nb(j,t)] u_j + gu_j b[nb(j,t)]
__global__ void k_band_gc(int N, int K, const float* __restrict__ y, const float* __restrict__ u,
                          const float* __restrict__ gu, const float* __restrict__ b, const int* __restrict__ sst,
                          const int* __restrict__ sln, float* __restrict__ gc) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const int s = sst[j], L = sln[j], P = 2 * K + 1;
  for (int t = -K; t <= K; ++t) {
    const int q = nbr(j, s, L, t);
    gc[(size_t)j * P + t + K] = y[q] * u[j] + gu[j] * b[q];
  }
}

__global__ void k_to_bf16(size_t n, const float* __restrict__ a, __nv_bfloat16* __restrict__ o) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    o[i] = __float2bfloat16_rn(a[i]);
}

// Adam (Kingma & Ba 2015) on the FP32 masters, then the BF16 copy
__global__ void k_adam(size_t n, float* __restrict__ th, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ thb) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float t = th[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    th[i] = t;
    thb[i] = __float2bfloat16_rn(t);
  }
}

size_t conv_smem(int Cin, int Cout) { return ((size_t)NK * Cin * Cout + (size_t)NK * TP * Cin) * sizeof(float); }

}  // namespace
}  // namespace ilm

using namespace ilm;

struct ilm_net_s {
  int nfeat = 8, width = 64, nlayers = 4, band = 4;
  std::vector<int> cin, cout;
  std::vector<size_t> woff, boff;
  size_t nparam = 0;
  DevBuf theta, thb, grad, m, v;
  // work (grown on demand)
  size_t cap = 0, pair_cap = 0;
  DevBuf acts, g0, g1, c, u, e, y, gu, gc, sums, loss, part, partb;
  int step = 0;
  // forward layers on the tcgen05 tensor cores (default) or FP32 FMA; the
  // tensor-core kernels' timeout flag (one int on the device)
  bool tensor_cores = true;
  DevBuf tc_err;
  // the end of the last stream-ordered use of the work buffers and
  // parameters above (a batch's learned set-up, a training step): the next
  // stream-ordered use waits for it on the device (net_after / net_mark),
  // the host-side parameter copies on the host (net_idle), so two launches
  // never share the buffers at once
  cudaEvent_t busy = nullptr;
  int P() const { return 2 * band + 1; }
  ~ilm_net_s() {
    if (busy) {
      cudaEventSynchronize(busy);
      cudaEventDestroy(busy);
    }
  }
};

namespace {

int net_idle(ilm_net_s* n) {
  if (n->busy) ILM_CHECK_CUDA(cudaEventSynchronize(n->busy));
  return ILM_OK;
}
int net_after(ilm_net_s* n, cudaStream_t st) {
  if (n->busy) ILM_CHECK_CUDA(cudaStreamWaitEvent(st, n->busy, 0));
  return ILM_OK;
}
int net_mark(ilm_net_s* n, cudaStream_t st) {
  if (!n->busy) ILM_CHECK_CUDA(cudaEventCreateWithFlags(&n->busy, cudaEventDisableTiming));
  ILM_CHECK_CUDA(cudaEventRecord(n->busy, st));
  return ILM_OK;
}

int net_reserve(ilm_net_s* n, int N, int npair) {
  if ((size_t)N > n->cap) {
    const size_t cap = std::max<size_t>(N, 1024);
    size_t tot = 0;
    for (int l = 0; l < n->nlayers; ++l) tot += (size_t)cap * n->cout[l];
    ILM_TRY(n->acts.alloc(tot * sizeof(float)));
    ILM_TRY(n->g0.alloc(cap * MAXC * sizeof(float)));
    ILM_TRY(n->g1.alloc(cap * MAXC * sizeof(float)));
    ILM_TRY(n->c.alloc(cap * n->P() * sizeof(float)));
    ILM_TRY(n->gc.alloc(cap * n->P() * sizeof(float)));
    ILM_TRY(n->u.alloc(cap * sizeof(float)));
    ILM_TRY(n->e.alloc(cap * sizeof(float)));
    ILM_TRY(n->y.alloc(cap * sizeof(float)));
    ILM_TRY(n->gu.alloc(cap * sizeof(float)));
    const size_t nbx = (cap + WCH - 1) / WCH;
    size_t maxw = 0;
    for (int l = 0; l < n->nlayers; ++l) maxw = std::max(maxw, (size_t)n->cin[l] * n->cout[l] * NK);
    ILM_TRY(n->part.alloc(nbx * maxw * sizeof(float)));
    ILM_TRY(n->partb.alloc(nbx * MAXC * sizeof(float)));
    n->cap = cap;
  }
  if ((size_t)npair > n->pair_cap) {
    ILM_TRY(n->sums.alloc(std::max<size_t>(npair, 64) * 2 * sizeof(double)));
    n->pair_cap = std::max<size_t>(npair, 64);
  }
  if (!n->loss.p) ILM_TRY(n->loss.alloc(sizeof(double)));
  return ILM_OK;
}

float* act_ptr(ilm_net_s* n, int l) {  // output of layer l
  size_t o = 0;
  for (int q = 0; q < l; ++q) o += n->cap * n->cout[q];
  return n->acts.as<float>() + o;
}

int launch_conv(int N, int Cin, int Cout, int mode, bool relu, const __nv_bfloat16* W, const float* bias,
                const float* in, const int* sst, const int* sln, float* out, cudaStream_t st) {
  const size_t smem = conv_smem(Cin, Cout);
  const int blocks = (N + TP - 1) / TP;
  if (blocks == 0) return ILM_OK;
  if (relu) {
    ILM_CHECK_CUDA(cudaFuncSetAttribute(k_conv<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_conv<true><<<blocks, CT, smem, st>>>(N, Cin, Cout, mode, W, bias, in, sst, sln, out);
  } else {
    ILM_CHECK_CUDA(cudaFuncSetAttribute(k_conv<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_conv<false><<<blocks, CT, smem, st>>>(N, Cin, Cout, mode, W, bias, in, sst, sln, out);
  }
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

// forward through all layers; c = band coefficients (N x P)
int net_forward(ilm_net_s* n, int N, const float* feat, const int* sst, const int* sln, float* c, cudaStream_t st) {
  const float* in = feat;
  if (n->tensor_cores && !n->tc_err.p) {
    ILM_TRY(n->tc_err.alloc(sizeof(int)));
    ILM_CHECK_CUDA(cudaMemsetAsync(n->tc_err.p, 0, sizeof(int), st));
  }
  for (int l = 0; l < n->nlayers; ++l) {
    float* out = act_ptr(n, l);
    const bool relu = l < n->nlayers - 1;
    const __nv_bfloat16* W = n->thb.as<__nv_bfloat16>() + n->woff[l];
    const float* bias = n->theta.as<float>() + n->boff[l];
    // the tensor-core kernel gathers 16-byte rows of the input
    if (n->tensor_cores && conv_tc_supported(n->cin[l], n->cout[l]) && (reinterpret_cast<uintptr_t>(in) & 15) == 0)
      ILM_TRY(launch_conv_tc(N, n->cin[l], n->cout[l], relu, W, bias, in, sst, sln, out, n->tc_err.as<int>(), st));
    else
      ILM_TRY(launch_conv(N, n->cin[l], n->cout[l], 0, relu, W, bias, in, sst, sln, out, st));
    in = out;
  }
  const int tot = N * n->P();
  k_band_c<<<std::min(1024, (tot + 255) / 256), 256, 0, st>>>(N, n->band, in, c);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

int net_loss_grad(ilm_net_s* n, int N, int npair, const int* off, const float* feat, const int* sst, const int* sln,
                  const float* w, const float* b, const float* x, cudaStream_t st) {
  ILM_TRY(net_reserve(n, N, npair));
  ILM_TRY(net_forward(n, N, feat, sst, sln, n->c.as<float>(), st));
  const int pb = (N + 255) / 256, K = n->band;
  k_band_fwd<<<pb, 256, 0, st>>>(N, K, n->c.as<float>(), b, sst, sln, n->u.as<float>());
  k_band_z<<<pb, 256, 0, st>>>(N, K, n->c.as<float>(), n->u.as<float>(), w, x, sst, sln, n->e.as<float>());
  k_pair_sums<<<npair, 256, 0, st>>>(off, n->e.as<float>(), x, n->sums.as<double>());
  k_loss_total<<<1, 32, 0, st>>>(npair, n->sums.as<double>(), n->loss.as<double>());
  k_band_gy<<<pb, 256, 0, st>>>(N, npair, off, n->e.as<float>(), w, n->sums.as<double>(), n->y.as<float>());
  k_band_fwd<<<pb, 256, 0, st>>>(N, K, n->c.as<float>(), n->y.as<float>(), sst, sln, n->gu.as<float>());
  k_band_gc<<<pb, 256, 0, st>>>(N, K, n->y.as<float>(), n->u.as<float>(), n->gu.as<float>(), b, sst, sln,
                                n->gc.as<float>());
  ILM_CHECK_LAUNCH();
  // backward through the layers: g holds dL/d(output of layer l)
  float* g = n->gc.as<float>();
  float* gnext = n->g0.as<float>();
  const int nbx = (N + WCH - 1) / WCH;
  for (int l = n->nlayers - 1; l >= 0; --l) {
    const int Ci = n->cin[l], Co = n->cout[l];
    if (l < n->nlayers - 1) {
      k_relu_mask<<<std::min<size_t>(2048, ((size_t)N * Co + 255) / 256), 256, 0, st>>>((size_t)N * Co,
                                                                                         act_ptr(n, l), g);
      ILM_CHECK_LAUNCH();
    }
    const float* a = l == 0 ? feat : act_ptr(n, l - 1);
    k_conv_wgrad<<<dim3(nbx, (Ci + WKS - 1) / WKS), CT, 0, st>>>(N, Ci, Co, g, a, sst, sln, n->part.as<float>(),
                                                                  n->partb.as<float>());
    ILM_CHECK_LAUNCH();
    const int nw = Ci * Co * NK;
    k_reduce_parts<<<(nw + 255) / 256, 256, 0, st>>>(nbx, nw, n->part.as<float>(), n->grad.as<float>() + n->woff[l]);
    k_reduce_parts<<<1, 64, 0, st>>>(nbx, Co, n->partb.as<float>(), n->grad.as<float>() + n->boff[l]);
    ILM_CHECK_LAUNCH();
    if (l > 0) {
      ILM_TRY(launch_conv(N, Co, Ci, 1, false, n->thb.as<__nv_bfloat16>() + n->woff[l], nullptr, g, sst, sln, gnext,
                          st));
      g = gnext;
      gnext = (gnext == n->g0.as<float>()) ? n->g1.as<float>() : n->g0.as<float>();
    }
  }
  return ILM_OK;
}

int check_net_inputs(ilm_net_s* n, int N, const float* feat, const int* sst, const int* sln) {
  ILM_REQUIRE(n && feat && sst && sln, "net: null argument");
  ILM_REQUIRE(N > 0, "net: no points");
  return ILM_OK;
}

}  // namespace

extern "C" {

int ilm_net_create(int nfeat, int width, int nlayers, int band, ilm_net_t* out) {
  ILM_REQUIRE(out, "net: null output");
  ILM_REQUIRE(nfeat >= 1 && nfeat <= MAXC && width >= 1 && width <= MAXC && nlayers >= 2 && nlayers <= 8 &&
                  band >= 0 && 2 * band + 1 <= MAXC,
              "net: unsupported shape (features %d, width %d, layers %d, band %d)", nfeat, width, nlayers, band);
  auto* n = new (std::nothrow) ilm_net_s();
  if (!n) return ILM_ERR_NO_MEMORY;
  std::unique_ptr<ilm_net_s> guard(n);
  n->nfeat = nfeat;
  n->width = width;
  n->nlayers = nlayers;
  n->band = band;
  size_t o = 0;
  for (int l = 0; l < nlayers; ++l) {
    const int ci = l == 0 ? nfeat : width;
    const int co = l == nlayers - 1 ? 2 * band + 1 : width;
    n->cin.push_back(ci);
    n->cout.push_back(co);
    n->woff.push_back(o);
    o += (size_t)co * ci * NK;
    n->boff.push_back(o);
    o += co;
  }
  n->nparam = o;
  ILM_TRY(n->theta.alloc(o * sizeof(float)));
  ILM_TRY(n->thb.alloc(o * sizeof(__nv_bfloat16)));
  ILM_TRY(n->grad.alloc(o * sizeof(float)));
  ILM_TRY(n->m.alloc(o * sizeof(float)));
  ILM_TRY(n->v.alloc(o * sizeof(float)));
  ILM_CHECK_CUDA(cudaMemset(n->theta.p, 0, o * sizeof(float)));
  ILM_CHECK_CUDA(cudaMemset(n->thb.p, 0, o * sizeof(__nv_bfloat16)));
  ILM_CHECK_CUDA(cudaMemset(n->m.p, 0, o * sizeof(float)));
  ILM_CHECK_CUDA(cudaMemset(n->v.p, 0, o * sizeof(float)));
  *out = guard.release();
  return ILM_OK;
}

int ilm_net_destroy(ilm_net_t n) {
  delete n;
  return ILM_OK;
}

int ilm_net_nparams(ilm_net_t n, size_t* count) {
  ILM_REQUIRE(n && count, "net: null argument");
  *count = n->nparam;
  return ILM_OK;
}

int ilm_net_set_params(ilm_net_t n, const float* host) {
  ILM_REQUIRE(n && host, "net: null argument");
  ILM_TRY(net_idle(n));
  ILM_CHECK_CUDA(cudaMemcpy(n->theta.p, host, n->nparam * sizeof(float), cudaMemcpyHostToDevice));
  k_to_bf16<<<256, 256>>>(n->nparam, n->theta.as<float>(), n->thb.as<__nv_bfloat16>());
  ILM_CHECK_LAUNCH();
  ILM_CHECK_CUDA(cudaMemset(n->m.p, 0, n->nparam * sizeof(float)));
  ILM_CHECK_CUDA(cudaMemset(n->v.p, 0, n->nparam * sizeof(float)));
  ILM_CHECK_CUDA(cudaDeviceSynchronize());
  n->step = 0;
  return ILM_OK;
}

int ilm_net_get_params(ilm_net_t n, float* host) {
  ILM_REQUIRE(n && host, "net: null argument");
  ILM_TRY(net_idle(n));
  ILM_CHECK_CUDA(cudaMemcpy(host, n->theta.p, n->nparam * sizeof(float), cudaMemcpyDeviceToHost));
  return ILM_OK;
}

int ilm_net_forward(ilm_net_t n, int npts, const float* feat, const int* seg_start, const int* seg_len,
                    float* band_out, ilm_stream_t stream) {
  ILM_TRY(check_net_inputs(n, npts, feat, seg_start, seg_len));
  ILM_REQUIRE(band_out, "net: null output");
  cudaStream_t st = as_stream(stream);
  ILM_TRY(net_after(n, st));
  ILM_TRY(net_reserve(n, npts, 1));
  ILM_TRY(net_forward(n, npts, feat, seg_start, seg_len, band_out, st));
  ILM_TRY(net_mark(n, st));
  if (!n->tensor_cores) return ILM_OK;
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  return net_check_tc(n);
}

int ilm_net_set_tensor_cores(ilm_net_t n, int enable) {
  ILM_REQUIRE(n, "net: null handle");
  ILM_TRY(net_idle(n));
  n->tensor_cores = enable != 0;
  return ILM_OK;
}

int ilm_net_loss_grad(ilm_net_t n, int npts, int npairs, const int* pair_off, const float* feat,
                      const int* seg_start, const int* seg_len, const float* w, const float* b, const float* x,
                      double* loss_out, float* grad_out, ilm_stream_t stream) {
  ILM_TRY(check_net_inputs(n, npts, feat, seg_start, seg_len));
  ILM_REQUIRE(npairs > 0 && pair_off && w && b && x, "net: bad training inputs");
  cudaStream_t st = as_stream(stream);
  ILM_TRY(net_after(n, st));
  ILM_TRY(net_loss_grad(n, npts, npairs, pair_off, feat, seg_start, seg_len, w, b, x, st));
  ILM_TRY(net_mark(n, st));
  if (loss_out) ILM_CHECK_CUDA(cudaMemcpyAsync(loss_out, n->loss.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  if (grad_out)
    ILM_CHECK_CUDA(cudaMemcpyAsync(grad_out, n->grad.p, n->nparam * sizeof(float), cudaMemcpyDeviceToHost, st));
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  return net_check_tc(n);
}

int ilm_net_train_step(ilm_net_t n, int npts, int npairs, const int* pair_off, const float* feat,
                       const int* seg_start, const int* seg_len, const float* w, const float* b, const float* x,
                       double lr, double* loss_dev, ilm_stream_t stream) {
  ILM_TRY(check_net_inputs(n, npts, feat, seg_start, seg_len));
  ILM_REQUIRE(npairs > 0 && pair_off && w && b && x && lr > 0, "net: bad training inputs");
  cudaStream_t st = as_stream(stream);
  ILM_TRY(net_after(n, st));
  ILM_TRY(net_loss_grad(n, npts, npairs, pair_off, feat, seg_start, seg_len, w, b, x, st));
  n->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)n->step), c2 = 1.f - powf(b2, (float)n->step);
  k_adam<<<std::min<size_t>(512, (n->nparam + 255) / 256), 256, 0, st>>>(
      n->nparam, n->theta.as<float>(), n->grad.as<float>(), n->m.as<float>(), n->v.as<float>(), (float)lr, b1, b2,
      1e-8f, c1, c2, n->thb.as<__nv_bfloat16>());
  ILM_CHECK_LAUNCH();
  if (loss_dev) ILM_CHECK_CUDA(cudaMemcpyAsync(loss_dev, n->loss.p, sizeof(double), cudaMemcpyDeviceToDevice, st));
  return net_mark(n, st);
}

int ilm_point_features(int npts, const double* x, const double* y, const double* nx, const double* ny,
                       const double* ds, const int* seg_start, const int* seg_len, double h, float* out) {
  ILM_REQUIRE(npts >= 0 && (npts == 0 || (x && y && nx && ny && ds && seg_start && seg_len && out)),
              "features: null argument");
  ILM_REQUIRE(h > 0, "features: bad spacing");
  for (int i = 0; i < npts; ++i) {
    const int s = seg_start[i], L = seg_len[i];
    ILM_REQUIRE(L >= 3 && s >= 0 && i >= s && i < s + L && s + L <= npts, "features: bad body segment at %d", i);
    const int ip = s + (i - s + 1) % L, im = s + (i - s + L - 1) % L;
    point_feature(x[i], y[i], nx[i], ny[i], ds[i], nx[ip], ny[ip], ds[ip], nx[im], ny[im], ds[im], h,
                  out + (size_t)i * 8);
  }
  return ILM_OK;
}

}  // extern "C"

// used by the batch solver: network forward over packed points
namespace ilm {
// after a forward has completed: a tensor-core wait that ran out is an error
// the device flag a tensor-core convolution of the forward sets when it gives
// up waiting (nullptr when the FP32 path runs); callers that do not
// synchronise copy it and check it later
int* net_tc_flag(ilm_net_t n) { return n->tensor_cores && n->tc_err.p ? n->tc_err.as<int>() : nullptr; }

int net_check_tc(ilm_net_t n) {
  if (!n->tensor_cores || !n->tc_err.p) return ILM_OK;
  int e = 0;
  ILM_CHECK_CUDA(cudaMemcpy(&e, n->tc_err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    ILM_CHECK_CUDA(cudaMemset(n->tc_err.p, 0, sizeof(int)));
    set_error("learned network: a tensor-core convolution did not complete in time");
    return ILM_ERR_TIMEOUT;
  }
  return ILM_OK;
}
int net_forward_packed(ilm_net_t n, int N, const float* feat, const int* sst, const int* sln, float* band,
                       cudaStream_t st) {
  ILM_TRY(net_after(n, st));
  ILM_TRY(net_reserve(n, N, 1));
  ILM_TRY(net_forward(n, N, feat, sst, sln, band, st));
  return net_mark(n, st);
}
int net_band(ilm_net_t n) { return n->band; }
int net_nfeat(ilm_net_t n) { return n->nfeat; }
}  // namespace ilm
