// Unbounded-domain inverse Laplacian: linear convolution with the lattice
// Green's function (LGF) of the 5-point Laplacian by zero-padded real FFTs.
//
// Replaces CartesianGrids' plan_laplacian(...; with_inverse=true) / `L \ w`
// (called from src/grid_operators.jl:177-179, built at src/cache.jl:321-324).
//
// Pipeline for an n1 x n2 field (x fastest) and padded sizes P1 >= 2 n1 - 1,
// P2 >= 2 n2 - 1 (P = 2^a or 3 * 2^a):
//   1. k_rfft_rows  : each of the n2 rows -> real FFT of length P1 (complex
//                     FFT of P1/2 + split), zero padding pruned on input.
//   2. k_cols       : each of the P1/2+1 spectral columns -> length-P2 complex
//                     FFT, multiply by the real LGF spectrum, inverse FFT; only
//                     the n2 input rows are read and the n2 output rows written.
//   3. k_irfft_rows : each of the n2 rows -> inverse real FFT, first n1 values.
// FP32 transforms of length 64..1024 run as register four-step FFTs (two
// in-register DFT passes, one shared-memory exchange); other lengths and FP64
// use Stockham auto-sort radix-4/3/2 transforms held in shared memory.
// The LGF table and its spectrum are built on the device in FP64 with the same
// kernels and cached per size.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <memory>

#include "ilm_internal.cuh"

namespace ilm {

template <typename T> struct CT;
template <> struct CT<float> { using t = float2; };
template <> struct CT<double> { using t = double2; };

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// s * i * a  (s = +1 or -1)
template <typename C> __device__ __forceinline__ C cmuli(C a, int s) {
  C r; r.x = -s * a.y; r.y = s * a.x; return r;
}

// Stockham auto-sort FFT of `ncol` columns of length L, column c at A[c*cs ..].
// tw: table of length twlen (multiple of L) with tw[m] = exp(-2 pi i m / twlen).
// SIGN = -1 forward, +1 inverse (unnormalised).  Returns the buffer holding
// the result (A or B).  Must be called by all threads of the block.
template <typename T, int SIGN>
__device__ typename CT<T>::t* stockham(typename CT<T>::t* A, typename CT<T>::t* B, int L, int ncol, int cs,
                                      const typename CT<T>::t* __restrict__ tw, int twlen) {
  using C = typename CT<T>::t;
  int Ns = 1;
  int rem = L;
  const T s3 = (T)0.86602540378443864676;
  while (rem > 1) {
    const int r = (rem % 4 == 0) ? 4 : ((rem % 3 == 0) ? 3 : 2);
    const int stride = L / r;
    const int tstep0 = twlen / (Ns * r);
    for (int idx = threadIdx.x; idx < ncol * stride; idx += blockDim.x) {
      const int c = idx / stride;
      const int j = idx - c * stride;
      const C* a_in = A + (size_t)c * cs;
      C* b_out = B + (size_t)c * cs;
      const int k = j % Ns;
      const int tstep = tstep0 * k;
      C a0 = a_in[j];
      C a1 = a_in[j + stride];
      C a2, a3;
      if (r > 2) a2 = a_in[j + 2 * stride];
      if (r > 3) a3 = a_in[j + 3 * stride];
      if (k != 0) {
        C w = tw[tstep];
        if (SIGN > 0) w.y = -w.y;
        a1 = cmul(a1, w);
        if (r > 2) {
          C w2 = tw[2 * tstep];
          if (SIGN > 0) w2.y = -w2.y;
          a2 = cmul(a2, w2);
        }
        if (r > 3) {
          C w3 = tw[3 * tstep];
          if (SIGN > 0) w3.y = -w3.y;
          a3 = cmul(a3, w3);
        }
      }
      const int base = (j / Ns) * Ns * r + k;
      if (r == 2) {
        b_out[base] = cadd(a0, a1);
        b_out[base + Ns] = csub(a0, a1);
      } else if (r == 4) {
        C s02 = cadd(a0, a2), d02 = csub(a0, a2);
        C s13 = cadd(a1, a3), d13 = csub(a1, a3);
        C id = cmuli(d13, SIGN);
        b_out[base] = cadd(s02, s13);
        b_out[base + Ns] = cadd(d02, id);
        b_out[base + 2 * Ns] = csub(s02, s13);
        b_out[base + 3 * Ns] = csub(d02, id);
      } else {  // r == 3
        C s12 = cadd(a1, a2), d12 = csub(a1, a2);
        C m;
        m.x = a0.x - (T)0.5 * s12.x;
        m.y = a0.y - (T)0.5 * s12.y;
        C id = cmuli(d12, SIGN);
        id.x *= s3;
        id.y *= s3;
        b_out[base] = cadd(a0, s12);
        b_out[base + Ns] = cadd(m, id);
        b_out[base + 2 * Ns] = csub(m, id);
      }
    }
    __syncthreads();
    C* t = A;
    A = B;
    B = t;
    Ns *= r;
    rem /= r;
  }
  return A;
}



__device__ __forceinline__ int find_job(const ConvJobDev* jobs, int njobs, int u, bool rows) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    int off = rows ? jobs[mid].row_off : jobs[mid].col_off;
    if (off <= u) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// 1. real row FFTs: in (n1 valid of each row, row-major n2 rows) -> work
template <typename T>
__global__ void k_rfft_rows(const ConvJobDev* __restrict__ jobs, int njobs) {
  using C = typename CT<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int jb = find_job(jobs, njobs, blockIdx.x, true);
  const ConvJobDev J = jobs[jb];
  const int row = blockIdx.x - J.row_off;
  const int H = J.P1 >> 1;
  C* A = reinterpret_cast<C*>(smem_raw);
  C* B = A + H;
  const T* __restrict__ x = static_cast<const T*>(J.in) + (size_t)row * J.n1;
  // input box: rows outside [ra, rb) and columns outside [ca, cb) are zero
  const bool rin = !J.has_box || (row >= J.ra && row < J.rb);
  const int clo = J.has_box ? J.ca : 0, chi = J.has_box ? J.cb : J.n1;
  for (int m = threadIdx.x; m < H; m += blockDim.x) {
    const int i0 = 2 * m;
    C z;
    z.x = rin && i0 >= clo && i0 < chi ? x[i0] : (T)0;
    z.y = rin && i0 + 1 >= clo && i0 + 1 < chi ? x[i0 + 1] : (T)0;
    A[m] = z;
  }
  __syncthreads();
  const C* tw = static_cast<const C*>(J.tw1);
  C* Z = stockham<T, -1>(A, B, H, 1, H, tw, J.P1);
  C* W = static_cast<C*>(J.work) + (size_t)row * (H + 1);
  for (int k = threadIdx.x; k <= H; k += blockDim.x) {
    C zk = Z[k == H ? 0 : k];
    C zc = Z[k == 0 ? 0 : H - k];
    zc.y = -zc.y;
    C e = tw[k];
    C s = cadd(zk, zc), d = csub(zk, zc);
    C ed = cmul(e, d);
    C X;
    X.x = (T)0.5 * (s.x + ed.y);
    X.y = (T)0.5 * (s.y - ed.x);
    W[k] = X;
  }
}

// 2. column pass.  mode 0: FFT, multiply by spectrum, inverse FFT (rows
// [0, n2out) written back).  mode 1: forward FFT only, real part scaled into
// the spectrum array (spectrum build; J.out is the spectrum).
template <typename T>
__global__ void k_cols(const ConvJobDev* __restrict__ jobs, int njobs, int CW, int mode) {
  using C = typename CT<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int jb = find_job(jobs, njobs, blockIdx.x, false);
  const ConvJobDev J = jobs[jb];
  const int H = J.P1 >> 1;
  const int ncols = H + 1;
  const int c0 = (blockIdx.x - J.col_off) * CW;
  const int nc = min(CW, ncols - c0);
  const int P2 = J.P2;
  const int cs = P2 + 1;  // padded column stride (bank conflicts)
  C* A = reinterpret_cast<C*>(smem_raw);
  C* B = A + (size_t)CW * cs;
  C* W = static_cast<C*>(J.work);
  for (int idx = threadIdx.x; idx < nc * P2; idx += blockDim.x) {
    const int row = idx / nc;
    const int c = idx - row * nc;
    C v;
    if (row < J.n2) v = W[(size_t)row * ncols + c0 + c];
    else { v.x = (T)0; v.y = (T)0; }
    A[(size_t)c * cs + row] = v;
  }
  __syncthreads();
  const C* tw = static_cast<const C*>(J.tw2);
  C* F = stockham<T, -1>(A, B, P2, nc, cs, tw, P2);
  C* G = (F == A) ? B : A;
  const int hp2 = P2 / 2 + 1;
  if (mode == 1) {
    T* spec = static_cast<T*>(J.out);
    for (int idx = threadIdx.x; idx < nc * hp2; idx += blockDim.x) {
      const int c = idx / hp2;
      const int ky = idx - c * hp2;
      spec[(size_t)(c0 + c) * hp2 + ky] = (T)(F[(size_t)c * cs + ky].x * J.scale);
    }
    return;
  }
  const T* __restrict__ spec = static_cast<const T*>(J.spec);
  for (int idx = threadIdx.x; idx < nc * P2; idx += blockDim.x) {
    const int c = idx / P2;
    const int ky = idx - c * P2;
    const int kk = ky <= P2 - ky ? ky : P2 - ky;
    const T sv = spec[(size_t)(c0 + c) * hp2 + kk];
    C v = F[(size_t)c * cs + ky];
    v.x *= sv;
    v.y *= sv;
    F[(size_t)c * cs + ky] = v;
  }
  __syncthreads();
  C* R = stockham<T, 1>(F, G, P2, nc, cs, tw, P2);
  for (int idx = threadIdx.x; idx < nc * J.n2out; idx += blockDim.x) {
    const int row = idx / nc;
    const int c = idx - row * nc;
    W[(size_t)row * ncols + c0 + c] = R[(size_t)c * cs + row];
  }
}

// 3. inverse real row FFTs: work -> out (first n1 values of each row) * scale
template <typename T>
__global__ void k_irfft_rows(const ConvJobDev* __restrict__ jobs, int njobs, void* out_base) {
  using C = typename CT<T>::t;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int jb = find_job(jobs, njobs, blockIdx.x, true);
  const ConvJobDev J = jobs[jb];
  const int row = blockIdx.x - J.row_off;
  const int H = J.P1 >> 1;
  C* X = reinterpret_cast<C*>(smem_raw);
  C* A = X + (H + 1);
  C* B = A + H;
  const C* W = static_cast<const C*>(J.work) + (size_t)row * (H + 1);
  for (int k = threadIdx.x; k <= H; k += blockDim.x) X[k] = W[k];
  __syncthreads();
  const C* tw = static_cast<const C*>(J.tw1);
  for (int k = threadIdx.x; k < H; k += blockDim.x) {
    C xk = X[k];
    C xc = X[H - k];
    xc.y = -xc.y;
    C e = tw[k];
    e.y = -e.y;  // exp(+2 pi i k / P1)
    C s = cadd(xk, xc), d = csub(xk, xc);
    C ed = cmul(e, d);
    C z;  // 0.5 * (s + i * ed)
    z.x = (T)0.5 * (s.x - ed.y);
    z.y = (T)0.5 * (s.y + ed.x);
    A[k] = z;
  }
  __syncthreads();
  C* Z = stockham<T, 1>(A, B, H, 1, H, tw, J.P1);
  T* obase = out_base ? reinterpret_cast<T*>(static_cast<unsigned char*>(out_base) + J.out_off)
                      : static_cast<T*>(J.out);
  T* __restrict__ out = obase + (size_t)row * J.n1;
  const T* __restrict__ add = J.add ? static_cast<const T*>(J.add) + (size_t)row * J.n1 : nullptr;
  const T sc = (T)J.scale;
  for (int m = threadIdx.x; m < H; m += blockDim.x) {
    const int i0 = 2 * m;
    C z = Z[m];
    if (i0 < J.n1) out[i0] = add ? add[i0] + z.x * sc : z.x * sc;
    if (i0 + 1 < J.n1) out[i0 + 1] = add ? add[i0 + 1] + z.y * sc : z.y * sc;
  }
}

// ---------------------------------------------------------------------------
// LGF table: G(m,n) = (1/2pi) int_0^pi (1 - cos(p a) e^{-q s}) / sinh s da,
// cosh s = 2 - cos a, p = min(m,n), q = max(m,n); G(0,0) = 0, L G = delta.
// ---------------------------------------------------------------------------
__global__ void k_lgf_table(int M, const double* __restrict__ a, const double* __restrict__ s,
                            const double* __restrict__ wt, int nq, double* __restrict__ out) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = blockIdx.y;
  if (m > M || n > m) return;
  const double p = (double)n, q = (double)m;
  double acc = 0.0;
  for (int j = 0; j < nq; ++j) {
    const double qs = q * s[j];
    const double e = exp(-qs);
    const double sp = sin(0.5 * p * a[j]);
    acc += (-expm1(-qs) + 2.0 * e * sp * sp) * wt[j];
  }
  acc *= 0.15915494309189533577;  // 1/(2 pi)
  out[(size_t)m * (M + 1) + n] = acc;
  out[(size_t)n * (M + 1) + m] = acc;
}

// circulant embedding K[j][i] = G(min(i,P1-i), min(j,P2-j))
__global__ void k_circulant(const double* __restrict__ G, int ld, int P1, int P2, double* __restrict__ K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= P1) return;
  const int ii = min(i, P1 - i), jj = min(j, P2 - j);
  K[(size_t)j * P1 + i] = G[(size_t)ii * ld + jj];
}

__global__ void k_d2f(const double* __restrict__ in, float* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

// ---------------------------------------------------------------------------
// host side: sizes, twiddles, library caches
// ---------------------------------------------------------------------------
// smallest 2^a or 3 * 2^a (>= 4) not below n: every such size from 64 to 1024
// has a register four-step factorisation (N1, N2 in {8, 12, 16, 24, 32})
int good_fft_size(int n) {
  long p2 = 4;
  while (p2 < n) p2 *= 2;
  long p3 = 12;
  while (p3 < n) p3 *= 2;
  return (int)std::min(p2, p3);
}

namespace {

std::mutex g_mu;
struct OwnedDev {
  void* p = nullptr;
  ~OwnedDev() {}
};
std::map<std::pair<int, int>, void*> g_twiddles;             // (L, dtype) -> device table
std::map<std::tuple<int, int, int>, void*> g_spectra;        // (P1, P2, dtype) -> spectrum
int g_lgf_M = -1;
double* g_lgf = nullptr;
float2* g_lgf_ff = nullptr;        // float-float copy of g_lgf
const double* g_lgf_ff_src = nullptr;  // the FP64 table it was split from

void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < n; ++i) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = 0.0;
      for (int k = 1; k <= n; ++k) {
        double p2 = p1;
        p1 = p0;
        p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
      }
      double dp = n * (z * p0 - p1) / (z * z - 1.0);
      double dz = p0 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) {
        p0 = 1.0; p1 = 0.0;
        for (int k = 1; k <= n; ++k) {
          double p2 = p1;
          p1 = p0;
          p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
        }
        dp = n * (z * p0 - p1) / (z * z - 1.0);
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
        break;
      }
    }
  }
}

int twiddle_table(int L, int dtype, const void** out) {
  auto key = std::make_pair(L, dtype);
  auto it = g_twiddles.find(key);
  if (it != g_twiddles.end()) {
    *out = it->second;
    return ILM_OK;
  }
  size_t esz = dtype == ILM_F64 ? 16 : 8;
  std::vector<unsigned char> h((size_t)L * esz);
  for (int m = 0; m < L; ++m) {
    // exact values at the quarter points
    double c, s;
    long long mm = m;
    if ((4LL * mm) % L == 0) {
      int q = (int)((4LL * mm) / L);
      const double cq[4] = {1.0, 0.0, -1.0, 0.0};
      const double sq[4] = {0.0, -1.0, 0.0, 1.0};
      c = cq[q];
      s = sq[q];
    } else {
      double ang = -2.0 * M_PI * (double)m / (double)L;
      c = cos(ang);
      s = sin(ang);
    }
    if (dtype == ILM_F64) {
      double v[2] = {c, s};
      memcpy(&h[(size_t)m * esz], v, esz);
    } else {
      float v[2] = {(float)c, (float)s};
      memcpy(&h[(size_t)m * esz], v, esz);
    }
  }
  void* d = nullptr;
  if (cudaMalloc(&d, h.size()) != cudaSuccess) {
    set_error("cudaMalloc twiddles failed");
    return ILM_ERR_NO_MEMORY;
  }
  ILM_CHECK_CUDA(cudaMemcpy(d, h.data(), h.size(), cudaMemcpyHostToDevice));
  g_twiddles[key] = d;
  *out = d;
  return ILM_OK;
}

// ---------------------------------------------------------------------------
// Register four-step FFTs (FP32 path).  A length L = N1 * N2 transform with
// N1, N2 in {8, 12, 16, 24, 32} (every 2^a and 3 * 2^a from 64 to 1024) is
// done as N2 DFTs of length N1 held in registers, a twiddle by w_L^{k1 n2},
// and N1 DFTs of length N2 held in registers, with one shared-memory exchange
// between them.  The data of one transform sit in shared memory as an
// N1 x (N2 + 1) matrix (row padding keeps both passes free of bank
// conflicts); element n = n1 N2 + n2 is at n1 (N2 + 1) + n2, in natural order
// before and after the transform.
// ---------------------------------------------------------------------------
// exp(-2 pi i k / N) for N = 32 and 24 as literals: in the unrolled register
// DFTs k is a compile-time constant, so the switch folds to an immediate and
// the multiplications by the trivial factors (0, +-1, +-1/2) simplify
__device__ __forceinline__ float2 tw32(int k) {
  switch (k) {
    case 0: return make_float2(1.000000000e+00f, 0.000000000e+00f);
    case 1: return make_float2(9.807852804e-01f, -1.950903220e-01f);
    case 2: return make_float2(9.238795325e-01f, -3.826834324e-01f);
    case 3: return make_float2(8.314696123e-01f, -5.555702330e-01f);
    case 4: return make_float2(7.071067812e-01f, -7.071067812e-01f);
    case 5: return make_float2(5.555702330e-01f, -8.314696123e-01f);
    case 6: return make_float2(3.826834324e-01f, -9.238795325e-01f);
    case 7: return make_float2(1.950903220e-01f, -9.807852804e-01f);
    case 8: return make_float2(0.000000000e+00f, -1.000000000e+00f);
    case 9: return make_float2(-1.950903220e-01f, -9.807852804e-01f);
    case 10: return make_float2(-3.826834324e-01f, -9.238795325e-01f);
    case 11: return make_float2(-5.555702330e-01f, -8.314696123e-01f);
    case 12: return make_float2(-7.071067812e-01f, -7.071067812e-01f);
    case 13: return make_float2(-8.314696123e-01f, -5.555702330e-01f);
    case 14: return make_float2(-9.238795325e-01f, -3.826834324e-01f);
    case 15: return make_float2(-9.807852804e-01f, -1.950903220e-01f);
    case 16: return make_float2(-1.000000000e+00f, 0.000000000e+00f);
    case 17: return make_float2(-9.807852804e-01f, 1.950903220e-01f);
    case 18: return make_float2(-9.238795325e-01f, 3.826834324e-01f);
    case 19: return make_float2(-8.314696123e-01f, 5.555702330e-01f);
    case 20: return make_float2(-7.071067812e-01f, 7.071067812e-01f);
    case 21: return make_float2(-5.555702330e-01f, 8.314696123e-01f);
    case 22: return make_float2(-3.826834324e-01f, 9.238795325e-01f);
    case 23: return make_float2(-1.950903220e-01f, 9.807852804e-01f);
    case 24: return make_float2(0.000000000e+00f, 1.000000000e+00f);
    case 25: return make_float2(1.950903220e-01f, 9.807852804e-01f);
    case 26: return make_float2(3.826834324e-01f, 9.238795325e-01f);
    case 27: return make_float2(5.555702330e-01f, 8.314696123e-01f);
    case 28: return make_float2(7.071067812e-01f, 7.071067812e-01f);
    case 29: return make_float2(8.314696123e-01f, 5.555702330e-01f);
    case 30: return make_float2(9.238795325e-01f, 3.826834324e-01f);
    case 31: return make_float2(9.807852804e-01f, 1.950903220e-01f);
    default: return make_float2(1.f, 0.f);
  }
}
__device__ __forceinline__ float2 tw24(int k) {
  switch (k) {
    case 0: return make_float2(1.000000000e+00f, 0.000000000e+00f);
    case 1: return make_float2(9.659258263e-01f, -2.588190451e-01f);
    case 2: return make_float2(8.660254038e-01f, -5.000000000e-01f);
    case 3: return make_float2(7.071067812e-01f, -7.071067812e-01f);
    case 4: return make_float2(5.000000000e-01f, -8.660254038e-01f);
    case 5: return make_float2(2.588190451e-01f, -9.659258263e-01f);
    case 6: return make_float2(0.000000000e+00f, -1.000000000e+00f);
    case 7: return make_float2(-2.588190451e-01f, -9.659258263e-01f);
    case 8: return make_float2(-5.000000000e-01f, -8.660254038e-01f);
    case 9: return make_float2(-7.071067812e-01f, -7.071067812e-01f);
    case 10: return make_float2(-8.660254038e-01f, -5.000000000e-01f);
    case 11: return make_float2(-9.659258263e-01f, -2.588190451e-01f);
    case 12: return make_float2(-1.000000000e+00f, 0.000000000e+00f);
    case 13: return make_float2(-9.659258263e-01f, 2.588190451e-01f);
    case 14: return make_float2(-8.660254038e-01f, 5.000000000e-01f);
    case 15: return make_float2(-7.071067812e-01f, 7.071067812e-01f);
    case 16: return make_float2(-5.000000000e-01f, 8.660254038e-01f);
    case 17: return make_float2(-2.588190451e-01f, 9.659258263e-01f);
    case 18: return make_float2(0.000000000e+00f, 1.000000000e+00f);
    case 19: return make_float2(2.588190451e-01f, 9.659258263e-01f);
    case 20: return make_float2(5.000000000e-01f, 8.660254038e-01f);
    case 21: return make_float2(7.071067812e-01f, 7.071067812e-01f);
    case 22: return make_float2(8.660254038e-01f, 5.000000000e-01f);
    case 23: return make_float2(9.659258263e-01f, 2.588190451e-01f);
    default: return make_float2(1.f, 0.f);
  }
}

constexpr int FAST_THREADS = 256;

__host__ __device__ constexpr int bitrev_c(int i, int bits) {
  int r = 0;
  for (int b = 0; b < bits; ++b) r |= ((i >> b) & 1) << (bits - 1 - b);
  return r;
}
__host__ __device__ constexpr int ilog2_c(int n) { return n <= 1 ? 0 : 1 + ilog2_c(n / 2); }

// w_N^j (forward sign) for N dividing 32 or 24; conjugated for SIGN > 0
template <int N, int SIGN>
__device__ __forceinline__ float2 twr(int j) {
  float2 w;
  if (32 % N == 0) w = tw32(j * (32 / N));
  else w = tw24(j * (24 / N));
  if (SIGN > 0) w.y = -w.y;
  return w;
}

// in-register radix-2 DIT DFT, N a power of two
template <int N, int SIGN>
__device__ __forceinline__ void dft_pow2(float2 (&a)[N]) {
  constexpr int B = ilog2_c(N);
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const int j = bitrev_c(i, B);
    if (j > i) {
      const float2 t = a[i];
      a[i] = a[j];
      a[j] = t;
    }
  }
#pragma unroll
  for (int half = 1; half < N; half *= 2) {
#pragma unroll
    for (int k = 0; k < N; k += 2 * half) {
#pragma unroll
      for (int j = 0; j < half; ++j) {
        float2 t = a[k + j + half];
        if (j != 0) t = cmul(twr<N, SIGN>(j * (N / (2 * half))), t);
        a[k + j + half] = csub(a[k + j], t);
        a[k + j] = cadd(a[k + j], t);
      }
    }
  }
}

// N = 3 M: three interleaved DFTs of length M and a radix-3 combination
template <int M, int SIGN>
__device__ __forceinline__ void dft_3m(float2 (&a)[3 * M]) {
  constexpr int N = 3 * M;
  float2 b0[M], b1[M], b2[M];
#pragma unroll
  for (int m = 0; m < M; ++m) {
    b0[m] = a[3 * m];
    b1[m] = a[3 * m + 1];
    b2[m] = a[3 * m + 2];
  }
  dft_pow2<M, SIGN>(b0);
  dft_pow2<M, SIGN>(b1);
  dft_pow2<M, SIGN>(b2);
  const float s3 = 0.86602540378443864676f * (float)SIGN;
#pragma unroll
  for (int k = 0; k < M; ++k) {
    float2 t1 = b1[k], t2 = b2[k];
    if (k != 0) {
      t1 = cmul(twr<N, SIGN>(k), t1);
      t2 = cmul(twr<N, SIGN>(2 * k), t2);
    }
    const float2 s = cadd(t1, t2), d = csub(t1, t2);
    float2 m;
    m.x = b0[k].x - 0.5f * s.x;
    m.y = b0[k].y - 0.5f * s.y;
    float2 id;  // i * SIGN * sqrt(3)/2 * d
    id.x = -s3 * d.y;
    id.y = s3 * d.x;
    a[k] = cadd(b0[k], s);
    a[k + M] = cadd(m, id);
    a[k + 2 * M] = csub(m, id);
  }
}

template <int N, int SIGN>
__device__ __forceinline__ void dft_reg(float2 (&a)[N]) {
  if constexpr (N == 12) dft_3m<4, SIGN>(a);
  else if constexpr (N == 24) dft_3m<8, SIGN>(a);
  else dft_pow2<N, SIGN>(a);
}

// One transform of length N1 N2 on the padded matrix x, by the G threads
// g = 0..G-1 of a group (act: this group has a transform).  twL[j * tws] =
// exp(-2 pi i j / (N1 N2)).  Called by every thread of the CTA.
template <int N1, int N2, int SIGN>
__device__ __forceinline__ void fft4step(float2* x, int g, bool act, const float2* __restrict__ twL, int tws) {
  constexpr int ST = N2 + 1;
  if (act && g < N2) {
    float2 a[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) a[n1] = x[n1 * ST + g];
    dft_reg<N1, SIGN>(a);
#pragma unroll
    for (int k1 = 1; k1 < N1; ++k1) {
      float2 w = twL[(size_t)(k1 * g) * tws];
      if (SIGN > 0) w.y = -w.y;
      a[k1] = cmul(w, a[k1]);
    }
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) x[k1 * ST + g] = a[k1];
  }
  __syncthreads();
  float2 b[N2];
  if (act && g < N1) {
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) b[n2] = x[g * ST + n2];
    dft_reg<N2, SIGN>(b);
  }
  __syncthreads();
  if (act && g < N1) {
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
      const int k = g + N1 * k2;
      x[(k / N2) * ST + (k % N2)] = b[k2];
    }
  }
  __syncthreads();
}

template <int N1, int N2>
__device__ __forceinline__ int padpos(int k) {
  return (k / N2) * (N2 + 1) + (k % N2);
}

// Asynchronous global -> shared copies (cp.async, sm_80+): every load of a
// stage is issued before the first one is waited for, so a CTA has its whole
// tile in flight instead of one dependent load per loop trip.  valid = false
// copies nothing and zero-fills the destination (src must still be a valid
// address).
__device__ __forceinline__ void cpa4(void* dst, const void* src, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(src), "r"(valid ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cpa8(void* dst, const void* src, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(src), "r"(valid ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cpa_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// rows: real FFT of length 2H (H = N1 N2) per row, RB rows per CTA starting
// at row r0 (rows up to the job's box end rb); input columns outside the box
// [ca, cb) are zero
template <int N1, int N2>
__device__ void rfft_rows_body(const ConvJobDev& J, int r0, int rend, float2* sm) {
  constexpr int H = N1 * N2, G = N1 > N2 ? N1 : N2, CS = N1 * (N2 + 1);
  constexpr int RB = FAST_THREADS / G;
  const int nr = min(RB, rend - r0);
  const float* __restrict__ in = static_cast<const float*>(J.in);
  const int clo = J.has_box ? J.ca : 0, chi = J.has_box ? J.cb : J.n1;
  for (int idx = threadIdx.x; idx < RB * H; idx += FAST_THREADS) {
    const int r = idx / H, m = idx - r * H;
    float2* d = sm + r * CS + padpos<N1, N2>(m);
    const float* x = in + (size_t)(r0 + (r < nr ? r : 0)) * J.n1;
    const int i0 = 2 * m;
    const bool v0 = r < nr && i0 >= clo && i0 < chi;
    const bool v1 = r < nr && i0 + 1 >= clo && i0 + 1 < chi;
    cpa4(&d->x, v0 ? x + i0 : in, v0);
    cpa4(&d->y, v1 ? x + i0 + 1 : in, v1);
  }
  cpa_wait_all();
  __syncthreads();
  const int r = threadIdx.x / G, g = threadIdx.x - r * G;
  const float2* tw = static_cast<const float2*>(J.tw1);
  fft4step<N1, N2, -1>(sm + (r < RB ? r : 0) * CS, g, r < nr, tw, 2);
  float2* W = static_cast<float2*>(J.work);
  for (int idx = threadIdx.x; idx < nr * (H + 1); idx += FAST_THREADS) {
    const int rr = idx / (H + 1), k = idx - rr * (H + 1);
    const float2* Z = sm + rr * CS;
    const float2 zk = Z[padpos<N1, N2>(k == H ? 0 : k)];
    float2 zc = Z[padpos<N1, N2>(k == 0 ? 0 : H - k)];
    zc.y = -zc.y;
    const float2 e = tw[k];
    const float2 s = cadd(zk, zc), d = csub(zk, zc);
    const float2 ed = cmul(e, d);
    float2 X;
    X.x = 0.5f * (s.x + ed.y);
    X.y = 0.5f * (s.y - ed.x);
    W[(size_t)(r0 + rr) * (H + 1) + k] = X;
  }
}

// inverse rows: the rows' H + 1 spectral values are staged in `raw`
// (RB x (H + 1)).  The thread of k1 forms the half-length complex spectrum
// z[k1 + N1 k2] of the real inverse transform straight from the staged
// values (split of X[k] and X[H - k]) and runs the first inverse stage in
// registers (length-N2 DFT over k2, twiddle w_H^{-n2 k1}); after one
// exchange the thread of n2 runs the length-N1 DFTs over k1 and writes
// z[N2 n1 + n2] = (out[2 m], out[2 m + 1]), m = N2 n1 + n2, first n1 values
// (+ the `add` field, staged while the transforms run)
template <int N1, int N2>
__device__ void irfft_rows_body(const ConvJobDev& J, int r0, float2* sm, float2* raw, void* out_base) {
  constexpr int H = N1 * N2, G = N1 > N2 ? N1 : N2, CS = N1 * (N2 + 1), ST = N2 + 1;
  constexpr int RB = FAST_THREADS / G;
  const int nr = min(RB, J.n2 - r0);
  const float2* __restrict__ tw = static_cast<const float2*>(J.tw1);  // exp(-2 pi i j / 2H)
  const float2* W = static_cast<const float2*>(J.work) + (size_t)r0 * (H + 1);
  for (int idx = threadIdx.x; idx < nr * (H + 1); idx += FAST_THREADS) cpa8(raw + idx, W + idx, true);
  cpa_wait_all();
  __syncthreads();
  const int r = threadIdx.x / G, g = threadIdx.x - r * G;
  const bool act = r < nr;
  float2* x = sm + (r < RB ? r : 0) * CS;
  if (act && g < N1) {
    float2 b[N2];
    const float2* X = raw + r * (H + 1);
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
      const int k = g + N1 * k2;
      const float2 xk = X[k];
      float2 xc = X[H - k];
      xc.y = -xc.y;
      float2 e = tw[k];
      e.y = -e.y;
      const float2 s = cadd(xk, xc), d = csub(xk, xc);
      const float2 ed = cmul(e, d);
      b[k2].x = 0.5f * (s.x - ed.y);
      b[k2].y = 0.5f * (s.y + ed.x);
    }
    dft_reg<N2, 1>(b);
#pragma unroll
    for (int n2 = 1; n2 < N2; ++n2) {
      float2 w = tw[2 * n2 * g];
      w.y = -w.y;
      b[n2] = cmul(w, b[n2]);
    }
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) x[g * ST + n2] = b[n2];
  }
  __syncthreads();
  // the added field's rows go into `raw` (free now; RB (H + 1) float2 >= RB n1
  // floats) while the last stage runs
  const float* __restrict__ add = static_cast<const float*>(J.add);
  float* addr = reinterpret_cast<float*>(raw);
  const int n1 = J.n1;
  if (add) {
    const float* a0 = add + (size_t)r0 * n1;
    for (int idx = threadIdx.x; idx < nr * n1; idx += FAST_THREADS) cpa4(addr + idx, a0 + idx, true);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
  float2 a[N1];
  if (act && g < N2) {
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) a[k1] = x[k1 * ST + g];
    dft_reg<N1, 1>(a);
  }
  if (add) {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
  }
  if (act && g < N2) {
    float* obase = out_base ? reinterpret_cast<float*>(static_cast<unsigned char*>(out_base) + J.out_off)
                            : static_cast<float*>(J.out);
    float* o = obase + (size_t)(r0 + r) * n1;
    const float* ar = addr + r * n1;
    const float sc = (float)J.scale;
#pragma unroll
    for (int q = 0; q < N1; ++q) {
      const int i0 = 2 * (N2 * q + g);
      if (add) {
        if (i0 < n1) o[i0] = ar[i0] + a[q].x * sc;
        if (i0 + 1 < n1) o[i0 + 1] = ar[i0 + 1] + a[q].y * sc;
      } else {
        if (i0 < n1) o[i0] = a[q].x * sc;
        if (i0 + 1 < n1) o[i0 + 1] = a[q].y * sc;
      }
    }
  }
}

// Column pass geometry: CW spectral columns per CTA (8 for transforms whose
// register DFTs use 24 or 32 threads, 16 for 12 or 16, 32 for 8), thread t
// works on column t % CW.  Each column's N1 x (N2 + 1) matrix is padded to
// col_stride() float2 so that the 16 threads of a half-warp (16 columns, or
// 8 columns x 2 rows) hit 16 distinct 8-byte bank pairs.
__host__ __device__ constexpr int col_cw(int G) { return G >= 24 ? 8 : G >= 12 ? 16 : 32; }
__host__ __device__ constexpr int col_stride(int N1, int N2) {
  return col_cw(N1 > N2 ? N1 : N2) == 8 ? (N1 * (N2 + 1) % 4 == 2 ? N1 * (N2 + 1) : N1 * (N2 + 1) + ((6 - N1 * (N2 + 1) % 4) % 4))
                                        : (N1 * (N2 + 1)) | 1;
}

// columns: FFT of length L = N1 N2, spectrum multiply, inverse FFT; only the
// rows [ra, rb) of the row-pass output are read (the rest are zero).  The
// forward four-step transform leaves the thread of k1 holding X[k1 + N1 k2]
// for every k2; the spectrum multiply and the first inverse stage (a
// length-N2 DFT over k2, then the twiddle w_L^{-n2 k1}) run on those
// registers, and the last inverse stage (length-N1 DFTs over k1) gives the
// thread of n2 the outputs x[N2 n1 + n2], which go straight to global
// memory: three shared-memory exchanges for the transform pair.
template <int N1, int N2>
__device__ void cols_body(const ConvJobDev& J, int c0, float2* sm) {
  constexpr int L = N1 * N2, G = N1 > N2 ? N1 : N2, ST = N2 + 1;
  constexpr int CW = col_cw(G), CS = col_stride(N1, N2);
  const int ncols = (J.P1 >> 1) + 1;
  const int nc = min(CW, ncols - c0);
  const int ra = J.has_box ? J.ra : 0, rb = J.has_box ? J.rb : J.n2;
  float2* W = static_cast<float2*>(J.work);
  for (int idx = threadIdx.x; idx < CW * L; idx += FAST_THREADS) {
    const int c = idx % CW, row = idx / CW;
    const bool v = c < nc && row >= ra && row < rb;
    cpa8(sm + c * CS + padpos<N1, N2>(row), v ? W + (size_t)row * ncols + c0 + c : W, v);
  }
  cpa_wait_all();
  __syncthreads();
  const int c = threadIdx.x % CW, g = threadIdx.x / CW;
  const bool act = c < nc && g < G;
  float2* x = sm + c * CS;
  const float2* __restrict__ tw = static_cast<const float2*>(J.tw2);
  // forward stage 1: length-N1 DFTs over n1 (thread n2 = g), twiddle w_L^{k1 n2}
  if (act && g < N2) {
    float2 a[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) a[n1] = x[n1 * ST + g];
    dft_reg<N1, -1>(a);
#pragma unroll
    for (int k1 = 1; k1 < N1; ++k1) a[k1] = cmul(tw[k1 * g], a[k1]);
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) x[k1 * ST + g] = a[k1];
  }
  __syncthreads();
  // forward stage 2 (thread k1 = g): X[k1 + N1 k2]; spectrum; inverse stage A
  if (act && g < N1) {
    float2 b[N2];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) b[n2] = x[g * ST + n2];
    dft_reg<N2, -1>(b);
    const float* __restrict__ spec = static_cast<const float*>(J.spec) + (size_t)(c0 + c) * (L / 2 + 1);
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) {
      const int k = g + N1 * k2;
      const float sv = __ldg(spec + (k <= L - k ? k : L - k));
      b[k2].x *= sv;
      b[k2].y *= sv;
    }
    dft_reg<N2, 1>(b);
#pragma unroll
    for (int n2 = 1; n2 < N2; ++n2) {
      float2 w = tw[n2 * g];
      w.y = -w.y;
      b[n2] = cmul(w, b[n2]);
    }
    // the thread reads and writes only its own row g of the matrix
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) x[g * ST + n2] = b[n2];
  }
  __syncthreads();
  // inverse stage B (thread n2 = g): length-N1 DFTs over k1 -> x[N2 n1 + n2]
  if (act && g < N2) {
    float2 a[N1];
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) a[k1] = x[k1 * ST + g];
    dft_reg<N1, 1>(a);
    float2* wc = W + c0 + c;
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) {
      const int row = N2 * n1 + g;
      if (row < J.n2out) wc[(size_t)row * ncols] = a[n1];
    }
  }
}

// dispatch on the transform length (block-uniform)
#define ILM_FAST_SWITCH(L, CALL)                 \
  switch (L) {                                   \
    case 64: CALL(8, 8); break;                  \
    case 96: CALL(8, 12); break;                 \
    case 128: CALL(8, 16); break;                \
    case 192: CALL(8, 24); break;                \
    case 256: CALL(16, 16); break;               \
    case 384: CALL(16, 24); break;               \
    case 512: CALL(16, 32); break;               \
    case 768: CALL(24, 32); break;               \
    case 1024: CALL(32, 32); break;              \
    default: break;                              \
  }

// which: 0 forward rows (frow_off), 1 columns (col_off), 2 inverse rows (irow_off)
__device__ __forceinline__ int find_job_fast(const ConvJobDev* jobs, int njobs, int u, int which) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const int off = which == 0 ? jobs[mid].frow_off : which == 1 ? jobs[mid].col_off : jobs[mid].irow_off;
    if (off <= u) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(FAST_THREADS)
    k_rfft_rows_fast(const ConvJobDev* __restrict__ jobs, int njobs, const int* __restrict__ bmap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* sm = reinterpret_cast<float2*>(smem_raw);
  const int jb = bmap ? bmap[blockIdx.x] : find_job_fast(jobs, njobs, blockIdx.x, 0);
  const ConvJobDev J = jobs[jb];
  const int ra = J.has_box ? J.ra : 0, rb = J.has_box ? J.rb : J.n2;
  const int r0 = ra + (blockIdx.x - J.frow_off) * J.frb;
#define ILM_CALL_RF(a, b) rfft_rows_body<a, b>(J, r0, rb, sm)
  ILM_FAST_SWITCH(J.P1 >> 1, ILM_CALL_RF)
#undef ILM_CALL_RF
}

__global__ void __launch_bounds__(FAST_THREADS)
    k_irfft_rows_fast(const ConvJobDev* __restrict__ jobs, int njobs, void* out_base, const int* __restrict__ bmap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* sm = reinterpret_cast<float2*>(smem_raw);
  const int jb = bmap ? bmap[blockIdx.x] : find_job_fast(jobs, njobs, blockIdx.x, 2);
  const ConvJobDev J = jobs[jb];
  const int r0 = (blockIdx.x - J.irow_off) * J.frb;
  // layout: the transforms' padded matrices (frb x N1 (N2 + 1)), then the
  // staging rows (frb x (H + 1)); both sizes are multiples of 8 bytes
#define ILM_CALL_IRF(a, b) \
  irfft_rows_body<a, b>(J, r0, sm, sm + (size_t)J.frb * (a) * ((b) + 1), out_base)
  ILM_FAST_SWITCH(J.P1 >> 1, ILM_CALL_IRF)
#undef ILM_CALL_IRF
}

__global__ void __launch_bounds__(FAST_THREADS, 2)
    k_cols_fast(const ConvJobDev* __restrict__ jobs, int njobs, const int* __restrict__ bmap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* sm = reinterpret_cast<float2*>(smem_raw);
  const int jb = bmap ? bmap[blockIdx.x] : find_job_fast(jobs, njobs, blockIdx.x, 1);
  const ConvJobDev J = jobs[jb];
  const int c0 = (blockIdx.x - J.col_off) * J.fcw;
#define ILM_CALL_C(a, b) cols_body<a, b>(J, c0, sm)
  ILM_FAST_SWITCH(J.P2, ILM_CALL_C)
#undef ILM_CALL_C
}

// host: factor of a fast length (0 if none), threads per transform, smem
bool fast_len(int L, int* n1, int* n2) {
  static const int tab[][3] = {{64, 8, 8},    {96, 8, 12},   {128, 8, 16},  {192, 8, 24},   {256, 16, 16},
                               {384, 16, 24}, {512, 16, 32}, {768, 24, 32}, {1024, 32, 32}};
  for (const auto& t : tab)
    if (t[0] == L) {
      *n1 = t[1];
      *n2 = t[2];
      return true;
    }
  return false;
}

size_t fast_transform_floats2(int L) {  // padded matrix size of one transform (float2)
  int a, b;
  if (!fast_len(L, &a, &b)) return 0;
  return (size_t)a * (b + 1);
}

int fast_group(int L) {
  int a, b;
  fast_len(L, &a, &b);
  return a > b ? a : b;
}

int ensure_fast_tables() { return ILM_OK; }  // the register DFTs' factors are literals (tw32 / tw24)

template <typename T>
size_t rows_smem(int P1) { return (size_t)(3 * (P1 / 2) + 2) * sizeof(typename CT<T>::t); }

template <typename T>
int cols_cw(int P2) {
  const size_t budget = 200 * 1024;
  size_t per = (size_t)2 * (P2 + 1) * sizeof(typename CT<T>::t);
  int cw = (int)(budget / per);
  if (cw > 16) cw = 16;
  if (cw < 1) cw = 1;
  return cw;
}

template <typename T>
int launch_prepared(const ConvJobDev* jd, int nj, const ConvLaunch& L, int mode, cudaStream_t st,
                    void* out_base = nullptr) {
  if (L.fast && mode == 0 && sizeof(T) == 4) {
    ILM_CHECK_CUDA(cudaFuncSetAttribute(k_rfft_rows_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.fsm_rows));
    ILM_CHECK_CUDA(cudaFuncSetAttribute(k_cols_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.fsm_cols));
    ILM_CHECK_CUDA(cudaFuncSetAttribute(k_irfft_rows_fast, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)L.fsm_irows));
    if (L.frows > 0) k_rfft_rows_fast<<<L.frows, FAST_THREADS, L.fsm_rows, st>>>(jd, nj, L.dmap[0]);
    ILM_CHECK_LAUNCH();
    k_cols_fast<<<L.cols, FAST_THREADS, L.fsm_cols, st>>>(jd, nj, L.dmap[1]);
    ILM_CHECK_LAUNCH();
    k_irfft_rows_fast<<<L.firows, FAST_THREADS, L.fsm_irows, st>>>(jd, nj, out_base, L.dmap[2]);
    ILM_CHECK_LAUNCH();
    return ILM_OK;
  }
  size_t sm_rows = rows_smem<T>(L.maxP1);
  size_t sm_cols = (size_t)2 * L.CW * (L.maxP2 + 1) * sizeof(typename CT<T>::t);
  ILM_CHECK_CUDA(cudaFuncSetAttribute(k_rfft_rows<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_rows));
  ILM_CHECK_CUDA(cudaFuncSetAttribute(k_cols<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_cols));
  ILM_CHECK_CUDA(cudaFuncSetAttribute(k_irfft_rows<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_rows));
  k_rfft_rows<T><<<L.rows, 256, sm_rows, st>>>(jd, nj);
  ILM_CHECK_LAUNCH();
  k_cols<T><<<L.cols, 256, sm_cols, st>>>(jd, nj, L.CW, mode);
  ILM_CHECK_LAUNCH();
  if (mode == 0) {
    k_irfft_rows<T><<<L.rows, 256, sm_rows, st>>>(jd, nj, out_base);
    ILM_CHECK_LAUNCH();
  }
  return ILM_OK;
}

template <typename T>
int launch_conv_jobs(const std::vector<ConvJobDev>& jobs_in, int mode, cudaStream_t st, void* jobs_dev_buf) {
  std::vector<ConvJobDev> jobs = jobs_in;
  ConvLaunch L;
  ILM_TRY(conv_jobs_finalize(jobs, sizeof(T) == 8 ? ILM_F64 : ILM_F32, &L));
  ILM_CHECK_CUDA(cudaMemcpyAsync(jobs_dev_buf, jobs.data(), jobs.size() * sizeof(ConvJobDev),
                                 cudaMemcpyHostToDevice, st));
  return launch_prepared<T>(static_cast<const ConvJobDev*>(jobs_dev_buf), (int)jobs.size(), L, mode, st);
}

}  // namespace

int lgf_table_device(int M, const double** tab, int* ld, cudaStream_t st) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_lgf && g_lgf_M >= M) {
    *tab = g_lgf;
    *ld = g_lgf_M + 1;
    return ILM_OK;
  }
  // grow geometrically to limit rebuilds
  int MM = std::max(M, g_lgf_M > 0 ? std::min(2 * g_lgf_M, 1 << 14) : M);
  if (MM < M) MM = M;
  std::vector<double> xg, wg;
  gauss_legendre(24, xg, wg);
  const int levels = 40;
  std::vector<double> ha, hs, hw;
  std::vector<double> edges;
  edges.push_back(0.0);
  for (int k = levels; k >= 0; --k) edges.push_back(M_PI * ldexp(1.0, -k));
  for (size_t e = 0; e + 1 < edges.size(); ++e) {
    double lo = edges[e], hi = edges[e + 1];
    for (int i = 0; i < 24; ++i) {
      double al = 0.5 * (hi - lo) * xg[i] + 0.5 * (hi + lo);
      double w = 0.5 * (hi - lo) * wg[i];
      double sh2 = sin(0.5 * al);
      double u = 2.0 * sh2 * sh2;
      double sh = sqrt(u * (u + 2.0));
      double s = log1p(u + sh);
      ha.push_back(al);
      hs.push_back(s);
      hw.push_back(w / sh);
    }
  }
  const int nq = (int)ha.size();
  DevBuf da, ds, dw;
  ILM_TRY(da.alloc(nq * sizeof(double)));
  ILM_TRY(ds.alloc(nq * sizeof(double)));
  ILM_TRY(dw.alloc(nq * sizeof(double)));
  ILM_CHECK_CUDA(cudaMemcpy(da.p, ha.data(), nq * sizeof(double), cudaMemcpyHostToDevice));
  ILM_CHECK_CUDA(cudaMemcpy(ds.p, hs.data(), nq * sizeof(double), cudaMemcpyHostToDevice));
  ILM_CHECK_CUDA(cudaMemcpy(dw.p, hw.data(), nq * sizeof(double), cudaMemcpyHostToDevice));
  double* d = nullptr;
  size_t bytes = (size_t)(MM + 1) * (MM + 1) * sizeof(double);
  if (cudaMalloc(&d, bytes) != cudaSuccess) {
    set_error("cudaMalloc LGF table (%zu bytes) failed", bytes);
    return ILM_ERR_NO_MEMORY;
  }
  dim3 grid((MM + 1 + 127) / 128, MM + 1);
  k_lgf_table<<<grid, 128, 0, st>>>(MM, da.as<double>(), ds.as<double>(), dw.as<double>(), nq, d);
  ILM_CHECK_LAUNCH();
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  if (g_lgf) cudaFree(g_lgf);
  g_lgf = d;
  g_lgf_M = MM;
  *tab = g_lgf;
  *ld = MM + 1;
  return ILM_OK;
}

__global__ void k_split_ff(size_t n, const double* __restrict__ a, float2* __restrict__ out) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k < n) {
    const double v = a[k];
    const float h = (float)v;
    out[k] = make_float2(h, (float)(v - (double)h));
  }
}

// The LGF table as float-float pairs (hi, lo), for the float-float Schur
// build; rebuilt whenever the FP64 table grows.
int lgf_table_ff_device(int M, const float2** tab, int* ld, cudaStream_t st) {
  const double* G = nullptr;
  int ldd = 0;
  ILM_TRY(lgf_table_device(M, &G, &ldd, st));
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_lgf_ff && g_lgf_ff_src == G) {
    *tab = g_lgf_ff;
    *ld = ldd;
    return ILM_OK;
  }
  const size_t n = (size_t)ldd * ldd;
  float2* d = nullptr;
  if (cudaMalloc(&d, n * sizeof(float2)) != cudaSuccess) {
    set_error("cudaMalloc float-float LGF table (%zu bytes) failed", n * sizeof(float2));
    return ILM_ERR_NO_MEMORY;
  }
  k_split_ff<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, G, d);
  ILM_CHECK_LAUNCH();
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  if (g_lgf_ff) cudaFree(g_lgf_ff);
  g_lgf_ff = d;
  g_lgf_ff_src = G;
  *tab = g_lgf_ff;
  *ld = ldd;
  return ILM_OK;
}

static int spectrum_device(int P1, int P2, int dtype, const void** out, cudaStream_t st) {
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_spectra.find(std::make_tuple(P1, P2, dtype));
    if (it != g_spectra.end()) {
      *out = it->second;
      return ILM_OK;
    }
  }
  const double* G = nullptr;
  int ld = 0;
  ILM_TRY(lgf_table_device(std::max(P1, P2) / 2, &G, &ld, st));
  const void *tw1 = nullptr, *tw2 = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    ILM_TRY(twiddle_table(P1, ILM_F64, &tw1));
    ILM_TRY(twiddle_table(P2, ILM_F64, &tw2));
  }
  DevBuf K, W, S64, jobsb;
  ILM_TRY(K.alloc((size_t)P1 * P2 * sizeof(double)));
  ILM_TRY(W.alloc((size_t)P2 * (P1 / 2 + 1) * 2 * sizeof(double)));
  const size_t nspec = (size_t)(P1 / 2 + 1) * (P2 / 2 + 1);
  ILM_TRY(S64.alloc(nspec * sizeof(double)));
  ILM_TRY(jobsb.alloc(sizeof(ConvJobDev)));
  k_circulant<<<dim3((P1 + 255) / 256, P2), 256, 0, st>>>(G, ld, P1, P2, K.as<double>());
  ILM_CHECK_LAUNCH();
  ConvJobDev J;
  memset(&J, 0, sizeof(J));
  J.in = K.p;
  J.out = S64.p;
  J.work = W.p;
  J.tw1 = tw1;
  J.tw2 = tw2;
  J.n1 = P1;
  J.n2 = P2;
  J.n2out = P2;
  J.P1 = P1;
  J.P2 = P2;
  // unnormalised r2c -> column FFT pair -> c2r gives a factor (P1/2) * P2
  J.scale = 1.0 / ((double)(P1 / 2) * (double)P2);
  std::vector<ConvJobDev> jobs{J};
  ILM_TRY(launch_conv_jobs<double>(jobs, 1, st, jobsb.p));
  void* d = nullptr;
  if (dtype == ILM_F64) {
    if (cudaMalloc(&d, nspec * sizeof(double)) != cudaSuccess) return ILM_ERR_NO_MEMORY;
    ILM_CHECK_CUDA(cudaMemcpyAsync(d, S64.p, nspec * sizeof(double), cudaMemcpyDeviceToDevice, st));
  } else {
    if (cudaMalloc(&d, nspec * sizeof(float)) != cudaSuccess) return ILM_ERR_NO_MEMORY;
    k_d2f<<<256, 256, 0, st>>>(S64.as<double>(), static_cast<float*>(d), nspec);
    ILM_CHECK_LAUNCH();
  }
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  std::lock_guard<std::mutex> lk(g_mu);
  g_spectra[std::make_tuple(P1, P2, dtype)] = d;
  *out = d;
  return ILM_OK;
}

int conv_plan_init(ConvPlan* plan, int n1, int n2, int dtype, cudaStream_t st) {
  plan->n1 = n1;
  plan->n2 = n2;
  plan->dtype = dtype;
  plan->P1 = good_fft_size(2 * n1 - 1);
  plan->P2 = good_fft_size(2 * n2 - 1);
  if (plan->P1 > 8192 || plan->P2 > 8192) {
    set_error("grid too large for the FFT convolution (P=%d x %d)", plan->P1, plan->P2);
    return ILM_ERR_SIZE_LIMIT;
  }
  ILM_TRY(spectrum_device(plan->P1, plan->P2, dtype, &plan->spec, st));
  {
    std::lock_guard<std::mutex> lk(g_mu);
    ILM_TRY(twiddle_table(plan->P1, dtype, &plan->tw1));
    ILM_TRY(twiddle_table(plan->P2, dtype, &plan->tw2));
  }
  size_t csz = dtype == ILM_F64 ? 16 : 8;
  ILM_TRY(plan->work.alloc((size_t)n2 * (plan->P1 / 2 + 1) * csz + 256));
  return ILM_OK;
}

int conv_apply(ConvPlan* plan, const void* in, void* out, double inv_factor, cudaStream_t st) {
  ConvJobDev J;
  memset(&J, 0, sizeof(J));
  J.in = in;
  J.out = out;
  J.work = plan->work.p;
  J.spec = plan->spec;
  J.tw1 = plan->tw1;
  J.tw2 = plan->tw2;
  J.n1 = plan->n1;
  J.n2 = plan->n2;
  J.n2out = plan->n2;
  J.P1 = plan->P1;
  J.P2 = plan->P2;
  J.scale = inv_factor;
  std::vector<ConvJobDev> jobs{J};
  // job descriptor lives in the tail of the work buffer
  size_t csz = plan->dtype == ILM_F64 ? 16 : 8;
  size_t off = (size_t)plan->n2 * (plan->P1 / 2 + 1) * csz;
  void* jb = static_cast<unsigned char*>(plan->work.p) + ((off + 15) / 16) * 16;
  if (((off + 15) / 16) * 16 + sizeof(ConvJobDev) > plan->work.bytes) {
    set_error("conv work buffer too small");
    return ILM_ERR_INVALID_ARG;
  }
  if (plan->dtype == ILM_F64) return launch_conv_jobs<double>(jobs, 0, st, jb);
  return launch_conv_jobs<float>(jobs, 0, st, jb);
}

int conv_jobs_finalize(std::vector<ConvJobDev>& jobs, int dtype, ConvLaunch* L) {
  int rows = 0, cols = 0, maxP1 = 0, maxP2 = 0;
  bool fast = dtype == ILM_F32 && !jobs.empty();
  for (auto& J : jobs) {
    if (J.has_box && !(J.ra >= 0 && J.ra < J.rb && J.rb <= J.n2 && J.ca >= 0 && J.ca < J.cb && J.cb <= J.n1)) {
      set_error("convolution input box [%d,%d) x [%d,%d) outside the %d x %d field", J.ca, J.cb, J.ra, J.rb, J.n1,
                J.n2);
      return ILM_ERR_INVALID_ARG;
    }
    maxP1 = std::max(maxP1, J.P1);
    maxP2 = std::max(maxP2, J.P2);
    int a, b;
    fast = fast && fast_len(J.P1 / 2, &a, &b) && fast_len(J.P2, &a, &b);
  }
  if (fast) {  // register four-step FFTs: rows in groups, 8 spectral columns per CTA
    ILM_TRY(ensure_fast_tables());
    size_t smr = 0, smc = 0, smi = 0;
    int frows = 0, firows = 0;
    L->mrows.clear();
    L->mcols.clear();
    L->mirows.clear();
    for (size_t jn = 0; jn < jobs.size(); ++jn) {
      ConvJobDev& J = jobs[jn];
      const int H = J.P1 / 2;
      J.frb = FAST_THREADS / fast_group(H);
      J.frow_off = frows;
      const int nbox = J.has_box ? J.rb - J.ra : J.n2;
      frows += (nbox + J.frb - 1) / J.frb;
      J.irow_off = firows;
      firows += (J.n2 + J.frb - 1) / J.frb;
      J.row_off = 0;
      J.col_off = cols;
      int n1c, n2c;
      fast_len(J.P2, &n1c, &n2c);
      J.fcw = col_cw(std::max(n1c, n2c));
      cols += (H + 1 + J.fcw - 1) / J.fcw;
      L->mrows.resize(frows, (int)jn);
      L->mcols.resize(cols, (int)jn);
      L->mirows.resize(firows, (int)jn);
      const size_t tr = (size_t)J.frb * fast_transform_floats2(H) * sizeof(float2);
      smr = std::max(smr, tr);
      smi = std::max(smi, tr + (size_t)J.frb * (H + 1) * sizeof(float2));
      smc = std::max(smc, (size_t)J.fcw * col_stride(n1c, n2c) * sizeof(float2));
    }
    L->fast = 1;
    L->frows = frows;
    L->firows = firows;
    L->fsm_irows = smi;
    L->rows = 0;
    L->cols = cols;
    L->CW = 0;  // per job (ConvJobDev::fcw)
    L->maxP1 = maxP1;
    L->maxP2 = maxP2;
    L->fsm_rows = smr;
    L->fsm_cols = smc;
    return ILM_OK;
  }
  L->fast = 0;
  const int CW = dtype == ILM_F64 ? cols_cw<double>(maxP2) : cols_cw<float>(maxP2);
  for (auto& J : jobs) {
    J.row_off = rows;
    rows += J.n2;
    J.col_off = cols;
    cols += (J.P1 / 2 + 1 + CW - 1) / CW;
  }
  L->rows = rows;
  L->cols = cols;
  L->CW = CW;
  L->maxP1 = maxP1;
  L->maxP2 = maxP2;
  return ILM_OK;
}

int conv_jobs_launch(const ConvJobDev* jobs_dev, int njobs, const ConvLaunch& L, int dtype, cudaStream_t st,
                     void* out_base) {
  if (njobs == 0) return ILM_OK;
  if (dtype == ILM_F64) return launch_prepared<double>(jobs_dev, njobs, L, 0, st, out_base);
  return launch_prepared<float>(jobs_dev, njobs, L, 0, st, out_base);
}

int conv_resources(int P1, int P2, int dtype, const void** spec, const void** tw1, const void** tw2, cudaStream_t st) {
  ILM_TRY(spectrum_device(P1, P2, dtype, spec, st));
  std::lock_guard<std::mutex> lk(g_mu);
  ILM_TRY(twiddle_table(P1, dtype, tw1));
  ILM_TRY(twiddle_table(P2, dtype, tw2));
  return ILM_OK;
}

}  // namespace ilm
