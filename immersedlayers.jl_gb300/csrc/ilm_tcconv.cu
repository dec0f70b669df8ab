// Forward 1-D convolution of the learned preconditioner's network on the
// 5th-generation tensor cores (tcgen05, accumulators in tensor memory).
//
// One layer, out[i][o] = bias[o] + sum_{t,c} W[o][c][t] in[nb(i, t-2)][c]
// (optionally ReLU), is an implicit GEMM D = A B with M = points (128 per
// CTA), K = 5 taps x Cin (padded to a multiple of 16) and N = Cout (padded
// to a multiple of 16):
//   A[r][t Cin + c] = in[nb(p0 + r, t - 2)][c]   (gathered along arc length,
//                                                 circular per body)
//   B[o][t Cin + c] = W[o][c][t]                  (BF16 weights, K-major)
// The activations are FP32; they enter the BF16 MMA as a hi/lo pair
// (hi = bf16(a), lo = bf16(a - hi)) and D = A_hi B + A_lo B accumulates in
// FP32 in tensor memory, so the layer matches the FP32-FMA path (k_conv) to
// ~2^-16 relative per product instead of BF16's 2^-8.  A and B are staged in
// shared memory in the no-swizzle canonical K-major layout (8 x 16-byte core
// matrices; K-adjacent core matrices 128 B apart, 8-row groups K/8 x 128 B
// apart); one thread issues the MMAs (M = 128, N = Np, K = 16 each) and
// commits them to an mbarrier; the epilogue reads D back with tcgen05.ld
// (warp w: lanes 32 (w % 4) .. +31, column half w / 4), adds the bias,
// applies ReLU and stores FP32.
//
// Every wait is bounded: a CTA whose MMA completion does not arrive within
// the limit records an error flag (checked by the host after the forward),
// skips its epilogue and still frees its tensor memory.
#include "ilm_internal.cuh"

namespace ilm {
namespace {

constexpr int TC_M = 128;        // points per CTA (TMEM lanes)
constexpr int TC_THREADS = 256;  // 8 warps: staging by all, epilogue as 2 x 4 lane quarters
constexpr int TC_NK = 5;         // taps
constexpr long long TC_SPIN_LIMIT = 1ll << 24;

__device__ __forceinline__ int tc_nbr(int i, int s, int L, int t) {
  if (L < 1) return i;
  int q = (i - s + t) % L;
  q += q < 0 ? L : 0;
  return s + q;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor: no swizzle, K-major, start address,
// LBO = byte stride of K-adjacent core matrices, SBO = byte stride of
// 8-row groups, descriptor version 1
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// byte offset of element (row, k) in a K-major no-swizzle tile with kp
// (padded) columns
__device__ __forceinline__ uint32_t tc_off(int row, int k, int kp) {
  return (uint32_t)((row >> 3) * (kp >> 3) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

template <int NC>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t (&v)[NC]);

template <>
__device__ __forceinline__ void tmem_ld<8>(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr));
}

template <>
__device__ __forceinline__ void tmem_ld<32>(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}

// NP: padded output channels (16 or 64); CIN: input channels (a multiple of
// 4); TMEM columns allocated: max(NP, 32)
template <int NP, bool RELU, int CIN>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_conv_tc(int N, int Cout, const __nv_bfloat16* __restrict__ W, const float* __restrict__ bias,
          const float* __restrict__ in, const int* __restrict__ sst, const int* __restrict__ sln,
          float* __restrict__ out, int* __restrict__ err) {
  constexpr uint32_t TCOLS = NP < 32 ? 32 : NP;
  constexpr int K = TC_NK * CIN;
  constexpr int kp = ((K + 15) / 16) * 16;
  constexpr int Cin = CIN;
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_timeout;
  __shared__ int s_nb[TC_M * TC_NK];  // neighbour index of every (row, tap)
  unsigned char* a_hi = smem;                               // TC_M x kp BF16
  unsigned char* a_lo = a_hi + (size_t)TC_M * kp * 2;       // TC_M x kp BF16
  unsigned char* bm = a_lo + (size_t)TC_M * kp * 2;         // NP x kp BF16
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int p0 = blockIdx.x * TC_M;

  // tensor memory for the accumulator (one warp allocates for the CTA)
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    s_timeout = 0;
  }
  // neighbours along arc length of every row and tap (rows past N: -1)
  for (int e = tid; e < TC_M * TC_NK; e += TC_THREADS) {
    const int r = e / TC_NK, t = e % TC_NK, i = p0 + r;
    s_nb[e] = i < N ? tc_nbr(i, sst[i], sln[i], t - 2) : -1;
  }
  // B: weights, B[o][t Cin + c] = W[o][c][t]; zero padding rows / columns
  for (int e = tid; e < NP * kp; e += TC_THREADS) {
    const int o = e / kp, k = e % kp;
    __nv_bfloat16 v = __float2bfloat16(0.f);
    if (o < Cout && k < K) {
      const int t = k / Cin, c = k % Cin;
      v = W[((size_t)o * Cin + c) * TC_NK + t];
    }
    *reinterpret_cast<__nv_bfloat16*>(bm + tc_off(o, k, kp)) = v;
  }
  // zero K padding of A (columns K .. kp)
  if (kp > K)
    for (int e = tid; e < TC_M * (kp - K); e += TC_THREADS) {
      const int r = e / (kp - K), k = K + e % (kp - K);
      const uint32_t off = tc_off(r, k, kp);
      *reinterpret_cast<__nv_bfloat16*>(a_hi + off) = __float2bfloat16(0.f);
      *reinterpret_cast<__nv_bfloat16*>(a_lo + off) = __float2bfloat16(0.f);
    }
  __syncthreads();
  // A: gathered activations as a hi / lo BF16 pair, four channels per item
  // (one 16-byte load, two 8-byte shared stores: 4 consecutive k stay in one
  // 16-byte core-matrix row because t Cin + 4 c4 is a multiple of 4)
  constexpr int C4 = CIN / 4;
  for (int e = tid; e < TC_M * TC_NK * C4; e += TC_THREADS) {
    const int r = e / (TC_NK * C4), t = (e / C4) % TC_NK, c4 = e % C4;
    const int j = s_nb[r * TC_NK + t];
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (j >= 0) v = __ldg(reinterpret_cast<const float4*>(in + (size_t)j * Cin) + c4);
    const float vv[4] = {v.x, v.y, v.z, v.w};
    __nv_bfloat16 hi[4], lo[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      hi[q] = __float2bfloat16(vv[q]);
      lo[q] = __float2bfloat16(vv[q] - __bfloat162float(hi[q]));
    }
    const uint32_t off = tc_off(r, t * Cin + 4 * c4, kp);
    *reinterpret_cast<uint2*>(a_hi + off) = *reinterpret_cast<const uint2*>(hi);
    *reinterpret_cast<uint2*>(a_lo + off) = *reinterpret_cast<const uint2*>(lo);
  }
  // generic-proxy shared stores -> visible to the tensor cores (async proxy)
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (tid == 0) {
    // kind::f16: D F32 (bits 4-5 = 1), A BF16 (7-9 = 1), B BF16 (10-12 = 1),
    // both K-major, N >> 3 at bit 17, M >> 4 at bit 24
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NP >> 3) << 17) |
                           ((uint32_t)(TC_M >> 4) << 24);
    const uint32_t sbo = (uint32_t)(kp >> 3) * 128u;
    const uint32_t a0[2] = {smem_u32(a_hi), smem_u32(a_lo)};
    const uint32_t b0 = smem_u32(bm);
    for (int pass = 0; pass < 2; ++pass)
      for (int kk = 0; kk < kp / 16; ++kk) {
        const uint64_t da = tc_desc(a0[pass] + (uint32_t)kk * 256u, 128u, sbo);
        const uint64_t db = tc_desc(b0 + (uint32_t)kk * 256u, 128u, sbo);
        const uint32_t acc = (pass > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
            "l"(da), "l"(db), "r"(idesc), "r"(acc));
      }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
        smem_u32(&mbar)));
  }
  // wait for the MMAs (phase 0), bounded
  {
    uint32_t done = 0;
    long long spins = 0;
    while (!done) {
      asm volatile(
          "{\n\t.reg .pred p;\n\t"
          "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
          "selp.u32 %0, 1, 0, p;\n\t}\n"
          : "=r"(done)
          : "r"(smem_u32(&mbar)));
      if (!done && ++spins > TC_SPIN_LIMIT) {
        s_timeout = 1;
        break;
      }
    }
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  const bool ok = s_timeout == 0;
  if (ok) {
    // epilogue: warp w reads lanes 32 (w % 4) .. +31, columns [half * NP/2, +NP/2)
    constexpr int HC = NP / 2;
    const int quarter = warp & 3, half = warp >> 2;
    const int r = quarter * 32 + lane;
    const int i = p0 + r;
    uint32_t v[HC];
    tmem_ld<HC>(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(half * HC), v);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (i < N) {
#pragma unroll
      for (int q = 0; q < HC; ++q) {
        const int o = half * HC + q;
        if (o < Cout) {
          float x = __uint_as_float(v[q]) + (bias ? bias[o] : 0.f);
          out[(size_t)i * Cout + o] = RELU ? fmaxf(x, 0.f) : x;
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS));
}

template <int NP, bool RELU, int CIN>
int launch_tc(int N, int Cout, const __nv_bfloat16* W, const float* bias, const float* in, const int* sst,
              const int* sln, float* out, int* err, cudaStream_t st) {
  constexpr int kp = ((TC_NK * CIN + 15) / 16) * 16;
  const size_t smem = (size_t)(2 * TC_M + NP) * kp * 2;
  auto kern = k_conv_tc<NP, RELU, CIN>;
  ILM_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<(N + TC_M - 1) / TC_M, TC_THREADS, smem, st>>>(N, Cout, W, bias, in, sst, sln, out, err);
  ILM_CHECK_LAUNCH();
  return ILM_OK;
}

}  // namespace

bool conv_tc_supported(int Cin, int Cout) { return (Cin == 8 || Cin == 64) && Cout >= 1 && Cout <= 64; }

int launch_conv_tc(int N, int Cin, int Cout, bool relu, const __nv_bfloat16* W, const float* bias, const float* in,
                   const int* sst, const int* sln, float* out, int* err, cudaStream_t st) {
  if (N <= 0) return ILM_OK;
  if (!conv_tc_supported(Cin, Cout)) {
    set_error("tensor-core convolution: unsupported channels %d -> %d", Cin, Cout);
    return ILM_ERR_UNSUPPORTED;
  }
#define TC_CASE(NPV, RV, CV) return launch_tc<NPV, RV, CV>(N, Cout, W, bias, in, sst, sln, out, err, st)
  if (Cout <= 16) {
    if (Cin == 8) {
      if (relu) TC_CASE(16, true, 8);
      TC_CASE(16, false, 8);
    }
    if (relu) TC_CASE(16, true, 64);
    TC_CASE(16, false, 64);
  }
  if (Cin == 8) {
    if (relu) TC_CASE(64, true, 8);
    TC_CASE(64, false, 8);
  }
  if (relu) TC_CASE(64, true, 64);
  TC_CASE(64, false, 64);
#undef TC_CASE
}

}  // namespace ilm
