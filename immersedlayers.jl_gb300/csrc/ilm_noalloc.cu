// Weighted grid inner product that allocates no device memory.
//
// Who needs it: callers that cannot allocate device memory at the moment they
// need an inner product or norm of grid data -- services whose memory pool
// owns the whole device and forbids allocations outside it (a Julia process
// whose GPU arrays all come from its own pool, an inference server sized to
// the card), and latency-critical loops in which a cudaMalloc or cudaFree
// (which can synchronise the whole device) is not acceptable.  The regular
// entry point, ilm_dot_grid, needs a cache, whose creation allocates.
// ilm_dot_grid_noalloc needs no cache and calls no allocating routine: its
// only scratch is the fixed device array below, which every GPU that loads
// this library holds until the process exits.
//
// Contract:
//  * at most kNoAllocMaxRows grid rows (ny dual nodes) per grid component:
//    one FP64 partial sum per row lives in the array; rows are any length
//    (each is reduced by a loop), so nx is not limited.  Taller grids are
//    rejected with ILM_ERR_SIZE_LIMIT before anything is launched;
//  * `stream` must belong to the current device (the legacy default stream
//    always does); a stream of another device is rejected, because the
//    array's address differs per device;
//  * the first call on a device looks up the device address of the scratch
//    array (cudaGetSymbolAddress, once per device, with that device current);
//  * the call waits for `stream` (cudaStreamSynchronize) and copies the
//    result to host memory before it returns;
//  * every call on a device shares the one array: calls whose kernels may
//    overlap on the GPU (different streams, or different host threads) race
//    and must be serialised by the caller;
//  * the array keeps the last call's contents; each call overwrites every
//    element it reads, so nothing has to start at zero.
#include <mutex>

#include "ilm_internal.cuh"

namespace {

constexpr int kNoAllocMaxRows = 16384;  // one FP64 partial sum per grid row: 128 KiB
constexpr int kNoAllocSlots = 4;        // one FP64 result per grid component
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxRows + kNoAllocSlots];

std::mutex g_na_mu;
double* g_na_addr[kMaxDevices] = {};

// device address of g_noalloc_scratch on the current device (looked up once);
// `st` must belong to that device
int noalloc_scratch(cudaStream_t st, double** out) {
  int dev = 0;
  ILM_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    ilm::set_error("ilm_dot_grid_noalloc: device ordinal %d out of range", dev);
    return ILM_ERR_UNSUPPORTED;
  }
  if (st != nullptr) {
    int sdev = -1;
    ILM_CHECK_CUDA(cudaStreamGetDevice(st, &sdev));
    if (sdev != dev) {
      ilm::set_error("ilm_dot_grid_noalloc: the stream belongs to device %d, the current device is %d", sdev, dev);
      return ILM_ERR_INVALID_ARG;
    }
  }
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      ilm::set_error("ilm_dot_grid_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return ILM_ERR_CUDA;
    }
    g_na_addr[dev] = static_cast<double*>(p);
  }
  *out = g_na_addr[dev];
  return ILM_OK;
}

// one block per row: trapezoid weights on primal directions, ghosts excluded
// on dual directions; fixed-order tree reduction (deterministic)
template <typename T>
__global__ void k_na_rows(int n1, int n2, int dx, int dy, const T* __restrict__ a, const T* __restrict__ b,
                          double* __restrict__ part) {
  __shared__ double sh[256];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int i = threadIdx.x; i < n1; i += blockDim.x) {
    double wx = 1.0;
    if (i == 0 || i == n1 - 1) wx = dx ? 0.0 : 0.5;
    s += wx * (double)a[(size_t)j * n1 + i] * (double)b[(size_t)j * n1 + i];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double wy = 1.0;
    if (j == 0 || j == n2 - 1) wy = dy ? 0.0 : 0.5;
    part[j] = wy * sh[0];
  }
}

__global__ void k_na_sum(int n, const double* __restrict__ part, double* __restrict__ slot) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) slot[0] = sh[0];
}

}  // namespace

extern "C" int ilm_dot_grid_noalloc(int nx, int ny, double h, int scaling, int kind, int dtype, const void* a,
                                    const void* b, double* result, ilm_stream_t stream) {
  ILM_REQUIRE(nx >= 4 && ny >= 4, "ilm_dot_grid_noalloc: grid needs at least 4x4 dual nodes (got %d x %d)", nx,
              ny);
  if (ny > kNoAllocMaxRows) {
    ilm::set_error("ilm_dot_grid_noalloc: grid of %d x %d dual nodes exceeds the fixed scratch (at most %d rows, "
                   "ny <= %d); use ilm_dot_grid",
                   nx, ny, kNoAllocMaxRows, kNoAllocMaxRows);
    return ILM_ERR_SIZE_LIMIT;
  }
  ILM_REQUIRE(h > 0.0, "ilm_dot_grid_noalloc: cell size must be positive");
  ILM_REQUIRE(scaling == ILM_GRID_SCALING || scaling == ILM_INDEX_SCALING, "ilm_dot_grid_noalloc: bad scaling %d",
              scaling);
  ILM_REQUIRE(dtype == ILM_F64 || dtype == ILM_F32, "ilm_dot_grid_noalloc: bad dtype %d", dtype);
  ILM_REQUIRE(a && b && result, "ilm_dot_grid_noalloc: null argument");
  const ilm_grid_s g{nx, ny, h, nx / 2, ny / 2};
  int pcs[4];
  const int ncomp = ilm::gridkind_components(kind, pcs);
  ILM_REQUIRE(ncomp > 0 && ncomp <= kNoAllocSlots, "ilm_dot_grid_noalloc: bad grid kind %d", kind);
  cudaStream_t st = ilm::as_stream(stream);
  double* scratch = nullptr;
  ILM_TRY(noalloc_scratch(st, &scratch));
  const size_t es = dtype == ILM_F64 ? 8 : 4;
  size_t off = 0;
  for (int c = 0; c < ncomp; ++c) {
    const ilm::Shape2 sh = g.shape(pcs[c]);
    const unsigned char* ac = static_cast<const unsigned char*>(a) + off * es;
    const unsigned char* bc = static_cast<const unsigned char*>(b) + off * es;
    if (dtype == ILM_F64)
      k_na_rows<double><<<sh.n2, 256, 0, st>>>(sh.n1, sh.n2, ilm::pc_dx(pcs[c]), ilm::pc_dy(pcs[c]),
                                               reinterpret_cast<const double*>(ac),
                                               reinterpret_cast<const double*>(bc), scratch);
    else
      k_na_rows<float><<<sh.n2, 256, 0, st>>>(sh.n1, sh.n2, ilm::pc_dx(pcs[c]), ilm::pc_dy(pcs[c]),
                                              reinterpret_cast<const float*>(ac), reinterpret_cast<const float*>(bc),
                                              scratch);
    ILM_CHECK_LAUNCH();
    k_na_sum<<<1, 256, 0, st>>>(sh.n2, scratch, scratch + kNoAllocMaxRows + c);
    ILM_CHECK_LAUNCH();
    off += sh.numel();
  }
  double slots[kNoAllocSlots] = {0.0, 0.0, 0.0, 0.0};
  ILM_CHECK_CUDA(cudaMemcpyAsync(slots, scratch + kNoAllocMaxRows, ncomp * sizeof(double), cudaMemcpyDeviceToHost,
                                 st));
  ILM_CHECK_CUDA(cudaStreamSynchronize(st));
  double total = 0.0;
  for (int c = 0; c < ncomp; ++c) total += slots[c];
  *result = scaling == ILM_GRID_SCALING ? total * h * h : total;
  return ILM_OK;
}
