// fvs_noalloc.cu — an allocation-free variant of the residual-norm reduction.
//
// fvs_time_integration computes, after every RK step, the RMS over cells of
// |U - U0| per component (the log_res.plt columns).  Its two kernels reduce
// through a per-block partial-sum buffer that the handle allocates with
// cudaMalloc.  Some callers cannot allocate device memory at the point where
// they need this number: hosts whose device memory is entirely reserved up
// front by another allocator (a framework's caching pool), and time-critical
// loops that must not pay cudaMalloc's implicit device synchronisation.
// fvs_rms_delta_noalloc serves them: the caller passes the two device state
// arrays and a device output, and the partial sums live in the file-scope
// array g_rms_scratch below instead of a fresh allocation.
//
// Limits and sharing:
//  - at most FVS_NOALLOC_MAX_BLOCKS blocks of 256 cells, i.e.
//    FVS_NOALLOC_MAX_CELLS = 2,097,152 cells; larger inputs return
//    FVS_ERR_INVALID before any device work.  The array holds 256 KB on
//    every GPU that loads the library, for the life of the process.
//  - every call on a device shares the one array and leaves its partial sums
//    in it; each call writes every slot it later reads, so nothing needs
//    clearing.  Calls that overlap on the GPU (different streams, or host
//    threads without ordering) race on the array.
//  - the first call on a device, with that device current, looks up the
//    array's device address (cudaGetSymbolAddress); make that first call
//    before any stream capture.  The address is kept for the life of the
//    process, so a cudaDeviceReset after the first call is not supported
//    (the kept address would point into the destroyed context).
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/fvs2d.h"

namespace {

constexpr int kBlock = 256;
constexpr int kMaxBlocks = FVS_NOALLOC_MAX_BLOCKS;
constexpr int kMaxDevices = 64;

// per-block partial sums of |U-U0|^2, 4 components per block
static __device__ __align__(256) double g_rms_scratch[4 * kMaxBlocks];

std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

__global__ void __launch_bounds__(kBlock) k_rms_partials(const double* __restrict__ u, const double* __restrict__ u0,
                                                        int n, double* __restrict__ partials) {
  __shared__ double sh[4][kBlock];
  const int i = blockIdx.x * kBlock + threadIdx.x;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    double d = 0.0;
    if (i < n) d = fabs(u[4 * (size_t)i + k] - u0[4 * (size_t)i + k]);
    sh[k][threadIdx.x] = d * d;
  }
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int k = 0; k < 4; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < 4; k++) partials[4 * (size_t)blockIdx.x + k] = sh[k][0];
}

__global__ void __launch_bounds__(kBlock) k_rms_final(const double* __restrict__ partials, int nblk, int n,
                                                     double* __restrict__ out) {
  __shared__ double sh[4][kBlock];
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nblk; b += kBlock)
#pragma unroll
    for (int k = 0; k < 4; k++) s[k] += partials[4 * (size_t)b + k];
#pragma unroll
  for (int k = 0; k < 4; k++) sh[k][threadIdx.x] = s[k];
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int k = 0; k < 4; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < 4; k++) out[k] = sqrt(sh[k][0] / double(n));
}

// device address of g_rms_scratch for the current device, looked up once
int scratch_for_current_device(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return FVS_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return FVS_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    double* p = nullptr;
    e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_rms_scratch);
    if (e != cudaSuccess || !p) return FVS_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return FVS_OK;
}

}  // namespace

extern "C" int fvs_rms_delta_noalloc(const double* dev_u, const double* dev_u0, int32_t ncells, double* dev_norm4,
                                     void* stream) {
  // null pointers, empty input, or more cells than the fixed scratch holds
  // (FVS_NOALLOC_MAX_CELLS): rejected before any device work
  if (!dev_u || !dev_u0 || !dev_norm4 || ncells <= 0) return FVS_ERR_INVALID;
  const long long nblk = (static_cast<long long>(ncells) + kBlock - 1) / kBlock;
  if (nblk > kMaxBlocks) return FVS_ERR_INVALID;
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != FVS_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_rms_partials<<<(unsigned)nblk, kBlock, 0, s>>>(dev_u, dev_u0, ncells, scratch);
  k_rms_final<<<1, kBlock, 0, s>>>(scratch, (int)nblk, ncells, dev_norm4);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FVS_OK : FVS_ERR_CUDA;
}

