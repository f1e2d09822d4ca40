// pm_noalloc.cu — allocation-free variant of the L2_0 pressure projection.
//
// Some callers of this library cannot allocate device memory at the point
// where they need the projection: solvers that run inside an
// application-owned memory pool whose budget is fixed up front, and
// MPI-parallel ParMooN ranks that partition each GPU's memory before the
// time loop starts (a cudaMalloc there would also synchronise the device).  For them, pm_l20_project_noalloc keeps the scratch of its
// deterministic two-stage reduction (one partial sum per block, the mean and
// a completion counter) in the file-scope device array below instead of in
// memory owned by a pm_handle.
//
// Limits and sharing: the array holds kNoAllocMaxBlocks partial sums, so one
// call projects at most kNoAllocMaxN pressure entries (P1disc, four per cell:
// 8,388,608 entries = 2,097,152 cells).  Every GPU that loads the library
// holds the array (64 KB) until the process exits.  All calls on a device
// share it and it keeps the last call's contents: the completion counter is
// cleared by every call before its kernels run, and calls that overlap on the
// GPU (different streams without ordering) race on the array.
#include <cuda_runtime.h>

#include <mutex>

#include "pmgpu.h"

namespace {

constexpr int kNoAllocBlock = 256;
constexpr int kNoAllocMaxBlocks = 8192;
constexpr long long kNoAllocMaxN = 4LL * kNoAllocBlock * kNoAllocMaxBlocks;
// layout: [0, kNoAllocMaxBlocks) partial sums, [kNoAllocMaxBlocks] mean,
// [kNoAllocMaxBlocks + 1] completion counter (as unsigned int)
constexpr int kNoAllocScratch = kNoAllocMaxBlocks + 32;

static __device__ __align__(256) double g_pm_noalloc_scratch[kNoAllocScratch];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch_ptr[kMaxDevices] = {};

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[kNoAllocBlock / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = (l < kNoAllocBlock / 32) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;
}

// Sum of the constant modes p[4c] (one per thread); the last block to finish
// reduces the per-block sums in block order and stores the mean.
__global__ void __launch_bounds__(kNoAllocBlock) k_noalloc_l20_sum(const double *p, int np,
                                                                   double *scratch) {
  const long long i = 4LL * ((long long)blockIdx.x * kNoAllocBlock + threadIdx.x);
  double s = block_sum(i < np ? p[i] : 0.0);
  unsigned int *counter = reinterpret_cast<unsigned int *>(scratch + kNoAllocMaxBlocks + 1);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = s;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kNoAllocBlock)
    v += ((volatile double *)scratch)[b];
  v = block_sum(v);
  if (threadIdx.x == 0) {
    scratch[kNoAllocMaxBlocks] = v * (4.0 / (double)np);  // IntoL20Vector3D, case -11
    *counter = 0u;
  }
}

__global__ void __launch_bounds__(kNoAllocBlock) k_noalloc_l20_sub(double *p, int np,
                                                                   const double *scratch) {
  const long long i = 4LL * ((long long)blockIdx.x * kNoAllocBlock + threadIdx.x);
  if (i < np) p[i] -= scratch[kNoAllocMaxBlocks];
}

// Once per device, with that device current: the device address of the
// scratch array (its host-side name is only a stand-in).
pm_status scratch_for_current_device(double **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return PM_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_pm_noalloc_scratch) != cudaSuccess || !ptr) {
      cudaGetLastError();
      return PM_CUDA_ERROR;
    }
    g_scratch_ptr[dev] = static_cast<double *>(ptr);
  }
  *out = g_scratch_ptr[dev];
  return PM_OK;
}

}  // namespace

extern "C" pm_status pm_l20_project_noalloc(double *d_p, int n_p, void *stream) {
  if (!d_p || n_p <= 0 || (n_p & 3) != 0) return PM_BADARG;
  if ((long long)n_p > kNoAllocMaxN) return PM_BADARG;
  double *scratch = nullptr;
  pm_status st = scratch_for_current_device(&scratch);
  if (st != PM_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int modes = n_p / 4;
  const int blocks = (modes + kNoAllocBlock - 1) / kNoAllocBlock;
  if (cudaMemsetAsync(scratch + kNoAllocMaxBlocks + 1, 0, sizeof(double), s) != cudaSuccess) {
    cudaGetLastError();
    return PM_CUDA_ERROR;
  }
  k_noalloc_l20_sum<<<blocks, kNoAllocBlock, 0, s>>>(d_p, n_p, scratch);
  k_noalloc_l20_sub<<<blocks, kNoAllocBlock, 0, s>>>(d_p, n_p, scratch);
  if (cudaPeekAtLastError() != cudaSuccess) {
    cudaGetLastError();
    return PM_CUDA_ERROR;
  }
  return PM_OK;
}
