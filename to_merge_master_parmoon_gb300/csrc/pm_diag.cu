// pm_diag.cu — device diagnostics: the FP64 FMA rate of the current GPU,
// measured by a kernel of this library (the denominator of the FP64-pipe
// roofline of the FP64 sweeps and factorisations).
//
// Every thread keeps kChains independent FMA chains in registers (enough
// independent work to cover the FP64 pipe's latency), kIters dependent steps
// each; the grid holds 16 CTAs of 256 threads per SM.  The values stay
// bounded (x <- x * a + b with |a| < 1) and one sum per thread is written so
// the work cannot be removed.  Timed with CUDA events after one warm-up
// launch; flop = 2 per FMA.
#include <cuda_runtime.h>

#include "pmgpu.h"

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;
constexpr int kThreads = 256;
constexpr int kCtasPerSm = 16;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(double a, double b, double *out) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = 1e-3 * (threadIdx.x + c);
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  out[(size_t)blockIdx.x * kThreads + threadIdx.x] = s;
}

}  // namespace

extern "C" pm_status pm_measure_fp64_fma(int device, double *flops_per_s) {
  if (!flops_per_s) return PM_BADARG;
  *flops_per_s = 0.0;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) {
    cudaGetLastError();
    return PM_NO_DEVICE;
  }
  if (cudaSetDevice(device) != cudaSuccess) return PM_CUDA_ERROR;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int grid = sms * kCtasPerSm;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * (size_t)grid * kThreads) != cudaSuccess) {
    cudaGetLastError();
    return PM_OOM;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_fma<<<grid, kThreads>>>(0.999, 1e-6, out);  // warm-up
  cudaEventRecord(e0);
  const int reps = 5;
  for (int r = 0; r < reps; ++r) k_fp64_fma<<<grid, kThreads>>>(0.999, 1e-6, out);
  cudaEventRecord(e1);
  pm_status st = PM_OK;
  if (cudaEventSynchronize(e1) != cudaSuccess) st = PM_CUDA_ERROR;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (st != PM_OK || ms <= 0.f) return st != PM_OK ? st : PM_CUDA_ERROR;
  const double flop = 2.0 * kChains * (double)kIters * kThreads * grid * reps;
  *flops_per_s = flop / (ms * 1e-3);
  return PM_OK;
}
