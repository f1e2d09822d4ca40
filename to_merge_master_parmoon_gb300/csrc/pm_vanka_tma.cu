// pm_vanka_tma.cu — Vanka apply with the stored FP32 LU factors staged in
// shared memory by bulk (TMA) copies.
//
// The substitution of one cell (P A = L U, 85 forward + 85 backward steps)
// is a serial chain per warp, so a warp that loads its factor columns from
// HBM as it goes keeps only a few KB in flight and the sweep reaches about
// 40 % of the HBM bandwidth.  Here every warp owns two 28.9 KB buffers in
// shared memory and walks the cells of the colour with a stride: while it
// substitutes with cell i's factors (read from shared memory), one
// cp.async.bulk brings cell i + stride's whole block (the factors are stored
// with a 16-byte-aligned per-cell stride, kFacStride) under an mbarrier.
// Three warps per CTA, one CTA per SM (173 KB of buffers).
//
// Every wait on an mbarrier is bounded: after `limit` unsuccessful polls
// (non-blocking mbarrier.test_wait; kMaxPolls by default, a few hundred ms)
// the warp records PM_ERR_BULK_TIMEOUT in *err, stops issuing copies, waits
// for the copies it still has in flight (bounded by kMaxPolls, whatever the
// limit of the first waits) and returns.
#include <cuda_runtime.h>

#include <cstdint>

#include "pm_kernels.h"

namespace pm {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kTmaWarps = 3;
constexpr int kCellBytes = kFacStride * (int)sizeof(float);  // 28,912
static_assert(kCellBytes % 16 == 0, "bulk copies move multiples of 16 bytes");
constexpr size_t kTmaSmem = (size_t)kTmaWarps * 2 * kCellBytes;  // 173,472
constexpr long long kMaxPolls = 1ll << 22;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one thread: arm the barrier for `bytes` and start the copy global -> shared
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes,
                                          uint64_t *bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_test_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait by the whole warp (at most `polls` non-blocking tests); true
// when the phase completed.  The result is warp-uniform (every lane has
// observed the completion itself, so every lane's later shared-memory reads
// are ordered after the copy).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long polls) {
  for (long long it = 0; it < polls; ++it)
    if (__all_sync(kFull, mbar_test_wait(bar, parity))) return true;
  return false;
}

__device__ __forceinline__ void scatter_cell(int i, float v, const int *ud, const int *pd, int nu,
                                             float *u) {
  if (i < 3 * NU_LOC) {
    const int comp = i / NU_LOC, a = i - comp * NU_LOC;
    u[(size_t)comp * nu + ud[a]] += v;
  } else {
    u[(size_t)3 * nu + pd[i - 3 * NU_LOC]] += v;
  }
}

// Forward/back substitution with the factors of one cell in shared memory
// (column-major, unit L below the diagonal, 1/U_jj on it), lanes owning rows
// lane, lane+32, lane+64; returns delta in y0..y2.
__device__ __forceinline__ void substitute(const float *Fc, int lane, float &y0, float &y1,
                                           float &y2) {
  const bool has2 = lane + 64 < NLOC;
  for (int j = 0; j < NLOC - 1; ++j) {
    const float *col = Fc + j * NLOC;
    const float l0 = (lane > j) ? col[lane] : 0.f;
    const float l1 = (lane + 32 > j) ? col[lane + 32] : 0.f;
    const float l2 = (has2 && lane + 64 > j) ? col[lane + 64] : 0.f;
    const float ysel = (j < 32) ? y0 : ((j < 64) ? y1 : y2);
    const float yj = __shfl_sync(kFull, ysel, j & 31);
    y0 -= l0 * yj;
    y1 -= l1 * yj;
    y2 -= l2 * yj;
  }
  for (int j = NLOC - 1; j >= 0; --j) {
    const float *col = Fc + j * NLOC;
    const int owner = j & 31;
    const float d = col[j];
    if (lane == owner) {
      if (j < 32) y0 *= d;
      else if (j < 64) y1 *= d;
      else y2 *= d;
    }
    const float ysel = (j < 32) ? y0 : ((j < 64) ? y1 : y2);
    const float xj = __shfl_sync(kFull, ysel, owner);
    if (lane < j) y0 -= col[lane] * xj;
    if (lane + 32 < j) y1 -= col[lane + 32] * xj;
    if (has2 && lane + 64 < j) y2 -= col[lane + 64] * xj;
  }
}

__global__ void __launch_bounds__(kTmaWarps * 32, 1) k_vanka_apply_tma(
    DevCells cells, int nu, const int *__restrict__ list, int ncol, const float *__restrict__ F,
    const uint8_t *__restrict__ perm, const float *__restrict__ rbuf, float damp,
    float *__restrict__ u, int *err, long long limit) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[kTmaWarps][2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *buf[2] = {reinterpret_cast<float *>(smem + (size_t)(2 * warp) * kCellBytes),
                   reinterpret_cast<float *>(smem + (size_t)(2 * warp + 1) * kCellBytes)};
  if (lane == 0) {
    mbar_init(&bars[warp][0], 1);
    mbar_init(&bars[warp][1], 1);
    fence_mbar_init();
  }
  __syncwarp();
  const int stride = gridDim.x * kTmaWarps;
  int slot = blockIdx.x * kTmaWarps + warp;
  // copies issued / completed per buffer (their count gives the phase parity)
  unsigned issued[2] = {0u, 0u}, done[2] = {0u, 0u};
  bool ok = true;
  if (slot < ncol && lane == 0)
    bulk_load(buf[0], F + (size_t)list[slot] * kFacStride, kCellBytes, &bars[warp][0]);
  if (slot < ncol) issued[0] = 1;
  const bool has2 = lane + 64 < NLOC;
  for (int i = 0; slot < ncol; ++i, slot += stride) {
    const int b = i & 1;
    const int next = slot + stride;
    if (ok && next < ncol) {
      if (lane == 0)
        bulk_load(buf[b ^ 1], F + (size_t)list[next] * kFacStride, kCellBytes, &bars[warp][b ^ 1]);
      issued[b ^ 1] += 1;
    }
    if (!ok) break;
    if (!mbar_wait(&bars[warp][b], done[b] & 1u, limit)) {
      ok = false;
      break;
    }
    done[b] += 1;
    const int cell = list[slot];
    const uint8_t *pc = perm + (size_t)cell * NLOC;
    const float *R = rbuf + (size_t)slot * kRStride;
    float y0 = R[__ldg(pc + lane)];
    float y1 = R[__ldg(pc + lane + 32)];
    float y2 = has2 ? R[__ldg(pc + lane + 64)] : 0.f;
    substitute(buf[b], lane, y0, y1, y2);
    const int *ud = cells.udofs + (size_t)cell * NU_LOC;
    const int *pd = cells.pdofs + (size_t)cell * NP_LOC;
    scatter_cell(lane, damp * y0, ud, pd, nu, u);
    scatter_cell(lane + 32, damp * y1, ud, pd, nu, u);
    if (has2) scatter_cell(lane + 64, damp * y2, ud, pd, nu, u);
    __syncwarp();  // buffer b is read by every lane before it is refilled
  }
  if (!ok) {
    if (lane == 0) atomicOr(err, PM_ERR_BULK_TIMEOUT);
    // drain: wait (bounded) for the copies this warp still has in flight
    for (int b = 0; b < 2; ++b)
      while (done[b] < issued[b]) {
        if (!mbar_wait(&bars[warp][b], done[b] & 1u, kMaxPolls)) break;
        done[b] += 1;
      }
  }
}

inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

}  // namespace

int launch_vanka_apply_tma_init() {
  return cudaFuncSetAttribute(k_vanka_apply_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kTmaSmem) == cudaSuccess
             ? 0
             : -1;
}

int launch_vanka_apply_tma(const DevCells &cells, int nu, const int *cell_list, int ncol,
                           const float *factors, const uint8_t *perm, const float *rbuf, float damp,
                           float *u, int *err, int num_sms, long long wait_limit, cudaStream_t s) {
  if (ncol <= 0) return 0;
  int grid = (ncol + kTmaWarps - 1) / kTmaWarps;
  if (grid > num_sms) grid = num_sms;
  const long long limit = wait_limit > 0 ? wait_limit : kMaxPolls;
  k_vanka_apply_tma<<<grid, kTmaWarps * 32, kTmaSmem, s>>>(cells, nu, cell_list, ncol, factors,
                                                           perm, rbuf, damp, u, err, limit);
  return ok() < 0 ? -1 : 1;
}

}  // namespace pm
