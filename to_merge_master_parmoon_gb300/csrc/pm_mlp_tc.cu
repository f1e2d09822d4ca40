// pm_mlp_tc.cu — forward layers of the learned smoother's MLP on the 5th-generation
// tensor cores (tcgen05): C = act(A W^T + b) for A [M x K] BF16 (activations,
// K contiguous) and W [N x K] BF16 (weights, K contiguous), FP32 accumulation
// in tensor memory.
//
// One CTA of eight warps (two warpgroups) per 128-row tile of A (UMMA shape
// M = 128, N = the layer width 256 or 96, K = 16 per instruction).  K is staged through shared
// memory in chunks of KC columns, in the K-major canonical layout without
// swizzling: 8-row x 16-byte core matrices, LBO = 128 bytes between core
// matrices along K, SBO = KC/8 * 128 bytes between 8-row groups.  Thread 0
// issues the chunk's tcgen05.mma instructions and commits them to an
// mbarrier, which every thread waits on (bounded) before the chunk buffers
// are refilled.  The epilogue reads the accumulator with tcgen05.ld (warp w
// owns TMEM lanes 32(w%4)..32(w%4)+31, i.e. tile rows 32(w%4)..+31; the two
// warpgroups take alternate 32-column blocks), adds the bias,
// applies GELU and writes FP32 and/or BF16 rows.  The TMEM columns (256 or
// 128) are always released before the CTA exits; a barrier wait that gives
// up sets PM_ERR_BULK_TIMEOUT in *err and skips the epilogue.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "pm_learned.h"

namespace pm {

namespace {

constexpr int kTcThreads = 256;  // two warpgroups
constexpr long long kTcMaxPolls = 1ll << 22;
// dynamic shared memory per CTA: at most two CTAs per SM, so their TMEM
// allocations (<= 256 columns each) always fit the SM's 512 columns
constexpr int kTcSmem = 100 * 1024;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ float gelu_tc(float x) {
  return 0.5f * x * (1.f + erff(x * 0.70710678118654752f));
}

// shared-memory matrix descriptor: K-major, no swizzle (sm_100 layout:
// start >> 4 in bits 0-13, LBO >> 4 in 16-29, SBO >> 4 in 32-45, version 1 in
// bits 46-47, swizzle mode 0 in bits 61-63)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: D F32, A and B BF16, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                      // D format F32
         | (1u << 7)                    // A format BF16
         | (1u << 10)                   // B format BF16
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(M >> 4) << 24);  // M / 16
}

__device__ __forceinline__ bool tc_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ bool tc_wait(uint64_t *bar, uint32_t parity) {
  for (long long it = 0; it < kTcMaxPolls; ++it)
    if (tc_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

struct TcArgs {
  int M, lda, ldo;
  const __nv_bfloat16 *A, *W;
  const float *bias;
  int act;               // 0 identity, 1 GELU
  float *pre;            // pre-activation out (FP32) or null
  float *Cf;             // FP32 out or null
  __nv_bfloat16 *Cb;     // BF16 out or null
  const int *on;         // skip when *on == 0
  int *err;
};

template <int N, int K>
__global__ void __launch_bounds__(kTcThreads) k_mlp_layer_tc(TcArgs a) {
  constexpr int KC = (K % 80 == 0) ? 80 : 64;  // K chunk (multiple of 16)
  static_assert(K % KC == 0 && KC % 16 == 0, "K chunking");
  static_assert(N % 16 == 0 && N >= 16 && N <= 256, "UMMA N for M = 128");
  constexpr int NCH = K / KC;
  constexpr int KB = KC / 8;                 // 16-byte units per row of a chunk
  constexpr uint32_t SBO = KB * 128;         // bytes between 8-row groups
  constexpr int A_BYTES = 128 * KC * 2;
  constexpr int NCOLS = N <= 128 ? 128 : 256;
  static_assert(A_BYTES + N * KC * 2 <= kTcSmem, "chunk buffers fit");
  constexpr uint32_t IDESC = idesc_bf16(128, N);

  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  if (a.on && *a.on == 0) return;  // uniform over the grid
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * 128;
  unsigned char *As = smem, *Bs = smem + A_BYTES;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(NCOLS)
                 : "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_slot;

  bool ok = true;
  for (int c = 0; c < NCH; ++c) {
    // stage the chunk: A rows m0..m0+127 (zeros past M) and all N rows of W
    // thread u -> row r = 8 * (u / (8 KB)) + u % 8, 16-byte column kb =
    // (u / 8) % KB: eight consecutive threads fill one 128-byte core matrix
    // (conflict-free shared stores; the second half of each 32-byte global
    // sector is read from L1 by the next eight threads)
#pragma unroll 4
    for (int u = tid; u < 128 * KB; u += kTcThreads) {
      const int rl = u & 7, q = u >> 3, kb = q % KB, r = 8 * (q / KB) + rl;
      const int gm = m0 + r;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (gm < a.M)
        v = __ldg(reinterpret_cast<const uint4 *>(a.A + (size_t)gm * a.lda + c * KC + kb * 8));
      *reinterpret_cast<uint4 *>(As + (r >> 3) * SBO + kb * 128 + (r & 7) * 16) = v;
    }
#pragma unroll 4
    for (int u = tid; u < N * KB; u += kTcThreads) {
      const int rl = u & 7, q = u >> 3, kb = q % KB, r = 8 * (q / KB) + rl;
      const uint4 v =
          __ldg(reinterpret_cast<const uint4 *>(a.W + (size_t)r * K + c * KC + kb * 8));
      *reinterpret_cast<uint4 *>(Bs + (r >> 3) * SBO + kb * 128 + (r & 7) * 16) = v;
    }
    // make the generic-proxy stores visible to the tensor cores' async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int kk = 0; kk < KC / 16; ++kk) {
        const uint64_t ad = smem_desc(smem_u32(As) + kk * 256, 128, SBO);
        const uint64_t bd = smem_desc(smem_u32(Bs) + kk * 256, 128, SBO);
        const uint32_t accumulate = (c > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tbase),
            "l"(ad), "l"(bd), "r"(IDESC), "r"(accumulate)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&bar))
          : "memory");
    }
    // the chunk's MMAs are done before its buffers are refilled
    const bool waited = tc_wait(&bar, (uint32_t)(c & 1));
    ok = __syncthreads_and(waited) != 0;
    if (!ok) break;
  }
  tc_fence_after();

  if (ok) {
    const int q = warp & 3, half = warp >> 2;  // TMEM lane quarter, column parity
    const int row = m0 + q * 32 + lane;
#pragma unroll 1
    for (int cb = 32 * half; cb < N; cb += 64) {
      uint32_t v[32];
      const uint32_t taddr = tbase + ((uint32_t)(q * 32) << 16) + (uint32_t)cb;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
          "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
            "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
            "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]),
            "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
            "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
            "=r"(v[30]), "=r"(v[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < a.M) {
        // 16-byte stores of the row's 32 values (row * ldo + cb is a multiple
        // of 32 elements, so every store is aligned)
        const size_t o = (size_t)row * a.ldo + cb;
        float x[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) x[j] = __uint_as_float(v[j]) + __ldg(a.bias + cb + j);
        if (a.pre) {
#pragma unroll
          for (int j = 0; j < 32; j += 4)
            *reinterpret_cast<float4 *>(a.pre + o + j) = make_float4(x[j], x[j + 1], x[j + 2], x[j + 3]);
        }
        if (a.act == 1) {
#pragma unroll
          for (int j = 0; j < 32; ++j) x[j] = gelu_tc(x[j]);
        }
        if (a.Cf) {
#pragma unroll
          for (int j = 0; j < 32; j += 4)
            *reinterpret_cast<float4 *>(a.Cf + o + j) = make_float4(x[j], x[j + 1], x[j + 2], x[j + 3]);
        }
        if (a.Cb) {
#pragma unroll
          for (int j = 0; j < 32; j += 8) {
            uint4 w;
            __nv_bfloat162 h0 = __floats2bfloat162_rn(x[j], x[j + 1]);
            __nv_bfloat162 h1 = __floats2bfloat162_rn(x[j + 2], x[j + 3]);
            __nv_bfloat162 h2 = __floats2bfloat162_rn(x[j + 4], x[j + 5]);
            __nv_bfloat162 h3 = __floats2bfloat162_rn(x[j + 6], x[j + 7]);
            w.x = *reinterpret_cast<uint32_t *>(&h0);
            w.y = *reinterpret_cast<uint32_t *>(&h1);
            w.z = *reinterpret_cast<uint32_t *>(&h2);
            w.w = *reinterpret_cast<uint32_t *>(&h3);
            *reinterpret_cast<uint4 *>(a.Cb + o + j) = w;
          }
        }
      }
    }
  } else {
    // give the MMAs still in flight a last (bounded) chance before the
    // columns are released
    if (tid == 0) atomicOr(a.err, PM_ERR_BULK_TIMEOUT);
    tc_wait(&bar, 0u);
    tc_wait(&bar, 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
}

inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

template <int N, int K>
int launch_layer(const TcArgs &a, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(k_mlp_layer_tc<N, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kTcSmem) != cudaSuccess)
      return -1;
    attr = true;
  }
  const int grid = (a.M + 127) / 128;
  k_mlp_layer_tc<N, K><<<grid, kTcThreads, kTcSmem, s>>>(a);
  return ok() < 0 ? -1 : 1;
}

}  // namespace

int mlp_tc_init() {
  int r = 0;
  r |= cudaFuncSetAttribute(k_mlp_layer_tc<kMlpHidden, kMlpInPad>,
                            cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  r |= cudaFuncSetAttribute(k_mlp_layer_tc<kMlpHidden, kMlpHidden>,
                            cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  r |= cudaFuncSetAttribute(k_mlp_layer_tc<kMlpOutPad, kMlpHidden>,
                            cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  return r == 0 ? 0 : -1;
}

int mlp_layer_tc(int layer, const __nv_bfloat16 *A, int M, const __nv_bfloat16 *W,
                 const float *bias, int act, float *pre, float *Cf, __nv_bfloat16 *Cb,
                 const int *on, int *err, cudaStream_t s) {
  if (M <= 0) return 0;
  TcArgs a{};
  a.M = M;
  a.A = A;
  a.W = W;
  a.bias = bias;
  a.act = act;
  a.pre = pre;
  a.Cf = Cf;
  a.Cb = Cb;
  a.on = on;
  a.err = err;
  switch (layer) {
    case 1:
      a.lda = kMlpInPad;
      a.ldo = kMlpHidden;
      return launch_layer<kMlpHidden, kMlpInPad>(a, s);
    case 2:
      a.lda = kMlpHidden;
      a.ldo = kMlpHidden;
      return launch_layer<kMlpHidden, kMlpHidden>(a, s);
    case 3:
      a.lda = kMlpHidden;
      a.ldo = kMlpOutPad;
      return launch_layer<kMlpOutPad, kMlpHidden>(a, s);
    default:
      return -1;
  }
}

}  // namespace pm
