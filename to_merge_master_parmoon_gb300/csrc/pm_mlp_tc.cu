// pm_mlp_tc.cu — forward layers of the learned smoother's MLP on the 5th-generation
// tensor cores (tcgen05): C = act(A W^T + b) for A [M x K] BF16 (activations,
// K contiguous) and W [N x K] BF16 (weights, K contiguous), FP32 accumulation
// in tensor memory.
//
// Persistent CTAs (one per SM for the 256-wide layers) walk the 128-row
// tiles of A (UMMA shape M = 128, N = the layer width 256 or 96, K = 16 per
// instruction) with warp specialisation: one thread streams the K chunks by
// TMA (cp.async.bulk.tensor) through a three-stage shared-memory ring in the
// K-major canonical layout without swizzling, one thread issues the
// tcgen05.mma of each chunk as soon as its bytes have landed, into one of two
// TMEM accumulators, and eight warps drain the other accumulator (tcgen05.ld,
// bias, GELU, FP32 and/or BF16 rows), so loads, MMAs and the epilogue of
// consecutive tiles overlap.  The TMEM columns are always released before
// the CTA exits; a barrier wait that gives up sets PM_ERR_BULK_TIMEOUT in
// *err and stops the pipeline.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "pm_learned.h"

namespace pm {

namespace {

constexpr long long kTcMaxPolls = 1ll << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ float gelu_tc(float x) {
  return 0.5f * x * (1.f + erff(x * 0.70710678118654752f));
}

// shared-memory matrix descriptor of a K-major operand in the 128-byte
// swizzled layout that TMA writes with CU_TENSOR_MAP_SWIZZLE_128B: rows of
// 64 BF16 (128 bytes), 8-row atoms of 1024 bytes (SBO), LBO unused (1),
// version 1, layout type 2 (128-byte swizzle); the K = 16 slices of an atom
// start 32 bytes apart
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | (1ull << 16) | ((uint64_t)(1024 >> 4) << 32) |
         (1ull << 46) | (2ull << 61);
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
  int M, ldo;
  int nch;               // K chunks of 64 columns (columns past K read as zeros)
  int n_off;             // first row of W and first output column of this launch
  const __nv_bfloat16 *A, *W;
  const float *bias;     // per output column, or null
  int act;               // 0 identity, 1 GELU
  float *pre;            // pre-activation out (FP32) or null
  float *Cf;             // FP32 out or null
  __nv_bfloat16 *Cb;     // BF16 out or null
  const int *on;         // skip when *on == 0
  int *err;
};

// one elected thread: 2-D tile (8 K-elements x `rows` rows) of a BF16 tensor
// map into shared memory, completing on `bar` (transaction bytes)
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// Pipeline depth and chunking of a layer: K in chunks of 64 columns (one
// 128-byte swizzle atom per row; the last chunk of K = 400 reads columns
// 400..447 as zeros), up to three chunks in flight; two accumulators of
// NCOLS TMEM columns (512 for N = 256: one CTA per SM; 256 for N = 96).
template <int N>
struct TcPlan {
  static constexpr int KC = 64;
  static constexpr int S = 3;
  static constexpr int A_STAGE = 128 * KC * 2;  // bytes of the A tile of a chunk
  static constexpr int W_STAGE = N * KC * 2;    // bytes of the W rows of a chunk
  static constexpr int STAGE = A_STAGE + W_STAGE;
  static constexpr int SMEM = S * STAGE;
  static constexpr int NCOLS = N <= 128 ? 128 : 256;
  static constexpr int CTAS_PER_SM = 512 / (2 * NCOLS);
  static_assert(KC % 16 == 0 && STAGE % 1024 == 0, "K chunking, 1024-byte atoms");
  static_assert(N % 16 == 0 && N >= 16 && N <= 256, "UMMA N for M = 128");
  static_assert(N % 8 == 0, "16-byte stores of BF16 output rows");
  static_assert(SMEM <= 200 * 1024, "stages fit in shared memory");
};

constexpr int kTcWarps = 10;  // producer, MMA issuer, eight epilogue warps
constexpr int kEpiWarps = 8;

// Persistent, warp-specialised layer: each CTA walks the 128-row tiles
// blockIdx.x, blockIdx.x + gridDim.x, ...
// * warp 0, lane 0 streams every tile's K chunks with TMA
//   (cp.async.bulk.tensor) into an S-stage ring: per chunk one box of 64
//   K-elements x 128 rows of A and one of 64 x N rows of W, written by TMA in
//   the 128-byte swizzled K-major layout (8-row atoms of 1024 bytes) that
//   the MMA descriptors name;
// * warp 1, lane 0 issues a chunk's KC/16 tcgen05.mma once its bytes have
//   landed, into accumulator (tile & 1), commits them to the stage's `empty`
//   barrier (freeing it for the producer) and, after a tile's last chunk, to
//   the accumulator's `tfull` barrier;
// * warps 2..9 drain an accumulator with tcgen05.ld (warp w reads TMEM lanes
//   32(w%4)..+31 = tile rows, the two groups of four alternate 32-column
//   blocks), add the bias, apply GELU, store FP32 and/or BF16 rows and
//   release the accumulator (`tempty`), while the MMAs of the next tile run
//   into the other one.
// Every wait is bounded.  A wait that gives up sets PM_ERR_BULK_TIMEOUT and
// a shared flag that stops the other roles; the MMA thread still commits its
// MMAs to `done`, which all threads wait for (bounded), the producer waits
// for its loads in flight, and the TMEM columns are released before exit.
template <int N>
__global__ void __launch_bounds__(kTcWarps * 32, 1)
    k_mlp_layer_tc(const __grid_constant__ CUtensorMap mapA,
                   const __grid_constant__ CUtensorMap mapW, TcArgs a) {
  using PL = TcPlan<N>;
  constexpr int KC = PL::KC, S = PL::S, NCOLS = PL::NCOLS;
  const int NCH = a.nch;
  constexpr uint32_t IDESC = idesc_bf16(128, N);

  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[S], empty[S], tfull[2], tempty[2], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed, issued, consumed;
  if (a.on && *a.on == 0) return;  // uniform over the grid
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntiles = (a.M + 127) / 128;
  const int mine = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(2 * NCOLS)
                 : "memory");
  }
  if (tid == 0) {
    for (int st = 0; st < S; ++st) {
      mbar_init(&full[st], 1);
      mbar_init(&empty[st], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], kEpiWarps);
    }
    mbar_init(&done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    // the swizzled stages need 1024-byte alignment: otherwise nothing is
    // loaded and the layer reports the error flag
    failed = (smem_u32(smem) & 1023u) != 0 ? 1 : 0;
    issued = 0;
    consumed = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_slot;
  volatile int *vfailed = &failed;

  if (warp == 0) {
    if (lane == 0) {
      // producer: global chunk g = it * NCH + c into stage g % S once the
      // MMAs of chunk g - S are done
      int g = 0;
      for (int it = 0; it < mine && !*vfailed; ++it) {
        const int m0 = (blockIdx.x + it * gridDim.x) * 128;
        for (int c = 0; c < NCH; ++c, ++g) {
          const int st = g % S;
          if ((g >= S && !tc_wait(&empty[st], (uint32_t)((g / S - 1) & 1))) || *vfailed) {
            atomicOr(&failed, 1);
            break;
          }
          unsigned char *As = smem + st * PL::STAGE, *Ws = As + PL::A_STAGE;
          mbar_expect_tx(&full[st], (uint32_t)PL::STAGE);
          tma_load_2d(As, &mapA, c * KC, m0, &full[st]);
          tma_load_2d(Ws, &mapW, c * KC, a.n_off, &full[st]);
        }
      }
      issued = g;
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      int g = 0;
      for (int it = 0; it < mine && !*vfailed; ++it) {
        const int b = it & 1;
        if (it >= 2 && !tc_wait(&tempty[b], (uint32_t)((it / 2 - 1) & 1))) {
          atomicOr(&failed, 1);
          break;
        }
        tc_fence_after();
        const uint32_t acc = tbase + (uint32_t)(b * NCOLS);
        bool ok = true;
        for (int c = 0; c < NCH; ++c, ++g) {
          const int st = g % S;
          if (!tc_wait(&full[st], (uint32_t)((g / S) & 1)) || *vfailed) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t as = smem_u32(smem + st * PL::STAGE), ws = as + PL::A_STAGE;
#pragma unroll
          for (int kk = 0; kk < KC / 16; ++kk) {
            const uint64_t ad = smem_desc_sw128(as + kk * 32);
            const uint64_t bd = smem_desc_sw128(ws + kk * 32);
            const uint32_t accumulate = (c > 0 || kk > 0) ? 1u : 0u;
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "setp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(acc),
                "l"(ad), "l"(bd), "r"(IDESC), "r"(accumulate)
                : "memory");
          }
          tc_commit(&empty[st]);
        }
        if (!ok) {
          atomicOr(&failed, 1);
          break;
        }
        tc_commit(&tfull[b]);
      }
      consumed = g;
      tc_commit(&done);  // arrives once every MMA issued above has completed
    }
    __syncwarp();
  } else {
    // epilogue warps
    const int q = warp & 3, half = (warp - 2) >> 2;  // TMEM lane quarter, column parity
    for (int it = 0; it < mine; ++it) {
      const int b = it & 1;
      if (*vfailed || !tc_wait(&tfull[b], (uint32_t)((it / 2) & 1))) {
        atomicOr(&failed, 1);
        break;
      }
      tc_fence_after();
      const int row = (blockIdx.x + it * gridDim.x) * 128 + q * 32 + lane;
#pragma unroll 1
      for (int cb = 32 * half; cb < N; cb += 64) {
        uint32_t v[32];
        const uint32_t taddr = tbase + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * NCOLS + cb);
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
          // 16-byte stores of the row's 32 values (row * ldo + cb is a
          // multiple of 32 elements, so every store is aligned)
          const size_t o = (size_t)row * a.ldo + a.n_off + cb;
          float x[32];
          if (a.bias) {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              x[j] = __uint_as_float(v[j]) + __ldg(a.bias + a.n_off + cb + j);
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) x[j] = __uint_as_float(v[j]);
          }
          // columns of the last block past N (N = 144: half a block) are not stored
          const int nv = N - cb < 32 ? N - cb : 32;
          if (a.pre) {
#pragma unroll
            for (int j = 0; j < 32; j += 4)
              if (j < nv)
                *reinterpret_cast<float4 *>(a.pre + o + j) =
                    make_float4(x[j], x[j + 1], x[j + 2], x[j + 3]);
          }
          if (a.act == 1) {
#pragma unroll
            for (int j = 0; j < 32; ++j) x[j] = gelu_tc(x[j]);
          }
          if (a.Cf) {
#pragma unroll
            for (int j = 0; j < 32; j += 4)
              if (j < nv)
                *reinterpret_cast<float4 *>(a.Cf + o + j) =
                    make_float4(x[j], x[j + 1], x[j + 2], x[j + 3]);
          }
          if (a.Cb) {
#pragma unroll
            for (int j = 0; j < 32; j += 8) {
              if (j >= nv) break;
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
      // this warp is done reading accumulator b
      tc_fence_before();
      __syncwarp();
      if (lane == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b]))
                     : "memory");
    }
  }
  // every MMA issued has completed (or the wait gave up)
  const bool fin = tc_wait(&done, 0u);
  __syncthreads();
  if (tid == 0 && (failed || !fin)) {
    atomicOr(a.err, PM_ERR_BULK_TIMEOUT);
    // loads issued but never consumed: let them land (bounded) before exit
    for (int g = consumed; g < issued; ++g) tc_wait(&full[g % S], (uint32_t)((g / S) & 1));
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase),
                 "r"(2 * NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
}

inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

// cuTensorMapEncodeTiled from the driver (no link against libcuda)
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                 const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                 const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled encode_fn() {
  static EncodeTiled fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  }
  return fn;
}

// 2-D BF16 map of a row-major [rows x cols] matrix (cols contiguous, row
// pitch ld elements) read in boxes of 64 columns x box_rows rows, written to
// shared memory with the 128-byte swizzle; columns and rows past the end
// read as zeros
bool make_map(CUtensorMap *m, const __nv_bfloat16 *base, int cols, int rows, int ld,
              int box_rows) {
  EncodeTiled f = encode_fn();
  if (!f) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(__nv_bfloat16)};
  const cuuint32_t box[2] = {64u, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1u, 1u};
  return f(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16 *>(base), dims,
           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int N>
int set_smem_limit() {
  return cudaFuncSetAttribute(k_mlp_layer_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              TcPlan<N>::SMEM) == cudaSuccess
             ? 0
             : -1;
}

// C[rows x N] (columns n_off.. of the output) = act(A W^T + bias) with A
// [rows x K] (row pitch lda) and W [>= n_off + N rows x K] (row pitch ldw)
template <int N>
int launch_n(TcArgs a, const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *W, int ldw, int K,
             int w_rows, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    if (set_smem_limit<N>() < 0) return -1;
    attr = true;
  }
  CUtensorMap ma, mw;
  if (!make_map(&ma, A, K, a.M, lda, 128) || !make_map(&mw, W, K, w_rows, ldw, N)) return -1;
  a.A = A;
  a.W = W;
  a.nch = (K + TcPlan<N>::KC - 1) / TcPlan<N>::KC;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return -1;
  const int tiles = (a.M + 127) / 128;
  const int grid = std::min(tiles, sms * TcPlan<N>::CTAS_PER_SM);
  k_mlp_layer_tc<N><<<grid, kTcWarps * 32, TcPlan<N>::SMEM, s>>>(ma, mw, a);
  return ok() < 0 ? -1 : 1;
}

}  // namespace

int mlp_tc_init() {
  int r = 0;
  r |= set_smem_limit<kMlpHidden>();
  r |= set_smem_limit<kMlpOutPad>();
  r |= set_smem_limit<kMlpInPad - kMlpHidden>();
  if (!encode_fn()) r = -1;
  return r == 0 ? 0 : -1;
}

int mlp_layer_tc(int layer, const __nv_bfloat16 *A, int M, const __nv_bfloat16 *W,
                 const float *bias, int act, float *pre, float *Cf, __nv_bfloat16 *Cb,
                 const int *on, int *err, cudaStream_t s) {
  if (M <= 0) return 0;
  TcArgs a{};
  a.M = M;
  a.bias = bias;
  a.act = act;
  a.pre = pre;
  a.Cf = Cf;
  a.Cb = Cb;
  a.on = on;
  a.err = err;
  switch (layer) {
    case 1:
      a.ldo = kMlpHidden;
      return launch_n<kMlpHidden>(a, A, kMlpInPad, W, kMlpInPad, kMlpInPad, kMlpHidden, s);
    case 2:
      a.ldo = kMlpHidden;
      return launch_n<kMlpHidden>(a, A, kMlpHidden, W, kMlpHidden, kMlpHidden, kMlpHidden, s);
    case 3:
      a.ldo = kMlpOutPad;
      return launch_n<kMlpOutPad>(a, A, kMlpHidden, W, kMlpHidden, kMlpHidden, kMlpOutPad, s);
    default:
      return -1;
  }
}

int mlp_gemm_tc(const __nv_bfloat16 *A, int lda, int rows, const __nv_bfloat16 *B, int ldb,
                int n, int k, float *C, int ldc, int *err, cudaStream_t s) {
  if (rows <= 0) return 0;
  TcArgs a{};
  a.M = rows;
  a.ldo = ldc;
  a.Cf = C;
  a.err = err;
  int launches = 0, r;
  // output columns in tiles of at most 256 (the widths this library needs:
  // 96, 256 and 400 = 256 + 144)
  for (int n0 = 0; n0 < n; n0 += kMlpHidden) {
    const int w = std::min(kMlpHidden, n - n0);
    a.n_off = n0;
    if (w == kMlpHidden)
      r = launch_n<kMlpHidden>(a, A, lda, B, ldb, k, n, s);
    else if (w == kMlpOutPad)
      r = launch_n<kMlpOutPad>(a, A, lda, B, ldb, k, n, s);
    else if (w == kMlpInPad - kMlpHidden)
      r = launch_n<kMlpInPad - kMlpHidden>(a, A, lda, B, ldb, k, n, s);
    else
      return -1;
    if (r < 0) return -1;
    launches += r;
  }
  return launches;
}

}  // namespace pm
