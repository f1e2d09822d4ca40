// pm_learned.cu — learned per-cell smoother on sm_103a (no counterpart in the
// reference; inserted as one extra post-smoothing step per level, with cell
// Vanka as fallback).
//
// Network: 397 -> 256 -> 256 -> 85, GELU, BF16 weights and activations,
// FP32 accumulation.  All GEMMs run on the tensor cores through
// mma.sync.m16n8k16 (BF16 x BF16 -> FP32) in one tiled kernel with generic
// operand strides, so the same kernel computes the forward layers
// (X W^T), the activation gradients (dY W) and the weight gradients (dA^T H).
// Training: MSE loss, backward through GELU, AdamW on FP32 master weights.
#include "pm_learned.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

namespace pm {

namespace {

inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

// ------------------------------------------------------------------ GEMM ---
// C(m, n) = alpha * sum_k A(m, k) B(k, n)  [+ bias(n)]  [GELU]
// A(m, k) = A[m*sam + k*sak], B(k, n) = B[k*sbk + n*sbn] (BF16), FP32 accumulate.
struct GemmArgs {
  int M, N, K;
  const __nv_bfloat16 *A;
  long long sam, sak;
  const __nv_bfloat16 *B;
  long long sbk, sbn;
  float alpha;
  const float *bias;     // [N] or null
  int act;               // 0 identity, 1 GELU
  float *pre;            // pre-activation out (FP32), ld = ldo
  float *Cf;             // FP32 out, ld = ldo
  __nv_bfloat16 *Cb;     // BF16 out, ld = ldo
  long long ldo;
  const int *on;         // optional device flag: skip the launch's work when 0
};

constexpr int BM = 64, BN = 64, BK = 32, KPAD = 8;
constexpr int kGemmThreads = 128;

__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.f + erff(x * 0.70710678118654752f)) +
         x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(kGemmThreads) k_gemm_bf16(GemmArgs g) {
  __shared__ __align__(16) __nv_bfloat16 As[BM][BK + KPAD];
  __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + KPAD];
  if (g.on && *g.on == 0) return;  // uniform over the grid
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;  // 2 x 2 warps, 32 x 32 each
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int gq = lane >> 2, cq = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int k0 = 0; k0 < g.K; k0 += BK) {
    // tiles: lanes run along the operand's contiguous dimension
    for (int t = tid; t < BM * BK; t += kGemmThreads) {
      int mm, kk;
      if (g.sak == 1) {
        mm = t / BK;
        kk = t % BK;
      } else {
        mm = t % BM;
        kk = t / BM;
      }
      const int gm = m0 + mm, gk = k0 + kk;
      As[mm][kk] = (gm < g.M && gk < g.K) ? g.A[gm * g.sam + gk * g.sak] : zero;
    }
    for (int t = tid; t < BN * BK; t += kGemmThreads) {
      int nn, kk;
      if (g.sbk == 1) {
        nn = t / BK;
        kk = t % BK;
      } else {
        nn = t % BN;
        kk = t / BN;
      }
      const int gn = n0 + nn, gk = k0 + kk;
      Bs[nn][kk] = (gn < g.N && gk < g.K) ? g.B[gk * g.sbk + gn * g.sbn] : zero;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < BK; ks += 16) {
      uint32_t a[2][4], b[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm * 32 + i * 16 + gq;
        a[i][0] = *reinterpret_cast<const uint32_t *>(&As[r][ks + 2 * cq]);
        a[i][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][ks + 2 * cq]);
        a[i][2] = *reinterpret_cast<const uint32_t *>(&As[r][ks + 2 * cq + 8]);
        a[i][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][ks + 2 * cq + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn * 32 + j * 8 + gq;
        b[j][0] = *reinterpret_cast<const uint32_t *>(&Bs[c][ks + 2 * cq]);
        b[j][1] = *reinterpret_cast<const uint32_t *>(&Bs[c][ks + 2 * cq + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int m = m0 + wm * 32 + i * 16 + gq + (r >= 2 ? 8 : 0);
        const int n = n0 + wn * 32 + j * 8 + 2 * cq + (r & 1);
        if (m >= g.M || n >= g.N) continue;
        float v = g.alpha * acc[i][j][r];
        if (g.bias) v += g.bias[n];
        const long long o = (long long)m * g.ldo + n;
        if (g.pre) g.pre[o] = v;
        if (g.act == 1) v = gelu(v);
        if (g.Cf) g.Cf[o] = v;
        if (g.Cb) g.Cb[o] = __float2bfloat16(v);
      }
}

int gemm(const GemmArgs &g, cudaStream_t s) {
  dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM);
  k_gemm_bf16<<<grid, kGemmThreads, 0, s>>>(g);
  return ok() < 0 ? -1 : 1;
}

// ------------------------------------------------------ elementwise / misc --
__global__ void k_init_params(float *P, unsigned long long seed) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kNumParams) return;
  // SplitMix64 hash of (seed, i) -> uniform in [-1, 1)
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  const float u = (float)((z >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f;
  float v = 0.f;
  if (i < kOffB1) {
    const int col = (int)((i - kOffW1) % kMlpInPad);
    v = col < kMlpIn ? u * rsqrtf((float)kMlpIn) : 0.f;
  } else if (i >= kOffW2 && i < kOffB2) {
    v = u * rsqrtf((float)kMlpHidden);
  } else if (i >= kOffW3 && i < kOffB3) {
    const int row = (int)((i - kOffW3) / kMlpHidden);
    v = row < kMlpOut ? 0.1f * u * rsqrtf((float)kMlpHidden) : 0.f;
  }
  P[i] = v;
}

__global__ void k_params_to_bf16(const float *P, __nv_bfloat16 *W1, __nv_bfloat16 *W2,
                                 __nv_bfloat16 *W3, __nv_bfloat16 *W2t, __nv_bfloat16 *W3t) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kOffB1) W1[i] = __float2bfloat16(P[kOffW1 + i]);
  if (i < (long long)kMlpHidden * kMlpHidden) {
    const __nv_bfloat16 w = __float2bfloat16(P[kOffW2 + i]);
    W2[i] = w;
    // W2t[c][r] = W2[r][c]
    W2t[(i % kMlpHidden) * kMlpHidden + i / kMlpHidden] = w;
  }
  if (i < (long long)kMlpOutPad * kMlpHidden) {
    const __nv_bfloat16 w = __float2bfloat16(P[kOffW3 + i]);
    W3[i] = w;
    W3t[(i % kMlpHidden) * kMlpOutPad + i / kMlpHidden] = w;
  }
}

// out[c * ldo + r] = in[r * ldi + c] for a rows x cols BF16 matrix (32 x 32
// tiles through shared memory)
__global__ void k_transpose_bf16(const __nv_bfloat16 *in, int rows, int cols, int ldi,
                                 __nv_bfloat16 *out, int ldo) {
  __shared__ __nv_bfloat16 t[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) t[k][threadIdx.x] = in[(size_t)r * ldi + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[(size_t)c * ldo + r] = t[threadIdx.x][k];
  }
}

__global__ void k_pad_input(const float *X, int M, __nv_bfloat16 *Xb) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)M * kMlpInPad) return;
  const int m = (int)(t / kMlpInPad), c = (int)(t % kMlpInPad);
  Xb[t] = __float2bfloat16(c < kMlpIn ? X[(long long)m * kMlpIn + c] : 0.f);
}

// dY = 2 (Y - T) / (M * 85) on the 85 real outputs; loss accumulated in FP64
__global__ void k_mse_grad(const float *Y, const float *T, int M, float *dY,
                           __nv_bfloat16 *dYb, double *loss) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (t < (long long)M * kMlpOutPad) {
    const int m = (int)(t / kMlpOutPad), c = (int)(t % kMlpOutPad);
    float g = 0.f;
    if (c < kMlpOut) {
      const float e = Y[t] - T[(long long)m * kMlpOut + c];
      l = e * e;
      g = 2.f * e / ((float)M * (float)kMlpOut);
    }
    dY[t] = g;
    dYb[t] = __float2bfloat16(g);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, (double)l / ((double)M * kMlpOut));
}

// dA = dH * GELU'(pre) (FP32 in, BF16 + FP32 out)
__global__ void k_gelu_back(const float *dH, const float *pre, long long n, float *dA,
                            __nv_bfloat16 *dAb) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float v = dH[t] * gelu_grad(pre[t]);
  dA[t] = v;
  dAb[t] = __float2bfloat16(v);
}

// column sums of a row-major [M x N] FP32 matrix -> out[n] (bias gradients)
__global__ void k_colsum(const float *A, int M, int N, float *out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; ++m) s += A[(long long)m * N + n];
  out[n] = s;
}

// zero the gradients of the padding (W1 columns 397..399, W3/b3 rows 85..95)
__global__ void k_mask_grads(float *G) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kNumParams) return;
  bool pad = false;
  if (i < kOffB1) pad = ((i - kOffW1) % kMlpInPad) >= kMlpIn;
  else if (i >= kOffW3 && i < kOffB3) pad = ((i - kOffW3) / kMlpHidden) >= kMlpOut;
  else if (i >= kOffB3) pad = (i - kOffB3) >= kMlpOut;
  if (pad) G[i] = 0.f;
}

__global__ void k_adamw(float *P, const float *G, float *Mo, float *Vo, float lr, float b1,
                        float b2, float eps, float wd, float c1, float c2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kNumParams) return;
  const float g = G[i];
  const float m = b1 * Mo[i] + (1.f - b1) * g;
  const float v = b2 * Vo[i] + (1.f - b2) * g * g;
  Mo[i] = m;
  Vo[i] = v;
  const bool is_bias = (i >= kOffB1 && i < kOffW2) || (i >= kOffB2 && i < kOffW3) || i >= kOffB3;
  const float mh = m / c1, vh = v / c2;
  P[i] -= lr * (mh / (sqrtf(vh) + eps) + (is_bias ? 0.f : wd * P[i]));
}

// -------------------------------------------------------------- features ---
template <typename T>
__device__ __forceinline__ float local_res(const T *d, const int *ud, const int *pd, int nu, int i) {
  if (i < 3 * NU_LOC) {
    const int comp = i / NU_LOC, a = i - comp * NU_LOC;
    return (float)d[(size_t)comp * nu + ud[a]];
  }
  return (float)d[(size_t)3 * nu + pd[i - 3 * NU_LOC]];
}

template <typename T>
__global__ void k_cell_summary(DevCells cells, int nu, const T *d, float *summary, const int *on) {
  if (on && *on == 0) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= cells.ncells) return;
  const int *ud = cells.udofs + (size_t)warp * NU_LOC;
  const int *pd = cells.pdofs + (size_t)warp * NP_LOC;
  float r1 = 0.f, r2 = 0.f, r3 = 0.f, pv = 0.f;
  if (lane < NU_LOC) {
    r1 = (float)d[ud[lane]];
    r2 = (float)d[(size_t)nu + ud[lane]];
    r3 = (float)d[(size_t)2 * nu + ud[lane]];
  }
  if (lane < NP_LOC) pv = (float)d[(size_t)3 * nu + pd[lane]];
  float v[8] = {r1, r2, r3, r1 * r1, r2 * r2, r3 * r3, fabsf(r1) + fabsf(r2) + fabsf(r3), pv * pv};
#pragma unroll
  for (int k = 0; k < 8; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  const float p0 = __shfl_sync(0xffffffffu, pv, 0), p1 = __shfl_sync(0xffffffffu, pv, 1);
  const float p2 = __shfl_sync(0xffffffffu, pv, 2), p3 = __shfl_sync(0xffffffffu, pv, 3);
  if (lane == 0) {
    float *s = summary + (size_t)warp * kSummary;
    const float inv = 1.f / NU_LOC;
    s[0] = v[0] * inv;
    s[1] = v[1] * inv;
    s[2] = v[2] * inv;
    s[3] = sqrtf(v[3] * inv);
    s[4] = sqrtf(v[4] * inv);
    s[5] = sqrtf(v[5] * inv);
    s[6] = p0;
    s[7] = p1;
    s[8] = p2;
    s[9] = p3;
    s[10] = sqrtf((v[3] + v[4] + v[5] + v[7]) / NLOC);
    s[11] = v[6] / (3 * NU_LOC);
  }
}

template <typename T>
__global__ void k_cell_features(DevCells cells, int nu, const T *d, const float *summary,
                                const int *nbr, __nv_bfloat16 *Xb, float *Xf, float *scale,
                                const int *on) {
  if (on && *on == 0) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= cells.ncells) return;
  const int c = warp;
  const int *ud = cells.udofs + (size_t)c * NU_LOC;
  const int *pd = cells.pdofs + (size_t)c * NP_LOC;
  float r[3];
  float ss = 0.f;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int i = lane + 32 * q;
    r[q] = i < NLOC ? local_res(d, ud, pd, nu, i) : 0.f;
    ss += r[q] * r[q];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  // scale: the largest residual RMS of the cell and its 26 neighbours, so
  // every feature is O(1) even where the cell's own residual is small
  float sc = sqrtf(ss / NLOC);
  {
    const int nb = lane < kNeighbours ? nbr[(size_t)c * kNeighbours + lane] : -1;
    float m = nb >= 0 ? summary[(size_t)nb * kSummary + 10] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    sc = fmaxf(sc, m);
  }
  const float inv = sc > 0.f ? 1.f / sc : 0.f;
  if (lane == 0) scale[c] = sc;
  for (int i = lane; i < kMlpInPad; i += 32) {
    float v = 0.f;
    if (i < NLOC) {
      v = r[i >> 5] * inv;  // i = lane + 32q -> q = i >> 5
    } else if (i < kMlpIn) {
      const int j = i - NLOC, n = j / kSummary, q = j - n * kSummary;
      const int nb = nbr[(size_t)c * kNeighbours + n];
      v = nb >= 0 ? summary[(size_t)nb * kSummary + q] * inv : 0.f;
    }
    // a cell whose own residual is tiny against its neighbours' would give
    // unbounded features (and BF16 GEMM overflow): clamp
    v = fminf(fmaxf(v, -kFeatureClamp), kFeatureClamp);
    if (Xb) Xb[(size_t)c * kMlpInPad + i] = __float2bfloat16(v);
    if (Xf && i < kMlpIn) Xf[(size_t)c * kMlpIn + i] = v;
  }
}

template <typename T>
__global__ void k_learned_apply(DevCells cells, int nu, int nact, const int *list, int ncol,
                                const float *Y, const float *scale, const float *inv_mult_u,
                                T omega, T *u, const int *on) {
  if (on && *on == 0) return;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ncol * NLOC) return;
  const int slot = (int)(t / NLOC), i = (int)(t % NLOC);
  const int c = list[slot];
  const float y = Y[(size_t)c * kMlpOutPad + i] * scale[c];
  if (i < 3 * NU_LOC) {
    const int comp = i / NU_LOC, a = i - comp * NU_LOC;
    const int dof = cells.udofs[(size_t)c * NU_LOC + a];
    if (dof < nact) u[(size_t)comp * nu + dof] += omega * (T)(inv_mult_u[dof] * y);
  } else {
    u[(size_t)3 * nu + cells.pdofs[(size_t)c * NP_LOC + (i - 3 * NU_LOC)]] += omega * (T)y;
  }
}

template <typename T>
__global__ void k_cell_targets(DevCells cells, int nu, const T *e, const float *scale, float *Tg) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)cells.ncells * NLOC) return;
  const int c = (int)(t / NLOC), i = (int)(t % NLOC);
  const int *ud = cells.udofs + (size_t)c * NU_LOC;
  const int *pd = cells.pdofs + (size_t)c * NP_LOC;
  const float sc = scale[c];
  Tg[t] = sc > 0.f ? local_res(e, ud, pd, nu, i) / sc : 0.f;
}

inline unsigned blocks_for(long long n, int b = 256) { return (unsigned)((n + b - 1) / b); }

constexpr int kMrBlocks = 608;  // fixed grid: fixed summation order

__device__ __forceinline__ double block_sum_d(double v) {
  __shared__ double sh[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = l < 8 ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;
}

template <typename T>
__global__ void __launch_bounds__(256) k_mr_step(const T *d, const T *q, int n, double *partials,
                                                 unsigned int *counter, double omega_max,
                                                 double *omega, const int *on) {
  if (on && *on == 0) return;
  double dq = 0.0, qq = 0.0;
  for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) {
    const double a = (double)d[i], b = (double)q[i];
    dq += a * b;
    qq += b * b;
  }
  dq = block_sum_d(dq);
  qq = block_sum_d(qq);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = dq;
    partials[2 * blockIdx.x + 1] = qq;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double a = 0.0, b = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += 256) {
    a += ((volatile double *)partials)[2 * k];
    b += ((volatile double *)partials)[2 * k + 1];
  }
  a = block_sum_d(a);
  b = block_sum_d(b);
  if (threadIdx.x == 0) {
    double w = b > 0.0 ? -a / b : 0.0;
    w = w < 0.0 ? 0.0 : (w > omega_max ? omega_max : w);
    *omega = w;
    *counter = 0u;
  }
}

template <typename T>
__global__ void k_axpy_dev(T *u, const double *omega, const T *c, int n, const int *on) {
  if (on && *on == 0) return;
  const T w = (T)(*omega);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    u[i] += w * c[i];
}

}  // namespace

template <typename T>
int launch_mr_step(const T *d, const T *q, int n, double *partials, unsigned int *counter,
                   double omega_max, double *omega, const int *on, cudaStream_t s) {
  k_mr_step<T><<<kMrBlocks, 256, 0, s>>>(d, q, n, partials, counter, omega_max, omega, on);
  return ok() < 0 ? -1 : 1;
}

template <typename T>
int launch_axpy_dev(T *u, const double *omega, const T *c, int n, const int *on, cudaStream_t s) {
  unsigned g = blocks_for(n);
  if (g > 8 * 152) g = 8 * 152;
  k_axpy_dev<T><<<g, 256, 0, s>>>(u, omega, c, n, on);
  return ok() < 0 ? -1 : 1;
}
template int launch_mr_step<double>(const double *, const double *, int, double *, unsigned int *,
                                    double, double *, const int *, cudaStream_t);
template int launch_mr_step<float>(const float *, const float *, int, double *, unsigned int *,
                                   double, double *, const int *, cudaStream_t);
template int launch_axpy_dev<double>(double *, const double *, const double *, int, const int *,
                                     cudaStream_t);
template int launch_axpy_dev<float>(float *, const double *, const float *, int, const int *,
                                    cudaStream_t);

// ================================================================== MLP ====
cudaError_t mlp_create(Mlp &m, int device, unsigned long long seed, int max_batch) {
  m.device = device;
  m.max_batch = max_batch;
  m.step = 0;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return e;
  auto A = [&](void **p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  const size_t np = sizeof(float) * (size_t)kNumParams;
  A((void **)&m.P, np);
  A((void **)&m.G, np);
  A((void **)&m.Mo, np);
  A((void **)&m.Vo, np);
  A((void **)&m.W1, sizeof(__nv_bfloat16) * (size_t)kMlpHidden * kMlpInPad);
  A((void **)&m.W2, sizeof(__nv_bfloat16) * (size_t)kMlpHidden * kMlpHidden);
  A((void **)&m.W3, sizeof(__nv_bfloat16) * (size_t)kMlpOutPad * kMlpHidden);
  A((void **)&m.W2t, sizeof(__nv_bfloat16) * (size_t)kMlpHidden * kMlpHidden);
  A((void **)&m.W3t, sizeof(__nv_bfloat16) * (size_t)kMlpHidden * kMlpOutPad);
  const size_t B = (size_t)max_batch;
  m.ldt = (max_batch + 63) / 64 * 64;
  const size_t LT = (size_t)m.ldt;
  A((void **)&m.Tx, sizeof(__nv_bfloat16) * LT * kMlpInPad);
  A((void **)&m.Th, sizeof(__nv_bfloat16) * LT * kMlpHidden);
  A((void **)&m.Ta, sizeof(__nv_bfloat16) * LT * kMlpHidden);
  A((void **)&m.Ty, sizeof(__nv_bfloat16) * LT * kMlpOutPad);
  A((void **)&m.X, sizeof(__nv_bfloat16) * B * kMlpInPad);
  A((void **)&m.H1, sizeof(__nv_bfloat16) * B * kMlpHidden);
  A((void **)&m.H2, sizeof(__nv_bfloat16) * B * kMlpHidden);
  A((void **)&m.dYb, sizeof(__nv_bfloat16) * B * kMlpOutPad);
  A((void **)&m.dA2b, sizeof(__nv_bfloat16) * B * kMlpHidden);
  A((void **)&m.dA1b, sizeof(__nv_bfloat16) * B * kMlpHidden);
  A((void **)&m.pre1, sizeof(float) * B * kMlpHidden);
  A((void **)&m.pre2, sizeof(float) * B * kMlpHidden);
  A((void **)&m.Y, sizeof(float) * B * kMlpOutPad);
  A((void **)&m.dY, sizeof(float) * B * kMlpOutPad);
  A((void **)&m.dH, sizeof(float) * B * kMlpHidden);
  A((void **)&m.loss, sizeof(double));
  A((void **)&m.err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(m.err, 0, sizeof(int));
  if (e == cudaSuccess && mlp_tc_init() < 0) e = cudaErrorInvalidValue;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m.stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(m.Mo, 0, np, m.stream);
  cudaMemsetAsync(m.Vo, 0, np, m.stream);
  cudaMemsetAsync(m.G, 0, np, m.stream);
  k_init_params<<<blocks_for(kNumParams), 256, 0, m.stream>>>(m.P, seed);
  mlp_sync_bf16(m, m.stream);
  e = cudaStreamSynchronize(m.stream);
  return e;
}

void mlp_destroy(Mlp &m) {
  cudaSetDevice(m.device);
  if (m.stream) cudaStreamSynchronize(m.stream);
  void *ptrs[] = {m.P,   m.G,    m.Mo,   m.Vo,   m.W1,   m.W2,   m.W3,  m.W2t, m.W3t,
                  m.Tx,  m.Th,   m.Ta,   m.Ty,   m.X,    m.H1,   m.H2,  m.dYb, m.dA2b,
                  m.dA1b, m.pre1, m.pre2, m.Y,   m.dY,   m.dH,   m.loss, m.err};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (m.stream) cudaStreamDestroy(m.stream);
  m = Mlp();
}

int mlp_sync_bf16(const Mlp &m, cudaStream_t s) {
  k_params_to_bf16<<<blocks_for(kOffB1), 256, 0, s>>>(m.P, m.W1, m.W2, m.W3, m.W2t, m.W3t);
  return ok() < 0 ? -1 : 1;
}

int mlp_forward(const Mlp &m, const __nv_bfloat16 *X, int M, __nv_bfloat16 *H1, __nv_bfloat16 *H2,
                float *Y, cudaStream_t s, const int *on, int *err) {
  if (M <= 0) return 0;
  int n = 0, r;
  if (m.tc) {
    int *e = err ? err : m.err;
    if ((r = mlp_layer_tc(1, X, M, m.W1, m.P + kOffB1, 1, nullptr, nullptr, H1, on, e, s)) < 0)
      return -1;
    n += r;
    if ((r = mlp_layer_tc(2, H1, M, m.W2, m.P + kOffB2, 1, nullptr, nullptr, H2, on, e, s)) < 0)
      return -1;
    n += r;
    if ((r = mlp_layer_tc(3, H2, M, m.W3, m.P + kOffB3, 0, nullptr, Y, nullptr, on, e, s)) < 0)
      return -1;
    return n + r;
  }
  GemmArgs g{};
  // layer 1: H1 = GELU(X W1^T + b1)
  g = GemmArgs{M, kMlpHidden, kMlpInPad, X, kMlpInPad, 1, m.W1, 1, kMlpInPad, 1.f,
               m.P + kOffB1, 1, nullptr, nullptr, H1, kMlpHidden, on};
  if ((r = gemm(g, s)) < 0) return -1;
  n += r;
  g = GemmArgs{M, kMlpHidden, kMlpHidden, H1, kMlpHidden, 1, m.W2, 1, kMlpHidden, 1.f,
               m.P + kOffB2, 1, nullptr, nullptr, H2, kMlpHidden, on};
  if ((r = gemm(g, s)) < 0) return -1;
  n += r;
  g = GemmArgs{M, kMlpOutPad, kMlpHidden, H2, kMlpHidden, 1, m.W3, 1, kMlpHidden, 1.f,
               m.P + kOffB3, 0, nullptr, Y, nullptr, kMlpOutPad, on};
  if ((r = gemm(g, s)) < 0) return -1;
  return n + r;
}

__global__ void k_copy_out(const float *Y, int M, float *out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)M * kMlpOut) return;
  out[t] = Y[(t / kMlpOut) * kMlpOutPad + t % kMlpOut];
}

int mlp_forward_f32(Mlp &m, const float *X, int M, float *Yout, cudaStream_t s) {
  if (M <= 0 || M > m.max_batch) return -1;
  k_pad_input<<<blocks_for((long long)M * kMlpInPad), 256, 0, s>>>(X, M, m.X);
  const int r = mlp_forward(m, m.X, M, m.H1, m.H2, m.Y, s);
  if (r < 0) return -1;
  k_copy_out<<<blocks_for((long long)M * kMlpOut), 256, 0, s>>>(m.Y, M, Yout);
  return ok() < 0 ? -1 : r + 2;
}

int mlp_loss_grad(Mlp &m, const float *X, const float *T, int M, cudaStream_t s) {
  if (M <= 0 || M > m.max_batch) return -1;
  int n = 0, r;
  cudaMemsetAsync(m.loss, 0, sizeof(double), s);
  k_pad_input<<<blocks_for((long long)M * kMlpInPad), 256, 0, s>>>(X, M, m.X);
  n++;
  GemmArgs g{};
  // forward, keeping pre-activations
  if (m.tc) {
    if ((r = mlp_layer_tc(1, m.X, M, m.W1, m.P + kOffB1, 1, m.pre1, nullptr, m.H1, nullptr, m.err,
                          s)) < 0)
      return -1;
    n += r;
    if ((r = mlp_layer_tc(2, m.H1, M, m.W2, m.P + kOffB2, 1, m.pre2, nullptr, m.H2, nullptr,
                          m.err, s)) < 0)
      return -1;
    n += r;
    if ((r = mlp_layer_tc(3, m.H2, M, m.W3, m.P + kOffB3, 0, nullptr, m.Y, nullptr, nullptr,
                          m.err, s)) < 0)
      return -1;
    n += r;
  } else {
    g = GemmArgs{M, kMlpHidden, kMlpInPad, m.X, kMlpInPad, 1, m.W1, 1, kMlpInPad, 1.f,
                 m.P + kOffB1, 1, m.pre1, nullptr, m.H1, kMlpHidden};
    if ((r = gemm(g, s)) < 0) return -1;
    n += r;
    g = GemmArgs{M, kMlpHidden, kMlpHidden, m.H1, kMlpHidden, 1, m.W2, 1, kMlpHidden, 1.f,
                 m.P + kOffB2, 1, m.pre2, nullptr, m.H2, kMlpHidden};
    if ((r = gemm(g, s)) < 0) return -1;
    n += r;
    g = GemmArgs{M, kMlpOutPad, kMlpHidden, m.H2, kMlpHidden, 1, m.W3, 1, kMlpHidden, 1.f,
                 m.P + kOffB3, 0, nullptr, m.Y, nullptr, kMlpOutPad};
    if ((r = gemm(g, s)) < 0) return -1;
    n += r;
  }
  k_mse_grad<<<blocks_for((long long)M * kMlpOutPad), 256, 0, s>>>(m.Y, T, M, m.dY, m.dYb, m.loss);
  n++;
  if (m.tc) {
    // the six backward GEMMs on tcgen05: weight gradients as (batch-major
    // operands transposed to K-major) products over the batch, data
    // gradients against the transposed weights
    const int lt = m.ldt;
    auto tr = [&](const __nv_bfloat16 *in, int cols, __nv_bfloat16 *out) {
      k_transpose_bf16<<<dim3((cols + 31) / 32, (M + 31) / 32), dim3(32, 8), 0, s>>>(in, M, cols,
                                                                                    cols, out, lt);
      n++;
    };
    const long long nh = (long long)M * kMlpHidden;
    // layer 3: dW3 = dY^T H2, db3, dH2 = dY W3
    tr(m.dYb, kMlpOutPad, m.Ty);
    tr(m.H2, kMlpHidden, m.Th);
    if ((r = mlp_gemm_tc(m.Ty, lt, kMlpOutPad, m.Th, lt, kMlpHidden, M, m.G + kOffW3, kMlpHidden,
                         m.err, s)) < 0)
      return -1;
    n += r;
    k_colsum<<<1, 128, 0, s>>>(m.dY, M, kMlpOutPad, m.G + kOffB3);
    n++;
    if ((r = mlp_gemm_tc(m.dYb, kMlpOutPad, M, m.W3t, kMlpOutPad, kMlpHidden, kMlpOutPad, m.dH,
                         kMlpHidden, m.err, s)) < 0)
      return -1;
    n += r;
    // layer 2 (dA2 in pre2's buffer)
    k_gelu_back<<<blocks_for(nh), 256, 0, s>>>(m.dH, m.pre2, nh, m.pre2, m.dA2b);
    n++;
    tr(m.dA2b, kMlpHidden, m.Ta);
    tr(m.H1, kMlpHidden, m.Th);
    if ((r = mlp_gemm_tc(m.Ta, lt, kMlpHidden, m.Th, lt, kMlpHidden, M, m.G + kOffW2, kMlpHidden,
                         m.err, s)) < 0)
      return -1;
    n += r;
    k_colsum<<<2, 128, 0, s>>>(m.pre2, M, kMlpHidden, m.G + kOffB2);
    n++;
    if ((r = mlp_gemm_tc(m.dA2b, kMlpHidden, M, m.W2t, kMlpHidden, kMlpHidden, kMlpHidden, m.dH,
                         kMlpHidden, m.err, s)) < 0)
      return -1;
    n += r;
    // layer 1 (dA1 in pre1's buffer)
    k_gelu_back<<<blocks_for(nh), 256, 0, s>>>(m.dH, m.pre1, nh, m.pre1, m.dA1b);
    n++;
    tr(m.dA1b, kMlpHidden, m.Ta);
    tr(m.X, kMlpInPad, m.Tx);
    if ((r = mlp_gemm_tc(m.Ta, lt, kMlpHidden, m.Tx, lt, kMlpInPad, M, m.G + kOffW1, kMlpInPad,
                         m.err, s)) < 0)
      return -1;
    n += r;
    k_colsum<<<2, 128, 0, s>>>(m.pre1, M, kMlpHidden, m.G + kOffB1);
    n++;
  } else {
    // layer 3: dW3 = dY^T H2, db3, dH2 = dY W3
    g = GemmArgs{kMlpOutPad, kMlpHidden, M, m.dYb, 1, kMlpOutPad, m.H2, kMlpHidden, 1, 1.f,
                 nullptr, 0, nullptr, m.G + kOffW3, nullptr, kMlpHidden};
    if ((r = gemm(g, s)) < 0) return -1;
    n += r;
    k_colsum<<<1, 128, 0, s>>>(m.dY, M, kMlpOutPad, m.G + kOffB3);
    n++;
    g = GemmArgs{M, kMlpHidden, kMlpOutPad, m.dYb, kMlpOutPad, 1, m.W3, kMlpHidden, 1, 1.f,
                 nullptr, 0, nullptr, m.dH, nullptr, kMlpHidden};
    if ((r = gemm(g, s)) < 0) return -1;
    n += r;
    const long long nh = (long long)M * kMlpHidden;
    // layer 2 (dA2 in pre2's buffer)
    k_gelu_back<<<blocks_for(nh), 256, 0, s>>>(m.dH, m.pre2, nh, m.pre2, m.dA2b);
    n++;
    g = GemmArgs{kMlpHidden, kMlpHidden, M, m.dA2b, 1, kMlpHidden, m.H1, kMlpHidden, 1, 1.f,
                 nullptr, 0, nullptr, m.G + kOffW2, nullptr, kMlpHidden};
    if ((r = gemm(g, s)) < 0) return -1;
    n += r;
    k_colsum<<<2, 128, 0, s>>>(m.pre2, M, kMlpHidden, m.G + kOffB2);
    n++;
    g = GemmArgs{M, kMlpHidden, kMlpHidden, m.dA2b, kMlpHidden, 1, m.W2, kMlpHidden, 1, 1.f,
                 nullptr, 0, nullptr, m.dH, nullptr, kMlpHidden};
    if ((r = gemm(g, s)) < 0) return -1;
    n += r;
    // layer 1 (dA1 in pre1's buffer)
    k_gelu_back<<<blocks_for(nh), 256, 0, s>>>(m.dH, m.pre1, nh, m.pre1, m.dA1b);
    n++;
    g = GemmArgs{kMlpHidden, kMlpInPad, M, m.dA1b, 1, kMlpHidden, m.X, kMlpInPad, 1, 1.f,
                 nullptr, 0, nullptr, m.G + kOffW1, nullptr, kMlpInPad};
    if ((r = gemm(g, s)) < 0) return -1;
    n += r;
    k_colsum<<<2, 128, 0, s>>>(m.pre1, M, kMlpHidden, m.G + kOffB1);
    n++;
  }
  k_mask_grads<<<blocks_for(kNumParams), 256, 0, s>>>(m.G);
  n++;
  return ok() < 0 ? -1 : n;
}

int mlp_adamw(Mlp &m, float lr, float b1, float b2, float eps, float wd, cudaStream_t s) {
  m.step++;
  const float c1 = 1.f - powf(b1, (float)m.step), c2 = 1.f - powf(b2, (float)m.step);
  k_adamw<<<blocks_for(kNumParams), 256, 0, s>>>(m.P, m.G, m.Mo, m.Vo, lr, b1, b2, eps, wd, c1, c2);
  if (ok() < 0) return -1;
  return mlp_sync_bf16(m, s) < 0 ? -1 : 2;
}

// ============================================================ features ====
template <typename T>
int launch_cell_summary(const DevCells &cells, int nu, const T *d, float *summary, const int *on,
                        cudaStream_t s) {
  if (cells.ncells <= 0) return 0;
  k_cell_summary<T><<<blocks_for((long long)cells.ncells * 32), 256, 0, s>>>(cells, nu, d, summary, on);
  return ok() < 0 ? -1 : 1;
}

template <typename T>
int launch_cell_features(const DevCells &cells, int nu, const T *d, const float *summary,
                         const int *nbr, __nv_bfloat16 *Xb, float *Xf, float *scale, const int *on,
                         cudaStream_t s) {
  if (cells.ncells <= 0) return 0;
  k_cell_features<T><<<blocks_for((long long)cells.ncells * 32), 256, 0, s>>>(
      cells, nu, d, summary, nbr, Xb, Xf, scale, on);
  return ok() < 0 ? -1 : 1;
}

template <typename T>
int launch_learned_apply(const DevCells &cells, int nu, int nact, const int *cell_list, int ncol,
                         const float *Y, const float *scale, const float *inv_mult_u, T omega,
                         T *u, const int *on, cudaStream_t s) {
  if (ncol <= 0) return 0;
  k_learned_apply<T><<<blocks_for((long long)ncol * NLOC), 256, 0, s>>>(
      cells, nu, nact, cell_list, ncol, Y, scale, inv_mult_u, omega, u, on);
  return ok() < 0 ? -1 : 1;
}

template <typename T>
int launch_cell_targets(const DevCells &cells, int nu, const T *e, const float *scale, float *Tg,
                        cudaStream_t s) {
  if (cells.ncells <= 0) return 0;
  k_cell_targets<T><<<blocks_for((long long)cells.ncells * NLOC), 256, 0, s>>>(cells, nu, e, scale, Tg);
  return ok() < 0 ? -1 : 1;
}

#define PM_LINST(T)                                                                               \
  template int launch_cell_summary<T>(const DevCells &, int, const T *, float *, const int *,     \
                                      cudaStream_t);                                              \
  template int launch_cell_features<T>(const DevCells &, int, const T *, const float *,           \
                                       const int *, __nv_bfloat16 *, float *, float *,            \
                                       const int *, cudaStream_t);                                \
  template int launch_learned_apply<T>(const DevCells &, int, int, const int *, int,              \
                                       const float *, const float *, const float *, T, T *,       \
                                       const int *, cudaStream_t);                                \
  template int launch_cell_targets<T>(const DevCells &, int, const T *, const float *, float *,   \
                                      cudaStream_t);
PM_LINST(double)
PM_LINST(float)
#undef PM_LINST

}  // namespace pm
