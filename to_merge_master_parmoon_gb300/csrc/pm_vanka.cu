// pm_vanka.cu — cell-Vanka smoother and coarse direct solve on sm_103a.
//
// The reference assembles each hexahedron's 85x85 local saddle block
// (27 Q2 nodes x 3 components + 4 P1disc modes) and calls dgetrf/dgetrs on
// it in every sweep (TNSE_MGLevel4::CellVanka, src/FE/NSE_MGLevel4.C:1653-2087;
// SolveLinearSystemLapack, src/FE/LinAlg.C:106-131).  The local blocks do not
// change during a linear solve, so here they are gathered and factored once
// per matrix (k_vanka_factor) and every sweep only
//   1. forms each cell's local residual from the full CSR rows (the same
//      rows the reference reads, :1810-1941),
//   2. applies the stored factors (forward/back substitution),
//   3. adds damp * delta to the cell's DOFs (:2044-2059),
// colour by colour: cells of one colour share no DOF; their residuals are
// all taken from the state before the colour (CellVanka_GPU semantics,
// src/FE/NSE_CellVanka.cu:2181-2365), so step 3 runs after step 1-2 of the
// whole colour in a separate launch.
#include <cuda_runtime.h>

#include <cstdint>

#include "pm_kernels.h"

namespace pm {

namespace {

constexpr unsigned kFull = 0xffffffffu;

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T ld_stream(const T *p) {
  return __ldcs(p);
}

// ------------------------------------------------------------------ factor --
// One CTA per cell.  S is the local matrix, column-major (S[col*85+row]),
// exactly the reference's System layout.  Right-looking LU with partial
// pivoting (first maximal |pivot|, dgetrf's choice).
constexpr int kFactorThreads = 256;

template <typename TC, typename TF>
__global__ void __launch_bounds__(kFactorThreads) k_vanka_factor(DevOp<double> op, DevCells cells,
                                                                 TF *__restrict__ factors,
                                                                 uint8_t *__restrict__ perm,
                                                                 int *status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TC *S = reinterpret_cast<TC *>(smem_raw);
  __shared__ int ud[NU_LOC], pd[NP_LOC];
  __shared__ int piv_row;
  __shared__ unsigned char pm[NLOC];
  __shared__ int singular;
  const int cell = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = kFactorThreads / 32;

  for (int t = tid; t < NLOC * NLOC; t += kFactorThreads) S[t] = TC(0);
  if (tid < NU_LOC) ud[tid] = cells.udofs[(size_t)cell * NU_LOC + tid];
  if (tid < NP_LOC) pd[tid] = cells.pdofs[(size_t)cell * NP_LOC + tid];
  if (tid < NLOC) pm[tid] = (unsigned char)tid;
  if (tid == 0) singular = 0;
  __syncthreads();

  // gather: velocity rows (9 blocks + BT), pressure rows (B)
  for (int a = warp; a < NU_LOC; a += nwarps) {
    const int r = ud[a];
    const bool dir = r >= op.nact;
    for (int j = op.a_rowptr[r] + lane; j < op.a_rowptr[r + 1]; j += 32) {
      const int l = op.a_col[j];
      int m = -1;
      for (int q = 0; q < NU_LOC; ++q)
        if (ud[q] == l) {
          m = q;
          break;
        }
      if (m < 0) continue;
      const int c1 = m * NLOC, c2 = (m + NU_LOC) * NLOC, c3 = (m + 2 * NU_LOC) * NLOC;
      S[c1 + a] = (TC)op.a[0][j];
      S[c2 + a + NU_LOC] = (TC)op.a[4][j];
      S[c3 + a + 2 * NU_LOC] = (TC)op.a[8][j];
      if (!dir) {
        S[c2 + a] = (TC)op.a[1][j];
        S[c3 + a] = (TC)op.a[2][j];
        S[c1 + a + NU_LOC] = (TC)op.a[3][j];
        S[c3 + a + NU_LOC] = (TC)op.a[5][j];
        S[c1 + a + 2 * NU_LOC] = (TC)op.a[6][j];
        S[c2 + a + 2 * NU_LOC] = (TC)op.a[7][j];
      }
    }
    if (!dir) {
      for (int j = op.bt_rowptr[r] + lane; j < op.bt_rowptr[r + 1]; j += 32) {
        const int l = op.bt_col[j];
        int m = -1;
        for (int q = 0; q < NP_LOC; ++q)
          if (pd[q] == l) {
            m = q;
            break;
          }
        if (m < 0) continue;
        const int c = (m + 3 * NU_LOC) * NLOC;
        S[c + a] = (TC)op.bt[0][j];
        S[c + a + NU_LOC] = (TC)op.bt[1][j];
        S[c + a + 2 * NU_LOC] = (TC)op.bt[2][j];
      }
    }
  }
  for (int k = warp; k < NP_LOC; k += nwarps) {
    const int r = pd[k], row = 3 * NU_LOC + k;
    for (int j = op.b_rowptr[r] + lane; j < op.b_rowptr[r + 1]; j += 32) {
      const int l = op.b_col[j];
      int m = -1;
      for (int q = 0; q < NU_LOC; ++q)
        if (ud[q] == l) {
          m = q;
          break;
        }
      if (m < 0) continue;
      S[m * NLOC + row] = (TC)op.b[0][j];
      S[(m + NU_LOC) * NLOC + row] = (TC)op.b[1][j];
      S[(m + 2 * NU_LOC) * NLOC + row] = (TC)op.b[2][j];
    }
  }
  __syncthreads();

  for (int k = 0; k < NLOC; ++k) {
    if (warp == 0) {
      TC best = TC(-1);
      int bi = k;
      for (int i = k + lane; i < NLOC; i += 32) {
        const TC v = fabs(S[k * NLOC + i]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const TC ob = __shfl_xor_sync(kFull, best, o);
        const int oi = __shfl_xor_sync(kFull, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (lane == 0) piv_row = bi;
    }
    __syncthreads();
    const int p = piv_row;
    if (p != k) {
      for (int j = tid; j < NLOC; j += kFactorThreads) {
        const TC t = S[j * NLOC + k];
        S[j * NLOC + k] = S[j * NLOC + p];
        S[j * NLOC + p] = t;
      }
      if (tid == 0) {
        const unsigned char t = pm[k];
        pm[k] = pm[p];
        pm[p] = t;
      }
    }
    __syncthreads();
    const TC piv = S[k * NLOC + k];
    if (piv == TC(0)) {
      if (tid == 0) singular = 1;
    } else {
      const TC rp = TC(1) / piv;
      for (int i = k + 1 + tid; i < NLOC; i += kFactorThreads) S[k * NLOC + i] *= rp;
    }
    __syncthreads();
    for (int jj = k + 1 + warp; jj < NLOC; jj += nwarps) {
      const TC ukj = S[jj * NLOC + k];
      if (ukj != TC(0))
        for (int ii = k + 1 + lane; ii < NLOC; ii += 32) S[jj * NLOC + ii] -= S[k * NLOC + ii] * ukj;
    }
    __syncthreads();
  }
  TF *F = factors + (size_t)cell * NLOC * NLOC;
  for (int t = tid; t < NLOC * NLOC; t += kFactorThreads) {
    const int i = t % NLOC, j = t / NLOC;
    TC v = S[t];
    if (i == j) v = (v != TC(0)) ? TC(1) / v : TC(0);
    F[t] = (TF)v;
  }
  if (tid < NLOC) perm[(size_t)cell * NLOC + tid] = pm[tid];
  if (tid == 0 && singular) atomicOr(status, 1);
}

// ------------------------------------------------------------------ apply ---
// One warp per cell of the colour.  Lane l owns local rows l, l+32, l+64 of
// the permuted system during the substitutions.
constexpr int kSolveWarps = 8;

template <typename T>
__global__ void __launch_bounds__(kSolveWarps * 32) k_vanka_solve(
    DevOp<T> op, DevCells cells, const int *__restrict__ list, int ncol, const T *__restrict__ F,
    const uint8_t *__restrict__ perm, const T *__restrict__ u, const T *__restrict__ rhs,
    T *__restrict__ dbuf) {
  __shared__ T sres[kSolveWarps][NLOC + 3];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = blockIdx.x * kSolveWarps + warp;
  if (slot >= ncol) return;  // whole warp leaves; no block-wide barrier below
  const int cell = list[slot];
  const int nu = op.nu;
  const int my_ud = lane < NU_LOC ? cells.udofs[(size_t)cell * NU_LOC + lane] : 0;
  const int my_pd = lane < NP_LOC ? cells.pdofs[(size_t)cell * NP_LOC + lane] : 0;
  T *R = sres[warp];
  const T *u1 = u, *u2 = u + nu, *u3 = u + 2 * nu, *p = u + 3 * nu;

  // 1. local residual over the full rows of the cell's 85 DOFs
  for (int a = 0; a < NU_LOC; ++a) {
    const int r = __shfl_sync(kFull, my_ud, a);
    T s1 = 0, s2 = 0, s3 = 0;
    const int rs = op.a_rowptr[r], re = op.a_rowptr[r + 1];
    for (int j = rs + lane; j < re; j += 32) {
      const int c = __ldg(op.a_col + j);
      const T x1 = u1[c], x2 = u2[c], x3 = u3[c];
      s1 += ld_stream(op.a[0] + j) * x1 + ld_stream(op.a[1] + j) * x2 + ld_stream(op.a[2] + j) * x3;
      s2 += ld_stream(op.a[3] + j) * x1 + ld_stream(op.a[4] + j) * x2 + ld_stream(op.a[5] + j) * x3;
      s3 += ld_stream(op.a[6] + j) * x1 + ld_stream(op.a[7] + j) * x2 + ld_stream(op.a[8] + j) * x3;
    }
    if (r < op.nact) {
      const int bs = op.bt_rowptr[r], be = op.bt_rowptr[r + 1];
      for (int j = bs + lane; j < be; j += 32) {
        const T pv = p[__ldg(op.bt_col + j)];
        s1 += ld_stream(op.bt[0] + j) * pv;
        s2 += ld_stream(op.bt[1] + j) * pv;
        s3 += ld_stream(op.bt[2] + j) * pv;
      }
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    s3 = warp_sum(s3);
    if (lane == 0) {
      R[a] = rhs[r] - s1;
      R[a + NU_LOC] = rhs[nu + r] - s2;
      R[a + 2 * NU_LOC] = rhs[2 * nu + r] - s3;
    }
  }
  for (int k = 0; k < NP_LOC; ++k) {
    const int r = __shfl_sync(kFull, my_pd, k);
    T s = 0;
    for (int j = op.b_rowptr[r] + lane; j < op.b_rowptr[r + 1]; j += 32) {
      const int c = __ldg(op.b_col + j);
      s += ld_stream(op.b[0] + j) * u1[c] + ld_stream(op.b[1] + j) * u2[c] +
           ld_stream(op.b[2] + j) * u3[c];
    }
    s = warp_sum(s);
    if (lane == 0) R[3 * NU_LOC + k] = rhs[3 * nu + r] - s;
  }
  __syncwarp();

  // 2. P A = L U: y = P r, L y' = y, U x = y'
  const uint8_t *pc = perm + (size_t)cell * NLOC;
  const T *Fc = F + (size_t)cell * NLOC * NLOC;
  const bool has2 = lane + 64 < NLOC;
  T y0 = R[__ldg(pc + lane)];
  T y1 = R[__ldg(pc + lane + 32)];
  T y2 = has2 ? R[__ldg(pc + lane + 64)] : T(0);
  for (int j = 0; j < NLOC - 1; ++j) {
    const T *col = Fc + (size_t)j * NLOC;
    const T l0 = (lane > j) ? ld_stream(col + lane) : T(0);
    const T l1 = (lane + 32 > j) ? ld_stream(col + lane + 32) : T(0);
    const T l2 = (has2 && lane + 64 > j) ? ld_stream(col + lane + 64) : T(0);
    const int owner = j & 31;
    const T ysel = (j < 32) ? y0 : ((j < 64) ? y1 : y2);
    const T yj = __shfl_sync(kFull, ysel, owner);
    y0 -= l0 * yj;
    y1 -= l1 * yj;
    y2 -= l2 * yj;
  }
  for (int j = NLOC - 1; j >= 0; --j) {
    const T *col = Fc + (size_t)j * NLOC;
    const T u0 = (lane <= j) ? ld_stream(col + lane) : T(0);
    const T u1v = (lane + 32 <= j) ? ld_stream(col + lane + 32) : T(0);
    const T u2v = (has2 && lane + 64 <= j) ? ld_stream(col + lane + 64) : T(0);
    const int owner = j & 31;
    // diagonal holds 1/U_jj
    if (lane == owner) {
      if (j < 32)
        y0 *= u0;
      else if (j < 64)
        y1 *= u1v;
      else
        y2 *= u2v;
    }
    const T ysel = (j < 32) ? y0 : ((j < 64) ? y1 : y2);
    const T xj = __shfl_sync(kFull, ysel, owner);
    if (lane < j) y0 -= u0 * xj;
    if (lane + 32 < j) y1 -= u1v * xj;
    if (has2 && lane + 64 < j) y2 -= u2v * xj;
  }
  T *D = dbuf + (size_t)slot * NLOC;
  D[lane] = y0;
  D[lane + 32] = y1;
  if (has2) D[lane + 64] = y2;
}

template <typename T>
__global__ void k_vanka_update(DevCells cells, int nu, const int *__restrict__ list, int ncol,
                               const T *__restrict__ dbuf, T damp, T *__restrict__ u) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ncol * NLOC) return;
  const int slot = (int)(t / NLOC), i = (int)(t % NLOC);
  const int cell = list[slot];
  const T d = damp * dbuf[t];
  if (i < 3 * NU_LOC) {
    const int comp = i / NU_LOC, a = i % NU_LOC;
    u[(size_t)comp * nu + cells.udofs[(size_t)cell * NU_LOC + a]] += d;
  } else {
    u[(size_t)3 * nu + cells.pdofs[(size_t)cell * NP_LOC + (i - 3 * NU_LOC)]] += d;
  }
}

// ----------------------------------------------------------------- coarse ---
// Dense column-major coarse matrix a[col*N + row] (SolveExact layout).
__global__ void k_coarse_scatter(DevOp<double> op, double *a, int N) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nu = op.nu, nu2 = 2 * nu, nug = 3 * nu;
  if (t < op.nact) {
    const int i = t;
    for (int j = op.a_rowptr[i]; j < op.a_rowptr[i + 1]; ++j) {
      const size_t idx = op.a_col[j];
      a[idx * N + i] = op.a[0][j];
      a[(idx + nu) * N + i] = op.a[1][j];
      a[idx * N + i + nu] = op.a[3][j];
      a[(idx + nu) * N + i + nu] = op.a[4][j];
      a[(idx + nu2) * N + i] = op.a[2][j];
      a[(idx + nu2) * N + i + nu] = op.a[5][j];
      a[idx * N + i + nu2] = op.a[6][j];
      a[(idx + nu) * N + i + nu2] = op.a[7][j];
      a[(idx + nu2) * N + i + nu2] = op.a[8][j];
    }
    for (int j = op.bt_rowptr[i]; j < op.bt_rowptr[i + 1]; ++j) {
      const size_t l = ((size_t)op.bt_col[j] + nug) * N;
      a[l + i] = op.bt[0][j];
      a[l + i + nu] = op.bt[1][j];
      a[l + i + 2 * nu] = op.bt[2][j];
    }
  } else if (t < nu) {
    const int i = t;
    for (int j = op.a_rowptr[i]; j < op.a_rowptr[i + 1]; ++j) {
      const size_t idx = op.a_col[j];
      a[i + N * idx] = op.a[0][j];
      a[(idx + nu) * N + i + nu] = op.a[4][j];
      a[(idx + nu2) * N + i + nu2] = op.a[8][j];
    }
  } else if (t < nu + op.np) {
    const int i = t - nu;
    for (int j = op.b_rowptr[i]; j < op.b_rowptr[i + 1]; ++j) {
      const size_t idx = op.b_col[j];
      a[idx * N + i + nug] = op.b[0][j];
      a[(idx + nu) * N + i + nug] = op.b[1][j];
      a[(idx + nu2) * N + i + nug] = op.b[2][j];
    }
  }
}

// replace the first pressure equation by p_0 = 0 (:5824-5827)
__global__ void k_coarse_pin(double *a, int N, int row) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    a[(size_t)i * N + row] = (i == row) ? 1.0 : 0.0;
}

constexpr int kDenseThreads = 1024;

__global__ void __launch_bounds__(kDenseThreads) k_dense_lu(double *a, int N, int *ipiv,
                                                            int *status) {
  __shared__ double bv[32];
  __shared__ int bi[32];
  __shared__ int piv_row;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = kDenseThreads / 32;
  for (int k = 0; k < N; ++k) {
    double best = -1.0;
    int bidx = k;
    for (int i = k + tid; i < N; i += kDenseThreads) {
      const double v = fabs(a[(size_t)k * N + i]);
      if (v > best) {
        best = v;
        bidx = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(kFull, best, o);
      const int oi = __shfl_xor_sync(kFull, bidx, o);
      if (ob > best || (ob == best && oi < bidx)) {
        best = ob;
        bidx = oi;
      }
    }
    if (lane == 0) {
      bv[warp] = best;
      bi[warp] = bidx;
    }
    __syncthreads();
    if (warp == 0) {
      best = bv[lane];
      bidx = bi[lane];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(kFull, best, o);
        const int oi = __shfl_xor_sync(kFull, bidx, o);
        if (ob > best || (ob == best && oi < bidx)) {
          best = ob;
          bidx = oi;
        }
      }
      if (lane == 0) {
        piv_row = bidx;
        ipiv[k] = bidx;
      }
    }
    __syncthreads();
    const int p = piv_row;
    if (p != k)
      for (int j = tid; j < N; j += kDenseThreads) {
        const double t = a[(size_t)j * N + k];
        a[(size_t)j * N + k] = a[(size_t)j * N + p];
        a[(size_t)j * N + p] = t;
      }
    __syncthreads();
    const double piv = a[(size_t)k * N + k];
    if (piv == 0.0) {
      if (tid == 0) atomicOr(status, 2);
    } else {
      const double rp = 1.0 / piv;
      for (int i = k + 1 + tid; i < N; i += kDenseThreads) a[(size_t)k * N + i] *= rp;
    }
    __syncthreads();
    for (int jj = k + 1 + warp; jj < N; jj += nwarps) {
      const double ukj = a[(size_t)jj * N + k];
      if (ukj != 0.0)
        for (int ii = k + 1 + lane; ii < N; ii += 32)
          a[(size_t)jj * N + ii] -= a[(size_t)k * N + ii] * ukj;
    }
    __syncthreads();
  }
}

constexpr int kDenseSolveThreads = 512;

__global__ void __launch_bounds__(kDenseSolveThreads) k_dense_solve(const double *lu,
                                                                    const int *ipiv, int N,
                                                                    const double *b, double *x,
                                                                    int pin_row) {
  extern __shared__ double xs[];
  const int tid = threadIdx.x;
  for (int i = tid; i < N; i += kDenseSolveThreads) xs[i] = b[i];
  __syncthreads();
  if (tid == 0) {
    if (pin_row >= 0) xs[pin_row] = 0.0;
    for (int k = 0; k < N; ++k) {
      const int p = ipiv[k];
      if (p != k) {
        const double t = xs[k];
        xs[k] = xs[p];
        xs[p] = t;
      }
    }
  }
  __syncthreads();
  for (int j = 0; j < N; ++j) {
    const double xj = xs[j];
    if (xj != 0.0)
      for (int i = j + 1 + tid; i < N; i += kDenseSolveThreads) xs[i] -= lu[(size_t)j * N + i] * xj;
    __syncthreads();
  }
  for (int j = N - 1; j >= 0; --j) {
    if (tid == 0) xs[j] /= lu[(size_t)j * N + j];
    __syncthreads();
    const double xj = xs[j];
    if (xj != 0.0)
      for (int i = tid; i < j; i += kDenseSolveThreads) xs[i] -= lu[(size_t)j * N + i] * xj;
    __syncthreads();
  }
  for (int i = tid; i < N; i += kDenseSolveThreads) x[i] = xs[i];
}

inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

}  // namespace

template <typename TF>
int launch_vanka_factor(const DevOp<double> &op, const DevCells &cells, TF *factors, uint8_t *perm,
                        bool factor_fp32, int *status, cudaStream_t s) {
  if (cells.ncells <= 0) return 0;
  if (factor_fp32) {
    const size_t sm = sizeof(float) * NLOC * NLOC;
    cudaFuncSetAttribute(k_vanka_factor<float, TF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    k_vanka_factor<float, TF><<<cells.ncells, kFactorThreads, sm, s>>>(op, cells, factors, perm,
                                                                      status);
  } else {
    const size_t sm = sizeof(double) * NLOC * NLOC;
    cudaFuncSetAttribute(k_vanka_factor<double, TF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
    k_vanka_factor<double, TF><<<cells.ncells, kFactorThreads, sm, s>>>(op, cells, factors, perm,
                                                                       status);
  }
  return ok() < 0 ? -1 : 1;
}

template <typename T>
int launch_vanka_solve(const DevOp<T> &op, const DevCells &cells, const int *cell_list, int ncol,
                       const T *factors, const uint8_t *perm, const T *u, const T *rhs, T *dbuf,
                       cudaStream_t s) {
  if (ncol <= 0) return 0;
  const int grid = (ncol + kSolveWarps - 1) / kSolveWarps;
  k_vanka_solve<T><<<grid, kSolveWarps * 32, 0, s>>>(op, cells, cell_list, ncol, factors, perm, u,
                                                    rhs, dbuf);
  return ok() < 0 ? -1 : 1;
}

template <typename T>
int launch_vanka_update(const DevCells &cells, int nu, const int *cell_list, int ncol,
                        const T *dbuf, T damp, T *u, cudaStream_t s) {
  if (ncol <= 0) return 0;
  const long long n = (long long)ncol * NLOC;
  k_vanka_update<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(cells, nu, cell_list, ncol, dbuf,
                                                                damp, u);
  return ok() < 0 ? -1 : 1;
}

int launch_coarse_assemble(const DevOp<double> &op, double *dense, int project_pressure,
                           cudaStream_t s) {
  const int N = 3 * op.nu + op.np;
  if (cudaMemsetAsync(dense, 0, sizeof(double) * (size_t)N * N, s) != cudaSuccess) return -1;
  const int rows = op.nu + op.np;
  k_coarse_scatter<<<(rows + 127) / 128, 128, 0, s>>>(op, dense, N);
  if (ok() < 0) return -1;
  if (project_pressure) {
    k_coarse_pin<<<(N + 255) / 256, 256, 0, s>>>(dense, N, 3 * op.nu);
    return ok() < 0 ? -1 : 2;
  }
  return 1;
}

int launch_dense_lu(double *a, int n, int *ipiv, int *status, cudaStream_t s) {
  k_dense_lu<<<1, kDenseThreads, 0, s>>>(a, n, ipiv, status);
  return ok() < 0 ? -1 : 1;
}

int launch_dense_solve(const double *lu, const int *ipiv, int n, const double *b, double *x,
                       int pin_row, cudaStream_t s) {
  const size_t sm = sizeof(double) * n;
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_dense_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_dense_solve<<<1, kDenseSolveThreads, sm, s>>>(lu, ipiv, n, b, x, pin_row);
  return ok() < 0 ? -1 : 1;
}

template int launch_vanka_factor<double>(const DevOp<double> &, const DevCells &, double *,
                                         uint8_t *, bool, int *, cudaStream_t);
template int launch_vanka_factor<float>(const DevOp<double> &, const DevCells &, float *,
                                        uint8_t *, bool, int *, cudaStream_t);
template int launch_vanka_solve<double>(const DevOp<double> &, const DevCells &, const int *, int,
                                        const double *, const uint8_t *, const double *,
                                        const double *, double *, cudaStream_t);
template int launch_vanka_solve<float>(const DevOp<float> &, const DevCells &, const int *, int,
                                       const float *, const uint8_t *, const float *,
                                       const float *, float *, cudaStream_t);
template int launch_vanka_update<double>(const DevCells &, int, const int *, int, const double *,
                                         double, double *, cudaStream_t);
template int launch_vanka_update<float>(const DevCells &, int, const int *, int, const float *,
                                        float, float *, cudaStream_t);

}  // namespace pm
