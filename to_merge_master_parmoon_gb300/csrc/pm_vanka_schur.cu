// pm_vanka_schur.cu — cell Vanka for one-block velocity operators (NSTYPE 2).
//
// The reference's NSTYPE-2 level (TNSE_MGLevel2, src/FE/NSE_MGLevel2.C) holds
// one velocity block A shared by the three components, and CellVanka
// (:336-700) builds the same 85x85 local system as NSTYPE 4 with that block
// on the three diagonal positions (:481-505) and no velocity coupling.  The
// local matrix is then
//
//        [ A 0 0 G1 ]         A  : 27x27 (cell rows/columns of the block)
//    M = [ 0 A 0 G2 ]         Gc : 27x4  (BTc, zero on Dirichlet rows)
//        [ 0 0 A G3 ]         Dc : 4x27  (Bc)
//        [ D1 D2 D3 0 ]
//
// and M x = r has the exact block solution
//    y_c = A^{-1} r_c,   p = S^{-1} (r_p - sum_c D_c y_c),   x_c = y_c - W_c p
// with W_c = A^{-1} G_c and S = -sum_c D_c W_c (4x4).  Per cell this stores
// 729 + 324 + 324 + 16 = 1393 values instead of the 7225 of the 85x85
// factors and factors in ~6e4 flops instead of 4.1e5; the result equals the
// 85x85 LU solve up to rounding.
//
//  k_schur_factor: one warp per cell, FP64 Gauss-Jordan with partial pivoting
//    (first maximal |pivot|) on [A | I | G1 G2 G3] in shared memory, lane i
//    owning row i; then S, and S^{-1} by lane 0.
//  k_schur_apply: one warp per cell, lane i < 27 owning velocity row i of the
//    three components; every load of the stored block is independent of the
//    previous arithmetic (three GEMVs and two small reductions).
#include <cuda_runtime.h>

#include <cstdint>

#include "pm_kernels.h"

namespace pm {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kGW = 2 * NU_LOC + 3 * NP_LOC;  // 66 columns of [A | I | G]: 27 + 27 + 12
static_assert(kGW == 66, "[A | I | G1 G2 G3] width");
constexpr int kMS = 67;                      // odd row stride (doubles): conflict-free rows
static_assert(kMS > kGW, "row stride covers the row");
constexpr int kGOff = 2 * NU_LOC;            // first G column (54)
constexpr int kFactorWarps = 2;
constexpr int kApplyWarps = 8;

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

__device__ __forceinline__ int find_local(const int *ids, int n, int g) {
  for (int q = 0; q < n; ++q)
    if (ids[q] == g) return q;
  return -1;
}

struct FactorSmem {
  double M[NU_LOC * kMS];           // [A | I | G], row-major, stride kMS
  double D[NP_LOC * 3 * NU_LOC];    // D[(k*3+c)*27 + i] = Bc(pdof_k, udof_i)
  int ud[NU_LOC], pd[NP_LOC];
};

template <typename TF>
__global__ void __launch_bounds__(kFactorWarps * 32) k_schur_factor(DevOp<double> op,
                                                                    DevCells cells,
                                                                    TF *__restrict__ factors,
                                                                    int *status) {
  __shared__ FactorSmem sm_all[kFactorWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cell = blockIdx.x * kFactorWarps + warp;
  if (cell >= cells.ncells) return;  // whole warp; no block-wide barrier below
  FactorSmem &sm = sm_all[warp];
  double *M = sm.M;
  for (int t = lane; t < NU_LOC * kMS; t += 32) M[t] = 0.0;
  for (int t = lane; t < NP_LOC * 3 * NU_LOC; t += 32) sm.D[t] = 0.0;
  if (lane < NU_LOC) sm.ud[lane] = cells.udofs[(size_t)cell * NU_LOC + lane];
  if (lane < NP_LOC) sm.pd[lane] = cells.pdofs[(size_t)cell * NP_LOC + lane];
  __syncwarp();
  if (lane < NU_LOC) M[lane * kMS + NU_LOC + lane] = 1.0;
  // gather A and G from the velocity rows (NSE_MGLevel2.C:470-540), D from
  // the pressure rows (:543-580)
  for (int a = 0; a < NU_LOC; ++a) {
    const int r = sm.ud[a];
    for (int j = op.a_rowptr[r] + lane; j < op.a_rowptr[r + 1]; j += 32) {
      const int m = find_local(sm.ud, NU_LOC, op.a_col[j]);
      if (m >= 0) M[a * kMS + m] = op.a[0][j];
    }
    if (r < op.nact) {
      for (int j = op.bt_rowptr[r] + lane; j < op.bt_rowptr[r + 1]; j += 32) {
        const int q = find_local(sm.pd, NP_LOC, op.bt_col[j]);
        if (q >= 0) {
#pragma unroll
          for (int c = 0; c < 3; ++c) M[a * kMS + kGOff + c * NP_LOC + q] = op.bt[c][j];
        }
      }
    }
  }
  for (int k = 0; k < NP_LOC; ++k) {
    const int r = sm.pd[k];
    for (int j = op.b_rowptr[r] + lane; j < op.b_rowptr[r + 1]; j += 32) {
      const int m = find_local(sm.ud, NU_LOC, op.b_col[j]);
      if (m >= 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) sm.D[(k * 3 + c) * NU_LOC + m] = op.b[c][j];
      }
    }
  }
  __syncwarp();

  // Gauss-Jordan: [A | I | G] -> [I | A^{-1} | A^{-1} G]
  bool singular = false;
  double *my = M + (lane < NU_LOC ? lane : 0) * kMS;
  for (int k = 0; k < NU_LOC; ++k) {
    double best = (lane >= k && lane < NU_LOC) ? fabs(my[k]) : -1.0;
    int bi = lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(kFull, best, o);
      const int oi = __shfl_xor_sync(kFull, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    bi = __shfl_sync(kFull, bi, 0);       // one choice for the warp (NaN-safe)
    if (bi < k || bi >= NU_LOC) bi = k;   // and always a row of the block
    if (bi != k) {
      for (int c = lane; c < kGW; c += 32) {
        const double t = M[k * kMS + c];
        M[k * kMS + c] = M[bi * kMS + c];
        M[bi * kMS + c] = t;
      }
    }
    __syncwarp();
    const double piv = M[k * kMS + k];
    if (piv == 0.0) singular = true;
    const double rp = piv != 0.0 ? 1.0 / piv : 0.0;
    __syncwarp();
    for (int c = k + 1 + lane; c < kGW; c += 32) M[k * kMS + c] *= rp;
    __syncwarp();
    if (lane < NU_LOC && lane != k) {
      const double f = my[k];
      if (f != 0.0)
        for (int c = k + 1; c < kGW; ++c) my[c] -= f * M[k * kMS + c];
    }
    __syncwarp();
  }

  // S = -sum_c D_c W_c: lane i's share of the 16 dot products over the 81
  // velocity rows, then warp sums
  double S[NP_LOC * NP_LOC];
#pragma unroll
  for (int k = 0; k < NP_LOC; ++k)
#pragma unroll
    for (int m = 0; m < NP_LOC; ++m) {
      double part = 0.0;
      if (lane < NU_LOC) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
          part += sm.D[(k * 3 + c) * NU_LOC + lane] * my[kGOff + c * NP_LOC + m];
      }
      S[k * NP_LOC + m] = -warp_sum(part);
    }
  // S^{-1} by Gauss-Jordan with partial pivoting (every lane, same values)
  double Si[NP_LOC * NP_LOC];
#pragma unroll
  for (int t = 0; t < NP_LOC * NP_LOC; ++t) Si[t] = (t / NP_LOC == t % NP_LOC) ? 1.0 : 0.0;
#pragma unroll
  for (int k = 0; k < NP_LOC; ++k) {
    int p = k;
#pragma unroll
    for (int i = k + 1; i < NP_LOC; ++i)
      if (fabs(S[i * NP_LOC + k]) > fabs(S[p * NP_LOC + k])) p = i;
#pragma unroll
    for (int c = 0; c < NP_LOC; ++c) {
      if (p != k) {
        const double t = S[k * NP_LOC + c];
        S[k * NP_LOC + c] = S[p * NP_LOC + c];
        S[p * NP_LOC + c] = t;
        const double u = Si[k * NP_LOC + c];
        Si[k * NP_LOC + c] = Si[p * NP_LOC + c];
        Si[p * NP_LOC + c] = u;
      }
    }
    const double piv = S[k * NP_LOC + k];
    if (piv == 0.0) singular = true;
    const double rp = piv != 0.0 ? 1.0 / piv : 0.0;
#pragma unroll
    for (int c = 0; c < NP_LOC; ++c) {
      S[k * NP_LOC + c] *= rp;
      Si[k * NP_LOC + c] *= rp;
    }
#pragma unroll
    for (int i = 0; i < NP_LOC; ++i) {
      if (i == k) continue;
      const double f = S[i * NP_LOC + k];
#pragma unroll
      for (int c = 0; c < NP_LOC; ++c) {
        S[i * NP_LOC + c] -= f * S[k * NP_LOC + c];
        Si[i * NP_LOC + c] -= f * Si[k * NP_LOC + c];
      }
    }
  }

  // store: A^{-1} column-major, D, W, S^{-1} column-major, zero padding
  TF *F = factors + (size_t)cell * kSchurStride;
  if (lane < NU_LOC) {
    for (int j = 0; j < NU_LOC; ++j) F[j * NU_LOC + lane] = (TF)my[NU_LOC + j];
#pragma unroll
    for (int k = 0; k < NP_LOC; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        F[kSchurOffD + (k * 3 + c) * NU_LOC + lane] = (TF)sm.D[(k * 3 + c) * NU_LOC + lane];
        F[kSchurOffW + (k * 3 + c) * NU_LOC + lane] = (TF)my[kGOff + c * NP_LOC + k];
      }
  }
  if (lane < NP_LOC * NP_LOC) {
    const int row = lane % NP_LOC, col = lane / NP_LOC;
    F[kSchurOffS + lane] = (TF)Si[row * NP_LOC + col];
  }
  if (lane < kSchurStride - kSchurOffS - NP_LOC * NP_LOC)
    F[kSchurOffS + NP_LOC * NP_LOC + lane] = TF(0);
  if (lane == 0 && singular) atomicOr(status, 1);
}

template <typename T>
__global__ void __launch_bounds__(kApplyWarps * 32) k_schur_apply(
    DevCells cells, int nu, const int *__restrict__ list, int ncol, const T *__restrict__ factors,
    const T *__restrict__ rbuf, T damp, T *__restrict__ u) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = blockIdx.x * kApplyWarps + warp;
  if (slot >= ncol) return;  // whole warp
  const int cell = list[slot];
  const bool vr = lane < NU_LOC;
  const T *R = rbuf + (size_t)slot * kRStride;
  const T r0 = vr ? R[lane] : T(0), r1 = vr ? R[NU_LOC + lane] : T(0),
          r2 = vr ? R[2 * NU_LOC + lane] : T(0);
  const T *F = factors + (size_t)cell * kSchurStride;
  // y_c = A^{-1} r_c
  T y0 = 0, y1 = 0, y2 = 0;
#pragma unroll 9
  for (int j = 0; j < NU_LOC; ++j) {
    const T a = vr ? __ldcs(F + j * NU_LOC + lane) : T(0);
    y0 += a * __shfl_sync(kFull, r0, j);
    y1 += a * __shfl_sync(kFull, r1, j);
    y2 += a * __shfl_sync(kFull, r2, j);
  }
  // t = r_p - sum_c D_c y_c
  T t[NP_LOC];
#pragma unroll
  for (int k = 0; k < NP_LOC; ++k) {
    const T *Dk = F + kSchurOffD + k * 3 * NU_LOC;
    T part = T(0);
    if (vr)
      part = __ldcs(Dk + lane) * y0 + __ldcs(Dk + NU_LOC + lane) * y1 +
             __ldcs(Dk + 2 * NU_LOC + lane) * y2;
    t[k] = R[3 * NU_LOC + k] - warp_sum(part);
  }
  // p = S^{-1} t (column-major S^{-1}, loaded by every lane)
  T p[NP_LOC];
#pragma unroll
  for (int k = 0; k < NP_LOC; ++k) p[k] = T(0);
#pragma unroll
  for (int m = 0; m < NP_LOC; ++m)
#pragma unroll
    for (int k = 0; k < NP_LOC; ++k) p[k] += F[kSchurOffS + m * NP_LOC + k] * t[m];
  // x_c = y_c - W_c p, then u += damp * x on the cell's DOFs
  if (vr) {
#pragma unroll
    for (int k = 0; k < NP_LOC; ++k) {
      const T *Wk = F + kSchurOffW + k * 3 * NU_LOC;
      y0 -= __ldcs(Wk + lane) * p[k];
      y1 -= __ldcs(Wk + NU_LOC + lane) * p[k];
      y2 -= __ldcs(Wk + 2 * NU_LOC + lane) * p[k];
    }
    const int d = cells.udofs[(size_t)cell * NU_LOC + lane];
    u[d] += damp * y0;
    u[(size_t)nu + d] += damp * y1;
    u[(size_t)2 * nu + d] += damp * y2;
  }
  if (lane < NP_LOC) {
    const T pl = lane == 0 ? p[0] : (lane == 1 ? p[1] : (lane == 2 ? p[2] : p[3]));
    u[(size_t)3 * nu + cells.pdofs[(size_t)cell * NP_LOC + lane]] += damp * pl;
  }
}

inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

}  // namespace

template <typename TF>
int launch_schur_factor(const DevOp<double> &op, const DevCells &cells, TF *factors, int *status,
                        cudaStream_t s) {
  if (cells.ncells <= 0) return 0;
  if (!op.structured) return -1;
  const int grid = (cells.ncells + kFactorWarps - 1) / kFactorWarps;
  k_schur_factor<TF><<<grid, kFactorWarps * 32, 0, s>>>(op, cells, factors, status);
  return ok() < 0 ? -1 : 1;
}

template <typename T>
int launch_schur_apply(const DevCells &cells, int nu, const int *cell_list, int ncol,
                       const T *factors, const T *rbuf, T damp, T *u, cudaStream_t s) {
  if (ncol <= 0) return 0;
  const int grid = (ncol + kApplyWarps - 1) / kApplyWarps;
  k_schur_apply<T><<<grid, kApplyWarps * 32, 0, s>>>(cells, nu, cell_list, ncol, factors, rbuf,
                                                    damp, u);
  return ok() < 0 ? -1 : 1;
}

template int launch_schur_factor<double>(const DevOp<double> &, const DevCells &, double *, int *,
                                         cudaStream_t);
template int launch_schur_factor<float>(const DevOp<double> &, const DevCells &, float *, int *,
                                        cudaStream_t);
template int launch_schur_apply<double>(const DevCells &, int, const int *, int, const double *,
                                        const double *, double, double *, cudaStream_t);
template int launch_schur_apply<float>(const DevCells &, int, const int *, int, const float *,
                                       const float *, float, float *, cudaStream_t);

}  // namespace pm
