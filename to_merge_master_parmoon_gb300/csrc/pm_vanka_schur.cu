// pm_vanka_schur.cu — cell Vanka by exact block elimination for levels
// without velocity coupling: one-block operators (NSTYPE 2) and nine-block
// levels (NSTYPE 4) whose off-diagonal blocks A12..A32 are zero.
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
// A nine-block level whose off-diagonal blocks vanish (the Galerkin Oseen
// form, NSType4Galerkin3D, src/FE/NSE3D_FixPo.C:1919-2071, and the theta
// systems built from it) has the same structure with three distinct
// diagonal blocks A_1 = A11, A_2 = A22, A_3 = A33: y_c = A_c^{-1} r_c,
// W_c = A_c^{-1} G_c, everything else as above; 3 x 729 + 324 + 324 + 16 =
// 2851 stored values per cell (NB = 3), three 27x27 eliminations.  The
// reference's CellVanka (src/FE/NSE_MGLevel4.C:1784-2031) solves the 85x85
// system by LU; the block solution is the same solution of the same system.
//
//  k_schur_factor<TF,TC,NB>: one warp per cell, Gauss-Jordan with partial
//    pivoting (first maximal |pivot|) on [A_b | I | G] in shared memory in
//    the compute type TC (FP64, or FP32 with option factor_fp32), lane i
//    owning row i, once (NB = 1, all three G) or per component (NB = 3);
//    then S and S^{-1} in FP64 by every lane (16 dot products and a 4x4
//    inverse).  Stored in TF.
//  k_schur_apply<NB>: one warp per cell, lane i < 27 owning velocity row i
//    of the three components; every load of the stored block is independent
//    of the previous arithmetic (three GEMVs and two small reductions).
#include <cuda_runtime.h>

#include <cstdint>

#include "pm_kernels.h"

namespace pm {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kFactorWarps = 2;
constexpr int kApplyWarps = 8;

// Shape of the Gauss-Jordan tableau of one pass: [A_b | I | G] with the G
// columns of the three components (NB = 1) or of component b (NB = 3).
template <int NB>
struct Tab {
  static constexpr int ng = NB == 1 ? 3 * NP_LOC : NP_LOC;  // G columns: 12 / 4
  static constexpr int gw = 2 * NU_LOC + ng;                // 66 / 58
  static constexpr int ms = gw | 1;                         // odd row stride: 67 / 59
  static constexpr int goff = 2 * NU_LOC;                   // first G column (54)
};
static_assert(Tab<1>::gw == 66 && Tab<1>::ms == 67, "[A | I | G1 G2 G3]");
static_assert(Tab<3>::gw == 58 && Tab<3>::ms == 59, "[A_c | I | G_c]");

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

template <int NB, typename TC>
struct FactorSmem {
  TC M[NU_LOC * Tab<NB>::ms];       // [A_b | I | G], row-major
  double D[NP_LOC * 3 * NU_LOC];    // D[(k*3+c)*27 + i] = Bc(pdof_k, udof_i)
  int ud[NU_LOC], pd[NP_LOC];
};

template <typename T>
__device__ __forceinline__ T abs_of(T v) {
  return v < T(0) ? -v : v;
}

template <typename TF, typename TC, int NB>
__global__ void __launch_bounds__(kFactorWarps * 32) k_schur_factor(DevOp<double> op,
                                                                    DevCells cells,
                                                                    TF *__restrict__ factors,
                                                                    int *status) {
  using L = Schur<NB>;
  constexpr int MS = Tab<NB>::ms, GW = Tab<NB>::gw, GOFF = Tab<NB>::goff;
  __shared__ FactorSmem<NB, TC> sm_all[kFactorWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cell = blockIdx.x * kFactorWarps + warp;
  if (cell >= cells.ncells) return;  // whole warp; no block-wide barrier below
  FactorSmem<NB, TC> &sm = sm_all[warp];
  TC *M = sm.M;
  for (int t = lane; t < NP_LOC * 3 * NU_LOC; t += 32) sm.D[t] = 0.0;
  if (lane < NU_LOC) sm.ud[lane] = cells.udofs[(size_t)cell * NU_LOC + lane];
  if (lane < NP_LOC) sm.pd[lane] = cells.pdofs[(size_t)cell * NP_LOC + lane];
  __syncwarp();
  // D from the pressure rows (NSE_MGLevel2.C:543-580, NSE_MGLevel4.C:1921-1960)
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
  TF *F = factors + (size_t)cell * L::stride;
  bool singular = false;
  double S[NP_LOC * NP_LOC];
#pragma unroll
  for (int t = 0; t < NP_LOC * NP_LOC; ++t) S[t] = 0.0;
  TC *my = M + (lane < NU_LOC ? lane : 0) * MS;
  for (int b = 0; b < NB; ++b) {
    // gather A_b and G from the velocity rows (NSE_MGLevel2.C:470-540;
    // NSE_MGLevel4.C:1823-1918 with A12..A32 = 0)
    const double *Ab = op.a[NB == 1 ? 0 : 4 * b];
    __syncwarp();
    for (int t = lane; t < NU_LOC * MS; t += 32) M[t] = TC(0);
    __syncwarp();
    if (lane < NU_LOC) M[lane * MS + NU_LOC + lane] = TC(1);
    for (int a = 0; a < NU_LOC; ++a) {
      const int r = sm.ud[a];
      for (int j = op.a_rowptr[r] + lane; j < op.a_rowptr[r + 1]; j += 32) {
        const int m = find_local(sm.ud, NU_LOC, op.a_col[j]);
        if (m >= 0) M[a * MS + m] = (TC)Ab[j];
      }
      if (r < op.nact) {
        for (int j = op.bt_rowptr[r] + lane; j < op.bt_rowptr[r + 1]; j += 32) {
          const int q = find_local(sm.pd, NP_LOC, op.bt_col[j]);
          if (q >= 0) {
            if constexpr (NB == 1) {
#pragma unroll
              for (int c = 0; c < 3; ++c) M[a * MS + GOFF + c * NP_LOC + q] = (TC)op.bt[c][j];
            } else {
              M[a * MS + GOFF + q] = (TC)op.bt[b][j];
            }
          }
        }
      }
    }
    __syncwarp();

    // Gauss-Jordan: [A_b | I | G] -> [I | A_b^{-1} | A_b^{-1} G]
    for (int k = 0; k < NU_LOC; ++k) {
      TC best = (lane >= k && lane < NU_LOC) ? abs_of(my[k]) : TC(-1);
      int bi = lane;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const TC ob = __shfl_xor_sync(kFull, best, o);
        const int oi = __shfl_xor_sync(kFull, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      bi = __shfl_sync(kFull, bi, 0);       // one choice for the warp (NaN-safe)
      if (bi < k || bi >= NU_LOC) bi = k;   // and always a row of the block
      if (bi != k) {
        for (int c = lane; c < GW; c += 32) {
          const TC t = M[k * MS + c];
          M[k * MS + c] = M[bi * MS + c];
          M[bi * MS + c] = t;
        }
      }
      __syncwarp();
      const TC piv = M[k * MS + k];
      if (piv == TC(0)) singular = true;
      const TC rp = piv != TC(0) ? TC(1) / piv : TC(0);
      __syncwarp();
      for (int c = k + 1 + lane; c < GW; c += 32) M[k * MS + c] *= rp;
      __syncwarp();
      if (lane < NU_LOC && lane != k) {
        const TC f = my[k];
        if (f != TC(0))
          for (int c = k + 1; c < GW; ++c) my[c] -= f * M[k * MS + c];
      }
      __syncwarp();
    }

    // S -= sum_c D_c W_c over the components of this pass: lane i's share
    // of the 16 dot products over the velocity rows, then warp sums
#pragma unroll
    for (int k = 0; k < NP_LOC; ++k)
#pragma unroll
      for (int m = 0; m < NP_LOC; ++m) {
        double part = 0.0;
        if (lane < NU_LOC) {
          if constexpr (NB == 1) {
#pragma unroll
            for (int c = 0; c < 3; ++c)
              part += sm.D[(k * 3 + c) * NU_LOC + lane] * (double)my[GOFF + c * NP_LOC + m];
          } else {
            part = sm.D[(k * 3 + b) * NU_LOC + lane] * (double)my[GOFF + m];
          }
        }
        S[k * NP_LOC + m] -= warp_sum(part);
      }
    // store A_b^{-1} (column-major) and W of this pass's components
    if (lane < NU_LOC) {
      for (int j = 0; j < NU_LOC; ++j)
        F[b * NU_LOC * NU_LOC + j * NU_LOC + lane] = (TF)my[NU_LOC + j];
#pragma unroll
      for (int k = 0; k < NP_LOC; ++k) {
        if constexpr (NB == 1) {
#pragma unroll
          for (int c = 0; c < 3; ++c)
            F[L::offW + (k * 3 + c) * NU_LOC + lane] = (TF)my[GOFF + c * NP_LOC + k];
        } else {
          F[L::offW + (k * 3 + b) * NU_LOC + lane] = (TF)my[GOFF + k];
        }
      }
    }
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

  // store D, S^{-1} (column-major), zero padding
  if (lane < NU_LOC) {
#pragma unroll
    for (int k = 0; k < NP_LOC; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        F[L::offD + (k * 3 + c) * NU_LOC + lane] = (TF)sm.D[(k * 3 + c) * NU_LOC + lane];
  }
  if (lane < NP_LOC * NP_LOC) {
    const int row = lane % NP_LOC, col = lane / NP_LOC;
    F[L::offS + lane] = (TF)Si[row * NP_LOC + col];
  }
  if (lane < L::stride - L::values) F[L::values + lane] = TF(0);
  if (lane == 0 && singular) atomicOr(status, 1);
}

// AOS (FP32): the velocity update goes to the interleaved copy ux (node d
// at ux[d]: three components and a pad; one 16-byte read-modify-write per
// node), the pressure update to u
template <typename T, int NB, bool AOS = false>
__global__ void __launch_bounds__(kApplyWarps * 32) k_schur_apply(
    DevCells cells, int nu, const int *__restrict__ list, int ncol, const T *__restrict__ factors,
    const T *__restrict__ rbuf, T damp, T *__restrict__ u, float4 *__restrict__ ux) {
  static_assert(!AOS || sizeof(T) == sizeof(float), "interleaved velocity: FP32 only");
  using L = Schur<NB>;
  constexpr int B1 = NB == 1 ? 0 : NU_LOC * NU_LOC;  // offset of A_2^{-1} (A_3^{-1}: 2 B1)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = blockIdx.x * kApplyWarps + warp;
  if (slot >= ncol) return;  // whole warp
  const int cell = list[slot];
  const bool vr = lane < NU_LOC;
  const T *R = rbuf + (size_t)slot * kRStride;
  const T r0 = vr ? R[lane] : T(0), r1 = vr ? R[NU_LOC + lane] : T(0),
          r2 = vr ? R[2 * NU_LOC + lane] : T(0);
  const T *F = factors + (size_t)cell * L::stride;
  // every load of the cell's block is issued before the arithmetic needs
  // it (one memory round trip per cell where the registers allow: all of
  // A^{-1}, D and W for one block; D and W up front for three blocks)
  T Dv[NP_LOC][3], Wv[NP_LOC][3];
#pragma unroll
  for (int k = 0; k < NP_LOC; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      Dv[k][c] = vr ? __ldcs(F + L::offD + (k * 3 + c) * NU_LOC + lane) : T(0);
      Wv[k][c] = vr ? __ldcs(F + L::offW + (k * 3 + c) * NU_LOC + lane) : T(0);
    }
  // y_c = A_c^{-1} r_c
  T y0 = 0, y1 = 0, y2 = 0;
  if constexpr (NB == 1) {
    T a[NU_LOC];
#pragma unroll
    for (int j = 0; j < NU_LOC; ++j) a[j] = vr ? __ldcs(F + j * NU_LOC + lane) : T(0);
#pragma unroll
    for (int j = 0; j < NU_LOC; ++j) {
      y0 += a[j] * __shfl_sync(kFull, r0, j);
      y1 += a[j] * __shfl_sync(kFull, r1, j);
      y2 += a[j] * __shfl_sync(kFull, r2, j);
    }
  } else {
#pragma unroll 9
    for (int j = 0; j < NU_LOC; ++j) {
      const T *Fj = F + j * NU_LOC + lane;
      const T a0 = vr ? __ldcs(Fj) : T(0), a1 = vr ? __ldcs(Fj + B1) : T(0),
              a2 = vr ? __ldcs(Fj + 2 * B1) : T(0);
      y0 += a0 * __shfl_sync(kFull, r0, j);
      y1 += a1 * __shfl_sync(kFull, r1, j);
      y2 += a2 * __shfl_sync(kFull, r2, j);
    }
  }
  // t = r_p - sum_c D_c y_c
  T t[NP_LOC];
#pragma unroll
  for (int k = 0; k < NP_LOC; ++k)
    t[k] = R[3 * NU_LOC + k] - warp_sum(Dv[k][0] * y0 + Dv[k][1] * y1 + Dv[k][2] * y2);
  // p = S^{-1} t (column-major S^{-1}, loaded by every lane)
  T p[NP_LOC];
#pragma unroll
  for (int k = 0; k < NP_LOC; ++k) p[k] = T(0);
#pragma unroll
  for (int m = 0; m < NP_LOC; ++m)
#pragma unroll
    for (int k = 0; k < NP_LOC; ++k) p[k] += F[L::offS + m * NP_LOC + k] * t[m];
  // x_c = y_c - W_c p, then u += damp * x on the cell's DOFs
  if (vr) {
#pragma unroll
    for (int k = 0; k < NP_LOC; ++k) {
      y0 -= Wv[k][0] * p[k];
      y1 -= Wv[k][1] * p[k];
      y2 -= Wv[k][2] * p[k];
    }
    const int d = cells.udofs[(size_t)cell * NU_LOC + lane];
    if constexpr (AOS) {
      float4 v = ux[d];
      v.x += damp * y0;
      v.y += damp * y1;
      v.z += damp * y2;
      ux[d] = v;
    } else {
      u[d] += damp * y0;
      u[(size_t)nu + d] += damp * y1;
      u[(size_t)2 * nu + d] += damp * y2;
    }
  }
  if (lane < NP_LOC) {
    const T pl = lane == 0 ? p[0] : (lane == 1 ? p[1] : (lane == 2 ? p[2] : p[3]));
    u[(size_t)3 * nu + cells.pdofs[(size_t)cell * NP_LOC + lane]] += damp * pl;
  }
}

// flag |= 1 when an off-diagonal velocity block holds a nonzero entry,
// |= 2 when the diagonal blocks differ somewhere (A22 != A11 or A33 != A11,
// compared as values; a NaN counts as different)
__global__ void __launch_bounds__(256) k_block_structure(DevOp<double> op, long long n,
                                                         int *flag) {
  bool nz = false, differ = false;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    nz |= op.a[1][i] != 0.0 || op.a[2][i] != 0.0 || op.a[3][i] != 0.0 || op.a[5][i] != 0.0 ||
          op.a[6][i] != 0.0 || op.a[7][i] != 0.0;
    const double d = op.a[0][i];
    differ |= !(op.a[4][i] == d) || !(op.a[8][i] == d);
  }
  const int bits = (__any_sync(kFull, nz) ? 1 : 0) | (__any_sync(kFull, differ) ? 2 : 0);
  if (bits && (threadIdx.x & 31) == 0) atomicOr(flag, bits);
}

inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

template <typename TF, int NB>
int factor_impl(const DevOp<double> &op, const DevCells &cells, TF *factors, int *status,
                bool fp32, cudaStream_t s) {
  if (cells.ncells <= 0) return 0;
  if (cells.nl != NU_LOC) return -1;  // Q2 hexahedra only
  const int grid = (cells.ncells + kFactorWarps - 1) / kFactorWarps;
  if constexpr (sizeof(TF) == sizeof(float)) {
    if (fp32) {
      k_schur_factor<TF, float, NB><<<grid, kFactorWarps * 32, 0, s>>>(op, cells, factors,
                                                                       status);
      return ok() < 0 ? -1 : 1;
    }
  } else {
    if (fp32) return -1;  // FP32 elimination only for FP32 factors
  }
  k_schur_factor<TF, double, NB><<<grid, kFactorWarps * 32, 0, s>>>(op, cells, factors, status);
  return ok() < 0 ? -1 : 1;
}

template <typename T, int NB>
int apply_impl(const DevCells &cells, int nu, const int *cell_list, int ncol, const T *factors,
               const T *rbuf, T damp, T *u, cudaStream_t s) {
  if (ncol <= 0) return 0;
  const int grid = (ncol + kApplyWarps - 1) / kApplyWarps;
  k_schur_apply<T, NB><<<grid, kApplyWarps * 32, 0, s>>>(cells, nu, cell_list, ncol, factors,
                                                        rbuf, damp, u, nullptr);
  return ok() < 0 ? -1 : 1;
}

}  // namespace

template <typename TF>
int launch_schur_factor(const DevOp<double> &op, const DevCells &cells, TF *factors, int *status,
                        bool fp32, cudaStream_t s) {
  if (!op.structured) return -1;
  return factor_impl<TF, 1>(op, cells, factors, status, fp32, s);
}

template <typename TF>
int launch_schur3_factor(const DevOp<double> &op, const DevCells &cells, TF *factors, int *status,
                         bool fp32, cudaStream_t s) {
  if (op.structured || !op.diag) return -1;
  return factor_impl<TF, 3>(op, cells, factors, status, fp32, s);
}

template <typename T>
int launch_schur_apply(const DevCells &cells, int nu, const int *cell_list, int ncol,
                       const T *factors, const T *rbuf, T damp, T *u, cudaStream_t s) {
  return apply_impl<T, 1>(cells, nu, cell_list, ncol, factors, rbuf, damp, u, s);
}

template <typename T>
int launch_schur3_apply(const DevCells &cells, int nu, const int *cell_list, int ncol,
                        const T *factors, const T *rbuf, T damp, T *u, cudaStream_t s) {
  return apply_impl<T, 3>(cells, nu, cell_list, ncol, factors, rbuf, damp, u, s);
}

int launch_schur_apply_aos(const DevCells &cells, int nu, const int *cell_list, int ncol,
                           const float *factors, const float *rbuf, float damp, float *u,
                           float4 *ux, cudaStream_t s) {
  if (ncol <= 0) return 0;
  if (cells.nl != NU_LOC || ux == nullptr) return -1;
  const int grid = (ncol + kApplyWarps - 1) / kApplyWarps;
  k_schur_apply<float, 1, true><<<grid, kApplyWarps * 32, 0, s>>>(cells, nu, cell_list, ncol,
                                                                 factors, rbuf, damp, u, ux);
  return ok() < 0 ? -1 : 1;
}

int launch_block_structure(const DevOp<double> &op, long long n, int *flag, cudaStream_t s) {
  if (n <= 0) return 0;
  long long g = (n + 255) / 256;
  if (g > 4 * 152) g = 4 * 152;
  k_block_structure<<<(unsigned)g, 256, 0, s>>>(op, n, flag);
  return ok() < 0 ? -1 : 1;
}

#define PM_SINST(T)                                                                              \
  template int launch_schur_factor<T>(const DevOp<double> &, const DevCells &, T *, int *, bool,  \
                                      cudaStream_t);                                              \
  template int launch_schur3_factor<T>(const DevOp<double> &, const DevCells &, T *, int *, bool, \
                                       cudaStream_t);                                             \
  template int launch_schur_apply<T>(const DevCells &, int, const int *, int, const T *,          \
                                     const T *, T, T *, cudaStream_t);                            \
  template int launch_schur3_apply<T>(const DevCells &, int, const int *, int, const T *,         \
                                      const T *, T, T *, cudaStream_t);
PM_SINST(double)
PM_SINST(float)
#undef PM_SINST

}  // namespace pm
