// pm_vanka.cu — cell-Vanka smoother and coarse direct solve on sm_103a.
//
// The reference assembles each hexahedron's 85x85 local saddle block
// (27 Q2 nodes x 3 components + 4 P1disc modes) and calls dgetrf/dgetrs on
// it in every sweep (TNSE_MGLevel4::CellVanka, src/FE/NSE_MGLevel4.C:1653-2087;
// SolveLinearSystemLapack, src/FE/LinAlg.C:106-131).  The local blocks do not
// change during a linear solve, so here they are gathered and factored once
// per matrix (k_vanka_factor) and every sweep only
//   1. forms each cell's local residual from the full CSR rows (the same
//      rows the reference reads, :1810-1941) -> k_vanka_residual,
//   2. applies the stored factors (forward/back substitution) and adds
//      damp * delta to the cell's DOFs (:2044-2059) -> k_vanka_apply,
// colour by colour: cells of one colour share no DOF; their residuals are
// all taken from the state before the colour (CellVanka_GPU semantics,
// src/FE/NSE_CellVanka.cu:2181-2365), so step 2 runs after step 1 of the
// whole colour in a separate launch.
#include <cuda_runtime.h>

#include <algorithm>
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

template <typename TC, typename TF, int NU>
__global__ void __launch_bounds__(kFactorThreads) k_vanka_factor(DevOp<double> op, DevCells cells,
                                                                 TF *__restrict__ factors,
                                                                 uint8_t *__restrict__ perm,
                                                                 int *status) {
  constexpr int NU_LOC = NU, NLOC = Elem<NU>::nloc, kFacStride = Elem<NU>::fac_stride;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TC *S = reinterpret_cast<TC *>(smem_raw);
  __shared__ int ud[NU_LOC], pd[NP_LOC];
  __shared__ int skey[NU_LOC], sloc[NU_LOC];  // the cell's DOFs sorted, with local indices
  __shared__ int piv_row;
  __shared__ TC piv_rcp, piv_val, piv_d0;  // 1 / pivot, the pivot, the old diagonal
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
  if (tid < NU_LOC) {  // rank sort (the DOFs of a cell are distinct)
    const int v = ud[tid];
    int rank = 0;
    for (int q = 0; q < NU_LOC; ++q) rank += ud[q] < v;
    skey[rank] = v;
    sloc[rank] = tid;
  }
  __syncthreads();
  // local index of velocity DOF l in the cell, -1 if absent (binary search)
  auto local_of = [&](int l) {
    int lo = 0, hi = NU_LOC;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (skey[mid] < l) lo = mid + 1; else hi = mid;
    }
    return (lo < NU_LOC && skey[lo] == l) ? sloc[lo] : -1;
  };

  // gather: velocity rows (9 blocks + BT), pressure rows (B)
  for (int a = warp; a < NU_LOC; a += nwarps) {
    const int r = ud[a];
    const bool dir = r >= op.nact;
    for (int j = op.a_rowptr[r] + lane; j < op.a_rowptr[r + 1]; j += 32) {
      const int l = op.a_col[j];
      const int m = local_of(l);
      if (m < 0) continue;
      const int c1 = m * NLOC, c2 = (m + NU_LOC) * NLOC, c3 = (m + 2 * NU_LOC) * NLOC;
      if (op.structured) {  // one block for the three components, no coupling
        const TC v = (TC)op.a[0][j];
        S[c1 + a] = v;
        S[c2 + a + NU_LOC] = v;
        S[c3 + a + 2 * NU_LOC] = v;
        continue;
      }
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
      const int m = local_of(l);
      if (m < 0) continue;
      S[m * NLOC + row] = (TC)op.b[0][j];
      S[(m + NU_LOC) * NLOC + row] = (TC)op.b[1][j];
      S[(m + 2 * NU_LOC) * NLOC + row] = (TC)op.b[2][j];
    }
  }
  __syncthreads();

  // Right-looking LU, two barriers per step: (1) the interchange of rows k
  // and p in every column with the scaling of column k (disjoint memory),
  // (2) the rank-1 update, during which warp 0 -- the warp that updates
  // column k+1 -- also finds the next pivot (look-ahead) from its own
  // freshly updated entries.
  // pivot of column k (rows k..): first maximal |a|, with its signed value
  auto pivot_search = [&](int k) {
    TC best = TC(-1), bv = TC(0);
    int bi = k;
    for (int i = k + lane; i < NLOC; i += 32) {
      const TC v = S[k * NLOC + i];
      if (fabs(v) > best) {
        best = fabs(v);
        bv = v;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const TC ob = __shfl_xor_sync(kFull, best, o);
      const TC ov = __shfl_xor_sync(kFull, bv, o);
      const int oi = __shfl_xor_sync(kFull, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bv = ov;
        bi = oi;
      }
    }
    if (lane == 0) {
      piv_row = bi;
      piv_val = bv;
      piv_d0 = S[k * NLOC + k];  // lane 0 holds row k (its own entry)
      piv_rcp = bv != TC(0) ? TC(1) / bv : TC(0);
      if (bv == TC(0)) singular = 1;
    }
  };
  if (warp == 0) pivot_search(0);
  __syncthreads();
  for (int k = 0; k < NLOC; ++k) {
    const int p = piv_row;
    const TC pv = piv_val, d0 = piv_d0, rp = piv_rcp;
    if (p != k)
      for (int j = tid; j < NLOC; j += kFactorThreads) {
        if (j == k) continue;
        const TC t = S[j * NLOC + k];
        S[j * NLOC + k] = S[j * NLOC + p];
        S[j * NLOC + p] = t;
      }
    // column k after the interchange: pv on the diagonal, row p holds the
    // old diagonal d0; below the diagonal scaled by 1 / pivot
    const TC sc = rp != TC(0) ? rp : TC(1);
    for (int i = k + 1 + tid; i < NLOC; i += kFactorThreads)
      S[k * NLOC + i] = (i == p ? d0 : S[k * NLOC + i]) * sc;
    if (tid == 0) {
      S[k * NLOC + k] = pv;
      if (p != k) {
        const unsigned char t = pm[k];
        pm[k] = pm[p];
        pm[p] = t;
      }
    }
    __syncthreads();
    for (int jj = k + 1 + warp; jj < NLOC; jj += nwarps) {
      const TC ukj = S[jj * NLOC + k];
      if (ukj != TC(0))
        for (int ii = k + 1 + lane; ii < NLOC; ii += 32) S[jj * NLOC + ii] -= S[k * NLOC + ii] * ukj;
    }
    if (warp == 0 && k + 1 < NLOC) {
      __syncwarp();
      pivot_search(k + 1);
    }
    __syncthreads();
  }
  TF *F = factors + (size_t)cell * kFacStride;
  for (int t = tid; t < NLOC * NLOC; t += kFactorThreads) {
    const int i = t % NLOC, j = t / NLOC;
    TC v = S[t];
    if (i == j) v = (v != TC(0)) ? TC(1) / v : TC(0);
    F[t] = (TF)v;
  }
  if (tid < NLOC) perm[(size_t)cell * NLOC + tid] = pm[tid];
  if (tid == 0 && singular) atomicOr(status, 1);
}

// ---------------------------------------------------------------- inverse ---
// A^{-1} = U^{-1} L^{-1} P in FP32 from the stored FP32 factors of one cell
// (column-major, unit L below the diagonal, 1/U_jj on it), written over
// them.  One CTA per cell; thread j < 85 computes column j: y = P e_j, then
// column-oriented forward (y_i -= L_ik y_k, i > k) and backward
// (x_k = y_k / U_kk, y_i -= U_ik x_k, i < k) substitution, the factor
// columns read from shared memory as broadcasts.  85^3 FMA per cell.
constexpr int kInvThreadsLU = 96;
__global__ void __launch_bounds__(kInvThreadsLU) k_lu_inverse_f32(float *__restrict__ factors,
                                                                  const uint8_t *__restrict__ perm) {
  __shared__ float LU[NLOC * NLOC];
  __shared__ unsigned char pm[NLOC];
  const int cell = blockIdx.x, j = threadIdx.x;
  float *F = factors + (size_t)cell * kFacStride;
  for (int t = threadIdx.x; t < NLOC * NLOC; t += kInvThreadsLU) LU[t] = F[t];
  if (threadIdx.x < NLOC) pm[threadIdx.x] = perm[(size_t)cell * NLOC + threadIdx.x];
  __syncthreads();
  float y[NLOC];
#pragma unroll
  for (int i = 0; i < NLOC; ++i) y[i] = (j < NLOC && pm[i] == j) ? 1.f : 0.f;
#pragma unroll
  for (int k = 0; k < NLOC - 1; ++k) {
    const float yk = y[k];
#pragma unroll
    for (int i = k + 1; i < NLOC; ++i) y[i] -= LU[k * NLOC + i] * yk;
  }
#pragma unroll
  for (int k = NLOC - 1; k >= 0; --k) {
    const float xk = y[k] * LU[k * NLOC + k];
    y[k] = xk;
#pragma unroll
    for (int i = 0; i < k; ++i) y[i] -= LU[k * NLOC + i] * xk;
  }
  __syncthreads();  // every thread is done with the factors
  if (j < NLOC) {
#pragma unroll
    for (int i = 0; i < NLOC; ++i) LU[j * NLOC + i] = y[i];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < NLOC * NLOC; t += kInvThreadsLU) F[t] = LU[t];
}

// ------------------------------------------------------------------ apply ---
// Sweep of one colour = two launches:
//  k_vanka_residual: one warp per cell forms the local residual
//    r = f - K u on the cell's 85 DOFs from the full CSR rows.  The cell's
//    27 A rows, 27 BT rows and 4 B rows are walked as one flattened entry
//    stream, U x 32 entries per iteration with all their loads issued
//    together (memory-level parallelism), and summed per row with a
//    deterministic segmented warp reduction.  r goes to a small buffer.
//  k_vanka_apply: one warp per cell solves P A = L U with the stored
//    factors (factor columns prefetched a block ahead in registers) and adds
//    damp * delta to the cell's DOFs.  Cells of one colour share no DOF and
//    every residual of the colour was taken before this launch, so the
//    in-place update is race-free.
constexpr int kResWarps = 4;
constexpr int kApplyWarps = 8;

__device__ __forceinline__ int warp_excl_scan(int v, int lane, int &total) {
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  total = __shfl_sync(kFull, x, 31);
  return x - v;
}

// segment of entry e: the last a in [0,n) with off[a] <= e (empty segments
// share their offset with the next one and are skipped).
__device__ __forceinline__ int find_seg(const int *off, int n, int e) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= e) lo = mid; else hi = mid;
  }
  return lo;
}

// Segmented warp sum of NO values keyed by seg (contiguous keys, -1 = none);
// the first lane of each segment adds the sums to acc[seg + k*stride].
template <typename T, int NO>
__device__ __forceinline__ void seg_accumulate(int seg, T (&v)[NO], T *acc, int stride, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int so = __shfl_down_sync(kFull, seg, o);
#pragma unroll
    for (int k = 0; k < NO; ++k) {
      const T w = __shfl_down_sync(kFull, v[k], o);
      if (lane + o < 32 && so == seg) v[k] += w;
    }
  }
  const int sp = __shfl_up_sync(kFull, seg, 1);
  if (seg >= 0 && (lane == 0 || sp != seg)) {
#pragma unroll
    for (int k = 0; k < NO; ++k) acc[seg + k * stride] += v[k];
  }
  __syncwarp();
}

// Aligned vector loads of VEC consecutive CSR entries (value and column
// arrays are padded to a multiple of 4 entries at upload).
template <typename T, int VEC>
struct VecLd;
template <>
struct VecLd<float, 4> {
  static __device__ __forceinline__ void val(const float *p, float (&o)[4]) {
    const float4 v = __ldcs(reinterpret_cast<const float4 *>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
  static __device__ __forceinline__ void idx(const int *p, int (&o)[4]) {
    const int4 v = __ldg(reinterpret_cast<const int4 *>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
};
template <>
struct VecLd<float, 2> {
  static __device__ __forceinline__ void val(const float *p, float (&o)[2]) {
    const float2 v = __ldcs(reinterpret_cast<const float2 *>(p));
    o[0] = v.x; o[1] = v.y;
  }
  static __device__ __forceinline__ void idx(const int *p, int (&o)[2]) {
    const int2 v = __ldg(reinterpret_cast<const int2 *>(p));
    o[0] = v.x; o[1] = v.y;
  }
};
template <typename T>
struct VecLd<T, 1> {
  static __device__ __forceinline__ void val(const T *p, T (&o)[1]) { o[0] = __ldcs(p); }
  static __device__ __forceinline__ void idx(const int *p, int (&o)[1]) { o[0] = __ldg(p); }
};
template <>
struct VecLd<double, 2> {
  static __device__ __forceinline__ void val(const double *p, double (&o)[2]) {
    const double2 v = __ldcs(reinterpret_cast<const double2 *>(p));
    o[0] = v.x; o[1] = v.y;
  }
  static __device__ __forceinline__ void idx(const int *p, int (&o)[2]) {
    const int2 v = __ldg(reinterpret_cast<const int2 *>(p));
    o[0] = v.x; o[1] = v.y;
  }
};

// Row segments of one warp: row a spans entries [rs[a], re[a]) and the
// aligned VEC-entry groups qs[a] .. qs[a] + (off[a+1]-off[a]) - 1, which are
// flattened across rows (group offset off[a]).
struct SegTab {
  int *qs, *off, *rs, *re;
};

template <int VEC>
__device__ __forceinline__ int seg_setup(const SegTab &t, int lane, bool valid, int rs, int re) {
  int nq = 0, qs = 0;
  if (valid && re > rs) {
    qs = rs / VEC;
    nq = (re - 1) / VEC - qs + 1;
  }
  int total;
  t.off[lane] = warp_excl_scan(nq, lane, total);
  t.qs[lane] = qs;
  t.rs[lane] = valid ? rs : 0;
  t.re[lane] = valid ? re : 0;
  __syncwarp();
  return total;
}

// Walk the groups of nseg row segments of a CSR matrix with NV value
// arrays; each entry contributes NO products.
// MODE 0: A rows (9 values, gather u1,u2,u3 -> 3 outputs)
// MODE 1: BT rows (3 values, gather p -> 3 outputs)
// MODE 2: B rows (3 values, gather u1,u2,u3 -> 1 output)
// MODE 3: A rows of a one-block operator (1 value, gather u1,u2,u3 -> 3 outputs)
// MODE 4: A rows of a level without velocity coupling (the 3 diagonal
//         blocks, value k times u_k into output k)
template <typename T, int MODE, int VEC, int U>
__device__ __forceinline__ void flat_rows(const SegTab &t, int nseg, int total,
                                          const int *__restrict__ col, const T *const *vals,
                                          const T *__restrict__ x0, const T *__restrict__ x1,
                                          const T *__restrict__ x2, T *acc, int lane) {
  constexpr int NV = MODE == 0 ? 9 : (MODE == 3 ? 1 : 3);
  constexpr int NO = MODE == 2 ? 1 : 3;
  for (int base = 0; base < total; base += 32 * U) {
    int seg[U];
    long long gq[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int g = base + q * 32 + lane;
      seg[q] = -1;
      gq[q] = 0;
      if (g < total) {
        seg[q] = find_seg(t.off, nseg, g);
        gq[q] = (long long)t.qs[seg[q]] + (g - t.off[seg[q]]);
      }
    }
    int ci[U][VEC];
    T v[U][NV][VEC];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      if (seg[q] >= 0) {
        VecLd<T, VEC>::idx(col + gq[q] * VEC, ci[q]);
#pragma unroll
        for (int k = 0; k < NV; ++k) VecLd<T, VEC>::val(vals[k] + gq[q] * VEC, v[q][k]);
      } else {
#pragma unroll
        for (int m = 0; m < VEC; ++m) {
          ci[q][m] = 0;
#pragma unroll
          for (int k = 0; k < NV; ++k) v[q][k][m] = T(0);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      T s[NO];
#pragma unroll
      for (int k = 0; k < NO; ++k) s[k] = T(0);
      if (seg[q] >= 0) {
        const long long e0 = gq[q] * VEC;
        const int lo = t.rs[seg[q]], hi = t.re[seg[q]];
#pragma unroll
        for (int m = 0; m < VEC; ++m) {
          const long long e = e0 + m;
          if (e >= lo && e < hi) {
            const int c = ci[q][m];
            if constexpr (MODE == 1) {
              const T g0 = __ldg(x0 + c);
              s[0] += v[q][0][m] * g0;
              s[1 % NO] += v[q][1][m] * g0;
              s[2 % NO] += v[q][2][m] * g0;
            } else if constexpr (MODE == 3) {
              const T a = v[q][0][m];
              s[0] += a * __ldg(x0 + c);
              s[1 % NO] += a * __ldg(x1 + c);
              s[2 % NO] += a * __ldg(x2 + c);
            } else if constexpr (MODE == 4) {
              s[0] += v[q][0][m] * __ldg(x0 + c);
              s[1 % NO] += v[q][1][m] * __ldg(x1 + c);
              s[2 % NO] += v[q][2][m] * __ldg(x2 + c);
            } else {
              const T g0 = __ldg(x0 + c), g1 = __ldg(x1 + c), g2 = __ldg(x2 + c);
              if constexpr (MODE == 0) {
                s[0] += v[q][0][m] * g0 + v[q][1][m] * g1 + v[q][2][m] * g2;
                s[1 % NO] += v[q][3][m] * g0 + v[q][4][m] * g1 + v[q][5][m] * g2;
                s[2 % NO] += v[q][6][m] * g0 + v[q][7][m] * g1 + v[q][8][m] * g2;
              } else {
                s[0] += v[q][0][m] * g0 + v[q][1][m] * g1 + v[q][2][m] * g2;
              }
            }
          }
        }
      }
      seg_accumulate<T, NO>(seg[q], s, acc, NU_LOC, lane);
    }
  }
}

template <typename T, int VEC, int U>
__global__ void __launch_bounds__(kResWarps * 32) k_vanka_residual(
    DevOp<T> op, DevCells cells, const int *__restrict__ list, int ncol, const T *__restrict__ u,
    const T *__restrict__ rhs, T *__restrict__ rbuf) {
  __shared__ int s_tab[kResWarps][4][32];
  __shared__ T s_acc[kResWarps][kRStride];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = blockIdx.x * kResWarps + warp;
  if (slot >= ncol) return;  // whole warp; no block-wide barrier in this kernel
  const int cell = list[slot];
  const int nu = op.nu;
  const T *u1 = u, *u2 = u + nu, *u3 = u + 2 * nu, *p = u + 3 * nu;
  const SegTab tab{s_tab[warp][0], s_tab[warp][1], s_tab[warp][2], s_tab[warp][3]};
  T *acc = s_acc[warp];
  for (int i = lane; i < kRStride; i += 32) acc[i] = T(0);
  const bool vu = lane < NU_LOC, vp = lane < NP_LOC;
  const int my_r = vu ? cells.udofs[(size_t)cell * NU_LOC + lane] : 0;
  const int my_p = vp ? cells.pdofs[(size_t)cell * NP_LOC + lane] : 0;
  // A rows: nine blocks, the one block of a structured operator, or the
  // three diagonal blocks of a level without velocity coupling
  int total = seg_setup<VEC>(tab, lane, vu, vu ? op.a_rowptr[my_r] : 0,
                             vu ? op.a_rowptr[my_r + 1] : 0);
  if (op.structured)
    flat_rows<T, 3, VEC, U>(tab, NU_LOC, total, op.a_col, op.a, u1, u2, u3, acc, lane);
  else if (op.diag)
    flat_rows<T, 4, VEC, U>(tab, NU_LOC, total, op.a_col, op.ad, u1, u2, u3, acc, lane);
  else
    flat_rows<T, 0, VEC, U>(tab, NU_LOC, total, op.a_col, op.a, u1, u2, u3, acc, lane);
  // BT rows of active velocity DOFs
  const bool act = vu && my_r < op.nact;
  total = seg_setup<VEC>(tab, lane, act, act ? op.bt_rowptr[my_r] : 0,
                         act ? op.bt_rowptr[my_r + 1] : 0);
  flat_rows<T, 1, VEC, U>(tab, NU_LOC, total, op.bt_col, op.bt, p, p, p, acc, lane);
  // B rows of the cell's pressure DOFs
  total = seg_setup<VEC>(tab, lane, vp, vp ? op.b_rowptr[my_p] : 0, vp ? op.b_rowptr[my_p + 1] : 0);
  flat_rows<T, 2, VEC, U>(tab, NP_LOC, total, op.b_col, op.b, u1, u2, u3, acc + 3 * NU_LOC, lane);
  __syncwarp();
  T *R = rbuf + (size_t)slot * kRStride;
  if (vu) {
    R[lane] = rhs[my_r] - acc[lane];
    R[lane + NU_LOC] = rhs[nu + my_r] - acc[lane + NU_LOC];
    R[lane + 2 * NU_LOC] = rhs[2 * nu + my_r] - acc[lane + 2 * NU_LOC];
  }
  if (vp) R[3 * NU_LOC + lane] = rhs[3 * nu + my_p] - acc[3 * NU_LOC + lane];
}

// Row-group variant of the local residual: one warp per cell, the warp's
// four 8-lane groups each own one row at a time (its A entries, then its BT
// entries), VEC entries per lane per load, a fixed 3-step butterfly per row.
// The cell's 27 velocity rows are taken in order of stencil size (8 Q2
// vertices, 12 edge midpoints, 6 face centres, the centre: 125/75/45/27
// entries on interior cells) so the four rows of a step have similar
// lengths; the order only balances work, any local numbering is correct.
__constant__ unsigned char c_row_order[NU_LOC] = {0, 2, 6, 8, 18, 20, 24, 26, 1, 3, 5, 7, 9, 11,
                                                  15, 17, 19, 21, 23, 25, 4, 10, 12, 14, 16, 22,
                                                  13};

// NV = 9 (nine A blocks), 1 (one A block), 3 with gather3 (a B row: one
// output) or without (a BT row: gather p, three outputs); DIAG (NV = 3):
// the diagonal blocks A11, A22, A33, value k times x_k into s[k].  AOS
// (FP32, gather3): x0 holds the velocity interleaved, node c at x0[4c..4c+2],
// one 16-byte gather per entry instead of three 4-byte ones
// UR groups of VEC entries of a row for one lane of its 8-lane group, the
// groups from g on with stride 8 (zeros past the row end re)
template <typename T, int VEC, int NV, int UR>
__device__ __forceinline__ void rg_load(const int *__restrict__ col, const T *const *vals, int g,
                                        int re, int (&ci)[UR][VEC], T (&v)[UR][NV][VEC]) {
#pragma unroll
  for (int q = 0; q < UR; ++q) {
    const int gq = g + 8 * q;
    if (gq * VEC < re) {
      VecLd<T, VEC>::idx(col + (size_t)gq * VEC, ci[q]);
#pragma unroll
      for (int k = 0; k < NV; ++k) VecLd<T, VEC>::val(vals[k] + (size_t)gq * VEC, v[q][k]);
    } else {
#pragma unroll
      for (int m = 0; m < VEC; ++m) {
        ci[q][m] = 0;
#pragma unroll
        for (int k = 0; k < NV; ++k) v[q][k][m] = T(0);
      }
    }
  }
}

// the products of the loaded entries in [rs, re): gathers and FMAs
template <typename T, int VEC, int NV, int UR, bool DIAG, bool AOS>
__device__ __forceinline__ void rg_accum(const int (&ci)[UR][VEC], const T (&v)[UR][NV][VEC],
                                         int g, int rs, int re, const T *__restrict__ x0,
                                         const T *__restrict__ x1, const T *__restrict__ x2,
                                         bool gather3, T (&s)[3]) {
#pragma unroll
  for (int q = 0; q < UR; ++q) {
    const int e0 = (g + 8 * q) * VEC;
#pragma unroll
    for (int m = 0; m < VEC; ++m) {
      const int e = e0 + m;
      if (e >= rs && e < re) {
        const int c = ci[q][m];
        if (gather3) {
          T g0, g1, g2;
          if constexpr (AOS) {
            static_assert(sizeof(T) == sizeof(float), "interleaved velocity: FP32 only");
            const float4 g4 = __ldg(reinterpret_cast<const float4 *>(x0) + c);
            g0 = g4.x;
            g1 = g4.y;
            g2 = g4.z;
          } else {
            g0 = __ldg(x0 + c);
            g1 = __ldg(x1 + c);
            g2 = __ldg(x2 + c);
          }
          if constexpr (DIAG) {
            s[0] += v[q][0][m] * g0;
            s[1] += v[q][1][m] * g1;
            s[2] += v[q][2][m] * g2;
          } else if constexpr (NV == 1) {
            s[0] += v[q][0][m] * g0;
            s[1] += v[q][0][m] * g1;
            s[2] += v[q][0][m] * g2;
          } else if constexpr (NV == 9) {
            s[0] += v[q][0][m] * g0 + v[q][1][m] * g1 + v[q][2][m] * g2;
            s[1] += v[q][3][m] * g0 + v[q][4][m] * g1 + v[q][5][m] * g2;
            s[2] += v[q][6][m] * g0 + v[q][7][m] * g1 + v[q][8][m] * g2;
          } else {  // B row: one output
            s[0] += v[q][0][m] * g0 + v[q][1][m] * g1 + v[q][2][m] * g2;
          }
        } else {  // BT row: gather p, three outputs
          const T pc = __ldg(x0 + c);
          s[0] += v[q][0][m] * pc;
          if constexpr (NV >= 3) {
            s[1] += v[q][1][m] * pc;
            s[2] += v[q][2][m] * pc;
          }
        }
      }
    }
  }
}

template <typename T, int VEC, int NV, int UR, bool DIAG = false, bool AOS = false>
__device__ __forceinline__ void row_group_sum(const int *__restrict__ col, const T *const *vals,
                                              int rs, int re, int sl, const T *__restrict__ x0,
                                              const T *__restrict__ x1, const T *__restrict__ x2,
                                              bool gather3, T (&s)[3]) {
  for (int g = rs / VEC + sl; g * VEC < re; g += 8 * UR) {
    int ci[UR][VEC];
    T v[UR][NV][VEC];
    rg_load<T, VEC, NV, UR>(col, vals, g, re, ci, v);
    rg_accum<T, VEC, NV, UR, DIAG, AOS>(ci, v, g, rs, re, x0, x1, x2, gather3, s);
  }
}

// A row and BT row of one velocity DOF: the first chunk of both (UR and URB
// groups per lane) is loaded before any of its gathers, so that a row step
// waits for one matrix round trip and one gather round trip; longer rows
// continue in row_group_sum
template <typename T, int VEC, int NV, int UR, int URB, bool DIAG, bool AOS>
__device__ __forceinline__ void vel_row_sum(const DevOp<T> &op, const T *const *avals, int ars,
                                            int are, int trs, int tre, int sl,
                                            const T *__restrict__ x0, const T *__restrict__ x1,
                                            const T *__restrict__ x2, const T *__restrict__ p,
                                            T (&s)[3]) {
  const int ga = ars / VEC + sl, gt = trs / VEC + sl;
  int ci[UR][VEC], cj[URB][VEC];
  T v[UR][NV][VEC], w[URB][3][VEC];
  rg_load<T, VEC, NV, UR>(op.a_col, avals, ga, are, ci, v);
  rg_load<T, VEC, 3, URB>(op.bt_col, op.bt, gt, tre, cj, w);
  rg_accum<T, VEC, NV, UR, DIAG, AOS>(ci, v, ga, ars, are, x0, x1, x2, true, s);
  rg_accum<T, VEC, 3, URB, false, false>(cj, w, gt, trs, tre, p, p, p, false, s);
  const int ra = (ars / VEC + 8 * UR) * VEC, rt = (trs / VEC + 8 * URB) * VEC;
  if (ra < are) row_group_sum<T, VEC, NV, UR, DIAG, AOS>(op.a_col, avals, ra, are, sl, x0, x1, x2, true, s);
  if (rt < tre) row_group_sum<T, VEC, 3, URB>(op.bt_col, op.bt, rt, tre, sl, p, p, p, false, s);
}

// KIND 0: nine A blocks; 1: one A block; 2: the three diagonal blocks.
// AOS (FP32, KIND 1): the velocity is read from ux (node c at ux[c], the
// three components and a pad), the pressure from u
template <typename T, int VEC, int KIND, int URA, int NU, bool AOS = false, bool FUSE = false>
__global__ void __launch_bounds__(kResWarps * 32) k_vanka_residual_rows(
    DevOp<T> op, DevCells cells, const int *__restrict__ list, int ncol, const T *__restrict__ u,
    const T *__restrict__ rhs, T *__restrict__ rbuf, const float4 *__restrict__ ux) {
  static_assert(!AOS || (KIND == 1 && sizeof(T) == sizeof(float)), "interleaved: FP32 one block");
  constexpr int NU_LOC = NU, kRStride = Elem<NU>::r_stride;
  // BT and B rows (at most 32 and 27 entries on hexahedra): one load round
  // trip per row whatever the vector width
  constexpr int URB = (16 / (int)sizeof(T)) / VEC > 1 ? (16 / (int)sizeof(T)) / VEC : 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = blockIdx.x * kResWarps + warp;
  if (slot >= ncol) return;  // whole warp; no block-wide barrier in this kernel
  const int cell = list[slot];
  const int sub = lane >> 3, sl = lane & 7;
  const int nu = op.nu;
  const T *u1 = u, *u2 = u + nu, *u3 = u + 2 * nu, *p = u + 3 * nu;
  const int *ud = cells.udofs + (size_t)cell * NU_LOC;
  T *R = rbuf + (size_t)slot * kRStride;
  // The cell's rows, their row-pointer ranges and right-hand sides, loaded
  // once, all in parallel, by the lane that owns each (lane a: velocity DOF
  // a; lane q < 4 also pressure DOF q) and handed to the 8-lane groups by
  // shuffles, so that a row step waits only for its values and gathers.
  const bool own_u = lane < NU_LOC, own_p = lane < NP_LOC;
  const int my_r = own_u ? __ldg(ud + lane) : 0;
  const int my_q = own_p ? __ldg(cells.pdofs + (size_t)cell * NP_LOC + lane) : 0;
  int my_ars = 0, my_are = 0, my_trs = 0, my_tre = 0, my_brs = 0, my_bre = 0;
  T my_f0 = T(0), my_f1 = T(0), my_f2 = T(0), my_fp = T(0);
  if (own_u) {
    my_ars = __ldg(op.a_rowptr + my_r);
    my_are = __ldg(op.a_rowptr + my_r + 1);
    if (my_r < op.nact) {
      my_trs = __ldg(op.bt_rowptr + my_r);
      my_tre = __ldg(op.bt_rowptr + my_r + 1);
    }
    my_f0 = rhs[my_r];
    my_f1 = rhs[(size_t)nu + my_r];
    my_f2 = rhs[(size_t)2 * nu + my_r];
  }
  if (own_p) {
    my_brs = __ldg(op.b_rowptr + my_q);
    my_bre = __ldg(op.b_rowptr + my_q + 1);
    my_fp = rhs[(size_t)3 * nu + my_q];
  }
  // velocity rows: A (one, three or nine blocks) and, on active rows, BT
  for (int step = 0; step < (NU_LOC + 3) / 4; ++step) {
    const int k = step * 4 + sub;
    const bool valid = k < NU_LOC;
    const int a = valid ? (NU == 27 ? (int)c_row_order[k] : k) : 0;
    const int ars = __shfl_sync(kFull, my_ars, a), are = __shfl_sync(kFull, my_are, a);
    const int trs = __shfl_sync(kFull, my_trs, a), tre = __shfl_sync(kFull, my_tre, a);
    const T f0 = __shfl_sync(kFull, my_f0, a), f1 = __shfl_sync(kFull, my_f1, a),
            f2 = __shfl_sync(kFull, my_f2, a);
    T s[3] = {T(0), T(0), T(0)};
    if (valid && FUSE) {
      if constexpr (AOS)
        vel_row_sum<T, VEC, 1, URA, URB, false, true>(op, op.a, ars, are, trs, tre, sl,
                                                      reinterpret_cast<const T *>(ux), nullptr,
                                                      nullptr, p, s);
      else if constexpr (KIND == 2)
        vel_row_sum<T, VEC, 3, URA, URB, true, false>(op, op.ad, ars, are, trs, tre, sl, u1, u2,
                                                      u3, p, s);
      else
        vel_row_sum<T, VEC, KIND == 1 ? 1 : 9, URA, URB, false, false>(op, op.a, ars, are, trs,
                                                                       tre, sl, u1, u2, u3, p, s);
    } else if (valid) {
      if constexpr (AOS)
        row_group_sum<T, VEC, 1, URA, false, true>(op.a_col, op.a,
                                                   ars, are, sl, reinterpret_cast<const T *>(ux),
                                                   nullptr, nullptr, true, s);
      else if constexpr (KIND == 2)
        row_group_sum<T, VEC, 3, URA, true>(op.a_col, op.ad, ars, are, sl, u1, u2, u3, true, s);
      else
        row_group_sum<T, VEC, KIND == 1 ? 1 : 9, URA>(op.a_col, op.a, ars, are, sl, u1, u2, u3,
                                                      true, s);
      if (tre > trs)  // active rows only (Dirichlet rows carry no BT)
        row_group_sum<T, VEC, 3, URB>(op.bt_col, op.bt, trs, tre, sl, p, p, p, false, s);
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
#pragma unroll
      for (int c = 0; c < 3; ++c) s[c] += __shfl_xor_sync(kFull, s[c], o);
    }
    if (valid && sl == 0) {
      R[a] = f0 - s[0];
      R[NU_LOC + a] = f1 - s[1];
      R[2 * NU_LOC + a] = f2 - s[2];
    }
  }
  // pressure rows (B): group `sub` owns the cell's pressure DOF `sub`
  {
    const int brs = __shfl_sync(kFull, my_brs, sub), bre = __shfl_sync(kFull, my_bre, sub);
    const T fp = __shfl_sync(kFull, my_fp, sub);
    T s[3] = {T(0), T(0), T(0)};
    if constexpr (AOS)
      row_group_sum<T, VEC, 3, URB, false, true>(op.b_col, op.b, brs, bre, sl,
                                                 reinterpret_cast<const T *>(ux), nullptr, nullptr,
                                                 true, s);
    else
      row_group_sum<T, VEC, 3, URB>(op.b_col, op.b, brs, bre, sl, u1, u2, u3, true, s);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) s[0] += __shfl_xor_sync(kFull, s[0], o);
    if (sl == 0) R[3 * NU_LOC + sub] = fp - s[0];
  }
}

template <typename T, int NU = NU_LOC>
__device__ __forceinline__ void scatter_local(int i, T v, const int *ud, const int *pd, int nu,
                                              T *u) {
  constexpr int NU_LOC = NU;
  if (i < 3 * NU_LOC) {
    const int comp = i / NU_LOC, a = i - comp * NU_LOC;
    u[(size_t)comp * nu + ud[a]] += v;
  } else {
    u[(size_t)3 * nu + pd[i - 3 * NU_LOC]] += v;
  }
}

// Mixed-precision apply with the stored FP32 inverse: delta = A^{-1} r, a
// dense 85x85 GEMV whose column loads are all independent (no substitution
// chain), then u[dofs] += damp * delta.
template <typename T>
__global__ void __launch_bounds__(kApplyWarps * 32) k_vanka_apply_inv(
    DevCells cells, int nu, const int *__restrict__ list, int ncol, const T *__restrict__ X,
    const T *__restrict__ rbuf, T damp, T *__restrict__ u) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = blockIdx.x * kApplyWarps + warp;
  if (slot >= ncol) return;
  const int cell = list[slot];
  const bool has2 = lane + 64 < NLOC;
  const T *R = rbuf + (size_t)slot * kRStride;
  const T r0 = R[lane], r1 = R[lane + 32], r2 = has2 ? R[lane + 64] : T(0);
  const T *Xc = X + (size_t)cell * kFacStride;
  T a0 = 0, a1 = 0, a2 = 0;
#pragma unroll 17
  for (int j = 0; j < NLOC; ++j) {
    const T *col = Xc + (size_t)j * NLOC;
    const T x0 = ld_stream(col + lane), x1 = ld_stream(col + lane + 32);
    const T x2 = has2 ? ld_stream(col + lane + 64) : T(0);
    const T rj = __shfl_sync(kFull, (j < 32) ? r0 : ((j < 64) ? r1 : r2), j & 31);
    a0 += x0 * rj;
    a1 += x1 * rj;
    a2 += x2 * rj;
  }
  const int *ud = cells.udofs + (size_t)cell * NU_LOC;
  const int *pd = cells.pdofs + (size_t)cell * NP_LOC;
  scatter_local(lane, damp * a0, ud, pd, nu, u);
  scatter_local(lane + 32, damp * a1, ud, pd, nu, u);
  if (has2) scatter_local(lane + 64, damp * a2, ud, pd, nu, u);
}

template <typename T, int NU>
__global__ void __launch_bounds__(kApplyWarps * 32) k_vanka_apply(
    DevCells cells, int nu, const int *__restrict__ list, int ncol, const T *__restrict__ F,
    const uint8_t *__restrict__ perm, const T *__restrict__ rbuf, T damp, T *__restrict__ u) {
  constexpr int NU_LOC = NU, NLOC = Elem<NU>::nloc, kFacStride = Elem<NU>::fac_stride,
                kRStride = Elem<NU>::r_stride;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = blockIdx.x * kApplyWarps + warp;
  if (slot >= ncol) return;
  const int cell = list[slot];
  const bool has1 = lane + 32 < NLOC, has2 = lane + 64 < NLOC;
  const uint8_t *pc = perm + (size_t)cell * NLOC;
  const T *R = rbuf + (size_t)slot * kRStride;
  T y0 = R[__ldg(pc + lane)];
  T y1 = has1 ? R[__ldg(pc + lane + 32)] : T(0);
  T y2 = has2 ? R[__ldg(pc + lane + 64)] : T(0);
  const T *Fc = F + (size_t)cell * kFacStride;
  // L2 prefetch of the 4 columns from j0 (one 128-byte line per lane, inside
  // this cell's factor block), kPfDist columns ahead of their use: the demand
  // loads then hit L2
  constexpr int kPfDist = 16;
  const char *fend = reinterpret_cast<const char *>(Fc + (size_t)NLOC * NLOC);
  auto prefetch4 = [&](int j0) {
    if (j0 < 0 || j0 >= NLOC) return;
    const char *a = reinterpret_cast<const char *>(Fc + (size_t)j0 * NLOC) + 128 * lane;
    if (lane * 128 < 4 * NLOC * (int)sizeof(T) && a < fend)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
  };
  // forward substitution with the unit lower factor, columns 0..83 in blocks
  // of 4, the next block's column entries loaded while this one is used
  T cur[4][3], nxt[4][3];
  auto load_l = [&](T(&b)[4][3], int j0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = j0 + q;
      const T *col = Fc + (size_t)j * NLOC;
      b[q][0] = (lane > j) ? ld_stream(col + lane) : T(0);
      b[q][1] = (has1 && lane + 32 > j) ? ld_stream(col + lane + 32) : T(0);
      b[q][2] = (has2 && lane + 64 > j) ? ld_stream(col + lane + 64) : T(0);
    }
  };
  load_l(cur, 0);
  for (int j = 4; j < kPfDist; j += 4) prefetch4(j);
  for (int j0 = 0; j0 < NLOC - 1; j0 += 4) {
    prefetch4(j0 + kPfDist);
    if (j0 + 4 < NLOC - 1) load_l(nxt, j0 + 4);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = j0 + q;
      const T ysel = (j < 32) ? y0 : ((j < 64) ? y1 : y2);
      const T yj = __shfl_sync(kFull, ysel, j & 31);
      y0 -= cur[q][0] * yj;
      y1 -= cur[q][1] * yj;
      y2 -= cur[q][2] * yj;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int k = 0; k < 3; ++k) cur[q][k] = nxt[q][k];
  }
  // back substitution with U (diagonal stores 1/U_jj), columns 84..0
  auto load_u = [&](T(&b)[4][3], int jt) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = jt - q;
      const T *col = Fc + (size_t)(j < 0 ? 0 : j) * NLOC;
      b[q][0] = (j >= 0 && lane <= j) ? ld_stream(col + lane) : T(0);
      b[q][1] = (j >= 0 && has1 && lane + 32 <= j) ? ld_stream(col + lane + 32) : T(0);
      b[q][2] = (j >= 0 && has2 && lane + 64 <= j) ? ld_stream(col + lane + 64) : T(0);
    }
  };
  load_u(cur, NLOC - 1);
  for (int jt = NLOC - 1; jt >= 0; jt -= 4) {
    prefetch4(jt - kPfDist - 3);
    if (jt - 4 >= 0) load_u(nxt, jt - 4);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = jt - q;
      if (j >= 0) {
        const int owner = j & 31;
        if (lane == owner) {
          if (j < 32) y0 *= cur[q][0];
          else if (j < 64) y1 *= cur[q][1];
          else y2 *= cur[q][2];
        }
        const T ysel = (j < 32) ? y0 : ((j < 64) ? y1 : y2);
        const T xj = __shfl_sync(kFull, ysel, owner);
        if (lane < j) y0 -= cur[q][0] * xj;
        if (lane + 32 < j) y1 -= cur[q][1] * xj;
        if (has2 && lane + 64 < j) y2 -= cur[q][2] * xj;
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int k = 0; k < 3; ++k) cur[q][k] = nxt[q][k];
  }
  // u += damp * delta on the cell's DOFs (local order: u1 nodes, u2, u3, p)
  const int *ud = cells.udofs + (size_t)cell * NU_LOC;
  const int *pd = cells.pdofs + (size_t)cell * NP_LOC;
  scatter_local<T, NU>(lane, damp * y0, ud, pd, nu, u);
  if (has1) scatter_local<T, NU>(lane + 32, damp * y1, ud, pd, nu, u);
  if (has2) scatter_local<T, NU>(lane + 64, damp * y2, ud, pd, nu, u);
}

// Two cells per warp: each half-warp owns one cell of the colour and each of
// its lanes rows hl, hl+16, ..., hl+80 (six per lane), so a warp keeps the
// factor columns of two cells in flight (the substitution chain, not the
// bandwidth, bounds one cell per warp).  Columns are processed in blocks of
// four, the next block's entries loaded while the current one is used; the
// row owning column j is held by half-lane j & 15 in slot j >> 4, so every
// index below is a compile-time constant after unrolling.
template <typename T, int NU, int SL>
__device__ __forceinline__ void load_cols(T (&b)[4][SL], const T *Fc, int hl, int j0, int dir,
                                          bool lower) {
  constexpr int NLOC = Elem<NU>::nloc;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int j = j0 + dir * t;
    const bool jok = j >= 0 && j < NLOC;
    const T *col = Fc + (size_t)(jok ? j : 0) * NLOC;
#pragma unroll
    for (int q = 0; q < SL; ++q) {
      const int r = hl + 16 * q;
      const bool want = jok && r < NLOC && (lower ? r > j : r <= j);
      b[t][q] = want ? ld_stream(col + r) : T(0);
    }
  }
}

template <typename T, int WARPS, int NU>
__global__ void __launch_bounds__(WARPS * 32) k_vanka_apply2(
    DevCells cells, int nu, const int *__restrict__ list, int ncol, const T *__restrict__ F,
    const uint8_t *__restrict__ perm, const T *__restrict__ rbuf, T damp, T *__restrict__ u) {
  constexpr int NU_LOC = NU, NLOC = Elem<NU>::nloc, kFacStride = Elem<NU>::fac_stride,
                kRStride = Elem<NU>::r_stride;
  constexpr int SL = (NLOC + 15) / 16;   // rows per half-lane: 6 (85), 4 (49)
  constexpr int NB = (NLOC + 3) / 4;     // column blocks of the back substitution
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pair = blockIdx.x * WARPS + warp;
  if (2 * pair >= ncol) return;  // whole warp
  const int half = lane >> 4, hl = lane & 15;
  const int slot = 2 * pair + half;
  const bool live = slot < ncol;
  const int cslot = live ? slot : slot - 1;  // an idle half repeats its partner's cell
  const int cell = list[cslot];
  const uint8_t *pc = perm + (size_t)cell * NLOC;
  const T *R = rbuf + (size_t)cslot * kRStride;
  T y[SL];
#pragma unroll
  for (int q = 0; q < SL; ++q) {
    const int r = hl + 16 * q;
    y[q] = r < NLOC ? R[__ldg(pc + r)] : T(0);
  }
  const T *Fc = F + (size_t)cell * kFacStride;
  // L2 prefetch of the 4 columns from j0, 16 columns ahead of their use (two
  // 128-byte lines per half-lane, inside this cell's factor block)
  const char *fend = reinterpret_cast<const char *>(Fc + (size_t)NLOC * NLOC);
  auto prefetch4 = [&](int j0) {
    if (j0 < 0 || j0 >= NLOC) return;
    const char *base = reinterpret_cast<const char *>(Fc + (size_t)j0 * NLOC);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int off = 128 * (hl + 16 * h);
      if (off < 4 * NLOC * (int)sizeof(T) && base + off < fend)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(base + off));
    }
  };
  T cur[4][SL], nxt[4][SL];
  // forward substitution with the unit lower factor, columns 0..83
  load_cols<T, NU, SL>(cur, Fc, hl, 0, 1, true);
  for (int jp = 4; jp < 16; jp += 4) prefetch4(jp);
#pragma unroll
  for (int blk = 0; blk < (NLOC - 1) / 4; ++blk) {  // 21 (85) or 12 (49) blocks of 4 columns
    const int j0 = 4 * blk;
    prefetch4(j0 + 16);
    if (blk + 1 < (NLOC - 1) / 4) load_cols<T, NU, SL>(nxt, Fc, hl, j0 + 4, 1, true);
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int j = j0 + t;
      const T yj = __shfl_sync(kFull, y[j >> 4], j & 15, 16);
#pragma unroll
      for (int q = 0; q < SL; ++q) y[q] -= cur[t][q] * yj;
    }
#pragma unroll
    for (int t = 0; t < 4; ++t)
#pragma unroll
      for (int q = 0; q < SL; ++q) cur[t][q] = nxt[t][q];
  }
  // back substitution with U (diagonal stores 1/U_jj), columns NLOC-1..0 in
  // blocks of 4 from 4 NB - 1 down (85: 87..84 with only 84 real, ..., 3..0)
  load_cols<T, NU, SL>(cur, Fc, hl, 4 * NB - 1, -1, false);
#pragma unroll
  for (int blk = NB - 1; blk >= 0; --blk) {
    const int jt = 4 * blk + 3;
    prefetch4(jt - 19);
    if (blk > 0) load_cols<T, NU, SL>(nxt, Fc, hl, jt - 4, -1, false);
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int j = jt - t;
      if (j < NLOC) {
        const int qb = j >> 4, owner = j & 15;
        if (hl == owner) y[qb] *= cur[t][qb];
        const T xj = __shfl_sync(kFull, y[qb], owner, 16);
#pragma unroll
        for (int q = 0; q < SL; ++q)
          if (hl + 16 * q < j) y[q] -= cur[t][q] * xj;
      }
    }
#pragma unroll
    for (int t = 0; t < 4; ++t)
#pragma unroll
      for (int q = 0; q < SL; ++q) cur[t][q] = nxt[t][q];
  }
  if (live) {
    const int *ud = cells.udofs + (size_t)cell * NU_LOC;
    const int *pd = cells.pdofs + (size_t)cell * NP_LOC;
#pragma unroll
    for (int q = 0; q < SL; ++q) {
      const int r = hl + 16 * q;
      if (r < NLOC) scatter_local<T, NU>(r, damp * y[q], ud, pd, nu, u);
    }
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
      if (op.structured) {
        const double v = op.a[0][j];
        a[idx * N + i] = v;
        a[(idx + nu) * N + i + nu] = v;
        a[(idx + nu2) * N + i + nu2] = v;
        continue;
      }
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
      const int k4 = op.structured ? 0 : 4, k8 = op.structured ? 0 : 8;
      a[i + N * idx] = op.a[0][j];
      a[(idx + nu) * N + i + nu] = op.a[k4][j];
      a[(idx + nu2) * N + i + nu2] = op.a[k8][j];
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
  __shared__ double piv_rcp;  // 1 / pivot, computed once per step
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
        const double pv = a[(size_t)k * N + bidx];  // the pivot before the interchange
        piv_rcp = pv != 0.0 ? 1.0 / pv : 0.0;
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
    const double rp = piv_rcp;
    if (rp == 0.0) {
      if (tid == 0) atomicOr(status, 2);
    } else {
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

// Blocked right-looking LU with partial pivoting for larger coarse systems
// (a coarsest level of several hundred to thousands of DOFs): per panel of
// kLuNb columns, one CTA factors the panel (the same pivot rule as
// k_dense_lu: first maximal |a|), one warp per other column applies the
// panel's row interchanges and, right of the panel, the unit-lower
// triangular solve with L11, and a tiled kernel updates the trailing matrix
// A22 -= L21 U12 on all SMs.  The factors and ipiv have the same meaning as
// k_dense_lu's (LAPACK dgetrf's sequential interchanges).
constexpr int kLuNb = 32;

__global__ void __launch_bounds__(kDenseThreads) k_lu_panel(double *a, int N, int k0, int *ipiv,
                                                            int *status) {
  __shared__ double bv[32];
  __shared__ int bi[32];
  __shared__ int piv_row;
  __shared__ double piv_rcp;  // 1 / pivot, computed once per step
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = kDenseThreads / 32;
  const int kend = min(k0 + kLuNb, N);
  for (int k = k0; k < kend; ++k) {
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
        const double pv = a[(size_t)k * N + bidx];  // the pivot before the interchange
        piv_rcp = pv != 0.0 ? 1.0 / pv : 0.0;
      }
    }
    __syncthreads();
    const int p = piv_row;
    if (p != k)
      for (int j = k0 + tid; j < kend; j += kDenseThreads) {
        const double t = a[(size_t)j * N + k];
        a[(size_t)j * N + k] = a[(size_t)j * N + p];
        a[(size_t)j * N + p] = t;
      }
    __syncthreads();
    const double rp = piv_rcp;
    if (rp == 0.0) {
      if (tid == 0) atomicOr(status, 2);
    } else {
      for (int i = k + 1 + tid; i < N; i += kDenseThreads) a[(size_t)k * N + i] *= rp;
    }
    __syncthreads();
    for (int jj = k + 1 + warp; jj < kend; jj += nwarps) {
      const double ukj = a[(size_t)jj * N + k];
      if (ukj != 0.0)
        for (int ii = k + 1 + lane; ii < N; ii += 32)
          a[(size_t)jj * N + ii] -= a[(size_t)k * N + ii] * ukj;
    }
    __syncthreads();
  }
}

// one warp per column outside the panel: the panel's interchanges, then
// (right of the panel) U12 = L11^{-1} A12
__global__ void k_lu_swap_trsm(double *a, int N, int k0, const int *ipiv) {
  const int lane = threadIdx.x & 31;
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int kend = min(k0 + kLuNb, N), m = kend - k0;
  if (w >= N - m) return;  // whole warp
  const int j = w < k0 ? (int)w : (int)w + m;
  double *col = a + (size_t)j * N;
  if (lane == 0)
    for (int k = k0; k < kend; ++k) {
      const int p = ipiv[k];
      if (p != k) {
        const double t = col[k];
        col[k] = col[p];
        col[p] = t;
      }
    }
  __syncwarp();
  if (j < k0) return;
  double v = lane < m ? col[k0 + lane] : 0.0;
  for (int k = 0; k < m; ++k) {
    const double xk = __shfl_sync(kFull, v, k);
    if (lane > k && lane < m) v -= a[(size_t)(k0 + k) * N + k0 + lane] * xk;
  }
  if (lane < m) col[k0 + lane] = v;
}

// A22 -= L21 U12: 64 x 64 tiles, 256 threads with 4 x 4 outputs each
constexpr int kLuTile = 64;
__global__ void __launch_bounds__(256) k_lu_gemm(double *a, int N, int k0) {
  __shared__ double Ls[kLuNb][kLuTile + 1];  // [k][i]
  __shared__ double Us[kLuNb][kLuTile + 1];  // [k][j]
  const int kend = min(k0 + kLuNb, N), m = kend - k0;
  const int i0 = kend + blockIdx.x * kLuTile, j0 = kend + blockIdx.y * kLuTile;
  const int tid = threadIdx.x;
  for (int t = tid; t < m * kLuTile; t += 256) {
    const int k = t / kLuTile, i = t - kLuTile * k;
    Ls[k][i] = (i0 + i < N) ? a[(size_t)(k0 + k) * N + i0 + i] : 0.0;
  }
  for (int t = tid; t < m * kLuTile; t += 256) {
    const int jj = t / m, k = t - m * jj;
    Us[k][jj] = (j0 + jj < N) ? a[(size_t)(j0 + jj) * N + k0 + k] : 0.0;
  }
  __syncthreads();
  const int ti = tid & 15, tj = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = 0.0;
  for (int k = 0; k < m; ++k) {
    double l[4], u[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) l[r] = Ls[k][ti + 16 * r];
#pragma unroll
    for (int c = 0; c < 4; ++c) u[c] = Us[k][tj + 16 * c];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[r][c] += l[r] * u[c];
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int j = j0 + tj + 16 * c;
    if (j >= N) continue;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int i = i0 + ti + 16 * r;
      if (i < N) a[(size_t)j * N + i] -= acc[r][c];
    }
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

// Column j of A^{-1} from the LU factors (P A = L U): one CTA per column,
// forward and back substitution of P e_j with barriers per step.  Runs once
// per factorisation; every coarse solve is then one GEMV.
constexpr int kInvThreads = 256;
__global__ void __launch_bounds__(kInvThreads) k_dense_inverse(const double *lu, const int *ipiv,
                                                               int N, double *inv) {
  extern __shared__ double xs[];
  const int j = blockIdx.x, tid = threadIdx.x;
  for (int i = tid; i < N; i += kInvThreads) xs[i] = (i == j) ? 1.0 : 0.0;
  __syncthreads();
  if (tid == 0)
    for (int k = 0; k < N; ++k) {
      const int p = ipiv[k];
      if (p != k) {
        const double t = xs[k];
        xs[k] = xs[p];
        xs[p] = t;
      }
    }
  __syncthreads();
  for (int k = 0; k < N; ++k) {
    const double xk = xs[k];
    if (xk != 0.0)
      for (int i = k + 1 + tid; i < N; i += kInvThreads) xs[i] -= lu[(size_t)k * N + i] * xk;
    __syncthreads();
  }
  for (int k = N - 1; k >= 0; --k) {
    if (tid == 0) xs[k] /= lu[(size_t)k * N + k];
    __syncthreads();
    const double xk = xs[k];
    if (xk != 0.0)
      for (int i = tid; i < k; i += kInvThreads) xs[i] -= lu[(size_t)k * N + i] * xk;
    __syncthreads();
  }
  for (int i = tid; i < N; i += kInvThreads) inv[(size_t)j * N + i] = xs[i];
}

// x = A^{-1} b (A^{-1} column-major), b[pin_row] = 0 when pin_row >= 0
template <typename TB, typename TX>
__global__ void k_dense_gemv(const double *__restrict__ inv, int N, const TB *__restrict__ b,
                             TX *__restrict__ x, int pin_row) {
  extern __shared__ double bs[];
  for (int i = threadIdx.x; i < N; i += blockDim.x) bs[i] = (i == pin_row) ? 0.0 : (double)b[i];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double s0 = 0.0, s1 = 0.0;
  int j = 0;
  for (; j + 1 < N; j += 2) {
    s0 += inv[(size_t)j * N + i] * bs[j];
    s1 += inv[(size_t)(j + 1) * N + i] * bs[j + 1];
  }
  if (j < N) s0 += inv[(size_t)j * N + i] * bs[j];
  x[i] = (TX)(s0 + s1);
}

inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

}  // namespace

template <typename TC, typename TF, int NU>
int launch_factor_nu(const DevOp<double> &op, const DevCells &cells, TF *factors, uint8_t *perm,
                     int *status, cudaStream_t s) {
  constexpr int n = Elem<NU>::nloc;
  const size_t sm = sizeof(TC) * n * n;
  cudaFuncSetAttribute(k_vanka_factor<TC, TF, NU>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)sm);
  k_vanka_factor<TC, TF, NU><<<cells.ncells, kFactorThreads, sm, s>>>(op, cells, factors, perm,
                                                                     status);
  return ok() < 0 ? -1 : 1;
}

template <typename TC, typename TF>
int launch_factor_impl(const DevOp<double> &op, const DevCells &cells, TF *factors, uint8_t *perm,
                       int *status, cudaStream_t s) {
  if (cells.nl == NU_TET) return launch_factor_nu<TC, TF, NU_TET>(op, cells, factors, perm, status, s);
  if (cells.nl != NU_LOC) return -1;
  return launch_factor_nu<TC, TF, NU_LOC>(op, cells, factors, perm, status, s);
}

template <typename TF>
int launch_vanka_factor(const DevOp<double> &op, const DevCells &cells, TF *factors, uint8_t *perm,
                        bool factor_fp32, bool inverse, int *status, cudaStream_t s) {
  if (cells.ncells <= 0) return 0;
  const int n = factor_fp32 ? launch_factor_impl<float, TF>(op, cells, factors, perm, status, s)
                            : launch_factor_impl<double, TF>(op, cells, factors, perm, status, s);
  if (n < 0 || !inverse) return n;
  if (cells.nl != NU_LOC) return -1;  // the stored inverse: hexahedral blocks only
  if constexpr (sizeof(TF) == sizeof(float)) {
    k_lu_inverse_f32<<<cells.ncells, kInvThreadsLU, 0, s>>>(factors, perm);
    return ok() < 0 ? -1 : n + 1;
  }
  return -1;  // the inverse is stored in FP32 only
}

template <typename T>
int launch_vanka_residual(const DevOp<T> &op, const DevCells &cells, const int *cell_list, int ncol,
                          const T *u, const T *rhs, T *rbuf, int variant, cudaStream_t s) {
  if (ncol <= 0) return 0;
  constexpr int VEC = sizeof(T) == 4 ? 4 : 2;
  constexpr int U = sizeof(T) == 4 ? 1 : 2;
  const int grid = (ncol + kResWarps - 1) / kResWarps;
  if (cells.nl == NU_TET) {  // tetrahedra: the row-group kernel
    if (op.structured)
      k_vanka_residual_rows<T, VEC, 1, 2, NU_TET><<<grid, kResWarps * 32, 0, s>>>(
          op, cells, cell_list, ncol, u, rhs, rbuf, nullptr);
    else if (op.diag)
      k_vanka_residual_rows<T, VEC, 2, 2, NU_TET><<<grid, kResWarps * 32, 0, s>>>(
          op, cells, cell_list, ncol, u, rhs, rbuf, nullptr);
    else
      k_vanka_residual_rows<T, VEC, 0, 1, NU_TET><<<grid, kResWarps * 32, 0, s>>>(
          op, cells, cell_list, ncol, u, rhs, rbuf, nullptr);
    return ok() < 0 ? -1 : 1;
  }
  if (cells.nl != NU_LOC) return -1;
  if (variant == 1) {
    k_vanka_residual<T, VEC, U><<<grid, kResWarps * 32, 0, s>>>(op, cells, cell_list, ncol, u, rhs,
                                                               rbuf);
  } else if (op.structured) {
    // one A value per entry.  FP32: scalar entries, so that the 8 lanes of a
    // row gather u at 8 consecutive columns (a vector width of 4 spread each
    // gather instruction over 32 entries and about three times as many cache
    // lines, and the kernel is bound by L1 wavefronts: 0.317 -> 0.277 ms per
    // 64^3 colour), 16 per lane in flight so that a vertex row (125 entries)
    // needs one load round trip; FP64 keeps pairs (measured faster there)
    if constexpr (sizeof(T) == 4)
      k_vanka_residual_rows<T, 1, 1, 16, NU_LOC><<<grid, kResWarps * 32, 0, s>>>(
          op, cells, cell_list, ncol, u, rhs, rbuf, nullptr);
    else
      k_vanka_residual_rows<T, VEC, 1, 2, NU_LOC><<<grid, kResWarps * 32, 0, s>>>(
          op, cells, cell_list, ncol, u, rhs, rbuf, nullptr);
  } else if (op.diag) {
    // three diagonal blocks: scalar entries in FP32 as for one block
    if constexpr (sizeof(T) == 4)
      k_vanka_residual_rows<T, 1, 2, 8, NU_LOC><<<grid, kResWarps * 32, 0, s>>>(
          op, cells, cell_list, ncol, u, rhs, rbuf, nullptr);
    else
      k_vanka_residual_rows<T, VEC, 2, 2, NU_LOC><<<grid, kResWarps * 32, 0, s>>>(
          op, cells, cell_list, ncol, u, rhs, rbuf, nullptr);
  } else {
    k_vanka_residual_rows<T, VEC, 0, 1, NU_LOC><<<grid, kResWarps * 32, 0, s>>>(
        op, cells, cell_list, ncol, u, rhs, rbuf, nullptr);
  }
  return ok() < 0 ? -1 : 1;
}

int launch_vanka_residual_aos(const DevOp<float> &op, const DevCells &cells, const int *cell_list,
                              int ncol, const float *u, const float4 *ux, const float *rhs,
                              float *rbuf, cudaStream_t s) {
  if (ncol <= 0) return 0;
  if (!op.structured || cells.nl != NU_LOC || ux == nullptr) return -1;
  const int grid = (ncol + kResWarps - 1) / kResWarps;
  // A and BT rows of a step loaded together (fused), 8 entries per lane of
  // an A row in flight (0.281 -> 0.266 ms per 64^3 colour against the
  // unfused kernel with 16)
  k_vanka_residual_rows<float, 1, 1, 8, NU_LOC, true, true><<<grid, kResWarps * 32, 0, s>>>(
      op, cells, cell_list, ncol, u, rhs, rbuf, ux);
  return ok() < 0 ? -1 : 1;
}

template <typename T>
int launch_vanka_apply(const DevCells &cells, int nu, const int *cell_list, int ncol,
                       const T *factors, const uint8_t *perm, bool inverse, const T *rbuf, T damp,
                       T *u, bool pairs, cudaStream_t s) {
  if (ncol <= 0) return 0;
  const int grid = (ncol + kApplyWarps - 1) / kApplyWarps;
  constexpr int W = sizeof(T) == 4 ? 8 : 4;  // FP64 holds twice the registers
  const int g2 = (ncol + 2 * W - 1) / (2 * W);
  if (cells.nl == NU_TET) {
    if (inverse) return -1;  // the stored inverse: hexahedral blocks only
    if (pairs)
      k_vanka_apply2<T, W, NU_TET><<<g2, W * 32, 0, s>>>(cells, nu, cell_list, ncol, factors,
                                                         perm, rbuf, damp, u);
    else
      k_vanka_apply<T, NU_TET><<<grid, kApplyWarps * 32, 0, s>>>(cells, nu, cell_list, ncol,
                                                                factors, perm, rbuf, damp, u);
    return ok() < 0 ? -1 : 1;
  }
  if (cells.nl != NU_LOC) return -1;
  if (inverse)
    k_vanka_apply_inv<T><<<grid, kApplyWarps * 32, 0, s>>>(cells, nu, cell_list, ncol, factors,
                                                          rbuf, damp, u);
  else if (pairs)
    k_vanka_apply2<T, W, NU_LOC><<<g2, W * 32, 0, s>>>(cells, nu, cell_list, ncol, factors, perm,
                                                       rbuf, damp, u);
  else
    k_vanka_apply<T, NU_LOC><<<grid, kApplyWarps * 32, 0, s>>>(cells, nu, cell_list, ncol, factors,
                                                              perm, rbuf, damp, u);
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
  if (n <= 2 * kLuNb) {
    k_dense_lu<<<1, kDenseThreads, 0, s>>>(a, n, ipiv, status);
    return ok() < 0 ? -1 : 1;
  }
  int launches = 0;
  for (int k0 = 0; k0 < n; k0 += kLuNb) {
    const int m = std::min(kLuNb, n - k0), rest = n - k0 - m;
    k_lu_panel<<<1, kDenseThreads, 0, s>>>(a, n, k0, ipiv, status);
    ++launches;
    if (n - m > 0) {
      const long long threads = (long long)(n - m) * 32;
      k_lu_swap_trsm<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(a, n, k0, ipiv);
      ++launches;
    }
    if (rest > 0) {
      const unsigned t = (unsigned)((rest + kLuTile - 1) / kLuTile);
      k_lu_gemm<<<dim3(t, t), 256, 0, s>>>(a, n, k0);
      ++launches;
    }
    if (ok() < 0) return -1;
  }
  return launches;
}

int launch_dense_inverse(const double *lu, const int *ipiv, int n, double *inv, cudaStream_t s) {
  const size_t sm = sizeof(double) * n;
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_dense_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_dense_inverse<<<n, kInvThreads, sm, s>>>(lu, ipiv, n, inv);
  return ok() < 0 ? -1 : 1;
}

template <typename TB, typename TX>
int launch_dense_gemv(const double *inv, int n, const TB *b, TX *x, int pin_row, cudaStream_t s) {
  const size_t sm = sizeof(double) * n;
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_dense_gemv<TB, TX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_dense_gemv<TB, TX><<<(n + 127) / 128, 128, sm, s>>>(inv, n, b, x, pin_row);
  return ok() < 0 ? -1 : 1;
}
template int launch_dense_gemv<double, double>(const double *, int, const double *, double *, int,
                                               cudaStream_t);
template int launch_dense_gemv<float, float>(const double *, int, const float *, float *, int,
                                             cudaStream_t);

int launch_dense_solve(const double *lu, const int *ipiv, int n, const double *b, double *x,
                       int pin_row, cudaStream_t s) {
  const size_t sm = sizeof(double) * n;
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_dense_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_dense_solve<<<1, kDenseSolveThreads, sm, s>>>(lu, ipiv, n, b, x, pin_row);
  return ok() < 0 ? -1 : 1;
}

template int launch_vanka_factor<double>(const DevOp<double> &, const DevCells &, double *,
                                         uint8_t *, bool, bool, int *, cudaStream_t);
template int launch_vanka_factor<float>(const DevOp<double> &, const DevCells &, float *,
                                        uint8_t *, bool, bool, int *, cudaStream_t);
#define PM_VINST(T)                                                                                 \
  template int launch_vanka_residual<T>(const DevOp<T> &, const DevCells &, const int *, int,      \
                                        const T *, const T *, T *, int, cudaStream_t);             \
  template int launch_vanka_apply<T>(const DevCells &, int, const int *, int, const T *,           \
                                     const uint8_t *, bool, const T *, T, T *, bool, cudaStream_t);
PM_VINST(double)
PM_VINST(float)
#undef PM_VINST

}  // namespace pm
