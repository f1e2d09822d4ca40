// pm_cellstore.cu — local residuals of the cell-Vanka sweep from a per-cell
// copy of the matrix rows each cell reads.
//
// The multiplicative colour-block Vanka sweep (the reference's GPU
// smoother's order, src/FE/NSE_CellVanka.cu:2181-2365) computes, colour by
// colour, r = f - K u on every cell's 85 DOFs over the full CSR rows of its
// 27 velocity and 4 pressure DOFs (src/FE/NSE_MGLevel4.C:1823-1960).  Over
// one sweep every velocity row is read once per cell that contains it (8
// times at a vertex), and from the CSR arrays those reads are 27 short
// scattered row segments per cell behind a row-pointer load.  For levels
// without velocity coupling the rows are copied once per matrix (at every
// refactorisation) into a store laid out in the sweep's colour order: the
// cells of one colour read one contiguous stretch, every row padded to whole
// vector groups, each group tagged with its local row.  The residual kernel
// then streams its cell's groups with aligned vector loads, 32 groups per
// warp step, and sums rows with a segmented warp reduction (keys are
// contiguous: one shuffle tree per step, the first lane of each row adds
// the row's partial sum into shared memory); the order of every sum is
// fixed, so results repeat bit for bit.
#include <cuda_runtime.h>

#include <cstdint>

#include "pm_kernels.h"

namespace pm {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kCsWarps = 4;     // residual: warps (cells) per CTA
constexpr int kFillWarps = 4;   // fill: warps (cells) per CTA

template <typename T>
struct Vec;
template <>
struct Vec<float> {
  static constexpr int n = 4;
  static __device__ __forceinline__ void ld(const float *p, float (&o)[4]) {
    const float4 v = __ldcs(reinterpret_cast<const float4 *>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
  static __device__ __forceinline__ void ldi(const int *p, int (&o)[4]) {
    const int4 v = __ldcs(reinterpret_cast<const int4 *>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
};
template <>
struct Vec<double> {
  static constexpr int n = 2;
  static __device__ __forceinline__ void ld(const double *p, double (&o)[2]) {
    const double2 v = __ldcs(reinterpret_cast<const double2 *>(p));
    o[0] = v.x; o[1] = v.y;
  }
  static __device__ __forceinline__ void ldi(const int *p, int (&o)[2]) {
    const int2 v = __ldcs(reinterpret_cast<const int2 *>(p));
    o[0] = v.x; o[1] = v.y;
  }
};

// Segmented warp sum of NO values keyed by seg (keys contiguous over the
// lanes, -1 = none): the first lane of each key adds its key's sums to
// acc[seg + k * stride].  The shuffle tree is fixed, so is the order.
template <typename T, int NO>
__device__ __forceinline__ void seg_add(int seg, T (&v)[NO], T *acc, int stride, int lane) {
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

// One warp per cell.  KIND 0: A groups (NVA values, gather u1, u2, u3, three
// outputs); 1: BT groups (three values, gather p, three outputs); 2: B
// groups (three values, gather u1, u2, u3, one output).  Software-pipelined:
// the loads of the next 32 x UR groups are issued before the gathers, the
// products and the segmented sums of the current ones, so one memory round
// trip overlaps the other work of a step.
template <typename T, int KIND, int NVA, int UR>
struct Groups {
  static constexpr int VEC = Vec<T>::n;
  static constexpr int NV = KIND == 0 ? NVA : 3;
  int c[UR][VEC], seg[UR];
  T v[UR][NV][VEC];

  __device__ __forceinline__ void load(const int *__restrict__ col,
                                       const unsigned char *__restrict__ rid,
                                       const T *const *vals, long long g0, int ng, int b,
                                       int lane) {
#pragma unroll
    for (int q = 0; q < UR; ++q) {
      const int g = b + q * 32 + lane;
      seg[q] = -1;
      if (g < ng) {
        const long long e = (g0 + g) * VEC;
        seg[q] = rid[g0 + g];
        Vec<T>::ldi(col + e, c[q]);
#pragma unroll
        for (int k = 0; k < NV; ++k) Vec<T>::ld(vals[k] + e, v[q][k]);
      }
    }
  }
};

template <typename T, int KIND, int NVA, int UR>
__device__ __forceinline__ void stream_groups(const int *__restrict__ col,
                                              const unsigned char *__restrict__ rid,
                                              const T *const *vals, long long g0, int ng,
                                              const T *__restrict__ x0, const T *__restrict__ x1,
                                              const T *__restrict__ x2, T *acc, int lane) {
  constexpr int VEC = Vec<T>::n;
  constexpr int NV = KIND == 0 ? NVA : 3;
  constexpr int NO = KIND == 2 ? 1 : 3;
  if (ng <= 0) return;
  Groups<T, KIND, NVA, UR> cur, nxt;
  nxt.load(col, rid, vals, g0, ng, 0, lane);
  for (int b = 0; b < ng; b += 32 * UR) {
    cur = nxt;
    if (b + 32 * UR < ng) nxt.load(col, rid, vals, g0, ng, b + 32 * UR, lane);
#pragma unroll
    for (int q = 0; q < UR; ++q) {
      T s[NO];
#pragma unroll
      for (int k = 0; k < NO; ++k) s[k] = T(0);
      if (cur.seg[q] >= 0) {
#pragma unroll
        for (int m = 0; m < VEC; ++m) {
          const int cc = cur.c[q][m];
          if constexpr (KIND == 0) {
            if constexpr (NVA == 1) {
              const T a = cur.v[q][0][m];
              s[0] += a * __ldg(x0 + cc);
              s[1 % NO] += a * __ldg(x1 + cc);
              s[2 % NO] += a * __ldg(x2 + cc);
            } else {
              s[0] += cur.v[q][0][m] * __ldg(x0 + cc);
              s[1 % NO] += cur.v[q][1 % NV][m] * __ldg(x1 + cc);
              s[2 % NO] += cur.v[q][2 % NV][m] * __ldg(x2 + cc);
            }
          } else if constexpr (KIND == 1) {
            const T pc = __ldg(x0 + cc);
            s[0] += cur.v[q][0][m] * pc;
            s[1 % NO] += cur.v[q][1][m] * pc;
            s[2 % NO] += cur.v[q][2][m] * pc;
          } else {
            s[0] += cur.v[q][0][m] * __ldg(x0 + cc) + cur.v[q][1][m] * __ldg(x1 + cc) +
                    cur.v[q][2][m] * __ldg(x2 + cc);
          }
        }
      }
      seg_add<T, NO>(cur.seg[q], s, acc, NU_LOC, lane);
    }
  }
}

template <typename T, int NVA>
__global__ void __launch_bounds__(kCsWarps * 32) k_vanka_residual_cells(
    CellStore<T> cs, DevCells cells, int nu, int slot0, const int *__restrict__ list, int ncol,
    const T *__restrict__ u, const T *__restrict__ rhs, T *__restrict__ rbuf) {
  __shared__ T s_acc[kCsWarps][kRStride];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = blockIdx.x * kCsWarps + warp;
  if (slot >= ncol) return;  // whole warp; no block-wide barrier in this kernel
  const int s = slot0 + slot;
  const int cell = list[slot];
  T *acc = s_acc[warp];
  for (int i = lane; i < kRStride; i += 32) acc[i] = T(0);
  __syncwarp();
  const T *u1 = u, *u2 = u + nu, *u3 = u + 2 * (size_t)nu, *p = u + 3 * (size_t)nu;
  const int nA = cs.cnt[3 * s], nBT = cs.cnt[3 * s + 1], nB = cs.cnt[3 * s + 2];
  const long long gA = cs.offA[s], gP = cs.offP[s];
  stream_groups<T, 0, NVA, 2>(cs.colA, cs.ridA, cs.a, gA, nA, u1, u2, u3, acc, lane);
  stream_groups<T, 1, NVA, 1>(cs.colP, cs.ridP, cs.p, gP, nBT, p, p, p, acc, lane);
  stream_groups<T, 2, NVA, 1>(cs.colP, cs.ridP, cs.p, gP + nBT, nB, u1, u2, u3,
                              acc + 3 * NU_LOC, lane);
  T *R = rbuf + (size_t)slot * kRStride;
  if (lane < NU_LOC) {
    const int r = cells.udofs[(size_t)cell * NU_LOC + lane];
    R[lane] = rhs[r] - acc[lane];
    R[lane + NU_LOC] = rhs[(size_t)nu + r] - acc[lane + NU_LOC];
    R[lane + 2 * NU_LOC] = rhs[2 * (size_t)nu + r] - acc[lane + 2 * NU_LOC];
  }
  if (lane < NP_LOC) {
    const int r = cells.pdofs[(size_t)cell * NP_LOC + lane];
    R[3 * NU_LOC + lane] = rhs[3 * (size_t)nu + r] - acc[3 * NU_LOC + lane];
  }
}

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

// Copy rows of one kind into the store: the warp's rows are given per lane
// (valid, source range [rs, rs + len)); each row goes to groups starting at
// g0 + its exclusive prefix of group counts.  KIND 0: A rows (nva values),
// 1: BT rows, 2: B rows (three values each).
template <typename T, int KIND>
__device__ __forceinline__ void fill_rows(bool valid, int rs, int len, int local, long long g0,
                                          const int *__restrict__ src_col,
                                          const double *const *src, int nv, int *dst_col,
                                          unsigned char *dst_rid, T *const *dst, bool pattern,
                                          int lane) {
  constexpr int VEC = Vec<T>::n;
  const int ng = valid ? (len + VEC - 1) / VEC : 0;
  int total;
  const int start = warp_excl_scan(ng, lane, total);
  for (int w = 0; w < 32; ++w) {
    const int n = __shfl_sync(kFull, ng, w);
    if (n == 0) continue;
    const int r0 = __shfl_sync(kFull, rs, w), ln = __shfl_sync(kFull, len, w);
    const int st = __shfl_sync(kFull, start, w), lr = __shfl_sync(kFull, local, w);
    const long long e0 = (g0 + st) * VEC;
    for (int j = lane; j < n * VEC; j += 32) {
      const bool real = j < ln;
      const int sj = r0 + (real ? j : ln - 1);
      if (pattern) {
        dst_col[e0 + j] = src_col[sj];
        if (j % VEC == 0) dst_rid[g0 + st + j / VEC] = (unsigned char)lr;
      }
      for (int k = 0; k < nv; ++k) dst[k][e0 + j] = real ? (T)src[k][sj] : T(0);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kFillWarps * 32) k_cell_store_fill(
    CellStore<T> cs, DevOp<double> op, DevCells cells, const int *__restrict__ order, int nslots,
    int pattern) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.x * kFillWarps + warp;
  if (s >= nslots) return;  // whole warp
  const int cell = order[s];
  int *colA = const_cast<int *>(cs.colA), *colP = const_cast<int *>(cs.colP);
  unsigned char *ridA = const_cast<unsigned char *>(cs.ridA);
  unsigned char *ridP = const_cast<unsigned char *>(cs.ridP);
  T *a[3] = {const_cast<T *>(cs.a[0]), const_cast<T *>(cs.a[1]), const_cast<T *>(cs.a[2])};
  T *p[3] = {const_cast<T *>(cs.p[0]), const_cast<T *>(cs.p[1]), const_cast<T *>(cs.p[2])};
  // A rows of the 27 velocity DOFs: A11 (= A22 = A33) or A11, A22, A33
  const bool vu = lane < NU_LOC;
  const int r = vu ? cells.udofs[(size_t)cell * NU_LOC + lane] : 0;
  const double *srcA[3] = {op.a[0], op.structured ? op.a[0] : op.a[4],
                           op.structured ? op.a[0] : op.a[8]};
  fill_rows<T, 0>(vu, vu ? op.a_rowptr[r] : 0, vu ? op.a_rowptr[r + 1] - op.a_rowptr[r] : 0,
                  lane, cs.offA[s], op.a_col, srcA, cs.nva, colA, ridA, a, pattern != 0, lane);
  // BT rows of the active ones, then the 4 B rows
  const bool act = vu && r < op.nact;
  fill_rows<T, 1>(act, act ? op.bt_rowptr[r] : 0,
                  act ? op.bt_rowptr[r + 1] - op.bt_rowptr[r] : 0, lane, cs.offP[s], op.bt_col,
                  op.bt, 3, colP, ridP, p, pattern != 0, lane);
  const bool vp = lane < NP_LOC;
  const int q = vp ? cells.pdofs[(size_t)cell * NP_LOC + lane] : 0;
  fill_rows<T, 2>(vp, vp ? op.b_rowptr[q] : 0, vp ? op.b_rowptr[q + 1] - op.b_rowptr[q] : 0,
                  lane, cs.offP[s] + cs.cnt[3 * s + 1], op.b_col, op.b, 3, colP, ridP, p,
                  pattern != 0, lane);
}

inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

}  // namespace

void cell_store_layout(int nslots, const int *order, const int *udofs, const int *pdofs, int nact,
                       const int *a_rowptr, const int *b_rowptr, const int *bt_rowptr, int vec,
                       long long *offA, long long *offP, int *cnt) {
  auto groups = [vec](int len) { return (len + vec - 1) / vec; };
  offA[0] = offP[0] = 0;
  for (int s = 0; s < nslots; ++s) {
    const int c = order[s];
    int nA = 0, nBT = 0, nB = 0;
    for (int a = 0; a < NU_LOC; ++a) {
      const int r = udofs[(size_t)c * NU_LOC + a];
      nA += groups(a_rowptr[r + 1] - a_rowptr[r]);
      if (r < nact) nBT += groups(bt_rowptr[r + 1] - bt_rowptr[r]);
    }
    for (int k = 0; k < NP_LOC; ++k) {
      const int q = pdofs[(size_t)c * NP_LOC + k];
      nB += groups(b_rowptr[q + 1] - b_rowptr[q]);
    }
    cnt[3 * s] = nA;
    cnt[3 * s + 1] = nBT;
    cnt[3 * s + 2] = nB;
    offA[s + 1] = offA[s] + nA;
    offP[s + 1] = offP[s] + nBT + nB;
  }
}

template <typename T>
int launch_cell_store_fill(const CellStore<T> &cs, const DevOp<double> &op, const DevCells &cells,
                           const int *order, int nslots, bool write_pattern, cudaStream_t s) {
  if (nslots <= 0) return 0;
  if (cells.nl != NU_LOC) return -1;
  const int grid = (nslots + kFillWarps - 1) / kFillWarps;
  k_cell_store_fill<T><<<grid, kFillWarps * 32, 0, s>>>(cs, op, cells, order, nslots,
                                                       write_pattern ? 1 : 0);
  return ok() < 0 ? -1 : 1;
}

template <typename T>
int launch_vanka_residual_cells(const CellStore<T> &cs, const DevCells &cells, int nu, int slot0,
                                const int *cell_list, int ncol, const T *u, const T *rhs, T *rbuf,
                                cudaStream_t s) {
  if (ncol <= 0) return 0;
  if (cells.nl != NU_LOC) return -1;
  const int grid = (ncol + kCsWarps - 1) / kCsWarps;
  if (cs.nva == 1)
    k_vanka_residual_cells<T, 1><<<grid, kCsWarps * 32, 0, s>>>(cs, cells, nu, slot0, cell_list,
                                                               ncol, u, rhs, rbuf);
  else
    k_vanka_residual_cells<T, 3><<<grid, kCsWarps * 32, 0, s>>>(cs, cells, nu, slot0, cell_list,
                                                               ncol, u, rhs, rbuf);
  return ok() < 0 ? -1 : 1;
}

#define PM_CSINST(T)                                                                              \
  template int launch_cell_store_fill<T>(const CellStore<T> &, const DevOp<double> &,              \
                                         const DevCells &, const int *, int, bool, cudaStream_t);  \
  template int launch_vanka_residual_cells<T>(const CellStore<T> &, const DevCells &, int, int,    \
                                              const int *, int, const T *, const T *, T *,         \
                                              cudaStream_t);
PM_CSINST(double)
PM_CSINST(float)
#undef PM_CSINST

}  // namespace pm
