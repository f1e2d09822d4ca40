// pm_sparse.cu — HBM-bound sweeps of the saddle-point operator on sm_103a:
// the coupled defect / mat-vec over the nine A blocks + B + BT
// (CoupledDefect / CoupledMatVect, src/FE/MGComponents3D.C:2872-3209), the
// grid-transfer SpMVs, L2_0 projection (IntoL20Vector3D,
// src/FE/MGComponents3D.C:1756-1786), Dirichlet/relaxation updates and the
// FGMRES BLAS-1 with deterministic reductions.
//
// Layout: CSR exactly as the reference stores it (one row-pointer/column
// array shared by A11..A33, nine value arrays; B and BT likewise with three).
// Vectors are [u1|u2|u3|p].  Matrix values are streamed with evict-first
// loads so that the gathered vector stays resident in the 129 MB L2.
#include <cuda_runtime.h>

#include <cstdint>

#include "pm_kernels.h"

namespace pm {

namespace {

constexpr int kBlock = 256;
constexpr int kReduceBlocks = 4 * 152;  // fixed grid => fixed summation order

template <typename T>
__device__ __forceinline__ T ld_stream(const T *p) {
  return __ldcs(p);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int G, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Velocity rows with 8 lanes per row (four rows per warp) and aligned vector
// loads: each lane takes VEC consecutive entries of the column and value
// arrays (arrays are padded to a multiple of 8 entries at upload), UR such
// groups in flight, then a fixed 3-step butterfly per row.  Dirichlet rows
// (>= nact) carry only the diagonal-block values (off-diagonal blocks are
// zeroed at upload) and no BT; with zero_nonactive they are set to zero.
template <typename T, int VEC>
struct VLd;
template <>
struct VLd<float, 4> {
  static __device__ __forceinline__ void val(const float *p, float (&o)[4]) {
    const float4 v = __ldcs(reinterpret_cast<const float4 *>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
  static __device__ __forceinline__ void idx(const int *p, int (&o)[4]) {
    const int4 v = __ldg(reinterpret_cast<const int4 *>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
};
template <typename T>
struct VLd<T, 1> {
  static __device__ __forceinline__ void val(const T *p, T (&o)[1]) { o[0] = __ldcs(p); }
  static __device__ __forceinline__ void idx(const int *p, int (&o)[1]) { o[0] = __ldg(p); }
};
template <>
struct VLd<double, 2> {
  static __device__ __forceinline__ void val(const double *p, double (&o)[2]) {
    const double2 v = __ldcs(reinterpret_cast<const double2 *>(p));
    o[0] = v.x; o[1] = v.y;
  }
  static __device__ __forceinline__ void idx(const int *p, int (&o)[2]) {
    const int2 v = __ldg(reinterpret_cast<const int2 *>(p));
    o[0] = v.x; o[1] = v.y;
  }
};

// s[0..2] += the row's products; NV = 9 (A blocks) and 1 (one-block A)
// gather x0..x2; NV = 3 (BT) gathers x0 only; NV = 3 with DIAG (the
// diagonal blocks A11, A22, A33 of a level without velocity coupling)
// multiplies value k with x_k into s[k]
template <typename T, int VEC, int NV, int UR, bool DIAG = false>
__device__ __forceinline__ void rows8_sum(const int *__restrict__ col, const T *const *vals, int rs,
                                          int re, int sl, const T *__restrict__ x0,
                                          const T *__restrict__ x1, const T *__restrict__ x2,
                                          T (&s)[3]) {
  for (int g = rs / VEC + sl; g * VEC < re; g += 8 * UR) {
    int ci[UR][VEC];
    T v[UR][NV][VEC];
#pragma unroll
    for (int q = 0; q < UR; ++q) {
      const int gq = g + 8 * q;
      if (gq * VEC < re) {
        VLd<T, VEC>::idx(col + (size_t)gq * VEC, ci[q]);
#pragma unroll
        for (int k = 0; k < NV; ++k) VLd<T, VEC>::val(vals[k] + (size_t)gq * VEC, v[q][k]);
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
    for (int q = 0; q < UR; ++q) {
      const int e0 = (g + 8 * q) * VEC;
#pragma unroll
      for (int m = 0; m < VEC; ++m) {
        const int e = e0 + m;
        if (e >= rs && e < re) {
          const int c = ci[q][m];
          if constexpr (DIAG) {
            s[0] += v[q][0][m] * __ldg(x0 + c);
            s[1] += v[q][1][m] * __ldg(x1 + c);
            s[2] += v[q][2][m] * __ldg(x2 + c);
          } else if constexpr (NV == 3) {
            const T pc = __ldg(x0 + c);
            s[0] += v[q][0][m] * pc;
            s[1] += v[q][1][m] * pc;
            s[2] += v[q][2][m] * pc;
          } else if constexpr (NV == 1) {
            const T a = v[q][0][m];
            s[0] += a * __ldg(x0 + c);
            s[1] += a * __ldg(x1 + c);
            s[2] += a * __ldg(x2 + c);
          } else {
            const T g0 = __ldg(x0 + c), g1 = __ldg(x1 + c), g2 = __ldg(x2 + c);
            s[0] += v[q][0][m] * g0 + v[q][1][m] * g1 + v[q][2][m] * g2;
            s[1] += v[q][3][m] * g0 + v[q][4][m] * g1 + v[q][5][m] * g2;
            s[2] += v[q][6][m] * g0 + v[q][7][m] * g1 + v[q][8][m] * g2;
          }
        }
      }
    }
  }
}

// KIND 0: nine A blocks; 1: one A block for the three components; 2: the
// three diagonal blocks only (A12..A32 zero on the level)
template <typename T, int VEC, int KIND, int UR>
__global__ void __launch_bounds__(kBlock) k_coupled_velocity8(DevOp<T> op, const T *__restrict__ x,
                                                              const T *__restrict__ b,
                                                              T *__restrict__ r, int defect,
                                                              int zero_nonactive) {
  // BT rows (at most 32 entries on hexahedra): one load round trip
  constexpr int URB = (16 / (int)sizeof(T)) / VEC > 1 ? (16 / (int)sizeof(T)) / VEC : 1;
  // no early return before the group shuffles: every lane of the warp joins
  const int sl = threadIdx.x & 7;
  const long long row = ((long long)blockIdx.x * kBlock + threadIdx.x) >> 3;
  const int nu = op.nu;
  const bool valid = row < nu;
  const int i = valid ? (int)row : 0;
  const bool skip = !valid || (zero_nonactive && i >= op.nact);
  const T *u1 = x, *u2 = x + nu, *u3 = x + 2 * nu, *p = x + 3 * nu;
  T s[3] = {T(0), T(0), T(0)};
  if (!skip) {
    if constexpr (KIND == 2)
      rows8_sum<T, VEC, 3, UR, true>(op.a_col, op.ad, op.a_rowptr[i], op.a_rowptr[i + 1], sl, u1,
                                     u2, u3, s);
    else
      rows8_sum<T, VEC, KIND == 1 ? 1 : 9, UR>(op.a_col, op.a, op.a_rowptr[i], op.a_rowptr[i + 1],
                                               sl, u1, u2, u3, s);
    if (i < op.nact)
      rows8_sum<T, VEC, 3, URB>(op.bt_col, op.bt, op.bt_rowptr[i], op.bt_rowptr[i + 1], sl, p, p,
                                p, s);
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) s[c] = group_sum<8>(s[c]);
  if (valid && sl == 0) {
    if (skip) {
      r[i] = r[nu + i] = r[2 * nu + i] = T(0);
    } else if (defect) {
      r[i] = b[i] - s[0];
      r[nu + i] = b[nu + i] - s[1];
      r[2 * nu + i] = b[2 * nu + i] - s[2];
    } else {
      r[i] = s[0];
      r[nu + i] = s[1];
      r[2 * nu + i] = s[2];
    }
  }
}

// Pressure rows q - B u (or B u): G lanes per row.
template <typename T, int G>
__global__ void __launch_bounds__(kBlock) k_coupled_pressure(DevOp<T> op, const T *__restrict__ x,
                                                             const T *__restrict__ b,
                                                             T *__restrict__ r, int defect) {
  const int lane = threadIdx.x & (G - 1);
  const long long row = ((long long)blockIdx.x * kBlock + threadIdx.x) / G;
  const bool valid = row < op.np;
  const int nu = op.nu;
  const int i = valid ? (int)row : 0;
  const T *u1 = x, *u2 = x + nu, *u3 = x + 2 * nu;
  T s = 0;
  if (valid) {
    const int rs = op.b_rowptr[i], re = op.b_rowptr[i + 1];
    for (int j = rs + lane; j < re; j += G) {
      const int c = __ldg(op.b_col + j);
      s += ld_stream(op.b[0] + j) * __ldg(u1 + c) + ld_stream(op.b[1] + j) * __ldg(u2 + c) +
           ld_stream(op.b[2] + j) * __ldg(u3 + c);
    }
  }
  s = group_sum<G>(s);
  if (valid && lane == 0) r[3 * nu + i] = defect ? b[3 * nu + i] - s : s;
}

// y_k = M x_k for NC components (transfers): G lanes per row.
template <typename T, int G, int NC>
__global__ void __launch_bounds__(kBlock) k_csr_apply(DevCsr<T> m, const T *__restrict__ x,
                                                      int x_stride, T *__restrict__ y,
                                                      int y_stride) {
  const int lane = threadIdx.x & (G - 1);
  const long long row = ((long long)blockIdx.x * kBlock + threadIdx.x) / G;
  const bool valid = row < m.rows;
  const int i = valid ? (int)row : 0;
  T s[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) s[k] = 0;
  if (valid) {
    const int rs = m.rowptr[i], re = m.rowptr[i + 1];
    for (int j = rs + lane; j < re; j += G) {
      const int c = __ldg(m.col + j);
      const T v = __ldg(m.val + j);
#pragma unroll
      for (int k = 0; k < NC; ++k) s[k] += v * __ldg(x + (size_t)k * x_stride + c);
    }
  }
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    T t = group_sum<G>(s[k]);
    if (valid && lane == 0) y[(size_t)k * y_stride + i] = t;
  }
}

// ---------------------------------------------------------------------------
// Block sum in fixed order, then the last block reduces the partials in
// fixed order.  Deterministic for a fixed grid.
template <typename T>
__device__ __forceinline__ T block_sum(T v) {
  __shared__ T sh[kBlock / 32];
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  T t = 0;
  if (w == 0) {
    t = (l < kBlock / 32) ? sh[l] : T(0);
    t = warp_sum(t);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

__device__ __forceinline__ bool last_block_done(unsigned int *counter) {
  __shared__ bool last;
  __threadfence();
  if (threadIdx.x == 0) {
    unsigned int prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  return last;
}

__device__ __forceinline__ void final_reduce(const double *partials, int n, double *result,
                                             unsigned int *counter, double scale, bool sqrt_out) {
  double v = 0;
  for (int i = threadIdx.x; i < n; i += kBlock) v += ((volatile const double *)partials)[i];
  v = block_sum(v);
  if (threadIdx.x == 0) {
    v *= scale;
    *result = sqrt_out ? sqrt(v) : v;
    *counter = 0u;
  }
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_l20_sum(const T *__restrict__ p, int np,
                                                    double *partials, unsigned int *counter) {
  double s = 0;
  for (int i = (blockIdx.x * kBlock + threadIdx.x) * 4; i < np; i += gridDim.x * kBlock * 4)
    s += (double)p[i];
  s = block_sum(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
  if (last_block_done(counter)) {
    // mean of the constant modes: s / np * 4 (IntoL20Vector3D, case -11)
    final_reduce(partials, gridDim.x, partials + gridDim.x, counter, 4.0 / (double)np, false);
  }
}

template <typename T>
__global__ void k_l20_sub(T *p, int np, const double *mean) {
  const T m = (T)(*mean);
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) * 4; i < np; i += gridDim.x * blockDim.x * 4)
    p[i] -= m;
}

__global__ void __launch_bounds__(kBlock) k_dot(const double *__restrict__ a,
                                                const double *__restrict__ b, int n,
                                                double *partials, unsigned int *counter,
                                                double *result) {
  double s = 0;
  for (int i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) s += a[i] * b[i];
  s = block_sum(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
  if (last_block_done(counter)) final_reduce(partials, gridDim.x, result, counter, 1.0, false);
}

// Modified Gram-Schmidt step fused with the next dot product.
__global__ void __launch_bounds__(kBlock) k_mgs(double *__restrict__ w,
                                                const double *__restrict__ va,
                                                const double *__restrict__ ha,
                                                const double *__restrict__ vd, int n,
                                                double *partials, unsigned int *counter,
                                                double *result, int norm) {
  const double h = va ? *ha : 0.0;
  double s = 0;
  for (int i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
    double wi = w[i];
    if (va) {
      wi -= h * va[i];
      w[i] = wi;
    }
    s += vd ? wi * vd[i] : wi * wi;
  }
  s = block_sum(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
  if (last_block_done(counter)) final_reduce(partials, gridDim.x, result, counter, 1.0, norm != 0);
}

__global__ void k_scale_copy(double *v, const double *w, const double *h, int n) {
  const double hv = *h;
  const double r = hv != 0.0 ? 1.0 / hv : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    v[i] = hv != 0.0 ? w[i] * r : w[i];
}

__global__ void k_scale(double *v, double a, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] *= a;
}

__global__ void k_multi_axpy(double *x, const double *Z, size_t ld, const double *y, int nk, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = x[i];
    for (int k = 0; k < nk; ++k) s += Z[(size_t)k * ld + i] * y[k];
    x[i] = s;
  }
}

template <typename TD, typename TS>
__global__ void k_convert(TD *d, const TS *s, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    d[i] = (TD)s[i];
}

template <typename T>
__global__ void k_fill(T *x, T v, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = v;
}

template <typename T>
__global__ void k_axpy(T *y, T a, const T *x, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    y[i] += a * x[i];
}

template <typename T>
__global__ void k_dirichlet(T *u, const T *src, int nu, int hb, int ndir) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * ndir) return;
  const int c = t / ndir, i = hb + t % ndir;
  u[(size_t)c * nu + i] = src ? src[(size_t)c * nu + i] : T(0);
}

template <typename T>
__global__ void k_zero_nonactive(T *v, int nu, int nact) {
  const int m = nu - nact;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * m) return;
  v[(size_t)(t / m) * nu + nact + t % m] = T(0);
}

template <typename T>
__global__ void k_relax(T *u, const T *uold, T alpha, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    u[i] = uold[i] + alpha * (u[i] - uold[i]);
}

// the FP32 velocity between its three component arrays and the interleaved
// copy the one-block sweep gathers from (16 bytes per node, pad 0)
__global__ void k_pack_velocity(const float *__restrict__ u, float4 *__restrict__ ux, int nu) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nu; i += gridDim.x * blockDim.x)
    ux[i] = make_float4(u[i], u[(size_t)nu + i], u[(size_t)2 * nu + i], 0.f);
}
__global__ void k_unpack_velocity(const float4 *__restrict__ ux, float *__restrict__ u, int nu) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nu; i += gridDim.x * blockDim.x) {
    const float4 v = ux[i];
    u[i] = v.x;
    u[(size_t)nu + i] = v.y;
    u[(size_t)2 * nu + i] = v.z;
  }
}

struct Ptr9 {
  double *p[9];
};
__global__ void k_zero_dirichlet_offdiag(Ptr9 a, const int *rowptr, int nu, int nact) {
  const int i = nact + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nu) return;
  for (int j = rowptr[i]; j < rowptr[i + 1]; ++j) {
    a.p[1][j] = 0.0;
    a.p[2][j] = 0.0;
    a.p[3][j] = 0.0;
    a.p[5][j] = 0.0;
    a.p[6][j] = 0.0;
    a.p[7][j] = 0.0;
  }
}

// Upload by SM loads of the caller's host array (through the CPU-GPU link;
// the device must be able to read pageable host memory): d64 = src, and
// d32 = (float)src when d32 is given; entries i >= zero_from are written as
// zero (off-diagonal velocity blocks on the Dirichlet rows, which are
// numbered last).  Four independent 8-byte loads per thread and iteration.
__global__ void k_host_upload(const double *__restrict__ src, double *__restrict__ d64,
                              float *__restrict__ d32, long long n, long long zero_from) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    double v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = src[i + q * stride];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long k = i + q * stride;
      const double w = k < zero_from ? v[q] : 0.0;
      d64[k] = w;
      if (d32) d32[k] = (float)w;
    }
  }
  for (; i < n; i += stride) {
    const double w = i < zero_from ? src[i] : 0.0;
    d64[i] = w;
    if (d32) d32[i] = (float)w;
  }
}

__global__ void k_check_finite(const double *x, int n, int *flag) {
  int bad = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    bad |= !isfinite(x[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1);
}

inline int grid_for(long long threads, int block = kBlock) {
  long long g = (threads + block - 1) / block;
  if (g < 1) g = 1;
  if (g > 2147483647LL) g = 2147483647LL;
  return (int)g;
}
inline int stride_grid(int n) {
  int g = (n + kBlock - 1) / kBlock;
  return g < 1 ? 1 : (g > 8 * 152 ? 8 * 152 : g);
}
inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

}  // namespace

// ============================================================ launchers ====
template <typename T>
int launch_coupled(const DevOp<T> &op, const T *x, const T *b, T *r, bool defect,
                   bool zero_nonactive, cudaStream_t s) {
  constexpr int GP = 16;
  constexpr int VEC = sizeof(T) == 4 ? 4 : 2;
  const unsigned gv = grid_for((long long)op.nu * 8);
  if (op.structured) {
    // FP32: scalar entries, the 8 lanes of a row gathering consecutive
    // columns (fewer cache lines per gather instruction than vectors of 4)
    if constexpr (sizeof(T) == 4)
      k_coupled_velocity8<T, 1, 1, 8><<<gv, kBlock, 0, s>>>(op, x, b, r, defect ? 1 : 0,
                                                           zero_nonactive ? 1 : 0);
    else
      k_coupled_velocity8<T, VEC, 1, 2><<<gv, kBlock, 0, s>>>(op, x, b, r, defect ? 1 : 0,
                                                             zero_nonactive ? 1 : 0);
  } else if (op.diag) {
    if constexpr (sizeof(T) == 4)
      k_coupled_velocity8<T, 1, 2, 8><<<gv, kBlock, 0, s>>>(op, x, b, r, defect ? 1 : 0,
                                                           zero_nonactive ? 1 : 0);
    else
      k_coupled_velocity8<T, VEC, 2, 2><<<gv, kBlock, 0, s>>>(op, x, b, r, defect ? 1 : 0,
                                                             zero_nonactive ? 1 : 0);
  } else {
    k_coupled_velocity8<T, VEC, 0, 1><<<gv, kBlock, 0, s>>>(op, x, b, r, defect ? 1 : 0,
                                                           zero_nonactive ? 1 : 0);
  }
  if (ok() < 0) return -1;
  k_coupled_pressure<T, GP><<<grid_for((long long)op.np * GP), kBlock, 0, s>>>(op, x, b, r,
                                                                               defect ? 1 : 0);
  return ok() < 0 ? -1 : 2;
}

template <typename T>
int launch_csr_apply(const DevCsr<T> &m, int ncomp, const T *x, int x_stride, T *y, int y_stride,
                     cudaStream_t s) {
  constexpr int G = 8;
  const int g = grid_for((long long)m.rows * G);
  if (ncomp == 3)
    k_csr_apply<T, G, 3><<<g, kBlock, 0, s>>>(m, x, x_stride, y, y_stride);
  else if (ncomp == 1)
    k_csr_apply<T, G, 1><<<g, kBlock, 0, s>>>(m, x, x_stride, y, y_stride);
  else
    return -1;
  return ok() < 0 ? -1 : 1;
}

template <typename T>
int launch_l20_project(T *p, int np, double *scratch, unsigned int *counter, cudaStream_t s) {
  const int nb = 2 * 152;
  k_l20_sum<T><<<nb, kBlock, 0, s>>>(p, np, scratch, counter);
  if (ok() < 0) return -1;
  k_l20_sub<T><<<stride_grid(np / 4 + 1), kBlock, 0, s>>>(p, np, scratch + nb);
  return ok() < 0 ? -1 : 2;
}

int launch_dot(const double *a, const double *b, int n, double *partials, unsigned int *counter,
               double *result, cudaStream_t s) {
  k_dot<<<kReduceBlocks, kBlock, 0, s>>>(a, b, n, partials, counter, result);
  return ok() < 0 ? -1 : 1;
}

int launch_mgs_step(double *w, const double *v_axpy, const double *h_axpy, const double *v_dot,
                    int n, double *partials, unsigned int *counter, double *result,
                    cudaStream_t s) {
  k_mgs<<<kReduceBlocks, kBlock, 0, s>>>(w, v_axpy, h_axpy, v_dot, n, partials, counter, result,
                                         v_dot ? 0 : 1);
  return ok() < 0 ? -1 : 1;
}

int launch_scale_copy(double *v, const double *w, const double *h, int n, cudaStream_t s) {
  k_scale_copy<<<stride_grid(n), kBlock, 0, s>>>(v, w, h, n);
  return ok() < 0 ? -1 : 1;
}
int launch_scale(double *v, double alpha, int n, cudaStream_t s) {
  k_scale<<<stride_grid(n), kBlock, 0, s>>>(v, alpha, n);
  return ok() < 0 ? -1 : 1;
}
int launch_multi_axpy(double *x, const double *Z, size_t ld, const double *y, int nk, int n,
                      cudaStream_t s) {
  k_multi_axpy<<<stride_grid(n), kBlock, 0, s>>>(x, Z, ld, y, nk, n);
  return ok() < 0 ? -1 : 1;
}
template <typename TD, typename TS>
int launch_convert(TD *dst, const TS *src, int n, cudaStream_t s) {
  k_convert<TD, TS><<<stride_grid(n), kBlock, 0, s>>>(dst, src, n);
  return ok() < 0 ? -1 : 1;
}
template <typename T>
int launch_fill(T *x, T v, int n, cudaStream_t s) {
  k_fill<T><<<stride_grid(n), kBlock, 0, s>>>(x, v, n);
  return ok() < 0 ? -1 : 1;
}
template <typename T>
int launch_axpy(T *y, T a, const T *x, int n, cudaStream_t s) {
  k_axpy<T><<<stride_grid(n), kBlock, 0, s>>>(y, a, x, n);
  return ok() < 0 ? -1 : 1;
}
template <typename T>
int launch_dirichlet(T *u, const T *src, int nu, int hb, int ndir, cudaStream_t s) {
  if (ndir <= 0) return 0;
  k_dirichlet<T><<<grid_for(3LL * ndir), kBlock, 0, s>>>(u, src, nu, hb, ndir);
  return ok() < 0 ? -1 : 1;
}
template <typename T>
int launch_zero_nonactive(T *v, int nu, int nact, cudaStream_t s) {
  if (nu <= nact) return 0;
  k_zero_nonactive<T><<<grid_for(3LL * (nu - nact)), kBlock, 0, s>>>(v, nu, nact);
  return ok() < 0 ? -1 : 1;
}
template <typename T>
int launch_relax(T *u, const T *uold, T alpha, int n, cudaStream_t s) {
  k_relax<T><<<stride_grid(n), kBlock, 0, s>>>(u, uold, alpha, n);
  return ok() < 0 ? -1 : 1;
}
int launch_pack_velocity(const float *u, float4 *ux, int nu, cudaStream_t s) {
  if (nu <= 0) return 0;
  k_pack_velocity<<<stride_grid(nu), kBlock, 0, s>>>(u, ux, nu);
  return ok() < 0 ? -1 : 1;
}
int launch_unpack_velocity(const float4 *ux, float *u, int nu, cudaStream_t s) {
  if (nu <= 0) return 0;
  k_unpack_velocity<<<stride_grid(nu), kBlock, 0, s>>>(ux, u, nu);
  return ok() < 0 ? -1 : 1;
}
int launch_zero_dirichlet_offdiag(double *const a[9], const int *rowptr, int nu, int nact,
                                  cudaStream_t s) {
  if (nu <= nact) return 0;
  Ptr9 p;
  for (int k = 0; k < 9; ++k) p.p[k] = a[k];
  k_zero_dirichlet_offdiag<<<grid_for(nu - nact), kBlock, 0, s>>>(p, rowptr, nu, nact);
  return ok() < 0 ? -1 : 1;
}
int launch_host_upload(const double *src, double *d64, float *d32, long long n,
                       long long zero_from, int num_sms, cudaStream_t s) {
  if (n <= 0) return 0;
  long long g = (n + 4LL * kBlock - 1) / (4LL * kBlock);
  const long long cap = 8LL * num_sms;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  k_host_upload<<<(unsigned)g, kBlock, 0, s>>>(src, d64, d32, n, zero_from);
  return ok() < 0 ? -1 : 1;
}
int launch_check_finite(const double *x, int n, int *flag, cudaStream_t s) {
  k_check_finite<<<stride_grid(n), kBlock, 0, s>>>(x, n, flag);
  return ok() < 0 ? -1 : 1;
}

// explicit instantiations
#define PM_INST(T)                                                                                \
  template int launch_coupled<T>(const DevOp<T> &, const T *, const T *, T *, bool, bool,         \
                                 cudaStream_t);                                                   \
  template int launch_csr_apply<T>(const DevCsr<T> &, int, const T *, int, T *, int,              \
                                   cudaStream_t);                                                 \
  template int launch_l20_project<T>(T *, int, double *, unsigned int *, cudaStream_t);           \
  template int launch_fill<T>(T *, T, int, cudaStream_t);                                         \
  template int launch_axpy<T>(T *, T, const T *, int, cudaStream_t);                              \
  template int launch_dirichlet<T>(T *, const T *, int, int, int, cudaStream_t);                  \
  template int launch_zero_nonactive<T>(T *, int, int, cudaStream_t);                             \
  template int launch_relax<T>(T *, const T *, T, int, cudaStream_t);
PM_INST(double)
PM_INST(float)
#undef PM_INST
template int launch_convert<float, double>(float *, const double *, int, cudaStream_t);
template int launch_convert<double, float>(double *, const float *, int, cudaStream_t);
template int launch_convert<double, double>(double *, const double *, int, cudaStream_t);

}  // namespace pm
