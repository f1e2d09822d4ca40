// pm_batch.cu — kernels of the fused multi-system solve (pm_add_level_batch,
// pm_solve_fused): G independent Oseen systems of one mesh are stacked into
// one block-diagonal level per grid level, so that every V-cycle kernel
// covers all G systems in one launch.  The stacked vectors are component-
// major with active DOFs first ([U1 | U2 | U3 | P], each velocity block =
// the G systems' active DOFs, then their Dirichlet DOFs; P = the G systems'
// pressures one after the other), which keeps the single-system kernels
// valid on the stacked level.  What must stay per system is here: the L^2_0
// pressure projection, the coarse direct solve (one dense inverse per
// system), and FGMRES's inner products, scalings and updates (one Arnoldi
// process per system, as TFgmresIte::Iterate runs for one system,
// src/FE/FgmresIte.C:250-677).  The reference batches the cells of one
// colour of one system in a launch (src/FE/NSE_CellVanka.cu:2181-2365);
// here a launch covers one colour of all G systems.
#include <cuda_runtime.h>

#include "pm_kernels.h"

namespace pm {
namespace {

constexpr int kB = 256;         // threads per block of the segment kernels
constexpr int kSegRanges = 7;   // ranges of one system in the stacked vector

__device__ __forceinline__ double block_sum256(double v) {
  __shared__ double ws[kB / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();  // ws may still be read by a previous call
  if (lane == 0) ws[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (warp == 0) {
    s = lane < kB / 32 ? ws[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  return s;  // valid in thread 0
}

// range r of system s = blockIdx.y; false if the system is inactive
__device__ __forceinline__ bool seg_range(const SegLayout &L, const int *act, long long &start,
                                          int &len) {
  const int s = blockIdx.y;
  if (act && !act[s]) return false;
  L.range(s, blockIdx.z, start, len);
  return true;
}

__global__ void __launch_bounds__(kB) k_seg_dot(const double *__restrict__ a,
                                                const double *__restrict__ b, SegLayout L,
                                                const int *act, double *partials) {
  long long start;
  int len;
  double s = 0.0;
  if (seg_range(L, act, start, len))
    for (int i = blockIdx.x * kB + threadIdx.x; i < len; i += gridDim.x * kB)
      s += a[start + i] * (b ? b[start + i] : a[start + i]);
  s = block_sum256(s);
  if (threadIdx.x == 0)
    partials[((size_t)blockIdx.y * kSegRanges + blockIdx.z) * gridDim.x + blockIdx.x] = s;
}

// w -= h[s] * va (va != null), then partial sums of <w, vd> (or <w, w>)
__global__ void __launch_bounds__(kB) k_seg_mgs(double *__restrict__ w,
                                                const double *__restrict__ va,
                                                const double *__restrict__ ha,
                                                const double *__restrict__ vd, SegLayout L,
                                                const int *act, double *partials) {
  long long start;
  int len;
  double s = 0.0;
  if (seg_range(L, act, start, len)) {
    const double h = va ? ha[blockIdx.y] : 0.0;
    for (int i = blockIdx.x * kB + threadIdx.x; i < len; i += gridDim.x * kB) {
      double wi = w[start + i];
      if (va) {
        wi -= h * va[start + i];
        w[start + i] = wi;
      }
      s += vd ? wi * vd[start + i] : wi * wi;
    }
  }
  s = block_sum256(s);
  if (threadIdx.x == 0)
    partials[((size_t)blockIdx.y * kSegRanges + blockIdx.z) * gridDim.x + blockIdx.x] = s;
}

// out[s * ostride] = sum of system s's partials in a fixed order (sqrt if norm)
__global__ void __launch_bounds__(kB) k_seg_reduce(const double *partials, int per_sys,
                                                   double *out, int ostride, int norm) {
  const double *p = partials + (size_t)blockIdx.x * per_sys;
  double s = 0.0;
  for (int i = threadIdx.x; i < per_sys; i += kB) s += p[i];
  s = block_sum256(s);
  if (threadIdx.x == 0) out[(size_t)blockIdx.x * ostride] = norm ? sqrt(s) : s;
}

// v[system s] *= coef[s]
__global__ void k_seg_scale(double *v, SegLayout L, const double *coef) {
  long long start;
  int len;
  if (!seg_range(L, nullptr, start, len)) return;
  const double c = coef[blockIdx.y];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x)
    v[start + i] *= c;
}

// v = w / h[s] for active systems with h[s] != 0, else v = 0
__global__ void k_seg_scale_copy(double *v, const double *w, const double *h, SegLayout L,
                                 const int *act) {
  long long start;
  int len;
  L.range(blockIdx.y, blockIdx.z, start, len);
  const double hv = h[blockIdx.y];
  const bool on = (!act || act[blockIdx.y]) && hv != 0.0;
  const double r = on ? 1.0 / hv : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x)
    v[start + i] = on ? w[start + i] * r : 0.0;
}

// x[system s] += sum_{k<nk} y[k*G + s] * Z[k*ld + :]
__global__ void k_seg_multi_axpy(double *x, const double *Z, size_t ld, const double *y, int nk,
                                 SegLayout L) {
  long long start;
  int len;
  L.range(blockIdx.y, blockIdx.z, start, len);
  const int s = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
    double acc = x[start + i];
    for (int k = 0; k < nk; ++k) acc += Z[(size_t)k * ld + start + i] * y[(size_t)k * L.G + s];
    x[start + i] = acc;
  }
}

// stacked <-> system-major native layout (system s at s * ndof_sys,
// [u1 | u2 | u3 | p] within)
__global__ void k_seg_permute(double *stacked, double *native, SegLayout L, int to_stacked) {
  long long start;
  int len;
  const int s = blockIdx.y, r = blockIdx.z;
  L.range(s, r, start, len);
  const long long nd = (long long)s * L.ndof_sys() + L.native_start(r);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
    if (to_stacked)
      stacked[start + i] = native[nd + i];
    else
      native[nd + i] = stacked[start + i];
  }
}

// L^2_0 projection of every system's pressure block (IntoL20Vector3D per
// system: subtract the mean of the constant P1disc modes p[0], p[4], ...);
// one CTA per system, sum in FP64 in a fixed order
template <typename T>
__global__ void __launch_bounds__(kB) k_l20_seg(T *p, int np_sys) {
  T *q = p + (size_t)blockIdx.x * np_sys;
  double s = 0.0;
  for (int i = threadIdx.x * 4; i < np_sys; i += kB * 4) s += (double)q[i];
  s = block_sum256(s);
  __shared__ double mean;
  if (threadIdx.x == 0) mean = s * 4.0 / (double)np_sys;
  __syncthreads();
  const T m = (T)mean;
  for (int i = threadIdx.x * 4; i < np_sys; i += kB * 4) q[i] -= m;
}

// Dense coarse blocks: entry (row, col) of the stacked coarse matrix goes to
// block s = pos[row] / nc at (pos[row] % nc, pos[col] % nc), column-major.
// Same entries as the single-system coarse matrix of SolveExact
// (src/FE/NSE_MGLevel4.C:5728-5830): the nine A blocks (diagonal blocks only
// on Dirichlet rows), BT and B.
__global__ void k_coarse_scatter_seg(DevOp<double> op, const int *pos, int nc, double *blocks) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nu = op.nu, nug = 3 * nu;
  auto put = [&](int row, int col, double v) {
    const int pr = pos[row], pc = pos[col];
    const int s = pr / nc;
    blocks[(size_t)s * nc * nc + (size_t)(pc - s * nc) * nc + (pr - s * nc)] = v;
  };
  if (t < nu) {
    const int i = t;
    const bool act = i < op.nact;
    for (int j = op.a_rowptr[i]; j < op.a_rowptr[i + 1]; ++j) {
      const int c = op.a_col[j];
      for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) {
          if (r != q && (!act || op.structured)) continue;
          const double v = op.structured ? op.a[0][j] : op.a[3 * r + q][j];
          put(i + r * nu, c + q * nu, v);
        }
    }
    if (act)
      for (int j = op.bt_rowptr[i]; j < op.bt_rowptr[i + 1]; ++j)
        for (int r = 0; r < 3; ++r) put(i + r * nu, nug + op.bt_col[j], op.bt[r][j]);
  } else if (t < nu + op.np) {
    const int i = t - nu;
    for (int j = op.b_rowptr[i]; j < op.b_rowptr[i + 1]; ++j)
      for (int q = 0; q < 3; ++q) put(nug + i, op.b_col[j] + q * nu, op.b[q][j]);
  }
}

// replace each system's first pressure equation by p_0 = 0 (:5824-5827)
__global__ void k_coarse_pin_seg(double *blocks, int nc, int row) {
  double *a = blocks + (size_t)blockIdx.y * nc * nc;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x)
    a[(size_t)i * nc + row] = (i == row) ? 1.0 : 0.0;
}

// x = A_s^{-1} b for every system s = blockIdx.y, gathered and scattered
// through sup (local index -> stacked index); b[pin] = 0 (pin >= 0)
template <typename TB, typename TX>
__global__ void k_dense_gemv_seg(const double *__restrict__ inv, int nc, const int *sup,
                                 const TB *__restrict__ b, TX *__restrict__ x, int pin) {
  extern __shared__ double bs[];
  const int s = blockIdx.y;
  const int *m = sup + (size_t)s * nc;
  const double *A = inv + (size_t)s * nc * nc;
  for (int i = threadIdx.x; i < nc; i += blockDim.x) bs[i] = (i == pin) ? 0.0 : (double)b[m[i]];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  double s0 = 0.0, s1 = 0.0;
  int j = 0;
  for (; j + 1 < nc; j += 2) {
    s0 += A[(size_t)j * nc + i] * bs[j];
    s1 += A[(size_t)(j + 1) * nc + i] * bs[j + 1];
  }
  if (j < nc) s0 += A[(size_t)j * nc + i] * bs[j];
  x[m[i]] = (TX)(s0 + s1);
}

inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

// blocks per range so that all ranges of all systems give ~4 waves of 152 SMs
inline int seg_grid_x(const SegLayout &L) {
  const long long longest = L.na > L.np ? L.na : L.np;
  long long want = (4LL * 152 + (long long)L.G * kSegRanges - 1) / ((long long)L.G * kSegRanges);
  const long long cap = (longest + kB - 1) / kB;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  return (int)want;
}

}  // namespace

int seg_partials_size(const SegLayout &L) { return L.G * kSegRanges * seg_grid_x(L); }

int launch_seg_dot(const double *a, const double *b, const SegLayout &L, const int *act,
                   double *partials, double *out, int ostride, bool norm, cudaStream_t s) {
  const int gx = seg_grid_x(L);
  k_seg_dot<<<dim3(gx, L.G, kSegRanges), kB, 0, s>>>(a, b, L, act, partials);
  if (ok() < 0) return -1;
  k_seg_reduce<<<L.G, kB, 0, s>>>(partials, kSegRanges * gx, out, ostride, norm ? 1 : 0);
  return ok() < 0 ? -1 : 2;
}

int launch_seg_mgs(double *w, const double *va, const double *ha, const double *vd,
                   const SegLayout &L, const int *act, double *partials, double *out,
                   cudaStream_t s) {
  const int gx = seg_grid_x(L);
  k_seg_mgs<<<dim3(gx, L.G, kSegRanges), kB, 0, s>>>(w, va, ha, vd, L, act, partials);
  if (ok() < 0) return -1;
  k_seg_reduce<<<L.G, kB, 0, s>>>(partials, kSegRanges * gx, out, 1, vd ? 0 : 1);
  return ok() < 0 ? -1 : 2;
}

int launch_seg_scale(double *v, const SegLayout &L, const double *coef, cudaStream_t s) {
  k_seg_scale<<<dim3(seg_grid_x(L), L.G, kSegRanges), kB, 0, s>>>(v, L, coef);
  return ok() < 0 ? -1 : 1;
}

int launch_seg_scale_copy(double *v, const double *w, const double *h, const SegLayout &L,
                          const int *act, cudaStream_t s) {
  k_seg_scale_copy<<<dim3(seg_grid_x(L), L.G, kSegRanges), kB, 0, s>>>(v, w, h, L, act);
  return ok() < 0 ? -1 : 1;
}

int launch_seg_multi_axpy(double *x, const double *Z, size_t ld, const double *y, int nk,
                          const SegLayout &L, cudaStream_t s) {
  if (nk <= 0) return 0;
  k_seg_multi_axpy<<<dim3(seg_grid_x(L), L.G, kSegRanges), kB, 0, s>>>(x, Z, ld, y, nk, L);
  return ok() < 0 ? -1 : 1;
}

int launch_seg_permute(double *stacked, double *native, const SegLayout &L, bool to_stacked,
                       cudaStream_t s) {
  k_seg_permute<<<dim3(seg_grid_x(L), L.G, kSegRanges), kB, 0, s>>>(stacked, native, L,
                                                                    to_stacked ? 1 : 0);
  return ok() < 0 ? -1 : 1;
}

template <typename T>
int launch_l20_seg(T *p, int np_sys, int nsys, cudaStream_t s) {
  k_l20_seg<T><<<nsys, kB, 0, s>>>(p, np_sys);
  return ok() < 0 ? -1 : 1;
}
template int launch_l20_seg<float>(float *, int, int, cudaStream_t);
template int launch_l20_seg<double>(double *, int, int, cudaStream_t);

int launch_coarse_assemble_seg(const DevOp<double> &op, const int *pos, int nc, int nsys,
                               double *blocks, int project_pressure, cudaStream_t s) {
  if (cudaMemsetAsync(blocks, 0, sizeof(double) * (size_t)nsys * nc * nc, s) != cudaSuccess)
    return -1;
  const int rows = op.nu + op.np;
  k_coarse_scatter_seg<<<(rows + 127) / 128, 128, 0, s>>>(op, pos, nc, blocks);
  if (ok() < 0) return -1;
  if (project_pressure) {
    // the first pressure DOF of a system's native numbering: 3 * (nu / nsys)
    k_coarse_pin_seg<<<dim3((nc + 255) / 256, nsys), 256, 0, s>>>(blocks, nc, 3 * (op.nu / nsys));
    return ok() < 0 ? -1 : 2;
  }
  return 1;
}

template <typename TB, typename TX>
int launch_dense_gemv_seg(const double *inv, int nc, int nsys, const int *sup, const TB *b, TX *x,
                          int pin, cudaStream_t s) {
  const size_t sm = sizeof(double) * nc;
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_dense_gemv_seg<TB, TX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
  k_dense_gemv_seg<TB, TX><<<dim3((nc + 127) / 128, nsys), 128, sm, s>>>(inv, nc, sup, b, x, pin);
  return ok() < 0 ? -1 : 1;
}
template int launch_dense_gemv_seg<double, double>(const double *, int, int, const int *,
                                                   const double *, double *, int, cudaStream_t);
template int launch_dense_gemv_seg<float, float>(const double *, int, int, const int *,
                                                 const float *, float *, int, cudaStream_t);

}  // namespace pm
