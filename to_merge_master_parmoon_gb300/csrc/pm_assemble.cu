// pm_assemble.cu — Oseen matrix assembly of one level on the device.
//
// The reference assembles the Galerkin Oseen blocks of NSTYPE 4 cell by cell
// on the host (NSType4Galerkin3D, src/FE/NSE3D_FixPo.C:1919-2071, called
// from TAssembleMat3D::Assemble3D, src/System/AssembleMat3D.C:230) with the
// gradient form nu (grad u, grad v) + ((b . grad) u, v) on the three diagonal
// velocity blocks and -(p, div v) / -(q, div u) in B and BT; with Q2 velocity,
// P1disc pressure and the 4-point Gauss rule per direction (64 points).  A
// time-dependent run re-assembles these for every new convection field.
//
// Here one CTA of 256 threads assembles one cell of a colour and adds into
// the level's CSR values in place; cells of one colour share no DOF, so the
// additions need no atomics and the order of the sums is fixed.  The
// quadrature sums use the tensor-product structure of the Q2 basis and the
// Gauss rule (sum factorisation): b(q) from the nodal values and the
// convection integrals contract one direction at a time, 1.9e4 FMA per cell
// instead of 5.7e4 for the plain 64-point sums.  Cells are
// axis-aligned boxes (the Jacobian is diag(hx, hy, hz) / 2), as in the
// uniform and stretched box meshes of the workloads.  Per cell:
//   diffusion  nu * detJ * sum_d s_d^2 Kref_d           (reference tables)
//   convection detJ * sum_q w_q phi_i(q) (b(q) . grad phi_j(q)),
//              b(q) = sum_m b_m phi_m(q) from the nodal convection b_m
//   B_d[m][j]  = -detJ * s_d * Bref_d[m][j]             (= BT_d[j][m])
// with s_d = 2 / h_d and detJ = hx hy hz / 8.  Dirichlet rows get 1 on the
// diagonal of A11, A22, A33 and nothing else.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#include "pm_kernels.h"

namespace pm {

namespace {

constexpr int kNq = 64;          // 4 x 4 x 4 Gauss points, q = qa + 4 qb + 16 qc
constexpr int kAsmThreads = 256;
// padded row strides (odd) of the per-basis-function shared arrays: the
// threads of a warp take consecutive j
constexpr int kGS = 65, kT1S = 49, kT2S = 37;

// reference tables on the unit cube [-1, 1]^3, local Q2 order a + 3b + 9c.
// Global memory read through L1 (the threads of a warp read different
// entries, which constant memory would serialise).
__device__ double g_Kref[3][NU_LOC][NU_LOC];   // sum_q w dphi_i,d dphi_j,d
__device__ double g_Bref[3][NP_LOC][NU_LOC];   // sum_q w psi_m dphi_j,d
__device__ double g_Mref[NU_LOC][NU_LOC];      // sum_q w phi_i phi_j
__device__ double g_dphi[kNq][NU_LOC][3];      // grad phi_j(q) on the unit cube
__device__ double g_l1[4][3];                  // 1D quadratic Lagrange l_a(x_q)
__device__ double g_wl1[4][3];                 // w_q l_a(x_q)

struct HostTables {
  double M[NU_LOC][NU_LOC];
  double K[3][NU_LOC][NU_LOC];
  double B[3][NP_LOC][NU_LOC];
  double phi[kNq][NU_LOC];
  double dphi[kNq][NU_LOC][3];
  double l1[4][3], wl1[4][3];
};

void lagrange2(double t, double *v, double *d) {
  v[0] = 0.5 * t * (t - 1.0);
  v[1] = 1.0 - t * t;
  v[2] = 0.5 * t * (t + 1.0);
  d[0] = t - 0.5;
  d[1] = -2.0 * t;
  d[2] = t + 0.5;
}

void make_tables(HostTables &T) {
  // Gauss-Legendre, 4 points on [-1, 1]
  const double gp[4] = {-0.86113631159405257522, -0.33998104358485626480,
                        0.33998104358485626480, 0.86113631159405257522};
  const double gw[4] = {0.34785484513745385737, 0.65214515486254614263,
                        0.65214515486254614263, 0.34785484513745385737};
  std::memset(&T, 0, sizeof(T));
  for (int q = 0; q < 4; ++q) {
    double v[3], d[3];
    lagrange2(gp[q], v, d);
    for (int a = 0; a < 3; ++a) {
      T.l1[q][a] = v[a];
      T.wl1[q][a] = gw[q] * v[a];
    }
  }
  for (int qc = 0; qc < 4; ++qc)
    for (int qb = 0; qb < 4; ++qb)
      for (int qa = 0; qa < 4; ++qa) {
        const int q = qa + 4 * qb + 16 * qc;
        const double w = gw[qa] * gw[qb] * gw[qc];
        double vx[3], vy[3], vz[3], dx[3], dy[3], dz[3];
        lagrange2(gp[qa], vx, dx);
        lagrange2(gp[qb], vy, dy);
        lagrange2(gp[qc], vz, dz);
        const double psi[4] = {1.0, gp[qa], gp[qb], gp[qc]};
        for (int c = 0; c < 3; ++c)
          for (int b = 0; b < 3; ++b)
            for (int a = 0; a < 3; ++a) {
              const int i = a + 3 * b + 9 * c;
              T.phi[q][i] = vx[a] * vy[b] * vz[c];
              T.dphi[q][i][0] = dx[a] * vy[b] * vz[c];
              T.dphi[q][i][1] = vx[a] * dy[b] * vz[c];
              T.dphi[q][i][2] = vx[a] * vy[b] * dz[c];
            }
        for (int i = 0; i < NU_LOC; ++i)
          for (int j = 0; j < NU_LOC; ++j) T.M[i][j] += w * T.phi[q][i] * T.phi[q][j];
        for (int d = 0; d < 3; ++d) {
          for (int i = 0; i < NU_LOC; ++i)
            for (int j = 0; j < NU_LOC; ++j) T.K[d][i][j] += w * T.dphi[q][i][d] * T.dphi[q][j][d];
          for (int m = 0; m < NP_LOC; ++m)
            for (int j = 0; j < NU_LOC; ++j) T.B[d][m][j] += w * psi[m] * T.dphi[q][j][d];
        }
      }
}

// position of column key in the sorted row [lo, hi), or -1 if absent (a
// pattern that lacks a coupling of the cell: the entry is left out)
__device__ __forceinline__ int find_pos(const int *cols, int lo, int hi, int key) {
  const int end = hi;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (cols[mid] < key) lo = mid + 1; else hi = mid;
  }
  return (lo < end && cols[lo] == key) ? lo : -1;
}

__global__ void __launch_bounds__(kAsmThreads) k_assemble_cells(
    AsmOp op, DevCells cells, const int *__restrict__ list, int ncol,
    const double *__restrict__ cell_h, const double *__restrict__ conv, double nu) {
  __shared__ int ud[NU_LOC], pd[NP_LOC];
  __shared__ double l1[4][3], wl1[4][3];
  __shared__ double bl[3][NU_LOC];        // nodal convection of the cell [d][m]
  __shared__ double S1[3][9][4];          // [d][ia + 3 ib][qc]
  __shared__ double S2[3][3][16];         // [d][ia][qb + 4 qc]
  __shared__ double bq[3][kNq];           // convection at the Gauss points
  __shared__ double G[NU_LOC * kGS];      // [j][16 qa + qb + 4 qc]: b(q) . grad phi_j(q)
  __shared__ double T1[NU_LOC * kT1S];    // [j][16 ia + qb + 4 qc]: qa contracted
  __shared__ double T2[NU_LOC * kT2S];    // [j][4 (ia + 3 ib) + qc]: qb contracted
  const int slot = blockIdx.x, tid = threadIdx.x;
  if (slot >= ncol) return;  // whole block
  const int cell = list[slot];
  const int nu_ = op.nu;
  if (tid < NU_LOC) ud[tid] = cells.udofs[(size_t)cell * NU_LOC + tid];
  if (tid < NP_LOC) pd[tid] = cells.pdofs[(size_t)cell * NP_LOC + tid];
  if (tid < 12) {
    l1[tid / 3][tid % 3] = g_l1[tid / 3][tid % 3];
    wl1[tid / 3][tid % 3] = g_wl1[tid / 3][tid % 3];
  }
  const double hx = cell_h[(size_t)cell * 3], hy = cell_h[(size_t)cell * 3 + 1],
               hz = cell_h[(size_t)cell * 3 + 2];
  const double s0 = 2.0 / hx, s1 = 2.0 / hy, s2 = 2.0 / hz;
  const double detJ = hx * hy * hz * 0.125;
  __syncthreads();
  for (int t = tid; t < 3 * NU_LOC; t += kAsmThreads) {
    const int d = t / NU_LOC, m = t - NU_LOC * d;
    bl[d][m] = conv[(size_t)d * nu_ + ud[m]];
  }
  __syncthreads();
  // b(q) = sum_m b_m phi_m(q), one direction at a time: c, b, a
  for (int t = tid; t < 3 * 9 * 4; t += kAsmThreads) {
    const int qc = t & 3, ab = (t >> 2) % 9, d = t / 36;
    S1[d][ab][qc] = bl[d][ab] * l1[qc][0] + bl[d][ab + 9] * l1[qc][1] + bl[d][ab + 18] * l1[qc][2];
  }
  __syncthreads();
  for (int t = tid; t < 3 * 3 * 16; t += kAsmThreads) {
    const int r = t & 15, ia = (t >> 4) % 3, d = t / 48;
    const int qb = r & 3, qc = r >> 2;
    S2[d][ia][r] = S1[d][ia][qc] * l1[qb][0] + S1[d][ia + 3][qc] * l1[qb][1] +
                   S1[d][ia + 6][qc] * l1[qb][2];
  }
  __syncthreads();
  for (int t = tid; t < 3 * kNq; t += kAsmThreads) {
    const int q = t & 63, d = t >> 6;
    const int qa = q & 3, r = q >> 2;
    bq[d][q] = S2[d][0][r] * l1[qa][0] + S2[d][1][r] * l1[qa][1] + S2[d][2][r] * l1[qa][2];
  }
  __syncthreads();
  for (int t = tid; t < kNq * NU_LOC; t += kAsmThreads) {
    const int q = t / NU_LOC, j = t - NU_LOC * q;
    const int qa = q & 3, r = q >> 2;
    G[j * kGS + 16 * qa + r] = s0 * bq[0][q] * g_dphi[q][j][0] + s1 * bq[1][q] * g_dphi[q][j][1] +
                               s2 * bq[2][q] * g_dphi[q][j][2];
  }
  __syncthreads();
  // conv_ij = sum_q w_q phi_i(q) G_j(q): contract qa, then qb, then qc
  for (int t = tid; t < 48 * NU_LOC; t += kAsmThreads) {
    const int u = t / NU_LOC, j = t - NU_LOC * u;
    const int ia = u % 3, r = u / 3;
    const double *g = &G[j * kGS + r];
    T1[j * kT1S + 16 * ia + r] =
        wl1[0][ia] * g[0] + wl1[1][ia] * g[16] + wl1[2][ia] * g[32] + wl1[3][ia] * g[48];
  }
  __syncthreads();
  for (int t = tid; t < 36 * NU_LOC; t += kAsmThreads) {
    const int u = t / NU_LOC, j = t - NU_LOC * u;
    const int qc = u & 3, ab = u >> 2;
    const int ia = ab % 3, ib = ab / 3;
    const double *g = &T1[j * kT1S + 16 * ia + 4 * qc];
    T2[j * kT2S + 4 * ab + qc] =
        wl1[0][ib] * g[0] + wl1[1][ib] * g[1] + wl1[2][ib] * g[2] + wl1[3][ib] * g[3];
  }
  __syncthreads();
  const double k0 = nu * detJ * s0 * s0, k1 = nu * detJ * s1 * s1, k2 = nu * detJ * s2 * s2;
  // A entries (active rows only), j fastest over the threads
  for (int t = tid; t < NU_LOC * NU_LOC; t += kAsmThreads) {
    const int i = t / NU_LOC, j = t - NU_LOC * i;
    const int r = ud[i];
    if (r >= op.nact) continue;
    const int ab = i % 9, ic = i / 9;
    const double *g = &T2[j * kT2S + 4 * ab];
    const double conv_ij =
        wl1[0][ic] * g[0] + wl1[1][ic] * g[1] + wl1[2][ic] * g[2] + wl1[3][ic] * g[3];
    const double va = k0 * g_Kref[0][i][j] + k1 * g_Kref[1][i][j] + k2 * g_Kref[2][i][j] +
                      detJ * conv_ij;
    const double vm = detJ * g_Mref[i][j];
    const double v = op.c_mass * vm + op.c_a * va;
    const int pos = find_pos(op.a_col, op.a_rowptr[r], op.a_rowptr[r + 1], ud[j]);
    if (pos < 0) continue;
    op.a[0][pos] += v;
    if (op.a[4]) op.a[4][pos] += v;
    if (op.a[8]) op.a[8][pos] += v;
    if (op.Aonly) op.Aonly[pos] += va;
    if (op.Monly) op.Monly[pos] += vm;
  }
  // B rows of the cell's pressure DOFs and BT entries of its active velocity rows
  const double s[3] = {s0, s1, s2};
  for (int t = tid; t < NP_LOC * NU_LOC; t += kAsmThreads) {
    const int m = t / NU_LOC, j = t - NU_LOC * m;
    double v[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] = -detJ * s[d] * g_Bref[d][m][j];
    const int p = pd[m];
    const int bpos = find_pos(op.b_col, op.b_rowptr[p], op.b_rowptr[p + 1], ud[j]);
    if (bpos >= 0) {
#pragma unroll
      for (int d = 0; d < 3; ++d) op.b[d][bpos] += op.b_scale * v[d];
    }
    const int r = ud[j];
    if (r < op.nact) {
      const int tpos = find_pos(op.bt_col, op.bt_rowptr[r], op.bt_rowptr[r + 1], p);
      if (tpos >= 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) op.bt[d][tpos] += op.bt_scale * v[d];
      }
    }
  }
}

__global__ void k_assemble_dirichlet(AsmOp op) {
  const int r = op.nact + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= op.nu) return;
  const int pos = find_pos(op.a_col, op.a_rowptr[r], op.a_rowptr[r + 1], r);
  if (pos < 0) return;
  op.a[0][pos] = 1.0;
  if (op.a[4]) op.a[4][pos] = 1.0;
  if (op.a[8]) op.a[8][pos] = 1.0;
}

// one warp per velocity row: the working right-hand side of the theta scheme
__global__ void k_system_rhs(AsmOp op, const double *__restrict__ old_rhs,
                             const double *__restrict__ rhs, const double *__restrict__ sol,
                             double c_old, double c_new, double c2, double *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nu = op.nu;
  if (row >= nu) return;  // whole warp
  const int i = (int)row;
  if (i >= op.nact) {
    if (lane < 3) out[(size_t)lane * nu + i] = rhs[(size_t)lane * nu + i];
    return;
  }
  double acc[3] = {0.0, 0.0, 0.0};
  for (int e = op.a_rowptr[i] + lane; e < op.a_rowptr[i + 1]; e += 32) {
    const int j = op.a_col[e];
    const double m = op.Monly[e] - c2 * op.Aonly[e];
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[c] += m * sol[(size_t)c * nu + j];
  }
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  if (lane < 3) {
    const size_t k = (size_t)lane * nu + i;
    out[k] = c_old * old_rhs[k] + c_new * rhs[k] + acc[lane];
  }
}

__global__ void k_zero_pressure(double *p, int np) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < np) p[k] = 0.0;
}

inline int ok() { return cudaPeekAtLastError() == cudaSuccess ? 1 : -1; }

}  // namespace

int assemble_tables_init() {
  static HostTables T;
  static bool made = false;
  if (!made) {
    make_tables(T);
    made = true;
  }
  if (cudaMemcpyToSymbol(g_Kref, T.K, sizeof(T.K)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_Bref, T.B, sizeof(T.B)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_Mref, T.M, sizeof(T.M)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_dphi, T.dphi, sizeof(T.dphi)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_l1, T.l1, sizeof(T.l1)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_wl1, T.wl1, sizeof(T.wl1)) != cudaSuccess)
    return -1;
  return 0;
}

int launch_assemble_level(const AsmOp &op, const DevCells &cells, const int *colour_cells,
                          const int *colour_ptr, int ncolours, const double *cell_h,
                          const double *conv, double nu, cudaStream_t s) {
  int n = 0;
  for (int k = 0; k < 9; ++k)
    if (op.a[k] &&
        cudaMemsetAsync(op.a[k], 0, sizeof(double) * (size_t)op.a_nnz, s) != cudaSuccess)
      return -1;
  for (double *q : {op.Aonly, op.Monly})
    if (q && cudaMemsetAsync(q, 0, sizeof(double) * (size_t)op.a_nnz, s) != cudaSuccess)
      return -1;
  for (int k = 0; k < 3; ++k)
    if (cudaMemsetAsync(op.b[k], 0, sizeof(double) * (size_t)op.b_nnz, s) != cudaSuccess ||
        cudaMemsetAsync(op.bt[k], 0, sizeof(double) * (size_t)op.bt_nnz, s) != cudaSuccess)
      return -1;
  for (int k = 0; k < ncolours; ++k) {
    const int b = colour_ptr[k], m = colour_ptr[k + 1] - b;
    if (m <= 0) continue;
    k_assemble_cells<<<m, kAsmThreads, 0, s>>>(op, cells, colour_cells + b, m, cell_h, conv, nu);
    if (ok() < 0) return -1;
    ++n;
  }
  if (op.nu > op.nact) {
    k_assemble_dirichlet<<<(op.nu - op.nact + 255) / 256, 256, 0, s>>>(op);
    if (ok() < 0) return -1;
    ++n;
  }
  return n;
}

int launch_system_rhs(const AsmOp &op, const double *old_rhs, const double *rhs,
                      const double *sol, double c_old, double c_new, double c2, double *out,
                      cudaStream_t s) {
  if (!op.Aonly || !op.Monly) return -1;
  const long long threads = (long long)op.nu * 32;
  k_system_rhs<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(op, old_rhs, rhs, sol, c_old,
                                                                 c_new, c2, out);
  if (ok() < 0) return -1;
  k_zero_pressure<<<(op.np + 255) / 256, 256, 0, s>>>(out + (size_t)3 * op.nu, op.np);
  return ok() < 0 ? -1 : 2;
}

}  // namespace pm
