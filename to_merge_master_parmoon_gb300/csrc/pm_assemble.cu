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
// convection integrals use the tensor-product structure: with b the Q2
// interpolant (b_m at the nodes),
//   int phi_i (b_x d_x phi_j) = sum_m b_m,x X1(a,am,aj) Y0(b,bm,bj) Y0(c,cm,cj)
// with the 1D integrals Y0 = int l l l and X1 = int l l l' over [-1, 1]
// (likewise for y and z), which the 4-point Gauss rule integrates exactly, as
// it does the 3D integrand; the sum over m contracts one direction at a time
// (7.3e3 FMA per cell instead of 5.7e4 for the plain 64-point sums; the y and
// z terms share their x factor Y0 and are summed before the last step).
// Diffusion and mass are Kronecker products of the 1D matrices
// D1 = int l' l' and M1 = int l l, e.g. M = M1 (x) M1 (x) M1, combined per
// cell in the y-z factors so that an entry costs two FMA.  Cells are
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

// reference tables on the unit cube [-1, 1]^3, local Q2 order a + 3b + 9c.
// Global memory read through L1 (the threads of a warp read different
// entries, which constant memory would serialise).
__device__ double g_Bref[3][NP_LOC][NU_LOC];   // sum_q w psi_m dphi_j,d
__device__ double g_tri[2][3][3][3];           // [0]: int l_a l_m l_j, [1]: int l_a l_m l_j'
__device__ double g_dm[2][3][3];               // [0]: int l_a' l_j', [1]: int l_a l_j

struct HostTables {
  double B[3][NP_LOC][NU_LOC];
  double dphi[kNq][NU_LOC][3];
  double tri[2][3][3][3];
  double dm[2][3][3];
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
    for (int a = 0; a < 3; ++a)
      for (int m = 0; m < 3; ++m)
        for (int j = 0; j < 3; ++j) {
          T.tri[0][a][m][j] += gw[q] * v[a] * v[m] * v[j];
          T.tri[1][a][m][j] += gw[q] * v[a] * v[m] * d[j];
        }
    for (int a = 0; a < 3; ++a)
      for (int j = 0; j < 3; ++j) {
        T.dm[0][a][j] += gw[q] * d[a] * d[j];
        T.dm[1][a][j] += gw[q] * v[a] * v[j];
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
              T.dphi[q][i][0] = dx[a] * vy[b] * vz[c];
              T.dphi[q][i][1] = vx[a] * dy[b] * vz[c];
              T.dphi[q][i][2] = vx[a] * vy[b] * dz[c];
            }
        for (int d = 0; d < 3; ++d)
          for (int m = 0; m < NP_LOC; ++m)
            for (int j = 0; j < NU_LOC; ++j) T.B[d][m][j] += w * psi[m] * T.dphi[q][j][d];
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

// SYS: the system c_mass M + c_a A, with A and M also stored (Aonly, Monly);
// otherwise the Oseen block A alone
template <bool SYS>
__global__ void __launch_bounds__(kAsmThreads) k_assemble_cells(
    AsmOp op, DevCells cells, const int *__restrict__ list, int ncol,
    const double *__restrict__ cell_h, const double *__restrict__ conv, double nu) {
  __shared__ int ud[NU_LOC], pd[NP_LOC];
  __shared__ double F[2][27];             // 1D triple-product integrals [Y0 | X1][a][m][j]
  __shared__ double DM[2][9];             // 1D [D1 | M1][a][j]
  __shared__ double sb[3][NU_LOC];        // detJ s_d b_m,d: scaled nodal convection
  __shared__ double W1[3][9][9];          // [d][am + 3 bm][3 c + cj]: cm contracted
  __shared__ double W2x[3][81];           // [am][w], w = 9 (3 b + bj) + 3 c + cj: d = x
  __shared__ double W2yz[3][81];          // the same, d = y and z summed
  __shared__ double Pyz[81], Qyz[81], Myz[81];  // diffusion and mass y-z factors
  __shared__ double cs[4];                // s0, s1, s2, detJ
  const int slot = blockIdx.x, tid = threadIdx.x;
  if (slot >= ncol) return;  // whole block
  const int cell = list[slot];
  const int nu_ = op.nu;
  if (tid < NU_LOC) ud[tid] = cells.udofs[(size_t)cell * NU_LOC + tid];
  if (tid < NP_LOC) pd[tid] = cells.pdofs[(size_t)cell * NP_LOC + tid];
  if (tid < 54) F[tid / 27][tid % 27] = (&g_tri[0][0][0][0])[tid];
  if (tid >= 64 && tid < 82) DM[(tid - 64) / 9][(tid - 64) % 9] = (&g_dm[0][0][0])[tid - 64];
  // s_d = 2 / h_d and detJ = hx hy hz / 8, once per cell (an FP64 division
  // is a sequence of FMA: not on every thread)
  if (tid < 3) cs[tid] = 2.0 / cell_h[(size_t)cell * 3 + tid];
  if (tid == 3)
    cs[3] = cell_h[(size_t)cell * 3] * cell_h[(size_t)cell * 3 + 1] *
            cell_h[(size_t)cell * 3 + 2] * 0.125;
  __syncthreads();
  const double s0 = cs[0], s1 = cs[1], s2 = cs[2], detJ = cs[3];
  for (int t = tid; t < 3 * NU_LOC; t += kAsmThreads) {
    const int d = t / NU_LOC, m = t - NU_LOC * d;
    sb[d][m] = detJ * cs[d] * conv[(size_t)d * nu_ + ud[m]];
  }
  if (tid >= 128 && tid < 128 + 81) {
    const int w = tid - 128;
    const int bbj = w / 9, ccj = w - 9 * bbj;
    const double mb = DM[1][bbj], mc = DM[1][ccj], db = DM[0][bbj], dc = DM[0][ccj];
    const double nd = nu * detJ;
    Pyz[w] = nd * s0 * s0 * mb * mc;
    Qyz[w] = nd * (s1 * s1 * db * mc + s2 * s2 * mb * dc);
    Myz[w] = detJ * mb * mc;
  }
  __syncthreads();
  // direction z (cm): the derivative factor X1 for d = 2, else Y0
  for (int t = tid; t < 3 * 81; t += kAsmThreads) {
    const int d = t / 81, u = t - 81 * d;
    const int ab = u / 9, ccj = u - 9 * ab;
    const double *f = &F[d == 2][(ccj / 3) * 9 + (ccj % 3)];  // [c][cm][cj], stride 3 in cm
    W1[d][ab][ccj] = sb[d][ab] * f[0] + sb[d][ab + 9] * f[3] + sb[d][ab + 18] * f[6];
  }
  __syncthreads();
  // direction y (bm): X1 for d = 1, else Y0; d = y and z summed
  for (int t = tid; t < 3 * 81; t += kAsmThreads) {
    const int am = t / 81, w = t - 81 * am;
    const int bbj = w / 9, ccj = w - 9 * bbj;
    const int fo = (bbj / 3) * 9 + (bbj % 3);  // [b][bm][bj]
    const double *y0 = &F[0][fo], *x1 = &F[1][fo];
    W2x[am][w] = W1[0][am][ccj] * y0[0] + W1[0][am + 3][ccj] * y0[3] + W1[0][am + 6][ccj] * y0[6];
    W2yz[am][w] = W1[1][am][ccj] * x1[0] + W1[1][am + 3][ccj] * x1[3] +
                  W1[1][am + 6][ccj] * x1[6] + W1[2][am][ccj] * y0[0] +
                  W1[2][am + 3][ccj] * y0[3] + W1[2][am + 6][ccj] * y0[6];
  }
  __syncthreads();
  // A entries (active rows only), j fastest over the threads: direction x (am)
  for (int t = tid; t < NU_LOC * NU_LOC; t += kAsmThreads) {
    const int i = t / NU_LOC, j = t - NU_LOC * i;
    const int r = ud[i];
    if (r >= op.nact) continue;
    const int ia = i % 3, ib = (i / 3) % 3, ic = i / 9;
    const int ja = j % 3, jb = (j / 3) % 3, jc = j / 9;
    const int w = 9 * (3 * ib + jb) + 3 * ic + jc;
    const int fo = ia * 9 + ja;  // [a][am][aj]
    const double va = F[1][fo] * W2x[0][w] + F[1][fo + 3] * W2x[1][w] + F[1][fo + 6] * W2x[2][w] +
                      F[0][fo] * W2yz[0][w] + F[0][fo + 3] * W2yz[1][w] +
                      F[0][fo + 6] * W2yz[2][w] + DM[0][3 * ia + ja] * Pyz[w] +
                      DM[1][3 * ia + ja] * Qyz[w];
    const int pos = find_pos(op.a_col, op.a_rowptr[r], op.a_rowptr[r + 1], ud[j]);
    if (pos < 0) continue;
    double v = va;
    if (SYS) {
      const double vm = DM[1][3 * ia + ja] * Myz[w];
      v = op.c_mass * vm + op.c_a * va;
      op.Aonly[pos] += va;
      op.Monly[pos] += vm;
    }
    op.a[0][pos] += v;
    if (op.a[4]) op.a[4][pos] += v;
    if (op.a[8]) op.a[8][pos] += v;
  }
  // B rows of the cell's pressure DOFs and BT entries of its active velocity rows
  const double nb[3] = {-detJ * s0, -detJ * s1, -detJ * s2};
  for (int t = tid; t < NP_LOC * NU_LOC; t += kAsmThreads) {
    const int m = t / NU_LOC, j = t - NU_LOC * m;
    double v[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] = nb[d] * g_Bref[d][m][j];
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

__global__ void k_interpolate_coarse(const int *__restrict__ map, int nc, int nf,
                                     const double *__restrict__ fine,
                                     double *__restrict__ coarse) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const int f = map[i];
#pragma unroll
  for (int c = 0; c < 3; ++c) coarse[(size_t)c * nc + i] = fine[(size_t)c * nf + f];
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
  if (cudaMemcpyToSymbol(g_Bref, T.B, sizeof(T.B)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_tri, T.tri, sizeof(T.tri)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_dm, T.dm, sizeof(T.dm)) != cudaSuccess)
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
    if (op.Aonly && op.Monly)
      k_assemble_cells<true><<<m, kAsmThreads, 0, s>>>(op, cells, colour_cells + b, m, cell_h,
                                                       conv, nu);
    else
      k_assemble_cells<false><<<m, kAsmThreads, 0, s>>>(op, cells, colour_cells + b, m, cell_h,
                                                        conv, nu);
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

int launch_interpolate_coarse(const int *map, int nc, int nf, const double *fine, double *coarse,
                              cudaStream_t s) {
  if (nc <= 0) return 0;
  k_interpolate_coarse<<<(nc + 255) / 256, 256, 0, s>>>(map, nc, nf, fine, coarse);
  return ok() < 0 ? -1 : 1;
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
