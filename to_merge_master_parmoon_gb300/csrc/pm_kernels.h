// pm_kernels.h — host-callable launchers of the sm_103a kernels of libpmgpu.
// Every launcher enqueues on the given stream and returns the number of
// kernels it launched (for the launch counter), or -1 on a launch error.
#ifndef PM_KERNELS_H
#define PM_KERNELS_H

#include <cuda_runtime.h>
#include <stdint.h>

namespace pm {

constexpr int NU_LOC = 27;                 // Q2 local velocity nodes
constexpr int NP_LOC = 4;                  // P1disc local pressure DOFs
constexpr int NLOC = 3 * NU_LOC + NP_LOC;  // 85: local Vanka block size
constexpr int kRStride = 88;               // per-cell stride of the residual buffer
// per-cell stride (values) of the stored 85x85 factors: 7225 rounded up so
// every cell's block starts on a 16-byte boundary in FP32 and FP64 (bulk copies)
constexpr int kFacStride = 7228;
constexpr int NU_TET = 15;  // P2 + face and cell bubbles on tetrahedra (local block 49)
// local sizes of a cell with NU velocity nodes: block, factor and residual strides
template <int NU>
struct Elem {
  static constexpr int nloc = 3 * NU + NP_LOC;
  static constexpr int fac_stride = (nloc * nloc + 3) / 4 * 4;  // 7228 (85), 2404 (49)
  static constexpr int r_stride = (nloc + 7) / 8 * 8;           // 88 (85), 56 (49)
};
inline int elem_nloc(int nl) { return 3 * nl + NP_LOC; }
inline int elem_fac_stride(int nl) {
  return nl == NU_TET ? Elem<NU_TET>::fac_stride : Elem<NU_LOC>::fac_stride;
}
inline int elem_r_stride(int nl) {
  return nl == NU_TET ? Elem<NU_TET>::r_stride : Elem<NU_LOC>::r_stride;
}

// One level's operator in precision T (device pointers).  The nine velocity
// blocks share the CSR pattern; off-diagonal blocks are zero on Dirichlet rows
// (the reference ignores them there, src/FE/MGComponents3D.C:3143-3162).
template <typename T>
struct DevOp {
  int nu, np, nact;
  // 1: A12..A32 are zero and A11 = A22 = A33 (checked exactly at set-up);
  // only a[0] is read
  int structured;
  // 1 (nine-block levels only): the off-diagonal blocks A12..A32 are all
  // zero and the diagonal blocks differ (checked on the device after every
  // upload); the sweeps read only ad[0..2] = A11, A22, A33.  (A nine-block
  // level whose diagonal blocks are also identical runs with structured = 1.)
  int diag;
  const int *a_rowptr, *a_col;
  const T *a[9];
  const T *ad[3];
  const int *b_rowptr, *b_col;
  const T *b[3];
  const int *bt_rowptr, *bt_col;
  const T *bt[3];
};

// Scalar CSR (transfer operators).
template <typename T>
struct DevCsr {
  int rows, cols;
  const int *rowptr, *col;
  const T *val;
};

// Local-block data of one level for the Vanka kernels.
struct DevCells {
  int ncells;
  const int *udofs;   // ncells x nl
  const int *pdofs;   // ncells x 4
  int nl = NU_LOC;    // velocity nodes per cell: 27 (Q2 hexahedra) or 15 (P2+bubble tetrahedra)
};

// ---------------------------------------------------------------- sparse ---
// r = b - K x (defect = true) or y = K x; optionally zero non-active velocity
// rows (TNSE_MGLevel4::Defect).
template <typename T>
int launch_coupled(const DevOp<T> &op, const T *x, const T *b, T *r, bool defect,
                   bool zero_nonactive, cudaStream_t s);
// y_c = M x_c for ncomp components stored with strides (x_stride, y_stride);
// beta_accumulate: y += M x instead of y = M x.
template <typename T>
int launch_csr_apply(const DevCsr<T> &m, int ncomp, const T *x, int x_stride, T *y, int y_stride,
                     cudaStream_t s);

// ---------------------------------------------------------------- vectors ---
// Deterministic sums: partial sums per block, reduced in fixed order by the
// last block to finish (no waiting).  `counter` must be zero on entry and is
// reset to zero by the last block.
template <typename T>
int launch_l20_project(T *p, int np, double *scratch, unsigned int *counter, cudaStream_t s);
int launch_dot(const double *a, const double *b, int n, double *partials, unsigned int *counter,
               double *result, cudaStream_t s);
// w -= h[k_axpy]*v_axpy (if v_axpy), then result = <w, v_dot> (if v_dot) or
// <w, w> (if v_dot == nullptr and norm == true).
int launch_mgs_step(double *w, const double *v_axpy, const double *h_axpy, const double *v_dot,
                    int n, double *partials, unsigned int *counter, double *result,
                    cudaStream_t s);
// v = w / *h (h read on device)
int launch_scale_copy(double *v, const double *w, const double *h, int n, cudaStream_t s);
int launch_scale(double *v, double alpha, int n, cudaStream_t s);
// x += sum_{k<nk} y[k] * Z[k*ld + :]
int launch_multi_axpy(double *x, const double *Z, size_t ld, const double *y, int nk, int n,
                      cudaStream_t s);
template <typename TD, typename TS>
int launch_convert(TD *dst, const TS *src, int n, cudaStream_t s);
template <typename T>
int launch_fill(T *x, T v, int n, cudaStream_t s);
template <typename T>
int launch_axpy(T *y, T a, const T *x, int n, cudaStream_t s);
// u[c*nu + hb + i] = src ? src[c*nu + hb + i] : 0 for the Dirichlet block of
// the three velocity components.
template <typename T>
int launch_dirichlet(T *u, const T *src, int nu, int hb, int ndir, cudaStream_t s);
// zero velocity rows >= nact of the three components
template <typename T>
int launch_zero_nonactive(T *v, int nu, int nact, cudaStream_t s);
// u = uold + alpha (u - uold)
template <typename T>
int launch_relax(T *u, const T *uold, T alpha, int n, cudaStream_t s);
// FP32 velocity u[c*nu + d] (c = 0..2) <-> its interleaved copy ux[d] (pad 0)
int launch_pack_velocity(const float *u, float4 *ux, int nu, cudaStream_t s);
int launch_unpack_velocity(const float4 *ux, float *u, int nu, cudaStream_t s);
// zero off-diagonal velocity blocks on rows >= nact
int launch_zero_dirichlet_offdiag(double *const a[9], const int *rowptr, int nu, int nact,
                                  cudaStream_t s);
// d64 = src (host memory read by the SMs), d32 = (float)src if d32; entries
// from zero_from on are zero.  Needs cudaDevAttrPageableMemoryAccess.
int launch_host_upload(const double *src, double *d64, float *d32, long long n,
                       long long zero_from, int num_sms, cudaStream_t s);
// non-finite check: flag[0] |= 1 if any entry is not finite
int launch_check_finite(const double *x, int n, int *flag, cudaStream_t s);

// ---------------------------------------------------------------- Vanka ----
// Gather every cell's 85x85 block from the FP64 CSR, LU with partial
// pivoting (FP64, or FP32 with factor_fp32), store the factors column-major
// in TF with the reciprocal of U's diagonal on the diagonal, and the row
// permutation as uint8 (row i of PA = row perm[i] of A).
// With inverse (FP32 storage only) the stored block is A^{-1} (column-major),
// computed in FP32 from the stored LU factors by a second kernel; perm is
// still written.
template <typename TF>
int launch_vanka_factor(const DevOp<double> &op, const DevCells &cells, TF *factors,
                        uint8_t *perm, bool factor_fp32, bool inverse, int *status,
                        cudaStream_t s);
// For the ncol cells listed in cell_list: local residual r = f - K u over the
// full rows of the cell's 85 DOFs -> rbuf[slot*kRStride + i].
// variant 0: row groups (8 lanes per row); 1: flattened row stream with
// segmented sums.  Same result up to summation order.
template <typename T>
int launch_vanka_residual(const DevOp<T> &op, const DevCells &cells, const int *cell_list, int ncol,
                          const T *u, const T *rhs, T *rbuf, int variant, cudaStream_t s);
// The same (row groups) on an FP32 one-block hexahedral level with the
// velocity read from its interleaved copy ux (node d: ux[d].x/y/z) and the
// pressure from u; -1 for any other level.
int launch_vanka_residual_aos(const DevOp<float> &op, const DevCells &cells, const int *cell_list,
                              int ncol, const float *u, const float4 *ux, const float *rhs,
                              float *rbuf, cudaStream_t s);
// Local solve with the stored factors and u[dofs] += damp * delta, for the
// same cells (run after launch_vanka_residual of the whole colour).  pairs:
// two cells per warp (half-warp per cell) instead of one.
template <typename T>
int launch_vanka_apply(const DevCells &cells, int nu, const int *cell_list, int ncol,
                       const T *factors, const uint8_t *perm, bool inverse, const T *rbuf,
                       T damp, T *u, bool pairs, cudaStream_t s);

// Error bits of bounded device waits (sweep kernels, `err` arguments)
constexpr int PM_ERR_BULK_TIMEOUT = 1;
// Mixed-precision apply with the FP32 LU factors staged in shared memory by
// bulk copies (two cell buffers per warp, three warps per CTA, at most
// num_sms CTAs walking the colour's cells with a stride).  Same arithmetic
// as launch_vanka_apply.  _init sets the kernel's shared-memory limit (call
// once before any launch, outside stream capture).  wait_limit: polls of
// each wait for a cell's factors before the kernel gives up (0: default).
int launch_vanka_apply_tma_init();
int launch_vanka_apply_tma(const DevCells &cells, int nu, const int *cell_list, int ncol,
                           const float *factors, const uint8_t *perm, const float *rbuf, float damp,
                           float *u, int *err, int num_sms, long long wait_limit, cudaStream_t s);

// Block (Schur-complement) local solve of levels without velocity coupling,
// NB = 1 (one-block operators: one A for the three components) or NB = 3
// (nine-block levels whose A12..A32 are zero: A11, A22, A33).  Per cell:
// the NB inverses A_b^{-1} (27x27, column-major, one after the other), D
// (4x3x27), W = A^{-1} G (4x3x27) and S^{-1} (4x4, column-major), padded to
// a 16-byte multiple of the storage precision.
template <int NB>
struct Schur {
  static constexpr int offD = NB * NU_LOC * NU_LOC;           // 729 / 2187
  static constexpr int offW = offD + NP_LOC * 3 * NU_LOC;     // 1053 / 2511
  static constexpr int offS = offW + NP_LOC * 3 * NU_LOC;     // 1377 / 2835
  static constexpr int values = offS + NP_LOC * NP_LOC;       // 1393 / 2851
  static constexpr int stride = (values + 3) / 4 * 4;         // 1396 / 2852
};
constexpr int kSchurOffD = Schur<1>::offD;
constexpr int kSchurOffW = Schur<1>::offW;
constexpr int kSchurOffS = Schur<1>::offS;
constexpr int kSchurValues = Schur<1>::values;
constexpr int kSchurStride = Schur<1>::stride;
// fp32: eliminate in FP32 (TF = float only; option factor_fp32), else FP64
template <typename TF>
int launch_schur_factor(const DevOp<double> &op, const DevCells &cells, TF *factors, int *status,
                        bool fp32, cudaStream_t s);
template <typename T>
int launch_schur_apply(const DevCells &cells, int nu, const int *cell_list, int ncol,
                       const T *factors, const T *rbuf, T damp, T *u, cudaStream_t s);
// FP32 one-block apply updating the interleaved velocity ux and the pressure in u
int launch_schur_apply_aos(const DevCells &cells, int nu, const int *cell_list, int ncol,
                           const float *factors, const float *rbuf, float damp, float *u,
                           float4 *ux, cudaStream_t s);
// the same for NB = 3 (op.diag levels)
template <typename TF>
int launch_schur3_factor(const DevOp<double> &op, const DevCells &cells, TF *factors, int *status,
                         bool fp32, cudaStream_t s);
template <typename T>
int launch_schur3_apply(const DevCells &cells, int nu, const int *cell_list, int ncol,
                        const T *factors, const T *rbuf, T damp, T *u, cudaStream_t s);
// Block structure of a nine-block level (n entries per block): flag[0] |= 1
// if any entry of the off-diagonal blocks a[1], a[2], a[3], a[5], a[6], a[7]
// is nonzero, |= 2 if the diagonal blocks a[0], a[4], a[8] differ anywhere
int launch_block_structure(const DevOp<double> &op, long long n, int *flag, cudaStream_t s);

// --------------------------------------------------------------- assembly --
// Writable view of a level's FP64 values for device assembly: NSTYPE 4 fills
// a[0], a[4], a[8] and zeroes the other blocks; a one-block level has a[0]
// only (a[1..8] null).
struct AsmOp {
  int nu, np, nact, a_nnz, b_nnz, bt_nnz;
  const int *a_rowptr, *a_col, *b_rowptr, *b_col, *bt_rowptr, *bt_col;
  double *a[9];
  double *b[3], *bt[3];
  // system values c_mass * M + c_a * A in a[], b_scale * B, bt_scale * BT;
  // the Oseen block A and the mass matrix M also into Aonly / Monly if given
  double c_mass, c_a, b_scale, bt_scale;
  double *Aonly, *Monly;
};
// out = c_old * old_rhs + c_new * rhs + (M - c2 A) sol on the active velocity
// rows of the three components (one block for all three), rhs on the
// Dirichlet rows, zero pressure rows (TSystemTNSE3D::AssembleSystMat's
// working right-hand side).
int launch_system_rhs(const AsmOp &op, const double *old_rhs, const double *rhs,
                      const double *sol, double c_old, double c_new, double c2, double *out,
                      cudaStream_t s);
// coarse[c * nc + i] = fine[c * nf + map[i]] for the three velocity components
int launch_interpolate_coarse(const int *map, int nc, int nf, const double *fine, double *coarse,
                              cudaStream_t s);
// reference tables into the current device's constant / global memory
int assemble_tables_init();
// Galerkin Oseen (and mass) blocks of one level (pm_assemble.cu): zero the values, then
// colour by colour one CTA per cell; cell_h = (hx, hy, hz) per cell, conv =
// [b1|b2|b3] at the velocity nodes.  Returns the number of kernels launched.
int launch_assemble_level(const AsmOp &op, const DevCells &cells, const int *colour_cells,
                          const int *colour_ptr, int ncolours, const double *cell_h,
                          const double *conv, double nu, cudaStream_t s);

// ----------------------------------------------------------------- coarse --
// Dense column-major N x N coarse saddle matrix of SolveExact
// (src/FE/NSE_MGLevel4.C:5728-5830) from the FP64 CSR.
int launch_coarse_assemble(const DevOp<double> &op, double *dense, int project_pressure,
                           cudaStream_t s);
// In-place LU with partial pivoting (one CTA), ipiv as in dgetrf.
int launch_dense_lu(double *a, int n, int *ipiv, int *status, cudaStream_t s);
// x = A^{-1} b with the factors (one CTA); b[first_p] = 0 when project.
int launch_dense_solve(const double *lu, const int *ipiv, int n, const double *b, double *x,
                       int pin_row, cudaStream_t s);
// A^{-1} (column-major) from the LU factors, one CTA per column.
int launch_dense_inverse(const double *lu, const int *ipiv, int n, double *inv, cudaStream_t s);
// x = A^{-1} b in FP64 arithmetic (b[pin_row] = 0 when pin_row >= 0).
template <typename TB, typename TX>
int launch_dense_gemv(const double *inv, int n, const TB *b, TX *x, int pin_row, cudaStream_t s);

// ------------------------------------------------------- stacked systems ---
// G systems of one mesh stacked into one level (pm_batch.cu): velocity
// component c holds the G systems' na active DOFs (system s at c*G*nu +
// s*na), then their nu - na Dirichlet DOFs (at c*G*nu + G*na + s*(nu-na));
// the pressure block holds the systems' np DOFs one after the other (at
// 3*G*nu + s*np).  nu, na, np are per system.  Seven ranges per system:
// r = 2c (active part of component c), 2c+1 (its Dirichlet part), 6 (pressure).
struct SegLayout {
  int G = 1, nu = 0, na = 0, np = 0;
  __host__ __device__ int ndof_sys() const { return 3 * nu + np; }
  __host__ __device__ void range(int s, int r, long long &start, int &len) const {
    const long long NU = (long long)G * nu;
    if (r < 6) {
      const int c = r >> 1;
      if ((r & 1) == 0) {
        start = c * NU + (long long)s * na;
        len = na;
      } else {
        start = c * NU + (long long)G * na + (long long)s * (nu - na);
        len = nu - na;
      }
    } else {
      start = 3 * NU + (long long)s * np;
      len = np;
    }
  }
  // first native index ([u1 | u2 | u3 | p] of one system) of range r
  __host__ __device__ int native_start(int r) const {
    return r < 6 ? (r >> 1) * nu + ((r & 1) ? na : 0) : 3 * nu;
  }
  // stacked index of native index l of system s
  __host__ __device__ long long stacked(int s, int l) const {
    long long start;
    int len;
    int r = 6;
    if (l < 3 * nu) r = 2 * (l / nu) + ((l % nu) >= na ? 1 : 0);
    range(s, r, start, len);
    return start + (l - native_start(r));
  }
};
// partial-sum slots the segment reductions need
int seg_partials_size(const SegLayout &L);
// out[s*ostride] = <a, b> over system s (b == null: <a, a>; sqrt with norm);
// systems with act[s] == 0 give 0 (act may be null: all active)
int launch_seg_dot(const double *a, const double *b, const SegLayout &L, const int *act,
                   double *partials, double *out, int ostride, bool norm, cudaStream_t s);
// per system: w -= ha[s] * va (va != null), out[s] = <w, vd> (vd != null) or ||w||
int launch_seg_mgs(double *w, const double *va, const double *ha, const double *vd,
                   const SegLayout &L, const int *act, double *partials, double *out,
                   cudaStream_t s);
// v[system s] *= coef[s] (coef on the device)
int launch_seg_scale(double *v, const SegLayout &L, const double *coef, cudaStream_t s);
// v = w / h[s] where system s is active and h[s] != 0, else v = 0
int launch_seg_scale_copy(double *v, const double *w, const double *h, const SegLayout &L,
                          const int *act, cudaStream_t s);
// x[system s] += sum_{k<nk} y[k*G + s] * Z[k*ld + :]
int launch_seg_multi_axpy(double *x, const double *Z, size_t ld, const double *y, int nk,
                          const SegLayout &L, cudaStream_t s);
// stacked vector <-> G native vectors one after the other
int launch_seg_permute(double *stacked, double *native, const SegLayout &L, bool to_stacked,
                       cudaStream_t s);
// L^2_0 projection of each of nsys consecutive pressure blocks of np_sys
template <typename T>
int launch_l20_seg(T *p, int np_sys, int nsys, cudaStream_t s);
// one dense nc x nc coarse block per system (column-major, one after the
// other) from a stacked coarse level; pos[i] = s*nc + native index of
// stacked DOF i; each system's first pressure row pinned when projecting
int launch_coarse_assemble_seg(const DevOp<double> &op, const int *pos, int nc, int nsys,
                               double *blocks, int project_pressure, cudaStream_t s);
// x = A_s^{-1} b per system through sup[s*nc + l] = stacked index of native l
template <typename TB, typename TX>
int launch_dense_gemv_seg(const double *inv, int nc, int nsys, const int *sup, const TB *b, TX *x,
                          int pin, cudaStream_t s);

}  // namespace pm

#endif
