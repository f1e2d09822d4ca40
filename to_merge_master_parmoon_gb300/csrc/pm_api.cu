// pm_api.cu — host side of libpmgpu: the C ABI declared in include/pmgpu.h.
//
// Orchestrates, on one CUDA stream, the reference's solver path:
//   TFgmresIte::Iterate (flexible, src/FE/FgmresIte.C:250-677)
//     -> TMultiGridIte::Iterate (src/FE/MultiGridIte.C:76-132)
//        -> TNSE_MultiGrid::Cycle, V-cycle (src/FE/NSE_MultiGrid.C:434-1779)
//           -> TNSE_MGLevel4 Defect / CorrectNodes / CellVanka / SolveExact
// with every numerical step on the GPU.  The V-cycle is captured once into a
// CUDA graph and replayed for every preconditioner application.  FGMRES keeps
// its vectors, Arnoldi and Gram-Schmidt on the device; only the (restart+2)
// Hessenberg entries of the current column travel to the host, where the
// Givens rotations run exactly as in the reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "pm_kernels.h"
#include "pm_learned.h"
#include "pm_setup_host.h"
#include "pmgpu.h"

struct pm_mlp {
  pm::Mlp m;
};

using namespace pm;

namespace {
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

namespace {

struct CsrStore {
  int rows = 0, cols = 0, nnz = 0;
  int *rowptr = nullptr, *col = nullptr;
  double *v64 = nullptr;
  float *v32 = nullptr;
  template <typename T>
  DevCsr<T> view() const;
};
template <>
DevCsr<double> CsrStore::view<double>() const {
  return DevCsr<double>{rows, cols, rowptr, col, v64};
}
template <>
DevCsr<float> CsrStore::view<float>() const {
  return DevCsr<float>{rows, cols, rowptr, col, v32};
}

struct LevelDev {
  int nu = 0, np = 0, ndof = 0, nact = 0, hb = 0, ndir = 0, ncells = 0;
  int a_nnz = 0, b_nnz = 0, bt_nnz = 0;
  int structured = 0;  // one-block descriptor (NSTYPE 2: a[0] only)
  // decoupled nine-block level (A12..A32 all zero): 1 with distinct diagonal
  // blocks (three A arrays read, block solve with three inverses), 2 with
  // A11 = A22 = A33 (one array read, the one-block operator's solve)
  int diag = 0;
  int res_variant = 0;    // local-residual kernel of the sweep (0 row groups, 1 stream)
  int apply_variant = 0;  // LU apply: 0 two cells per warp, 1 bulk-staged (FP32), 2 one cell per warp
  std::vector<int> h_udofs, h_pdofs, h_parent, h_child, h_colour;
  int nl = NU_LOC;                // velocity nodes per cell (27 Q2, 15 P2+bubble tetrahedra)
  HostCsr h_pu, h_pp;             // handed-over prolongation from the next coarser level
  bool has_colour = false;
  int *a_rowptr = nullptr, *a_col = nullptr, *b_rowptr = nullptr, *b_col = nullptr;
  int *bt_rowptr = nullptr, *bt_col = nullptr;
  double *a64[9] = {}, *b64[3] = {}, *bt64[3] = {};
  float *a32[9] = {}, *b32[3] = {}, *bt32[3] = {};
  int *udofs = nullptr, *pdofs = nullptr;
  Colouring colouring;
  int *colour_cells = nullptr;
  void *factors = nullptr;
  uint8_t *perm = nullptr;
  CsrStore Pu, Ru, Pp, Rp;
  void *sol = nullptr, *rhs = nullptr, *def = nullptr, *uold = nullptr, *dbuf = nullptr;
  // interleaved FP32 velocity (16 bytes per node) that the one-block sweep
  // gathers from and updates; mixed precision, hexahedral smoothed levels
  float4 *ux = nullptr;
  double *x64 = nullptr, *y64 = nullptr, *z64 = nullptr;
  // unique bytes of one Vanka sweep per cell, split by kernel (see pm_setup)
  double vanka_res_bytes = 0.0, vanka_apply_bytes = 0.0;
  // learned smoother buffers (allocated on first attach / harvest)
  bool l_ready = false;
  int *l_nbr = nullptr;
  float *l_inv_mult = nullptr, *l_summary = nullptr, *l_Y = nullptr, *l_scale = nullptr;
  __nv_bfloat16 *l_X = nullptr, *l_H1 = nullptr, *l_H2 = nullptr;
  void *l_corr = nullptr, *l_q = nullptr, *l_zero = nullptr;  // V-cycle precision
  double *l_omega = nullptr;                                   // step length (device)
  // device assembly inputs (allocated on first pm_assemble_level)
  double *asm_h = nullptr, *asm_conv = nullptr;
  double *asm_A = nullptr, *asm_M = nullptr;  // Oseen block and mass matrix (system assembly)
  bool asm_theta = false;  // asm_A / asm_M hold the last system assembly
  int *coarse_nodes = nullptr;  // velocity DOF of this level at each node of level-1

  template <typename T>
  DevOp<T> op() const;
  DevCells cells() const { return DevCells{ncells, udofs, pdofs, nl}; }
  // one A block for the three components: a one-block descriptor, or a
  // decoupled nine-block level with A11 = A22 = A33
  bool one_block() const { return structured || diag == 2; }
  // the Schur block solve of one-block levels exists for Q2 hexahedra only
  bool schur() const { return one_block() && nl == NU_LOC; }
  // block elimination with three diagonal blocks (decoupled nine-block levels)
  bool schur3() const { return diag == 1 && nl == NU_LOC; }
  size_t fac_bytes = 0;  // allocated factor storage
  uint64_t pattern_key = 0;  // fingerprint of the CSR patterns (pattern_fingerprint)
  // stacked level of G systems (pm_add_level_batch): per-system layout and
  // cells; the colour lists of all systems, kept while a solve sweeps only
  // the systems still iterating
  SegLayout seg;
  int ncells_sys = 0;
  std::vector<int> colour_full_ptr, colour_full_order;
};
template <>
DevOp<double> LevelDev::op<double>() const {
  DevOp<double> o;
  o.nu = nu;
  o.structured = structured || diag == 2;
  o.diag = diag == 1;
  o.np = np;
  o.nact = nact;
  o.a_rowptr = a_rowptr;
  o.a_col = a_col;
  for (int k = 0; k < 9; ++k) o.a[k] = a64[k];
  for (int k = 0; k < 3; ++k) o.ad[k] = a64[4 * k];
  o.b_rowptr = b_rowptr;
  o.b_col = b_col;
  o.bt_rowptr = bt_rowptr;
  o.bt_col = bt_col;
  for (int k = 0; k < 3; ++k) {
    o.b[k] = b64[k];
    o.bt[k] = bt64[k];
  }
  return o;
}
template <>
DevOp<float> LevelDev::op<float>() const {
  DevOp<float> o;
  o.nu = nu;
  o.structured = structured || diag == 2;
  o.diag = diag == 1;
  o.np = np;
  o.nact = nact;
  o.a_rowptr = a_rowptr;
  o.a_col = a_col;
  for (int k = 0; k < 9; ++k) o.a[k] = a32[k];
  for (int k = 0; k < 3; ++k) o.ad[k] = a32[4 * k];
  o.b_rowptr = b_rowptr;
  o.b_col = b_col;
  o.bt_rowptr = bt_rowptr;
  o.bt_col = bt_col;
  for (int k = 0; k < 3; ++k) {
    o.b[k] = b32[k];
    o.bt[k] = bt32[k];
  }
  return o;
}

}  // namespace

struct pm_handle {
  pm_options opt;
  double t_update0 = 0.0;  // host clock at pm_update_matrices entry (verbose timing)
  cudaStream_t stream = nullptr;
  std::vector<LevelDev> L;
  bool setup_done = false;
  std::string err;
  long long launches = 0;
  long long bytes = 0;
  std::vector<void *> allocs;
  // reductions and scalars
  double *partials = nullptr;
  unsigned int *counter = nullptr;
  double *hcol = nullptr;
  double *ydev = nullptr;
  int *status_d = nullptr;
  int *sweep_err = nullptr;  // device flags of bounded waits inside sweep kernels
  int *diag_flags = nullptr; // per level: an off-diagonal velocity block is nonzero
  bool asm_tables = false;   // assembly reference tables on the device
  int num_sms = 0;
  // coarse direct solve
  int coarse_n = 0;
  double *coarse_lu = nullptr, *coarse_inv = nullptr, *coarse_b = nullptr, *coarse_x = nullptr;
  int *coarse_ipiv = nullptr;
  // FGMRES storage
  int restart = 0;
  double *V = nullptr, *Z = nullptr, *w = nullptr, *xd = nullptr, *bd = nullptr;
  // V-cycle graphs: [0] plain, [1] with the learned step
  cudaGraphExec_t vgraph_g[2] = {nullptr, nullptr};
  long long vgraph_kernels_g[2] = {0, 0};
  bool l_active = false;  // the cycle being run / captured includes the learned step
  // profiling of the Vanka solve kernel
  bool prof = false;
  std::vector<cudaEvent_t> evpool;
  size_t evused = 0;
  std::vector<double> prof_bytes;
  // [0] = k_vanka_residual, [1] = k_vanka_apply
  double prof_ms[2] = {0.0, 0.0}, prof_sum_bytes[2] = {0.0, 0.0};
  long long prof_launches[2] = {0, 0};
  double last_factor_ms = 0.0;
  std::vector<void *> pinned;
  long long pinned_bytes = 0;
  // learned smoother (borrowed network), device on/off flag read by its kernels
  pm::Mlp *mlp = nullptr;
  double l_omega = 1.0, l_fallback = 0.5;
  int *d_on = nullptr;
  int l_on_host = 0;
  int l_fallbacks = 0;
  // stacked systems (pm_add_level_batch / pm_solve_fused): system count,
  // per-system flags (1 = still iterating), per-system scale factors, the
  // native-layout staging vector, the coarse maps (stacked index -> s * nc +
  // native index, and back) and whether the sweeps currently skip systems
  int nsys = 1;
  bool adding_stacked = false;
  int *d_act = nullptr;
  double *d_coef = nullptr, *stage = nullptr;
  int *coarse_pos = nullptr, *coarse_sup = nullptr;
  bool colours_restricted = false;
};

namespace {

pm_status fail(pm_handle *h, pm_status s, const std::string &msg) {
  if (h) h->err = msg;
  return s;
}

pm_status cuda_fail(pm_handle *h, const char *what) {
  cudaError_t e = cudaGetLastError();
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  if (h) h->err = m;
  return (e == cudaErrorMemoryAllocation) ? PM_OOM : PM_CUDA_ERROR;
}

template <typename T>
pm_status dalloc(pm_handle *h, T **p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  if (h->opt.max_device_bytes > 0 &&
      h->bytes + (long long)(count * sizeof(T)) > h->opt.max_device_bytes) {
    h->err = "device allocation of " + std::to_string(count * sizeof(T)) +
             " bytes exceeds max_device_bytes (" + std::to_string(h->opt.max_device_bytes) +
             ", " + std::to_string(h->bytes) + " held)";
    return PM_OOM;
  }
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, count * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    h->err = "cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes failed: " +
             cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? PM_OOM : PM_CUDA_ERROR;
  }
  h->allocs.push_back(q);
  h->bytes += (long long)(count * sizeof(T));
  *p = static_cast<T *>(q);
  return PM_OK;
}

// CSR value / column arrays: padded by 8 zero entries so that the Vanka
// residual kernel's aligned 4-entry vector loads never leave the allocation.
constexpr size_t kCsrPad = 8;
template <typename T>
pm_status dalloc_padded(pm_handle *h, T **p, size_t count) {
  pm_status s = dalloc(h, p, count + kCsrPad);
  if (s != PM_OK) return s;
  if (cudaMemsetAsync(*p, 0, (count + kCsrPad) * sizeof(T), h->stream) != cudaSuccess)
    return cuda_fail(h, "padded alloc");
  return PM_OK;
}

template <typename T>
pm_status upload_padded(pm_handle *h, T **dst, const T *src, size_t count) {
  pm_status s = dalloc_padded(h, dst, count);
  if (s != PM_OK) return s;
  if (count && cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice, h->stream) !=
                   cudaSuccess)
    return cuda_fail(h, "upload");
  return PM_OK;
}

template <typename T>
pm_status upload(pm_handle *h, T **dst, const T *src, size_t count) {
  pm_status s = dalloc(h, dst, count);
  if (s != PM_OK) return s;
  if (count && cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice, h->stream) !=
                   cudaSuccess)
    return cuda_fail(h, "upload");
  return PM_OK;
}

#define PM_TRY(expr)                  \
  do {                                \
    pm_status _s = (expr);            \
    if (_s != PM_OK) return _s;       \
  } while (0)

#define PM_LAUNCH(expr)                                      \
  do {                                                       \
    int _n = (expr);                                         \
    if (_n < 0) return cuda_fail(h, #expr);                  \
    h->launches += _n;                                       \
  } while (0)

// entry points of one system: not for a handle of stacked systems
#define PM_SINGLE(h)                                                              \
  do {                                                                            \
    if ((h) && (h)->nsys > 1)                                                     \
      return fail((h), PM_BADARG, "not available on a handle of stacked systems"); \
  } while (0)

bool mixed(const pm_handle *h) { return h->opt.precision == PM_PREC_MIXED; }
// mixed mode stores each local block's FP32 inverse unless told otherwise
bool use_inverse(const pm_handle *h) { return mixed(h) && h->opt.vanka_inverse != 0; }

pm_status sync(pm_handle *h, const char *what) {
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return cuda_fail(h, what);
  if (h->sweep_err) {  // bounded device waits that gave up (bulk-copy barriers)
    int e = 0;
    if (cudaMemcpy(&e, h->sweep_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      return cuda_fail(h, what);
    if (e) {
      cudaMemset(h->sweep_err, 0, sizeof(int));
      return fail(h, PM_TIMEOUT, std::string(what) + ": a bulk copy into shared memory did not "
                                 "complete within the wait limit (sweep result invalid)");
    }
  }
  return PM_OK;
}

// ------------------------------------------------------------ level ops ---
template <typename T>
pm_status l20(pm_handle *h, T *p, int np) {
  if (!h->opt.project_pressure) return PM_OK;
  if (h->nsys > 1)  // stacked systems: each system's pressure block separately
    PM_LAUNCH(launch_l20_seg<T>(p, np / h->nsys, h->nsys, h->stream));
  else
    PM_LAUNCH(launch_l20_project<T>(p, np, h->partials, h->counter, h->stream));
  return PM_OK;
}

// TNSE_MGLevel4::Defect: CoupledDefect, L2_0 of the pressure part, zero
// non-active velocity rows.
template <typename T>
pm_status level_defect(pm_handle *h, const LevelDev &Lv, const T *u, const T *f, T *d) {
  PM_LAUNCH(launch_coupled<T>(Lv.op<T>(), u, f, d, true, true, h->stream));
  return l20<T>(h, d + 3 * Lv.nu, Lv.np);
}

template <typename T>
pm_status vanka_sweep(pm_handle *h, LevelDev &Lv, T *u, const T *rhs) {
  const T damp = (T)h->opt.smooth_damp;
  const bool relax = std::fabs(1.0 - h->opt.alpha) > 1e-3;
  PM_LAUNCH(launch_dirichlet<T>(u, rhs, Lv.nu, Lv.hb, Lv.ndir, h->stream));
  if (relax &&
      cudaMemcpyAsync(Lv.uold, u, sizeof(T) * Lv.ndof, cudaMemcpyDeviceToDevice, h->stream) !=
          cudaSuccess)
    return cuda_fail(h, "uold copy");
  const DevOp<T> op = Lv.op<T>();
  const DevCells cells = Lv.cells();
  const int ncol = (int)Lv.colouring.ptr.size() - 1;
  // FP32 one-block levels: the sweep gathers the velocity from its
  // interleaved copy (one 16-byte load per matrix entry instead of three
  // 4-byte loads, the residual being bound by the L1 wavefronts of its
  // gathers) and the apply updates that copy; packed before the colours,
  // unpacked after them
  const bool aos = sizeof(T) == sizeof(float) && Lv.ux && Lv.schur() && Lv.res_variant == 0;
  float *uf = reinterpret_cast<float *>(u);
  if (aos) PM_LAUNCH(launch_pack_velocity(uf, Lv.ux, Lv.nu, h->stream));
  for (int k = 0; k < ncol; ++k) {
    const int b = Lv.colouring.ptr[k], n = Lv.colouring.ptr[k + 1] - b;
    if (n == 0) continue;
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    if (h->prof && h->evused + 3 <= h->evpool.size()) {
      e0 = h->evpool[h->evused];
      e1 = h->evpool[h->evused + 1];
      e2 = h->evpool[h->evused + 2];
      h->evused += 3;
      cudaEventRecord(e0, h->stream);
    }
    if (aos)
      PM_LAUNCH(launch_vanka_residual_aos(Lv.op<float>(), cells, Lv.colour_cells + b, n, uf,
                                          Lv.ux, reinterpret_cast<const float *>(rhs),
                                          static_cast<float *>(Lv.dbuf), h->stream));
    else
      PM_LAUNCH(launch_vanka_residual<T>(op, cells, Lv.colour_cells + b, n, u, rhs,
                                         static_cast<T *>(Lv.dbuf), Lv.res_variant, h->stream));
    if (e1) cudaEventRecord(e1, h->stream);
    if (aos)
      PM_LAUNCH(launch_schur_apply_aos(cells, Lv.nu, Lv.colour_cells + b, n,
                                       static_cast<const float *>(Lv.factors),
                                       static_cast<const float *>(Lv.dbuf), (float)damp, uf,
                                       Lv.ux, h->stream));
    else if (Lv.schur())
      PM_LAUNCH(launch_schur_apply<T>(cells, Lv.nu, Lv.colour_cells + b, n,
                                      static_cast<const T *>(Lv.factors),
                                      static_cast<const T *>(Lv.dbuf), damp, u, h->stream));
    else if (Lv.schur3())
      PM_LAUNCH(launch_schur3_apply<T>(cells, Lv.nu, Lv.colour_cells + b, n,
                                       static_cast<const T *>(Lv.factors),
                                       static_cast<const T *>(Lv.dbuf), damp, u, h->stream));
    else if (sizeof(T) == sizeof(float) && !use_inverse(h) && Lv.apply_variant == 1 &&
             Lv.nl == NU_LOC)
      PM_LAUNCH(launch_vanka_apply_tma(cells, Lv.nu, Lv.colour_cells + b, n,
                                       static_cast<const float *>(Lv.factors), Lv.perm,
                                       reinterpret_cast<const float *>(Lv.dbuf), (float)damp,
                                       reinterpret_cast<float *>(u), h->sweep_err, h->num_sms,
                                       h->opt.wait_limit, h->stream));
    else
      PM_LAUNCH(launch_vanka_apply<T>(cells, Lv.nu, Lv.colour_cells + b, n,
                                      static_cast<const T *>(Lv.factors), Lv.perm, use_inverse(h),
                                      static_cast<const T *>(Lv.dbuf), damp, u,
                                      Lv.apply_variant == 0, h->stream));
    if (e2) {
      cudaEventRecord(e2, h->stream);
      // algorithmic bytes of this colour: the level's unique Vanka-sweep
      // bytes per cell (split into the residual part and the factor part)
      // times the cells of this colour
      h->prof_bytes.push_back(Lv.vanka_res_bytes * n);
      h->prof_bytes.push_back(Lv.vanka_apply_bytes * n);
    }
  }
  if (aos) PM_LAUNCH(launch_unpack_velocity(Lv.ux, uf, Lv.nu, h->stream));
  if (relax) PM_LAUNCH(launch_relax<T>(u, static_cast<const T *>(Lv.uold), (T)h->opt.alpha, Lv.ndof, h->stream));
  PM_LAUNCH(launch_dirichlet<T>(u, rhs, Lv.nu, Lv.hb, Lv.ndir, h->stream));
  return PM_OK;
}

template <typename T>
pm_status coarse_solve(pm_handle *h, LevelDev &Lv, const T *rhs, T *u) {
  // SolveExact with the inverse of the (pinned) coarse matrix, FP64 arithmetic
  if (h->nsys > 1) {  // one inverse per stacked system, pinned at its first pressure DOF
    const int pin = h->opt.project_pressure ? 3 * Lv.seg.nu : -1;
    PM_LAUNCH((launch_dense_gemv_seg<T, T>(h->coarse_inv, h->coarse_n, h->nsys, h->coarse_sup,
                                           rhs, u, pin, h->stream)));
    return PM_OK;
  }
  const int pin = h->opt.project_pressure ? 3 * Lv.nu : -1;
  PM_LAUNCH((launch_dense_gemv<T, T>(h->coarse_inv, h->coarse_n, rhs, u, pin, h->stream)));
  return PM_OK;
}

// Per-level buffers of the learned step: neighbour slots, inverse node
// multiplicities, cell summaries, BF16 features and activations, outputs.
pm_status ensure_learned_buffers(pm_handle *h, LevelDev &Lv) {
  if (Lv.l_ready || Lv.ncells == 0) return PM_OK;
  std::vector<int> nbr;
  build_neighbours(Lv.ncells, Lv.h_udofs.data(), Lv.nu, nbr);
  std::vector<float> inv;
  node_inverse_multiplicity(Lv.ncells, Lv.h_udofs.data(), Lv.nu, inv);
  PM_TRY(upload(h, &Lv.l_nbr, nbr.data(), nbr.size()));
  PM_TRY(upload(h, &Lv.l_inv_mult, inv.data(), inv.size()));
  const size_t nc = (size_t)Lv.ncells;
  PM_TRY(dalloc(h, &Lv.l_summary, nc * kSummary));
  PM_TRY(dalloc(h, &Lv.l_scale, nc));
  PM_TRY(dalloc(h, &Lv.l_Y, nc * kMlpOutPad));
  PM_TRY(dalloc(h, &Lv.l_X, nc * kMlpInPad));
  PM_TRY(dalloc(h, &Lv.l_H1, nc * kMlpHidden));
  PM_TRY(dalloc(h, &Lv.l_H2, nc * kMlpHidden));
  const size_t es = mixed(h) ? sizeof(float) : sizeof(double);
  PM_TRY(dalloc(h, reinterpret_cast<unsigned char **>(&Lv.l_corr), (size_t)Lv.ndof * es));
  PM_TRY(dalloc(h, reinterpret_cast<unsigned char **>(&Lv.l_q), (size_t)Lv.ndof * es));
  PM_TRY(dalloc(h, reinterpret_cast<unsigned char **>(&Lv.l_zero), (size_t)Lv.ndof * es));
  PM_TRY(dalloc(h, &Lv.l_omega, 1));
  if (cudaMemsetAsync(Lv.l_zero, 0, (size_t)Lv.ndof * es, h->stream) != cudaSuccess)
    return cuda_fail(h, "zero vector");
  PM_TRY(sync(h, "learned buffers"));
  Lv.l_ready = true;
  return PM_OK;
}

// Learned post-smoothing step on one level: d = f - K u, cell features,
// MLP, u += omega * (cell corrections averaged over the cells sharing a DOF)
// colour by colour (no two cells of a colour share a DOF).  All kernels read
// the device flag h->d_on and do nothing when it is 0.
template <typename T>
pm_status learned_step(pm_handle *h, LevelDev &C, T *u, const T *f) {
  T *d = static_cast<T *>(C.def);
  PM_TRY(level_defect<T>(h, C, u, f, d));
  const DevCells cells = C.cells();
  PM_LAUNCH(launch_cell_summary<T>(cells, C.nu, d, C.l_summary, h->d_on, h->stream));
  PM_LAUNCH(launch_cell_features<T>(cells, C.nu, d, C.l_summary, C.l_nbr, C.l_X, nullptr,
                                    C.l_scale, h->d_on, h->stream));
  PM_LAUNCH(mlp_forward(*h->mlp, C.l_X, C.ncells, C.l_H1, C.l_H2, C.l_Y, h->stream, h->d_on,
                        h->sweep_err));
  // correction c = cell predictions averaged over the cells sharing a DOF
  T *c = static_cast<T *>(C.l_corr), *q = static_cast<T *>(C.l_q);
  PM_LAUNCH(launch_fill<T>(c, T(0), C.ndof, h->stream));
  const int ncol = (int)C.colouring.ptr.size() - 1;
  for (int k = 0; k < ncol; ++k) {
    const int b = C.colouring.ptr[k], n = C.colouring.ptr[k + 1] - b;
    PM_LAUNCH(launch_learned_apply<T>(cells, C.nu, C.nact, C.colour_cells + b, n, C.l_Y,
                                      C.l_scale, C.l_inv_mult, T(1), c, h->d_on, h->stream));
  }
  // minimal-residual step length (as TNSE_MGLevel4::StepLengthControl
  // damps a correction, src/FE/NSE_MGLevel4.C:5878): q = P(0 - K c),
  // omega = argmin ||d + omega q|| in [0, omega_max], u += omega c
  PM_TRY(level_defect<T>(h, C, c, static_cast<const T *>(C.l_zero), q));
  PM_LAUNCH(launch_mr_step<T>(d, q, C.ndof, h->partials, h->counter, h->l_omega, C.l_omega,
                              h->d_on, h->stream));
  PM_LAUNCH(launch_axpy_dev<T>(u, C.l_omega, c, C.ndof, h->d_on, h->stream));
  return PM_OK;
}

// TNSE_MultiGrid::Cycle (V-cycle, cell Vanka, coarse SolveExact)
template <typename T>
pm_status cycle(pm_handle *h, int i) {
  LevelDev &C = h->L[i];
  T *u = static_cast<T *>(C.sol), *f = static_cast<T *>(C.rhs);
  // CorrectNodes + SetDirichletNodes
  PM_LAUNCH(launch_dirichlet<T>(u, f, C.nu, C.hb, C.ndir, h->stream));
  if (i == 0) return coarse_solve<T>(h, C, f, u);
  LevelDev &K = h->L[i - 1];
  T *d = static_cast<T *>(C.def);
  T *cu = static_cast<T *>(K.sol), *cf = static_cast<T *>(K.rhs);
  for (int s = 0; s < h->opt.pre_smooth; ++s) PM_TRY(vanka_sweep<T>(h, C, u, f));
  PM_LAUNCH(launch_dirichlet<T>(u, (const T *)nullptr, C.nu, C.hb, C.ndir, h->stream));
  PM_TRY(level_defect<T>(h, C, u, f, d));
  // DefectRestriction (u and p) + CorrectDefect + Reset
  PM_LAUNCH(launch_csr_apply<T>(C.Ru.view<T>(), 3, d, C.nu, cf, K.nu, h->stream));
  PM_LAUNCH(launch_csr_apply<T>(C.Rp.view<T>(), 1, d + 3 * C.nu, C.np, cf + 3 * K.nu, K.np, h->stream));
  PM_LAUNCH(launch_zero_nonactive<T>(cf, K.nu, K.nact, h->stream));
  PM_TRY(l20<T>(h, cf + 3 * K.nu, K.np));
  PM_LAUNCH(launch_fill<T>(cu, T(0), K.ndof, h->stream));
  PM_TRY(cycle<T>(h, i - 1));
  // Prolongate, CorrectNodes(defect), Update, CorrectNodes(u)
  PM_LAUNCH(launch_csr_apply<T>(C.Pu.view<T>(), 3, cu, K.nu, d, C.nu, h->stream));
  PM_LAUNCH(launch_csr_apply<T>(C.Pp.view<T>(), 1, cu + 3 * K.nu, K.np, d + 3 * C.nu, C.np, h->stream));
  PM_LAUNCH(launch_dirichlet<T>(d, (const T *)nullptr, C.nu, C.hb, C.ndir, h->stream));
  PM_LAUNCH(launch_axpy<T>(u, (T)h->opt.beta, d, C.ndof, h->stream));
  PM_LAUNCH(launch_dirichlet<T>(u, (const T *)nullptr, C.nu, C.hb, C.ndir, h->stream));
  for (int s = 0; s < h->opt.post_smooth; ++s) PM_TRY(vanka_sweep<T>(h, C, u, f));
  if (h->l_active &&
      (h->opt.learned_levels <= 0 || i >= (int)h->L.size() - h->opt.learned_levels))
    PM_TRY(learned_step<T>(h, C, u, f));
  return PM_OK;
}

// TMultiGridIte::Iterate body after rhs is in place: zero start,
// SetDirichletNodes, one cycle.
template <typename T>
pm_status vcycle_core(pm_handle *h) {
  LevelDev &F = h->L.back();
  PM_LAUNCH(launch_fill<T>(static_cast<T *>(F.sol), T(0), F.ndof, h->stream));
  PM_LAUNCH(launch_dirichlet<T>(static_cast<T *>(F.sol), static_cast<const T *>(F.rhs), F.nu, F.hb,
                                F.ndir, h->stream));
  return cycle<T>(h, (int)h->L.size() - 1);
}

void drop_graphs(pm_handle *h) {
  for (int k = 0; k < 2; ++k)
    if (h->vgraph_g[k]) {
      cudaGraphExecDestroy(h->vgraph_g[k]);
      h->vgraph_g[k] = nullptr;
    }
}

// One V-cycle; with a network attached and enabled the cycle includes the
// learned post-smoothing step.  The plain and the learned cycle are each
// captured once into their own graph.
pm_status run_vcycle_core(pm_handle *h) {
  h->l_active = h->mlp != nullptr && h->l_on_host != 0;
  const int gi = h->l_active ? 1 : 0;
  if (h->opt.use_graphs && !h->prof) {
    if (!h->vgraph_g[gi]) {
      cudaGraph_t g = nullptr;
      const long long before = h->launches;
      if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return cuda_fail(h, "begin capture");
      pm_status s = mixed(h) ? vcycle_core<float>(h) : vcycle_core<double>(h);
      cudaError_t e = cudaStreamEndCapture(h->stream, &g);
      if (s != PM_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
      }
      if (e != cudaSuccess) return cuda_fail(h, "end capture");
      h->vgraph_kernels_g[gi] = h->launches - before;
      h->launches = before;
      if (cudaGraphInstantiate(&h->vgraph_g[gi], g, 0) != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(h, "graph instantiate");
      }
      cudaGraphDestroy(g);
    }
    if (cudaGraphLaunch(h->vgraph_g[gi], h->stream) != cudaSuccess)
      return cuda_fail(h, "graph launch");
    h->launches += h->vgraph_kernels_g[gi];
    return PM_OK;
  }
  return mixed(h) ? vcycle_core<float>(h) : vcycle_core<double>(h);
}

// z = M v (FP64 in/out)
pm_status precondition(pm_handle *h, double *z, const double *v) {
  LevelDev &F = h->L.back();
  if (mixed(h))
    PM_LAUNCH((launch_convert<float, double>(static_cast<float *>(F.rhs), v, F.ndof, h->stream)));
  else if (cudaMemcpyAsync(F.rhs, v, sizeof(double) * F.ndof, cudaMemcpyDeviceToDevice,
                           h->stream) != cudaSuccess)
    return cuda_fail(h, "rhs copy");
  PM_TRY(run_vcycle_core(h));
  if (mixed(h))
    PM_LAUNCH((launch_convert<double, float>(z, static_cast<const float *>(F.sol), F.ndof, h->stream)));
  else if (cudaMemcpyAsync(z, F.sol, sizeof(double) * F.ndof, cudaMemcpyDeviceToDevice,
                           h->stream) != cudaSuccess)
    return cuda_fail(h, "sol copy");
  return PM_OK;
}

pm_status set_learned_flag(pm_handle *h, int on) {
  h->l_on_host = on;
  static const int kValues[2] = {0, 1};
  if (cudaMemcpyAsync(h->d_on, &kValues[on ? 1 : 0], sizeof(int), cudaMemcpyHostToDevice,
                      h->stream) != cudaSuccess)
    return cuda_fail(h, "learned flag");
  return PM_OK;
}

// Defect_NSE4 on the finest level in FP64
pm_status defect_nse4(pm_handle *h, const double *x, const double *b, double *r) {
  LevelDev &F = h->L.back();
  PM_LAUNCH(launch_coupled<double>(F.op<double>(), x, b, r, true, false, h->stream));
  return l20<double>(h, r + 3 * F.nu, F.np);
}

pm_status read_scalars(pm_handle *h, double *dst, const double *src, int n) {
  if (cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream) !=
      cudaSuccess)
    return cuda_fail(h, "scalar read");
  return sync(h, "scalar read");
}

pm_status norm2(pm_handle *h, const double *x, int n, double *out) {
  PM_LAUNCH(launch_dot(x, x, n, h->partials, h->counter, h->hcol, h->stream));
  PM_TRY(read_scalars(h, out, h->hcol, 1));
  *out = std::sqrt(*out);
  return PM_OK;
}

void gen_rot(double dx, double dy, double *cs, double *sn) {
  if (dy == 0.0) {
    *cs = 1.0;
    *sn = 0.0;
  } else if (std::fabs(dy) > std::fabs(dx)) {
    double t = dx / dy;
    *sn = 1.0 / std::sqrt(1.0 + t * t);
    *cs = t * *sn;
  } else {
    double t = dy / dx;
    *cs = 1.0 / std::sqrt(1.0 + t * t);
    *sn = t * *cs;
  }
}
void apply_rot(double *dx, double *dy, double cs, double sn) {
  double t = cs * *dx + sn * *dy;
  *dy = -sn * *dx + cs * *dy;
  *dx = t;
}

// TFgmresIte::Iterate, flexible branch
pm_status fgmres(pm_handle *h, double *x, const double *b, pm_result *res) {
  LevelDev &F = h->L.back();
  const int N = F.ndof;
  int restart = h->opt.restart;
  const int maxit = h->opt.maxit, minit = h->opt.minit;
  if (restart > maxit) restart = maxit;
  if (restart <= 0) restart = 10;
  if (restart > h->restart) return fail(h, PM_BADARG, "restart larger than allocated");
  const double red = h->opt.red_factor, resmin = h->opt.res_norm_min, divf = h->opt.div_factor;
  std::vector<double> s(restart + 1), cs(restart + 1), sn(restart + 1), y(restart + 1);
  std::vector<double> H((size_t)(restart + 1) * restart, 0.0), col(restart + 2);
  auto hh = [&](int r, int c) -> double & { return H[(size_t)r * restart + c]; };
  double *V = h->V, *Z = h->Z, *w = h->w;
  auto v = [&](int k) { return V + (size_t)k * N; };
  auto z = [&](int k) { return Z + (size_t)k * N; };
  res->vcycles = 0;

  PM_TRY(defect_nse4(h, x, b, v(0)));
  double r0;
  PM_TRY(norm2(h, v(0), N, &r0));
  double resv = r0, res0 = r0, beta = r0;
  res->res0 = r0;
  if (!std::isfinite(r0)) {
    res->res = r0;
    return fail(h, PM_NAN, "non-finite initial residual");
  }
  int maxite = maxit;
  if (beta <= resmin) {
    if (minit == 0 || beta < 1e-20) {
      res->iterations = 0;
      res->res = resv;
      return PM_OK;
    }
    maxite = minit;
  }
  // learned step on at the start of every solve; off for the rest of the
  // solve once an iteration reduces the residual by less than l_fallback
  if (h->mlp) PM_TRY(set_learned_flag(h, 1));
  double prev_res = r0;
  int j = 1;
  while (j <= maxite) {
    PM_LAUNCH(launch_scale(v(0), 1.0 / beta, N, h->stream));
    std::fill(s.begin(), s.end(), 0.0);
    s[0] = beta;
    int i;
    for (i = 0; i < restart && j <= maxite; i++, j++) {
      for (int attempt = 0;; ++attempt) {
        PM_TRY(precondition(h, z(i), v(i)));
        res->vcycles++;
        PM_LAUNCH(launch_coupled<double>(F.op<double>(), z(i), nullptr, w, false, false,
                                         h->stream));
        // modified Gram-Schmidt, each step fused with the next dot product
        PM_LAUNCH(launch_mgs_step(w, nullptr, nullptr, v(0), N, h->partials, h->counter, h->hcol,
                                  h->stream));
        for (int k = 1; k <= i; ++k)
          PM_LAUNCH(launch_mgs_step(w, v(k - 1), h->hcol + (k - 1), v(k), N, h->partials,
                                    h->counter, h->hcol + k, h->stream));
        PM_LAUNCH(launch_mgs_step(w, v(i), h->hcol + i, nullptr, N, h->partials, h->counter,
                                  h->hcol + i + 1, h->stream));
        PM_LAUNCH(launch_scale_copy(v(i + 1), w, h->hcol + i + 1, N, h->stream));
        PM_TRY(read_scalars(h, col.data(), h->hcol, i + 2));
        for (int k = 0; k <= i + 1; ++k) hh(k, i) = col[k];
        for (int k = 0; k <= i + 1; ++k)
          if (!std::isfinite(col[k])) {
            res->iterations = j;
            res->res = col[k];
            return fail(h, PM_NAN, "non-finite Arnoldi coefficient");
          }
        const double s_i = s[i], s_i1 = s[i + 1];
        for (int k = 0; k < i; ++k) apply_rot(&hh(k, i), &hh(k + 1, i), cs[k], sn[k]);
        gen_rot(hh(i, i), hh(i + 1, i), &cs[i], &sn[i]);
        apply_rot(&hh(i, i), &hh(i + 1, i), cs[i], sn[i]);
        apply_rot(&s[i], &s[i + 1], cs[i], sn[i]);
        resv = std::fabs(s[i + 1]);
        if (!(h->mlp && h->l_on_host && prev_res > 0.0 && resv > h->l_fallback * prev_res))
          break;
        // the learned step failed the reduction test: off for the rest of the
        // solve, and this column is computed again with the plain V-cycle, so
        // that the rejected direction never enters the Krylov basis
        PM_TRY(set_learned_flag(h, 0));
        h->l_fallbacks++;
        s[i] = s_i;
        s[i + 1] = s_i1;
      }
      prev_res = resv;
      if (j >= minit && (resv < resmin || resv < red * (h->opt.red_initial ? r0 : res0))) {
        for (int k = 0; k <= i; ++k) y[k] = s[k];
        for (int r = i; r >= 0; --r) {
          y[r] /= hh(r, r);
          for (int q = r - 1; q >= 0; --q) y[q] -= hh(q, r) * y[r];
        }
        if (cudaMemcpyAsync(h->ydev, y.data(), sizeof(double) * (i + 1), cudaMemcpyHostToDevice,
                            h->stream) != cudaSuccess)
          return cuda_fail(h, "y upload");
        PM_LAUNCH(launch_multi_axpy(x, Z, (size_t)N, h->ydev, i + 1, N, h->stream));
        PM_TRY(sync(h, "fgmres final"));
        res->iterations = j;
        res->res = resv;
        return PM_OK;
      }
      if (resv > divf * res0) {
        res->iterations = j;
        res->res = resv;
        return fail(h, PM_DIVERGED, "FGMRES residual exceeded SC_DIV_FACTOR * res0");
      }
    }
    // restart (src/FE/FgmresIte.C:574-590); only the i columns of this cycle
    for (int k = 0; k < i; ++k) y[k] = s[k];
    for (int r = i - 1; r >= 0; --r) {
      y[r] /= hh(r, r);
      for (int q = r - 1; q >= 0; --q) y[q] -= hh(q, r) * y[r];
    }
    if (cudaMemcpyAsync(h->ydev, y.data(), sizeof(double) * i, cudaMemcpyHostToDevice,
                        h->stream) != cudaSuccess)
      return cuda_fail(h, "y upload");
    PM_LAUNCH(launch_multi_axpy(x, Z, (size_t)N, h->ydev, i, N, h->stream));
    PM_TRY(defect_nse4(h, x, b, v(0)));
    PM_TRY(norm2(h, v(0), N, &resv));
    res0 = beta = resv;
    if (!std::isfinite(resv)) return fail(h, PM_NAN, "non-finite residual at restart");
  }
  if (j > maxite) j = maxite;
  res->iterations = j;
  res->res = resv;
  return PM_MAXIT;
}

// ---------------------------------------------------- stacked systems ----
// While a fused solve runs, the Vanka sweeps of systems that have finished
// are dropped from the colour lists (their vectors are zero from then on),
// and the V-cycle graphs are captured again for the shorter lists.
pm_status restrict_colours(pm_handle *h, const std::vector<int> &act) {
  for (size_t l = 1; l < h->L.size(); ++l) {
    LevelDev &Lv = h->L[l];
    if (Lv.colour_full_ptr.empty()) {
      Lv.colour_full_ptr = Lv.colouring.ptr;
      Lv.colour_full_order = Lv.colouring.order;
    }
    const int ncol = (int)Lv.colour_full_ptr.size() - 1;
    std::vector<int> ptr((size_t)ncol + 1, 0);
    Lv.colouring.order.clear();
    for (int k = 0; k < ncol; ++k) {
      for (int q = Lv.colour_full_ptr[k]; q < Lv.colour_full_ptr[k + 1]; ++q) {
        const int c = Lv.colour_full_order[(size_t)q];
        if (act[(size_t)(c / Lv.ncells_sys)]) Lv.colouring.order.push_back(c);
      }
      ptr[(size_t)k + 1] = (int)Lv.colouring.order.size();
    }
    Lv.colouring.ptr = ptr;
    if (!Lv.colouring.order.empty() &&
        cudaMemcpyAsync(Lv.colour_cells, Lv.colouring.order.data(),
                        sizeof(int) * Lv.colouring.order.size(), cudaMemcpyHostToDevice,
                        h->stream) != cudaSuccess)
      return cuda_fail(h, "colour lists");
  }
  drop_graphs(h);
  h->colours_restricted = true;
  return sync(h, "colour lists");
}

pm_status restore_colours(pm_handle *h) {
  if (!h->colours_restricted) return PM_OK;
  for (size_t l = 1; l < h->L.size(); ++l) {
    LevelDev &Lv = h->L[l];
    Lv.colouring.ptr = Lv.colour_full_ptr;
    Lv.colouring.order = Lv.colour_full_order;
    if (cudaMemcpyAsync(Lv.colour_cells, Lv.colouring.order.data(),
                        sizeof(int) * Lv.colouring.order.size(), cudaMemcpyHostToDevice,
                        h->stream) != cudaSuccess)
      return cuda_fail(h, "colour lists");
  }
  drop_graphs(h);
  h->colours_restricted = false;
  return sync(h, "colour lists");
}

// TFgmresIte::Iterate (src/FE/FgmresIte.C:250-677) for G stacked systems in
// lockstep: one Arnoldi process, Hessenberg matrix, Givens sequence and
// stopping test per system, every device step (V-cycle, mat-vec, Gram-
// Schmidt, updates) one launch over all systems.  A system leaves when it
// meets its stopping test (its update is applied then), diverges or hits a
// non-finite value; its vectors are zeroed and its sweeps dropped.  Returns
// per-system results in res[0..G-1].
pm_status fgmres_seg(pm_handle *h, double *x, const double *b, pm_result *res) {
  LevelDev &F = h->L.back();
  const int N = F.ndof, G = h->nsys;
  const SegLayout &SL = F.seg;
  int restart = h->opt.restart;
  const int maxit = h->opt.maxit, minit = h->opt.minit;
  if (restart > maxit) restart = maxit;
  if (restart <= 0) restart = 10;
  if (restart > h->restart) return fail(h, PM_BADARG, "restart larger than allocated");
  const double red = h->opt.red_factor, resmin = h->opt.res_norm_min, divf = h->opt.div_factor;
  const size_t R1 = (size_t)restart + 1;
  std::vector<double> sv(R1 * G), cs(R1 * G), sn(R1 * G), y(R1), yall(R1 * G);
  std::vector<double> H(R1 * restart * G, 0.0), col((R1 + 1) * G);
  auto hh = [&](int s, int r, int c) -> double & {
    return H[((size_t)s * R1 + r) * restart + c];
  };
  double *V = h->V, *Z = h->Z, *w = h->w;
  auto v = [&](int k) { return V + (size_t)k * N; };
  auto z = [&](int k) { return Z + (size_t)k * N; };
  std::vector<int> act((size_t)G, 1);
  std::vector<double> r0((size_t)G), res0((size_t)G), beta((size_t)G), resv((size_t)G);
  std::vector<double> coef((size_t)G);
  for (int s = 0; s < G; ++s) {
    std::memset(&res[s], 0, sizeof(pm_result));
    res[s].status = PM_OK;
  }
  auto upload_act = [&]() -> pm_status {
    if (cudaMemcpyAsync(h->d_act, act.data(), sizeof(int) * G, cudaMemcpyHostToDevice,
                        h->stream) != cudaSuccess)
      return cuda_fail(h, "flag upload");
    return PM_OK;
  };
  auto upload_coef = [&]() -> pm_status {
    if (cudaMemcpyAsync(h->d_coef, coef.data(), sizeof(double) * G, cudaMemcpyHostToDevice,
                        h->stream) != cudaSuccess)
      return cuda_fail(h, "scale upload");
    return PM_OK;
  };
  // systems that leave: flags, zeroed Arnoldi vector k, fewer sweeps
  auto retire = [&](int k, const std::vector<int> &was) -> pm_status {
    if (was == act) return PM_OK;
    PM_TRY(upload_act());
    for (int s = 0; s < G; ++s) coef[(size_t)s] = act[(size_t)s] ? 1.0 : 0.0;
    PM_TRY(upload_coef());
    PM_LAUNCH(launch_seg_scale(v(k), SL, h->d_coef, h->stream));
    bool any = false;
    for (int s = 0; s < G; ++s) any |= act[(size_t)s] != 0;
    return any ? restrict_colours(h, act) : PM_OK;
  };
  auto any_active = [&]() {
    for (int s = 0; s < G; ++s)
      if (act[(size_t)s]) return true;
    return false;
  };
  auto back_subst = [&](int s, int n) {  // y = H(0:n,0:n)^{-1} s(0:n) of system s
    for (int k = 0; k < n; ++k) y[(size_t)k] = sv[(size_t)k * G + s];
    for (int r = n - 1; r >= 0; --r) {
      y[(size_t)r] /= hh(s, r, r);
      for (int q = r - 1; q >= 0; --q) y[(size_t)q] -= hh(s, q, r) * y[(size_t)r];
    }
    for (int k = 0; k < n; ++k) yall[(size_t)k * G + s] = y[(size_t)k];
  };
  auto apply_updates = [&](int n) -> pm_status {  // x += Z yall (n columns)
    if (n <= 0) return PM_OK;
    if (cudaMemcpyAsync(h->ydev, yall.data(), sizeof(double) * (size_t)n * G,
                        cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
      return cuda_fail(h, "y upload");
    PM_LAUNCH(launch_seg_multi_axpy(x, Z, (size_t)N, h->ydev, n, SL, h->stream));
    return PM_OK;
  };

  PM_TRY(upload_act());
  PM_TRY(defect_nse4(h, x, b, v(0)));
  PM_LAUNCH(launch_seg_dot(v(0), nullptr, SL, nullptr, h->partials, h->hcol, 1, true, h->stream));
  PM_TRY(read_scalars(h, r0.data(), h->hcol, G));
  std::vector<int> was = act;
  for (int s = 0; s < G; ++s) {
    res[s].res0 = res[s].res = r0[(size_t)s];
    res0[(size_t)s] = beta[(size_t)s] = resv[(size_t)s] = r0[(size_t)s];
    if (!std::isfinite(r0[(size_t)s])) {
      res[s].status = PM_NAN;
      act[(size_t)s] = 0;
    } else if (r0[(size_t)s] <= resmin) {  // nothing to do (SC_MINIT is not applied here)
      act[(size_t)s] = 0;
    }
  }
  PM_TRY(retire(0, was));
  int j = 1;
  while (any_active() && j <= maxit) {
    for (int s = 0; s < G; ++s)
      coef[(size_t)s] = act[(size_t)s] ? 1.0 / beta[(size_t)s] : 0.0;
    PM_TRY(upload_coef());
    PM_LAUNCH(launch_seg_scale(v(0), SL, h->d_coef, h->stream));
    std::fill(sv.begin(), sv.end(), 0.0);
    for (int s = 0; s < G; ++s) sv[(size_t)s] = beta[(size_t)s];
    int i;
    for (i = 0; i < restart && j <= maxit; i++, j++) {
      PM_TRY(precondition(h, z(i), v(i)));
      for (int s = 0; s < G; ++s) res[s].vcycles += act[(size_t)s];
      PM_LAUNCH(launch_coupled<double>(F.op<double>(), z(i), nullptr, w, false, false, h->stream));
      // modified Gram-Schmidt per system, each step fused with the next dot
      PM_LAUNCH(launch_seg_mgs(w, nullptr, nullptr, v(0), SL, h->d_act, h->partials, h->hcol,
                               h->stream));
      for (int k = 1; k <= i; ++k)
        PM_LAUNCH(launch_seg_mgs(w, v(k - 1), h->hcol + (size_t)(k - 1) * G, v(k), SL, h->d_act,
                                 h->partials, h->hcol + (size_t)k * G, h->stream));
      PM_LAUNCH(launch_seg_mgs(w, v(i), h->hcol + (size_t)i * G, nullptr, SL, h->d_act,
                               h->partials, h->hcol + (size_t)(i + 1) * G, h->stream));
      PM_LAUNCH(launch_seg_scale_copy(v(i + 1), w, h->hcol + (size_t)(i + 1) * G, SL, h->d_act,
                                      h->stream));
      PM_TRY(read_scalars(h, col.data(), h->hcol, (i + 2) * G));
      was = act;
      bool finishing = false;
      std::fill(yall.begin(), yall.end(), 0.0);
      for (int s = 0; s < G; ++s) {
        if (!act[(size_t)s]) continue;
        bool bad = false;
        for (int k = 0; k <= i + 1; ++k) {
          hh(s, k, i) = col[(size_t)k * G + s];
          if (!std::isfinite(hh(s, k, i))) bad = true;
        }
        if (bad) {
          res[s].status = PM_NAN;
          res[s].iterations = j;
          res[s].res = NAN;
          act[(size_t)s] = 0;
          continue;
        }
        double *cs_s = &cs[(size_t)s * R1], *sn_s = &sn[(size_t)s * R1];
        for (int k = 0; k < i; ++k) apply_rot(&hh(s, k, i), &hh(s, k + 1, i), cs_s[k], sn_s[k]);
        gen_rot(hh(s, i, i), hh(s, i + 1, i), &cs_s[i], &sn_s[i]);
        apply_rot(&hh(s, i, i), &hh(s, i + 1, i), cs_s[i], sn_s[i]);
        apply_rot(&sv[(size_t)i * G + s], &sv[(size_t)(i + 1) * G + s], cs_s[i], sn_s[i]);
        const double rv = std::fabs(sv[(size_t)(i + 1) * G + s]);
        resv[(size_t)s] = rv;
        res[s].res = rv;
        res[s].iterations = j;
        if (j >= minit &&
            (rv < resmin || rv < red * (h->opt.red_initial ? r0[(size_t)s] : res0[(size_t)s]))) {
          back_subst(s, i + 1);
          finishing = true;
          act[(size_t)s] = 0;
        } else if (rv > divf * res0[(size_t)s]) {
          res[s].status = PM_DIVERGED;
          act[(size_t)s] = 0;
        }
      }
      if (finishing) PM_TRY(apply_updates(i + 1));
      PM_TRY(retire(i + 1, was));
      if (!any_active()) break;
    }
    if (!any_active()) break;
    // restart (src/FE/FgmresIte.C:574-590) of the systems still iterating
    std::fill(yall.begin(), yall.end(), 0.0);
    for (int s = 0; s < G; ++s)
      if (act[(size_t)s]) back_subst(s, i);
    PM_TRY(apply_updates(i));
    PM_TRY(defect_nse4(h, x, b, v(0)));
    PM_LAUNCH(launch_seg_dot(v(0), nullptr, SL, h->d_act, h->partials, h->hcol, 1, true,
                             h->stream));
    PM_TRY(read_scalars(h, col.data(), h->hcol, G));
    was = act;
    for (int s = 0; s < G; ++s) {
      if (!act[(size_t)s]) continue;
      res0[(size_t)s] = beta[(size_t)s] = resv[(size_t)s] = col[(size_t)s];
      res[s].res = col[(size_t)s];
      if (!std::isfinite(col[(size_t)s])) {
        res[s].status = PM_NAN;
        act[(size_t)s] = 0;
      }
    }
    PM_TRY(retire(0, was));
  }
  for (int s = 0; s < G; ++s)
    if (act[(size_t)s]) {
      res[s].status = PM_MAXIT;
      res[s].iterations = std::min(j, maxit);
    }
  return restore_colours(h);
}

// ------------------------------------------------------------- setup ------
// Factor storage for the level's local solve: the 85x85 (or 49x49) LU with
// its permutation, or the block-elimination data (one-block levels, and
// decoupled nine-block levels).  Grows the allocation when a level changes
// to a solve that stores more (a decoupled level whose matrices gain
// velocity coupling in pm_update_matrices).
pm_status ensure_factors(pm_handle *h, LevelDev &Lv) {
  if (Lv.ncells == 0) return PM_OK;
  const size_t es = mixed(h) ? sizeof(float) : sizeof(double);
  const size_t per_cell = Lv.schur() ? (size_t)kSchurStride
                          : Lv.schur3() ? (size_t)Schur<3>::stride
                                        : (size_t)elem_fac_stride(Lv.nl);
  const size_t need = (size_t)Lv.ncells * per_cell * es;
  if (need > Lv.fac_bytes) {
    PM_TRY(dalloc(h, reinterpret_cast<unsigned char **>(&Lv.factors), need));
    Lv.fac_bytes = need;
  }
  if (!Lv.schur() && !Lv.schur3() && !Lv.perm)
    PM_TRY(dalloc(h, &Lv.perm, (size_t)Lv.ncells * elem_nloc(Lv.nl)));
  return PM_OK;
}

// Unique bytes of one sweep per cell (each stored element counted once):
// residual kernel = matrix values (the A arrays the level reads: 9, 3 when
// decoupled, 1 for one-block levels) + column indices + row pointers, u and
// rhs read; apply kernel = factors (+ permutation), u read+write.
void level_bytes(pm_handle *h, LevelDev &Lv) {
  if (Lv.ncells <= 0) return;
  const double sv = mixed(h) ? 4.0 : 8.0;
  const double nblk = Lv.one_block() ? 1.0 : (Lv.diag == 1 ? 3.0 : 9.0);
  const double mat = nblk * sv * Lv.a_nnz + 4.0 * Lv.a_nnz + 4.0 * (Lv.nu + 1) +
                     (3.0 * sv + 4.0) * ((double)Lv.b_nnz + Lv.bt_nnz) + 4.0 * (Lv.np + 1) +
                     4.0 * (Lv.nu + 1);
  Lv.vanka_res_bytes = (mat + 2.0 * sv * Lv.ndof) / Lv.ncells;
  const double nloc = elem_nloc(Lv.nl);
  const double per_cell = Lv.schur()    ? (double)kSchurValues * sv
                          : Lv.schur3() ? (double)Schur<3>::values * sv
                                        : nloc * nloc * sv + nloc;
  Lv.vanka_apply_bytes = ((double)Lv.ncells * per_cell + 2.0 * sv * Lv.ndof) / Lv.ncells;
}

// Decoupled nine-block levels: one device pass per level over the nine
// velocity blocks (after the Dirichlet rows' off-diagonal entries were
// zeroed), then one read-back: A12..A32 all zero -> diag 1, and A11 = A22 =
// A33 as well -> diag 2.  Levels `only` (all when -1).  *changed reports
// levels whose mode flipped; the captured V-cycles are then dropped (the
// kernels differ).
pm_status detect_decoupled(pm_handle *h, bool *changed, int only = -1) {
  const int n = (int)h->L.size();
  if (changed) *changed = false;
  if (!h->diag_flags) PM_TRY(dalloc(h, &h->diag_flags, (size_t)n));
  if (cudaMemsetAsync(h->diag_flags, 0, sizeof(int) * n, h->stream) != cudaSuccess)
    return cuda_fail(h, "block check reset");
  auto checked = [&](int l) {
    return (only < 0 || l == only) && !h->L[l].structured && h->opt.decouple;
  };
  for (int l = 0; l < n; ++l) {
    if (!checked(l)) continue;
    LevelDev &Lv = h->L[l];
    PM_LAUNCH(launch_block_structure(Lv.op<double>(), Lv.a_nnz, h->diag_flags + l, h->stream));
  }
  std::vector<int> f(n, 1);
  if (cudaMemcpyAsync(f.data(), h->diag_flags, sizeof(int) * n, cudaMemcpyDeviceToHost,
                      h->stream) != cudaSuccess)
    return cuda_fail(h, "block check read");
  PM_TRY(sync(h, "block check"));
  bool any = false;
  for (int l = 0; l < n; ++l) {
    if (only >= 0 && l != only) continue;
    LevelDev &Lv = h->L[l];
    const int d = !checked(l) ? 0 : ((f[l] & 1) ? 0 : ((f[l] & 2) ? 1 : 2));
    if (d != Lv.diag) {
      Lv.diag = d;
      any = true;
    }
  }
  if (any) drop_graphs(h);
  if (changed) *changed = any;
  return PM_OK;
}

// Kernel choice per level (pm_options.residual_variant / apply_variant = -1):
// both variants timed with CUDA events on the level's largest colour (zeroed
// vectors, 3 launches after one warm-up launch), the faster one kept.
template <typename T>
pm_status tune_level(pm_handle *h, LevelDev &Lv) {
  // defaults (option 0): row groups except on FP32 nine-block levels that
  // read all nine blocks, where the flattened stream measured faster (0.64
  // against 0.91 ms per 64^3 colour launch); decoupled levels read three blocks and
  // the row groups are faster there (259 against 272 ms mixed, 549 against
  // 1087 ms FP64); LU apply with two cells per warp in FP64 (the FP64 chain
  // is the bound), one cell per warp in FP32 (each measured faster in the
  // full solve, with the L2 prefetch of the columns)
  // kernel index: 0 row groups, 1 flattened stream
  const int rule_res = (sizeof(T) == sizeof(float) && !Lv.structured && !Lv.diag) ? 1 : 0;
  const int ro = h->opt.residual_variant;
  Lv.res_variant = ro == 0 ? rule_res : (ro == 2 ? 1 : 0);
  const bool can_bulk = sizeof(T) == sizeof(float) && !use_inverse(h) && !Lv.structured &&
                        Lv.diag == 0 && Lv.nl == NU_LOC;
  const int ao = h->opt.apply_variant;
  const int rule_apply = sizeof(T) == sizeof(double) ? 0 : 2;
  Lv.apply_variant = ao == 0 ? rule_apply : (ao == 2 ? 2 : (can_bulk ? 1 : 0));
  const bool tune_res = h->opt.residual_variant < 0;
  const bool tune_apply =
      h->opt.apply_variant < 0 && !use_inverse(h) && !Lv.structured && Lv.diag == 0;
  if ((!tune_res && !tune_apply) || Lv.ncells == 0) return PM_OK;
  int kb = 0, nb = 0;
  for (size_t k = 0; k + 1 < Lv.colouring.ptr.size(); ++k) {
    const int n = Lv.colouring.ptr[k + 1] - Lv.colouring.ptr[k];
    if (n > nb) {
      nb = n;
      kb = (int)k;
    }
  }
  if (nb == 0) return PM_OK;
  if (cudaMemsetAsync(Lv.sol, 0, sizeof(T) * Lv.ndof, h->stream) != cudaSuccess ||
      cudaMemsetAsync(Lv.rhs, 0, sizeof(T) * Lv.ndof, h->stream) != cudaSuccess)
    return cuda_fail(h, "tuning buffers");
  const DevOp<T> op = Lv.op<T>();
  const int *list = Lv.colour_cells + Lv.colouring.ptr[kb];
  T *u = static_cast<T *>(Lv.sol), *rb = static_cast<T *>(Lv.dbuf);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto time_it = [&](auto &&launch, float &ms) -> pm_status {
    for (int rep = 0; rep < 4; ++rep) {
      if (rep == 1) cudaEventRecord(e0, h->stream);
      PM_LAUNCH(launch());
    }
    cudaEventRecord(e1, h->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) return cuda_fail(h, "tuning");
    cudaEventElapsedTime(&ms, e0, e1);
    return PM_OK;
  };
  pm_status st = PM_OK;
  if (tune_res) {
    float t[2] = {0.f, 0.f};
    for (int v = 0; v < 2 && st == PM_OK; ++v)
      st = time_it([&] {
        return launch_vanka_residual<T>(op, Lv.cells(), list, nb, u,
                                        static_cast<const T *>(Lv.rhs), rb, v, h->stream);
      }, t[v]);
    Lv.res_variant = t[1] < t[0] ? 1 : 0;  // kernel index: 0 row groups, 1 stream
  }
  if (tune_apply && st == PM_OK) {
    // kernel index: 0 two cells per warp, 1 bulk-staged (FP32 only), 2 one cell per warp
    float t[3] = {0.f, 1e30f, 0.f};
    const T *F = static_cast<const T *>(Lv.factors);
    for (int v = 0; v < 3 && st == PM_OK; ++v) {
      if (v == 1) {
        if (!can_bulk) continue;
        st = time_it([&] {
          return launch_vanka_apply_tma(Lv.cells(), Lv.nu, list, nb,
                                        reinterpret_cast<const float *>(F), Lv.perm,
                                        reinterpret_cast<const float *>(rb), 1.f,
                                        reinterpret_cast<float *>(u), h->sweep_err, h->num_sms,
                                        h->opt.wait_limit, h->stream);
        }, t[1]);
      } else {
        st = time_it([&] {
          return launch_vanka_apply<T>(Lv.cells(), Lv.nu, list, nb, F, Lv.perm, false, rb, T(1), u,
                                       v == 0, h->stream);
        }, t[v]);
      }
    }
    int best = 0;
    for (int v = 1; v < 3; ++v)
      if (t[v] < t[best]) best = v;
    Lv.apply_variant = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st == PM_OK) st = sync(h, "tuning");
  return st;
}

// After new matrix values: re-check which levels run decoupled and, for
// levels whose mode changed, the factor storage, byte counts and kernels.
pm_status refresh_modes(pm_handle *h, int only = -1) {
  bool changed = false;
  PM_TRY(detect_decoupled(h, &changed, only));
  if (!changed) return PM_OK;
  for (size_t l = 1; l < h->L.size(); ++l) {
    if (only >= 0 && (int)l != only) continue;
    LevelDev &Lv = h->L[l];
    PM_TRY(ensure_factors(h, Lv));
    level_bytes(h, Lv);
    if (mixed(h))
      PM_TRY(tune_level<float>(h, Lv));
    else
      PM_TRY(tune_level<double>(h, Lv));
  }
  return PM_OK;
}

pm_status factor_all(pm_handle *h) {
  if (cudaMemsetAsync(h->status_d, 0, sizeof(int), h->stream) != cudaSuccess)
    return cuda_fail(h, "status reset");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, h->stream);
  for (size_t l = 1; l < h->L.size(); ++l) {
    LevelDev &Lv = h->L[l];
    // block elimination in FP32 unless factor_fp32 = 0 (mixed only); the
    // 85x85 LU in FP32 only with factor_fp32 = 1
    const bool f32 = mixed(h) && h->opt.factor_fp32 != 0;
    if (Lv.schur()) {
      if (mixed(h))
        PM_LAUNCH(launch_schur_factor<float>(Lv.op<double>(), Lv.cells(),
                                             static_cast<float *>(Lv.factors), h->status_d, f32,
                                             h->stream));
      else
        PM_LAUNCH(launch_schur_factor<double>(Lv.op<double>(), Lv.cells(),
                                              static_cast<double *>(Lv.factors), h->status_d,
                                              false, h->stream));
    } else if (Lv.schur3()) {
      if (mixed(h))
        PM_LAUNCH(launch_schur3_factor<float>(Lv.op<double>(), Lv.cells(),
                                              static_cast<float *>(Lv.factors), h->status_d, f32,
                                              h->stream));
      else
        PM_LAUNCH(launch_schur3_factor<double>(Lv.op<double>(), Lv.cells(),
                                               static_cast<double *>(Lv.factors), h->status_d,
                                               false, h->stream));
    } else if (mixed(h))
      PM_LAUNCH(launch_vanka_factor<float>(Lv.op<double>(), Lv.cells(), static_cast<float *>(Lv.factors),
                                           Lv.perm, h->opt.factor_fp32 > 0, use_inverse(h),
                                           h->status_d, h->stream));
    else
      PM_LAUNCH(launch_vanka_factor<double>(Lv.op<double>(), Lv.cells(), static_cast<double *>(Lv.factors),
                                            Lv.perm, false, false, h->status_d, h->stream));
  }
  LevelDev &C = h->L[0];
  if (h->nsys > 1) {  // one dense block per stacked system
    const size_t nc = (size_t)h->coarse_n;
    PM_LAUNCH(launch_coarse_assemble_seg(C.op<double>(), h->coarse_pos, h->coarse_n, h->nsys,
                                         h->coarse_lu, h->opt.project_pressure, h->stream));
    for (int s = 0; s < h->nsys; ++s) {
      PM_LAUNCH(launch_dense_lu(h->coarse_lu + s * nc * nc, h->coarse_n, h->coarse_ipiv + s * nc,
                                h->status_d, h->stream));
      PM_LAUNCH(launch_dense_inverse(h->coarse_lu + s * nc * nc, h->coarse_ipiv + s * nc,
                                     h->coarse_n, h->coarse_inv + s * nc * nc, h->stream));
    }
  } else {
    PM_LAUNCH(launch_coarse_assemble(C.op<double>(), h->coarse_lu, h->opt.project_pressure,
                                     h->stream));
    PM_LAUNCH(launch_dense_lu(h->coarse_lu, h->coarse_n, h->coarse_ipiv, h->status_d, h->stream));
    PM_LAUNCH(launch_dense_inverse(h->coarse_lu, h->coarse_ipiv, h->coarse_n, h->coarse_inv,
                                   h->stream));
  }
  cudaEventRecord(e1, h->stream);
  int st = 0;
  if (cudaMemcpyAsync(&st, h->status_d, sizeof(int), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
    return cuda_fail(h, "status read");
  PM_TRY(sync(h, "factorisation"));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  h->last_factor_ms = ms;
  if (st & 1) return fail(h, PM_BADARG, "singular local Vanka block (zero pivot)");
  if (st & 2) return fail(h, PM_BADARG, "singular coarse system (zero pivot)");
  return PM_OK;
}

// Number of A value arrays of a level descriptor: 9 (NSTYPE 4) or 1 (NSTYPE 2:
// a[0] is the block of all three components, a[1..8] are NULL); 0 if mixed.
int desc_blocks(const pm_level_desc *d) {
  int given = 0;
  for (int k = 1; k < 9; ++k) given += d->a[k] != nullptr;
  if (!d->a[0]) return 0;
  return given == 8 ? 9 : (given == 0 ? 1 : 0);
}

pm_status upload_values(pm_handle *h, LevelDev &Lv, const pm_level_desc *d, bool first) {
  const int nblk = desc_blocks(d);
  if (nblk == 0) return fail(h, PM_BADARG, "A blocks: give all nine or only a[0]");
  if (first) Lv.structured = nblk == 1;
  if ((nblk == 1) != (Lv.structured != 0))
    return fail(h, PM_BADARG, "A block count differs from the level's first upload");
  if (h->opt.upload_mode == 1) {
    // the SMs read the caller's arrays and write the FP64 (and FP32) copies
    // in one pass; off-diagonal blocks are zeroed on the Dirichlet rows
    for (int k = 0; k < nblk; ++k) {
      if (first) {
        PM_TRY(dalloc_padded(h, &Lv.a64[k], Lv.a_nnz));
        if (mixed(h)) PM_TRY(dalloc_padded(h, &Lv.a32[k], Lv.a_nnz));
      }
      const bool offdiag = nblk == 9 && k != 0 && k != 4 && k != 8;
      const long long zero_from = offdiag ? (long long)d->a_rowptr[Lv.nact] : (long long)Lv.a_nnz;
      PM_LAUNCH(launch_host_upload(d->a[k], Lv.a64[k], mixed(h) ? Lv.a32[k] : nullptr, Lv.a_nnz,
                                   zero_from, h->num_sms, h->stream));
    }
    for (int k = 0; k < 3; ++k) {
      if (!d->b[k] || !d->bt[k]) return fail(h, PM_BADARG, "missing B/BT block");
      if (first) {
        PM_TRY(dalloc_padded(h, &Lv.b64[k], Lv.b_nnz));
        PM_TRY(dalloc_padded(h, &Lv.bt64[k], Lv.bt_nnz));
        if (mixed(h)) {
          PM_TRY(dalloc_padded(h, &Lv.b32[k], Lv.b_nnz));
          PM_TRY(dalloc_padded(h, &Lv.bt32[k], Lv.bt_nnz));
        }
      }
      PM_LAUNCH(launch_host_upload(d->b[k], Lv.b64[k], mixed(h) ? Lv.b32[k] : nullptr, Lv.b_nnz,
                                   Lv.b_nnz, h->num_sms, h->stream));
      PM_LAUNCH(launch_host_upload(d->bt[k], Lv.bt64[k], mixed(h) ? Lv.bt32[k] : nullptr,
                                   Lv.bt_nnz, Lv.bt_nnz, h->num_sms, h->stream));
    }
    return PM_OK;
  }
  for (int k = 0; k < nblk; ++k) {
    if (first) PM_TRY(dalloc_padded(h, &Lv.a64[k], Lv.a_nnz));
    if (cudaMemcpyAsync(Lv.a64[k], d->a[k], sizeof(double) * Lv.a_nnz, cudaMemcpyHostToDevice,
                        h->stream) != cudaSuccess)
      return cuda_fail(h, "A upload");
  }
  for (int k = 0; k < 3; ++k) {
    if (!d->b[k] || !d->bt[k]) return fail(h, PM_BADARG, "missing B/BT block");
    if (first) {
      PM_TRY(dalloc_padded(h, &Lv.b64[k], Lv.b_nnz));
      PM_TRY(dalloc_padded(h, &Lv.bt64[k], Lv.bt_nnz));
    }
    if (cudaMemcpyAsync(Lv.b64[k], d->b[k], sizeof(double) * Lv.b_nnz, cudaMemcpyHostToDevice,
                        h->stream) != cudaSuccess ||
        cudaMemcpyAsync(Lv.bt64[k], d->bt[k], sizeof(double) * Lv.bt_nnz, cudaMemcpyHostToDevice,
                        h->stream) != cudaSuccess)
      return cuda_fail(h, "B upload");
  }
  if (!Lv.structured)
    PM_LAUNCH(launch_zero_dirichlet_offdiag(Lv.a64, Lv.a_rowptr, Lv.nu, Lv.nact, h->stream));
  if (mixed(h)) {
    for (int k = 0; k < nblk; ++k) {
      if (first) PM_TRY(dalloc_padded(h, &Lv.a32[k], Lv.a_nnz));
      PM_LAUNCH((launch_convert<float, double>(Lv.a32[k], Lv.a64[k], Lv.a_nnz, h->stream)));
    }
    for (int k = 0; k < 3; ++k) {
      if (first) {
        PM_TRY(dalloc_padded(h, &Lv.b32[k], Lv.b_nnz));
        PM_TRY(dalloc_padded(h, &Lv.bt32[k], Lv.bt_nnz));
      }
      PM_LAUNCH((launch_convert<float, double>(Lv.b32[k], Lv.b64[k], Lv.b_nnz, h->stream)));
      PM_LAUNCH((launch_convert<float, double>(Lv.bt32[k], Lv.bt64[k], Lv.bt_nnz, h->stream)));
    }
  }
  return PM_OK;
}

pm_status upload_csr(pm_handle *h, CsrStore &c, const HostCsr &m) {
  c.rows = m.rows;
  c.cols = m.cols;
  c.nnz = (int)m.col.size();
  PM_TRY(upload(h, &c.rowptr, m.rowptr.data(), m.rowptr.size()));
  PM_TRY(upload(h, &c.col, m.col.data(), m.col.size()));
  PM_TRY(upload(h, &c.v64, m.val.data(), m.val.size()));
  if (mixed(h)) {
    PM_TRY(dalloc(h, &c.v32, m.val.size()));
    PM_LAUNCH((launch_convert<float, double>(c.v32, c.v64, c.nnz, h->stream)));
  }
  return PM_OK;
}

// Fingerprint of a level's CSR patterns: a multiply-xorshift hash over
// every row pointer of A, B and BT and every 61st column index (a strided
// sample, so that the check costs a few milliseconds at 64^3 instead of a
// pass over all 160 M indices).  pm_update_matrices compares it with the
// one pm_add_level took.
uint64_t pattern_fingerprint(const pm_level_desc *d) {
  uint64_t x = 0x243F6A8885A308D3ull;
  auto mix = [&x](uint32_t v) {
    x = (x ^ v) * 0x9E3779B97F4A7C15ull;
    x ^= x >> 29;
  };
  auto rows = [&](const int *p, int n) {
    for (int i = 0; i <= n; ++i) mix((uint32_t)p[i]);
  };
  auto cols = [&](const int *c, int nnz) {
    for (int j = 0; j < nnz; j += 61) mix((uint32_t)c[j]);
    if (nnz > 0) mix((uint32_t)c[nnz - 1]);
  };
  rows(d->a_rowptr, d->n_udof);
  rows(d->b_rowptr, d->n_pdof);
  rows(d->bt_rowptr, d->n_udof);
  cols(d->a_col, d->a_nnz);
  cols(d->b_col, d->b_nnz);
  cols(d->bt_col, d->bt_nnz);
  return x;
}

bool check_desc(pm_handle *h, const pm_level_desc *d) {
  if (!d) return fail(h, PM_BADARG, "null level"), false;
  if (d->n_udof <= 0 || d->n_pdof <= 0 || d->n_active < 0 || d->n_active > d->n_udof)
    return fail(h, PM_BADARG, "bad level sizes"), false;
  if (d->hanging_bound != d->n_active)
    return fail(h, PM_BADARG, "hanging nodes are not supported (hanging_bound != n_active)"), false;
  if (d->hanging_bound + d->n_dirichlet != d->n_udof)
    return fail(h, PM_BADARG, "n_dirichlet inconsistent with n_udof"), false;
  if ((d->n_ulocal != NU_LOC && d->n_ulocal != NU_TET) || d->n_plocal != NP_LOC)
    return fail(h, PM_BADARG,
                "local DOFs: Q2/P1disc hexahedra (27+4) or P2+bubble/P1disc tetrahedra (15+4)"),
           false;
  if (d->pu_rowptr && (!d->pu_col || !d->pu_val || !d->pp_rowptr || !d->pp_col || !d->pp_val ||
                       d->pu_rowptr[d->n_udof] != d->pu_nnz || d->pp_rowptr[d->n_pdof] != d->pp_nnz))
    return fail(h, PM_BADARG, "incomplete prolongation arrays"), false;
  if (!d->a_rowptr || !d->a_col || !d->b_rowptr || !d->b_col || !d->bt_rowptr || !d->bt_col ||
      !d->cell_udofs || !d->cell_pdofs)
    return fail(h, PM_BADARG, "missing arrays"), false;
  if (desc_blocks(d) == 0)
    return fail(h, PM_BADARG, "A blocks: give all nine or only a[0]"), false;
  if (d->a_rowptr[d->n_udof] != d->a_nnz || d->b_rowptr[d->n_pdof] != d->b_nnz ||
      d->bt_rowptr[d->n_udof] != d->bt_nnz)
    return fail(h, PM_BADARG, "row pointer totals do not match nnz"), false;
  return true;
}

}  // namespace

// ===================================================================== ABI ==
extern "C" {

void pm_default_options(pm_options *o) {
  std::memset(o, 0, sizeof(*o));
  o->precision = PM_PREC_FP64;
  o->factor_fp32 = -1;
  o->pre_smooth = 2;
  o->post_smooth = 2;
  o->smooth_damp = 1.0;
  o->alpha = 1.0;
  o->beta = 1.0;
  o->project_pressure = 1;
  o->restart = 20;
  o->maxit = 100;
  o->minit = 0;
  o->red_factor = 0.0;
  o->res_norm_min = 1e-10;
  o->div_factor = 1e10;
  o->device = 0;
  o->use_graphs = 1;
  o->verbose = 0;
  o->pin_host = 0;
  o->vanka_inverse = 0;
  o->residual_variant = 0;
  o->apply_variant = 0;
  o->upload_mode = 0;
  o->red_initial = 0;
  o->decouple = 1;
  o->wait_limit = 0;
  o->max_device_bytes = 0;
  o->learned_levels = 1;
}

const char *pm_status_string(int s) {
  switch (s) {
    case PM_OK: return "ok";
    case PM_MAXIT: return "maximum iterations reached";
    case PM_DIVERGED: return "diverged";
    case PM_NAN: return "non-finite residual";
    case PM_TIMEOUT: return "device wait timed out";
    case PM_OOM: return "out of device memory";
    case PM_BADARG: return "bad argument";
    case PM_CUDA_ERROR: return "CUDA error";
    case PM_NOT_SETUP: return "not set up";
    case PM_NO_DEVICE: return "no CUDA device";
    default: return "unknown";
  }
}

const char *pm_last_error(pm_handle *h) { return h ? h->err.c_str() : "null handle"; }

int pm_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

pm_status pm_create(pm_handle **out, const pm_options *opt) {
  if (!out) return PM_BADARG;
  *out = nullptr;
  pm_options o;
  if (opt)
    o = *opt;
  else
    pm_default_options(&o);
  if (o.precision != PM_PREC_FP64 && o.precision != PM_PREC_MIXED) return PM_BADARG;
  if (o.factor_fp32 < -1 || o.factor_fp32 > 1) return PM_BADARG;
  if (o.factor_fp32 > 0 && o.precision != PM_PREC_MIXED) return PM_BADARG;
  if (o.pre_smooth < 0 || o.post_smooth < 0 || o.restart <= 0 || o.maxit <= 0) return PM_BADARG;
  if (o.residual_variant < -1 || o.residual_variant > 2) return PM_BADARG;
  if (o.apply_variant < -1 || o.apply_variant > 2) return PM_BADARG;
  if (o.upload_mode < 0 || o.upload_mode > 1) return PM_BADARG;
  if (o.decouple < 0 || o.decouple > 1 || o.wait_limit < 0 || o.max_device_bytes < 0 ||
      o.learned_levels < 0)
    return PM_BADARG;
  if (pm_device_count() <= 0) return PM_NO_DEVICE;
  if (cudaSetDevice(o.device) != cudaSuccess) {
    cudaGetLastError();
    return PM_NO_DEVICE;
  }
  pm_handle *h = new pm_handle();
  h->opt = o;
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, o.device);
  if (h->num_sms <= 0) h->num_sms = 1;
  if (o.upload_mode == 1) {
    int pageable = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, o.device);
    if (!pageable) {
      delete h;
      return PM_BADARG;  // the SMs cannot read the caller's host arrays on this system
    }
  }
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return PM_CUDA_ERROR;
  }
  *out = h;
  return PM_OK;
}

pm_status pm_add_level(pm_handle *h, const pm_level_desc *d) {
  if (!h) return PM_BADARG;
  if (h->setup_done) return fail(h, PM_BADARG, "levels must be added before pm_setup");
  if (h->nsys > 1 && !h->adding_stacked)
    return fail(h, PM_BADARG, "a handle of stacked systems takes levels from pm_add_level_batch");
  if (!check_desc(h, d)) return PM_BADARG;
  if (cudaSetDevice(h->opt.device) != cudaSuccess) return cuda_fail(h, "set device");
  h->L.emplace_back();
  LevelDev &Lv = h->L.back();
  Lv.nu = d->n_udof;
  Lv.np = d->n_pdof;
  Lv.ndof = 3 * Lv.nu + Lv.np;
  Lv.nact = d->n_active;
  Lv.hb = d->hanging_bound;
  Lv.ndir = d->n_dirichlet;
  Lv.ncells = d->n_cells;
  Lv.a_nnz = d->a_nnz;
  Lv.b_nnz = d->b_nnz;
  Lv.bt_nnz = d->bt_nnz;
  Lv.nl = d->n_ulocal;
  Lv.h_udofs.assign(d->cell_udofs, d->cell_udofs + (size_t)Lv.ncells * Lv.nl);
  if (d->pu_rowptr) {
    auto take = [](HostCsr &m, int rows, const int *rp, const int *c, const double *v, int nnz) {
      m.rows = rows;
      m.rowptr.assign(rp, rp + rows + 1);
      m.col.assign(c, c + nnz);
      m.val.assign(v, v + nnz);
    };
    take(Lv.h_pu, d->n_udof, d->pu_rowptr, d->pu_col, d->pu_val, d->pu_nnz);
    take(Lv.h_pp, d->n_pdof, d->pp_rowptr, d->pp_col, d->pp_val, d->pp_nnz);
  }
  Lv.h_pdofs.assign(d->cell_pdofs, d->cell_pdofs + (size_t)Lv.ncells * NP_LOC);
  if (d->cell_parent && d->cell_child) {
    Lv.h_parent.assign(d->cell_parent, d->cell_parent + Lv.ncells);
    Lv.h_child.assign(d->cell_child, d->cell_child + Lv.ncells);
  }
  Lv.pattern_key = pattern_fingerprint(d);
  Lv.has_colour = d->cell_colour != nullptr;
  if (Lv.has_colour) Lv.h_colour.assign(d->cell_colour, d->cell_colour + Lv.ncells);
  PM_TRY(upload(h, &Lv.a_rowptr, d->a_rowptr, (size_t)Lv.nu + 1));
  PM_TRY(upload_padded(h, &Lv.a_col, d->a_col, (size_t)Lv.a_nnz));
  PM_TRY(upload(h, &Lv.b_rowptr, d->b_rowptr, (size_t)Lv.np + 1));
  PM_TRY(upload_padded(h, &Lv.b_col, d->b_col, (size_t)Lv.b_nnz));
  PM_TRY(upload(h, &Lv.bt_rowptr, d->bt_rowptr, (size_t)Lv.nu + 1));
  PM_TRY(upload_padded(h, &Lv.bt_col, d->bt_col, (size_t)Lv.bt_nnz));
  if (h->opt.pin_host && !h->adding_stacked) {  // stacked arrays are temporary
    auto pin = [h](const void *p, size_t bytes) {
      if (!p || bytes < (1u << 20)) return;
      if (cudaHostRegister(const_cast<void *>(p), bytes, cudaHostRegisterPortable) == cudaSuccess) {
        h->pinned.push_back(const_cast<void *>(p));
        h->pinned_bytes += (long long)bytes;
      } else
        cudaGetLastError();  // already registered / not registrable: copy unpinned
    };
    for (int k = 0; k < 9; ++k) pin(d->a[k], sizeof(double) * (size_t)Lv.a_nnz);
    for (int k = 0; k < 3; ++k) {
      pin(d->b[k], sizeof(double) * (size_t)Lv.b_nnz);
      pin(d->bt[k], sizeof(double) * (size_t)Lv.bt_nnz);
    }
  }
  PM_TRY(upload_values(h, Lv, d, true));
  PM_TRY(upload(h, &Lv.udofs, Lv.h_udofs.data(), Lv.h_udofs.size()));
  PM_TRY(upload(h, &Lv.pdofs, Lv.h_pdofs.data(), Lv.h_pdofs.size()));
  Lv.seg.G = 1;
  Lv.seg.nu = Lv.nu;
  Lv.seg.na = Lv.nact;
  Lv.seg.np = Lv.np;
  Lv.ncells_sys = Lv.ncells;
  return sync(h, "add level");
}

pm_status pm_add_level_batch(pm_handle *h, const pm_level_desc *descs, int n_sys) {
  if (!h || !descs || n_sys < 1) return PM_BADARG;
  if (h->setup_done) return fail(h, PM_BADARG, "levels must be added before pm_setup");
  if (h->L.empty())
    h->nsys = n_sys;
  else if (h->nsys != n_sys)
    return fail(h, PM_BADARG, "every level of a stacked handle needs the same system count");
  if (n_sys == 1) return pm_add_level(h, descs);
  for (int s = 0; s < n_sys; ++s)
    if (!check_desc(h, &descs[s])) return PM_BADARG;
  StackSizes coarse;
  if (!h->L.empty()) {
    const LevelDev &K = h->L.back();
    coarse.nu = K.seg.nu;
    coarse.na = K.seg.na;
    coarse.np = K.seg.np;
    coarse.ncells = K.ncells_sys;
  }
  StackedLevel st;
  pm_level_desc sd;
  std::string err;
  if (!stack_levels(descs, n_sys, coarse, st, sd, err)) return fail(h, PM_BADARG, err);
  h->adding_stacked = true;
  const pm_status r = pm_add_level(h, &sd);
  h->adding_stacked = false;
  if (r != PM_OK) return r;
  LevelDev &Lv = h->L.back();
  Lv.seg.G = n_sys;
  Lv.seg.nu = descs[0].n_udof;
  Lv.seg.na = descs[0].n_active;
  Lv.seg.np = descs[0].n_pdof;
  Lv.ncells_sys = descs[0].n_cells;
  return PM_OK;
}

pm_status pm_setup(pm_handle *h) {
  if (!h) return PM_BADARG;
  if (h->L.empty()) return fail(h, PM_BADARG, "no levels");
  if (h->setup_done) return fail(h, PM_BADARG, "pm_setup called twice");
  const size_t es = mixed(h) ? sizeof(float) : sizeof(double);
  for (const LevelDev &Lv : h->L)
    if (Lv.nl != NU_LOC && use_inverse(h))
      return fail(h, PM_BADARG, "vanka_inverse: Q2 hexahedral levels only");
  // which nine-block levels run decoupled (reads the uploaded values)
  PM_TRY(detect_decoupled(h, nullptr));
  // colouring, transfers, buffers
  size_t maxcol = 0;
  for (size_t l = 0; l < h->L.size(); ++l) {
    LevelDev &Lv = h->L[l];
    std::string err;
    if (!make_colouring(Lv.ncells, Lv.nl, NP_LOC, Lv.h_udofs.data(), Lv.h_pdofs.data(), Lv.nu,
                        Lv.np, Lv.has_colour ? Lv.h_colour.data() : nullptr, Lv.colouring, err))
      return fail(h, PM_BADARG, "level " + std::to_string(l) + ": " + err);
    PM_TRY(upload(h, &Lv.colour_cells, Lv.colouring.order.data(), Lv.colouring.order.size()));
    maxcol = std::max(maxcol, (size_t)Lv.colouring.max_size);
    if (l > 0) {
      LevelDev &K = h->L[l - 1];
      HostCsr Pu, Ru, Pp, Rp;
      if (!Lv.h_pu.rowptr.empty()) {  // handed over: restriction is the transpose
        Pu = Lv.h_pu;
        Pp = Lv.h_pp;
        Pu.cols = K.nu;
        Pp.cols = K.np;
        for (int c : Pu.col)
          if (c < 0 || c >= K.nu) return fail(h, PM_BADARG, "prolongation column out of range");
        for (int c : Pp.col)
          if (c < 0 || c >= K.np) return fail(h, PM_BADARG, "prolongation column out of range");
        Ru = transpose(Pu);
        Rp = transpose(Pp);
      } else {
        if (Lv.nl != NU_LOC || K.nl != NU_LOC)
          return fail(h, PM_BADARG, "tetrahedral levels need the prolongation arrays");
        if (Lv.h_parent.empty()) return fail(h, PM_BADARG, "fine level without cell_parent/cell_child");
        if (!build_transfers(K.ncells, K.h_udofs.data(), K.h_pdofs.data(), K.nu, K.np, Lv.ncells,
                             Lv.h_udofs.data(), Lv.h_pdofs.data(), Lv.nu, Lv.np,
                             Lv.h_parent.data(), Lv.h_child.data(), Pu, Ru, Pp, Rp, err))
          return fail(h, PM_BADARG, "level " + std::to_string(l) + ": " + err);
      }
      PM_TRY(upload_csr(h, Lv.Pu, Pu));
      PM_TRY(upload_csr(h, Lv.Ru, Ru));
      PM_TRY(upload_csr(h, Lv.Pp, Pp));
      PM_TRY(upload_csr(h, Lv.Rp, Rp));
      // local factors (FP64 or FP32 storage) and permutations, or the
      // block-solve data of a level without velocity coupling
      PM_TRY(ensure_factors(h, Lv));
      PM_TRY(dalloc(h, reinterpret_cast<unsigned char **>(&Lv.dbuf),
                    (size_t)Lv.colouring.max_size * elem_r_stride(Lv.nl) * es));
      if (std::fabs(1.0 - h->opt.alpha) > 1e-3)
        PM_TRY(dalloc(h, reinterpret_cast<unsigned char **>(&Lv.uold), (size_t)Lv.ndof * es));
      if (mixed(h) && Lv.nl == NU_LOC) PM_TRY(dalloc(h, &Lv.ux, (size_t)Lv.nu));
    }
    level_bytes(h, Lv);
    PM_TRY(dalloc(h, reinterpret_cast<unsigned char **>(&Lv.sol), (size_t)Lv.ndof * es));
    PM_TRY(dalloc(h, reinterpret_cast<unsigned char **>(&Lv.rhs), (size_t)Lv.ndof * es));
    PM_TRY(dalloc(h, reinterpret_cast<unsigned char **>(&Lv.def), (size_t)Lv.ndof * es));
    PM_TRY(dalloc(h, &Lv.x64, (size_t)Lv.ndof));
    PM_TRY(dalloc(h, &Lv.y64, (size_t)Lv.ndof));
    PM_TRY(dalloc(h, &Lv.z64, (size_t)Lv.ndof));
  }
  (void)maxcol;
  PM_TRY(dalloc(h, &h->partials,
                std::max<size_t>(8 * 152 + 64, (size_t)seg_partials_size(h->L.back().seg))));
  PM_TRY(dalloc(h, &h->counter, 4));
  if (cudaMemsetAsync(h->counter, 0, 4 * sizeof(unsigned int), h->stream) != cudaSuccess)
    return cuda_fail(h, "counter reset");
  PM_TRY(dalloc(h, &h->status_d, 4));
  PM_TRY(dalloc(h, &h->sweep_err, 4));
  if (cudaMemsetAsync(h->sweep_err, 0, sizeof(int), h->stream) != cudaSuccess)
    return cuda_fail(h, "flag reset");
  if (mixed(h) && launch_vanka_apply_tma_init() < 0) return cuda_fail(h, "bulk-copy apply set-up");
  h->restart = std::max(1, std::min(h->opt.restart, h->opt.maxit));
  PM_TRY(dalloc(h, &h->hcol, ((size_t)h->restart + 4) * h->nsys));
  PM_TRY(dalloc(h, &h->ydev, ((size_t)h->restart + 4) * h->nsys));
  LevelDev &C = h->L[0];
  // the coarse direct solve: one dense system, or one per stacked system
  h->coarse_n = C.ndof / h->nsys;
  const size_t ncoarse = (size_t)h->coarse_n * h->coarse_n * h->nsys;
  PM_TRY(dalloc(h, &h->coarse_lu, ncoarse));
  PM_TRY(dalloc(h, &h->coarse_inv, ncoarse));
  PM_TRY(dalloc(h, &h->coarse_ipiv, (size_t)C.ndof));
  if (h->nsys > 1) {
    std::vector<int> pos((size_t)C.ndof), sup((size_t)C.ndof);
    const int nc = h->coarse_n;
    for (int s = 0; s < h->nsys; ++s)
      for (int l = 0; l < nc; ++l) {
        const int q = (int)C.seg.stacked(s, l);
        pos[(size_t)q] = s * nc + l;
        sup[(size_t)s * nc + l] = q;
      }
    PM_TRY(upload(h, &h->coarse_pos, pos.data(), pos.size()));
    PM_TRY(upload(h, &h->coarse_sup, sup.data(), sup.size()));
    PM_TRY(dalloc(h, &h->d_act, (size_t)h->nsys));
    PM_TRY(dalloc(h, &h->d_coef, (size_t)h->nsys));
    PM_TRY(dalloc(h, &h->stage, (size_t)h->L.back().ndof));
  }
  PM_TRY(dalloc(h, &h->coarse_b, (size_t)C.ndof));
  PM_TRY(dalloc(h, &h->coarse_x, (size_t)C.ndof));
  const size_t N = h->L.back().ndof;
  PM_TRY(dalloc(h, &h->V, (size_t)(h->restart + 1) * N));
  PM_TRY(dalloc(h, &h->Z, (size_t)(h->restart + 1) * N));
  PM_TRY(dalloc(h, &h->w, N));
  PM_TRY(dalloc(h, &h->xd, N));
  PM_TRY(dalloc(h, &h->bd, N));
  PM_TRY(factor_all(h));
  for (size_t l = 1; l < h->L.size(); ++l) {
    if (mixed(h))
      PM_TRY(tune_level<float>(h, h->L[l]));
    else
      PM_TRY(tune_level<double>(h, h->L[l]));
  }
  h->setup_done = true;
  return PM_OK;
}

pm_status pm_update_matrices(pm_handle *h, const pm_level_desc *levels, int n) {
  if (!h || !levels) return PM_BADARG;
  PM_SINGLE(h);
  if (!h->setup_done) return PM_NOT_SETUP;
  h->t_update0 = now_s();
  if (n != (int)h->L.size()) return fail(h, PM_BADARG, "level count mismatch");
  for (int l = 0; l < n; ++l) {
    LevelDev &Lv = h->L[l];
    const pm_level_desc *d = &levels[l];
    if (d->n_udof != Lv.nu || d->n_pdof != Lv.np || d->a_nnz != Lv.a_nnz || d->b_nnz != Lv.b_nnz ||
        d->bt_nnz != Lv.bt_nnz || !d->a_rowptr || !d->a_col || !d->b_rowptr || !d->b_col ||
        !d->bt_rowptr || !d->bt_col || pattern_fingerprint(d) != Lv.pattern_key)
      return fail(h, PM_BADARG, "pattern changed (sizes, row pointers or sampled columns)");
    PM_TRY(upload_values(h, Lv, d, false));
  }
  PM_TRY(refresh_modes(h));
  if (h->opt.verbose) {
    // host timing of the two phases (the sync separates them)
    PM_TRY(sync(h, "upload"));
    const double t1 = now_s();
    PM_TRY(factor_all(h));
    const double t2 = now_s();
    double bytes = 0.0;
    for (const LevelDev &Lv : h->L)
      bytes += 8.0 * ((Lv.structured ? 1.0 : 9.0) * Lv.a_nnz + 3.0 * (Lv.b_nnz + Lv.bt_nnz));
    std::fprintf(stderr, "pm_update_matrices: upload %.4f s (%.1f GB/s), factor %.4f s\n",
                 t1 - h->t_update0, bytes / (t1 - h->t_update0) / 1e9, t2 - t1);
    return PM_OK;
  }
  return factor_all(h);
}

pm_status pm_refactor(pm_handle *h, double *ms) {
  if (!h) return PM_BADARG;
  if (!h->setup_done) return PM_NOT_SETUP;
  PM_TRY(factor_all(h));
  if (ms) *ms = h->last_factor_ms;
  return PM_OK;
}

pm_status pm_destroy(pm_handle *h) {
  if (!h) return PM_OK;
  cudaSetDevice(h->opt.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graphs(h);
  for (cudaEvent_t e : h->evpool) cudaEventDestroy(e);
  for (void *p : h->allocs) cudaFree(p);
  for (void *p : h->pinned) cudaHostUnregister(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return PM_OK;
}

pm_status pm_set_tolerances(pm_handle *h, int restart, int maxit, int minit, double red_factor,
                            double res_norm_min, double div_factor) {
  if (!h) return PM_BADARG;
  if (maxit < 0 || minit < 0 || restart <= 0 || !(red_factor >= 0.0) || !(res_norm_min >= 0.0) ||
      !(div_factor > 0.0))
    return fail(h, PM_BADARG, "pm_set_tolerances: invalid value");
  if (h->setup_done && std::min(restart, maxit) > h->restart)
    return fail(h, PM_BADARG, "pm_set_tolerances: restart larger than the set-up allocation");
  h->opt.restart = restart;
  h->opt.maxit = maxit;
  h->opt.minit = minit;
  h->opt.red_factor = red_factor;
  h->opt.res_norm_min = res_norm_min;
  h->opt.div_factor = div_factor;
  return PM_OK;
}

int pm_n_levels(pm_handle *h) { return h ? (int)h->L.size() : 0; }
int pm_level_ndof(pm_handle *h, int l) {
  return (h && l >= 0 && l < (int)h->L.size()) ? h->L[l].ndof : -1;
}
int pm_level_variant(pm_handle *h, int l) {
  return (h && l >= 0 && l < (int)h->L.size()) ? h->L[l].res_variant + 2 * h->L[l].apply_variant
                                                : -1;
}
int pm_level_blocks(pm_handle *h, int l) {
  return (h && l >= 0 && l < (int)h->L.size()) ? (h->L[l].structured ? 1 : 9) : -1;
}
int pm_level_decoupled(pm_handle *h, int l) {
  return (h && l >= 0 && l < (int)h->L.size()) ? h->L[l].diag : -1;
}

#define PM_CHECK_LEVEL(h, level)                                           \
  do {                                                                     \
    if (!(h)) return PM_BADARG;                                            \
    if (!(h)->setup_done) return PM_NOT_SETUP;                             \
    if ((level) < 0 || (level) >= (int)(h)->L.size())                      \
      return fail((h), PM_BADARG, "level out of range");                   \
  } while (0)

// Sweep-kernel timings recorded since the last collection (events of the
// residual and apply launches, after a synchronisation) into the totals.
static void collect_profile(pm_handle *h) {
  if (!h->prof) return;
  for (size_t k = 0; k + 2 < h->evused; k += 3) {
    float t0 = 0.f, t1 = 0.f;
    cudaEventElapsedTime(&t0, h->evpool[k], h->evpool[k + 1]);
    cudaEventElapsedTime(&t1, h->evpool[k + 1], h->evpool[k + 2]);
    h->prof_ms[0] += t0;
    h->prof_ms[1] += t1;
    h->prof_launches[0]++;
    h->prof_launches[1]++;
    h->prof_sum_bytes[0] += h->prof_bytes[2 * (k / 3)];
    h->prof_sum_bytes[1] += h->prof_bytes[2 * (k / 3) + 1];
  }
  h->evused = 0;
  h->prof_bytes.clear();
}

static pm_status h2d(pm_handle *h, double *d, const double *s, size_t n) {
  if (cudaMemcpyAsync(d, s, n * sizeof(double), cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
    return cuda_fail(h, "H2D");
  return PM_OK;
}
static pm_status d2h(pm_handle *h, double *d, const double *s, size_t n) {
  if (cudaMemcpyAsync(d, s, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
    return cuda_fail(h, "D2H");
  return sync(h, "D2H");
}

pm_status pm_coupled_defect(pm_handle *h, int level, const double *x, const double *b, double *r,
                            int project) {
  PM_CHECK_LEVEL(h, level);
  LevelDev &Lv = h->L[level];
  PM_TRY(h2d(h, Lv.x64, x, Lv.ndof));
  PM_TRY(h2d(h, Lv.y64, b, Lv.ndof));
  PM_LAUNCH(launch_coupled<double>(Lv.op<double>(), Lv.x64, Lv.y64, Lv.z64, true, false, h->stream));
  if (project) PM_LAUNCH(launch_l20_project<double>(Lv.z64 + 3 * Lv.nu, Lv.np, h->partials, h->counter, h->stream));
  return d2h(h, r, Lv.z64, Lv.ndof);
}

pm_status pm_defect(pm_handle *h, int level, const double *u, const double *f, double *d,
                    double *res) {
  PM_CHECK_LEVEL(h, level);
  LevelDev &Lv = h->L[level];
  PM_TRY(h2d(h, Lv.x64, u, Lv.ndof));
  PM_TRY(h2d(h, Lv.y64, f, Lv.ndof));
  PM_TRY(level_defect<double>(h, Lv, Lv.x64, Lv.y64, Lv.z64));
  if (res) {
    double r;
    PM_TRY(norm2(h, Lv.z64, Lv.ndof, &r));
    *res = r;
  }
  return d2h(h, d, Lv.z64, Lv.ndof);
}

pm_status pm_matvec(pm_handle *h, int level, const double *x, double *y) {
  PM_CHECK_LEVEL(h, level);
  LevelDev &Lv = h->L[level];
  PM_TRY(h2d(h, Lv.x64, x, Lv.ndof));
  PM_LAUNCH(launch_coupled<double>(Lv.op<double>(), Lv.x64, nullptr, Lv.z64, false, false, h->stream));
  return d2h(h, y, Lv.z64, Lv.ndof);
}

pm_status pm_cell_vanka(pm_handle *h, int level, double *u, const double *rhs, int sweeps) {
  PM_CHECK_LEVEL(h, level);
  if (level == 0) return fail(h, PM_BADARG, "the coarsest level is solved exactly");
  LevelDev &Lv = h->L[level];
  PM_TRY(h2d(h, Lv.x64, u, Lv.ndof));
  PM_TRY(h2d(h, Lv.y64, rhs, Lv.ndof));
  if (mixed(h)) {
    float *uu = static_cast<float *>(Lv.sol), *ff = static_cast<float *>(Lv.rhs);
    PM_LAUNCH((launch_convert<float, double>(uu, Lv.x64, Lv.ndof, h->stream)));
    PM_LAUNCH((launch_convert<float, double>(ff, Lv.y64, Lv.ndof, h->stream)));
    for (int s = 0; s < sweeps; ++s) PM_TRY(vanka_sweep<float>(h, Lv, uu, ff));
    PM_LAUNCH((launch_convert<double, float>(Lv.x64, uu, Lv.ndof, h->stream)));
  } else {
    for (int s = 0; s < sweeps; ++s) PM_TRY(vanka_sweep<double>(h, Lv, Lv.x64, Lv.y64));
  }
  const pm_status st = d2h(h, u, Lv.x64, Lv.ndof);
  collect_profile(h);
  return st;
}

pm_status pm_restrict(pm_handle *h, int level, const double *fine, double *coarse) {
  PM_CHECK_LEVEL(h, level);
  if (level == 0) return fail(h, PM_BADARG, "no coarser level");
  LevelDev &Fl = h->L[level], &Cl = h->L[level - 1];
  PM_TRY(h2d(h, Fl.x64, fine, Fl.ndof));
  PM_LAUNCH(launch_csr_apply<double>(Fl.Ru.view<double>(), 3, Fl.x64, Fl.nu, Cl.z64, Cl.nu, h->stream));
  PM_LAUNCH(launch_csr_apply<double>(Fl.Rp.view<double>(), 1, Fl.x64 + 3 * Fl.nu, Fl.np,
                                     Cl.z64 + 3 * Cl.nu, Cl.np, h->stream));
  return d2h(h, coarse, Cl.z64, Cl.ndof);
}

pm_status pm_prolongate(pm_handle *h, int level, const double *coarse, double *fine) {
  PM_CHECK_LEVEL(h, level);
  if (level == 0) return fail(h, PM_BADARG, "no coarser level");
  LevelDev &Fl = h->L[level], &Cl = h->L[level - 1];
  PM_TRY(h2d(h, Cl.x64, coarse, Cl.ndof));
  PM_LAUNCH(launch_csr_apply<double>(Fl.Pu.view<double>(), 3, Cl.x64, Cl.nu, Fl.z64, Fl.nu, h->stream));
  PM_LAUNCH(launch_csr_apply<double>(Fl.Pp.view<double>(), 1, Cl.x64 + 3 * Cl.nu, Cl.np,
                                     Fl.z64 + 3 * Fl.nu, Fl.np, h->stream));
  return d2h(h, fine, Fl.z64, Fl.ndof);
}

pm_status pm_solve_exact(pm_handle *h, const double *rhs, double *u) {
  PM_CHECK_LEVEL(h, 0);
  PM_SINGLE(h);
  LevelDev &C = h->L[0];
  PM_TRY(h2d(h, C.x64, rhs, C.ndof));
  PM_LAUNCH(launch_dense_solve(h->coarse_lu, h->coarse_ipiv, h->coarse_n, C.x64, C.z64,
                               h->opt.project_pressure ? 3 * C.nu : -1, h->stream));
  return d2h(h, u, C.z64, C.ndof);
}

pm_status pm_vcycle(pm_handle *h, double *z, const double *v) {
  PM_CHECK_LEVEL(h, 0);
  LevelDev &F = h->L.back();
  PM_TRY(h2d(h, h->bd, v, F.ndof));
  PM_TRY(precondition(h, h->xd, h->bd));
  return d2h(h, z, h->xd, F.ndof);
}

pm_status pm_solve_device(pm_handle *h, double *d_sol, const double *d_rhs, pm_result *out) {
  PM_CHECK_LEVEL(h, 0);
  PM_SINGLE(h);
  pm_result r;
  std::memset(&r, 0, sizeof(r));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  if (h->prof) {
    h->evused = 0;
    h->prof_bytes.clear();
  }
  cudaEventRecord(e0, h->stream);
  pm_status st = fgmres(h, d_sol, d_rhs, &r);
  cudaEventRecord(e1, h->stream);
  if (st == PM_OK || st == PM_MAXIT) {
    // true residual of the returned iterate (FP64)
    pm_status s2 = defect_nse4(h, d_sol, d_rhs, h->w);
    if (s2 == PM_OK) s2 = norm2(h, h->w, h->L.back().ndof, &r.true_res);
    if (s2 != PM_OK) st = s2;
  }
  cudaStreamSynchronize(h->stream);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  r.solve_ms = ms;
  r.setup_ms = h->last_factor_ms;
  r.status = st;
  collect_profile(h);
  if (out) *out = r;
  return st;
}

pm_status pm_solve(pm_handle *h, double *sol, const double *rhs, pm_result *out) {
  PM_CHECK_LEVEL(h, 0);
  LevelDev &F = h->L.back();
  PM_TRY(h2d(h, h->xd, sol, F.ndof));
  PM_TRY(h2d(h, h->bd, rhs, F.ndof));
  pm_status st = pm_solve_device(h, h->xd, h->bd, out);
  pm_status s2 = d2h(h, sol, h->xd, F.ndof);
  return st != PM_OK ? st : s2;
}

pm_status pm_solve_fused(pm_handle *h, double *const *sols, const double *const *rhss,
                         pm_result *results) {
  PM_CHECK_LEVEL(h, 0);
  if (!sols || !rhss) return PM_BADARG;
  for (int s = 0; s < h->nsys; ++s)
    if (!sols[s] || !rhss[s]) return PM_BADARG;
  if (h->nsys == 1) return pm_solve(h, sols[0], rhss[0], results);
  LevelDev &F = h->L.back();
  const SegLayout &SL = F.seg;
  const int G = h->nsys;
  const size_t nd = (size_t)SL.ndof_sys();
  // initial guesses and right-hand sides into the stacked layout
  for (int pass = 0; pass < 2; ++pass) {
    for (int s = 0; s < G; ++s)
      if (cudaMemcpyAsync(h->stage + (size_t)s * nd, pass == 0 ? sols[s] : rhss[s],
                          sizeof(double) * nd, cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
        return cuda_fail(h, "vector upload");
    PM_LAUNCH(launch_seg_permute(pass == 0 ? h->xd : h->bd, h->stage, SL, true, h->stream));
  }
  std::vector<pm_result> r((size_t)G);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, h->stream);
  pm_status st = fgmres_seg(h, h->xd, h->bd, r.data());
  cudaEventRecord(e1, h->stream);
  // every system sweeps again in the next solve, also after an error
  const pm_status rs = restore_colours(h);
  if (st == PM_OK) st = rs;
  if (st == PM_OK) {  // true residual of every returned iterate (FP64)
    std::vector<double> tr((size_t)G);
    st = defect_nse4(h, h->xd, h->bd, h->w);
    if (st == PM_OK) {
      const int n = launch_seg_dot(h->w, nullptr, SL, nullptr, h->partials, h->hcol, 1, true,
                                   h->stream);
      st = n < 0 ? cuda_fail(h, "true residual") : read_scalars(h, tr.data(), h->hcol, G);
      h->launches += n > 0 ? n : 0;
    }
    for (int s = 0; s < G && st == PM_OK; ++s) r[(size_t)s].true_res = tr[(size_t)s];
  }
  cudaStreamSynchronize(h->stream);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != PM_OK) return st;
  PM_LAUNCH(launch_seg_permute(h->xd, h->stage, SL, false, h->stream));
  for (int s = 0; s < G; ++s)
    if (cudaMemcpyAsync(sols[s], h->stage + (size_t)s * nd, sizeof(double) * nd,
                        cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
      return cuda_fail(h, "vector download");
  PM_TRY(sync(h, "fused solve"));
  pm_status first = PM_OK;
  for (int s = 0; s < G; ++s) {
    r[(size_t)s].solve_ms = ms;
    r[(size_t)s].setup_ms = h->last_factor_ms;
    if (results) results[s] = r[(size_t)s];
    if (first == PM_OK && r[(size_t)s].status != PM_OK) first = (pm_status)r[(size_t)s].status;
  }
  return first;
}

int pm_n_systems(pm_handle *h) { return h ? h->nsys : 0; }

static AsmOp asm_op(LevelDev &Lv) {
  AsmOp op{};
  op.nu = Lv.nu;
  op.np = Lv.np;
  op.nact = Lv.nact;
  op.a_nnz = Lv.a_nnz;
  op.b_nnz = Lv.b_nnz;
  op.bt_nnz = Lv.bt_nnz;
  op.a_rowptr = Lv.a_rowptr;
  op.a_col = Lv.a_col;
  op.b_rowptr = Lv.b_rowptr;
  op.b_col = Lv.b_col;
  op.bt_rowptr = Lv.bt_rowptr;
  op.bt_col = Lv.bt_col;
  const int nblk = Lv.structured ? 1 : 9;
  for (int k = 0; k < nblk; ++k) op.a[k] = Lv.a64[k];
  for (int k = 0; k < 3; ++k) {
    op.b[k] = Lv.b64[k];
    op.bt[k] = Lv.bt64[k];
  }
  op.c_mass = 0.0;
  op.c_a = 1.0;
  op.b_scale = 1.0;
  op.bt_scale = 1.0;
  op.Aonly = Lv.asm_A;
  op.Monly = Lv.asm_M;
  return op;
}

// SYS: the theta-scheme system (A and M kept for pm_system_rhs); otherwise
// the Oseen blocks alone
static pm_status assemble_impl(pm_handle *h, int level, const double *d_cell_h,
                               const double *d_conv, double nu, double c_mass, double c_a,
                               double b_scale, double bt_scale, bool sys) {
  PM_CHECK_LEVEL(h, level);
  PM_SINGLE(h);
  if (!d_cell_h || !d_conv) return fail(h, PM_BADARG, "missing cell sizes or convection");
  LevelDev &Lv = h->L[level];
  if (Lv.ncells <= 0) return fail(h, PM_BADARG, "level without cells");
  if (Lv.nl != NU_LOC) return fail(h, PM_BADARG, "device assembly: Q2 hexahedral levels only");
  if (!h->asm_tables) {
    if (assemble_tables_init() < 0) return cuda_fail(h, "assembly tables");
    h->asm_tables = true;
  }
  if (sys) {
    if (!Lv.asm_A) PM_TRY(dalloc(h, &Lv.asm_A, (size_t)Lv.a_nnz));
    if (!Lv.asm_M) PM_TRY(dalloc(h, &Lv.asm_M, (size_t)Lv.a_nnz));
  }
  AsmOp op = asm_op(Lv);
  op.c_mass = c_mass;
  op.c_a = c_a;
  op.b_scale = b_scale;
  op.bt_scale = bt_scale;
  if (!sys) op.Aonly = op.Monly = nullptr;
  Lv.asm_theta = false;
  PM_LAUNCH(launch_assemble_level(op, Lv.cells(), Lv.colour_cells, Lv.colouring.ptr.data(),
                                  (int)Lv.colouring.ptr.size() - 1, d_cell_h, d_conv, nu,
                                  h->stream));
  // the assembly zeroes A12..A32 and writes the same values into A11, A22
  // and A33 (k_assemble_cells): mode 2 by construction, no device check
  if (!Lv.structured) {
    const int d = h->opt.decouple ? 2 : 0;
    if (d != Lv.diag) {
      Lv.diag = d;
      drop_graphs(h);
      PM_TRY(ensure_factors(h, Lv));
      level_bytes(h, Lv);
      if (mixed(h))
        PM_TRY(tune_level<float>(h, Lv));
      else
        PM_TRY(tune_level<double>(h, Lv));
    }
  }
  if (mixed(h)) {
    const int nblk = Lv.structured ? 1 : 9;
    for (int k = 0; k < nblk; ++k)
      if (!Lv.diag || k % 4 == 0)  // a decoupled level reads A11, A22, A33 only
        PM_LAUNCH((launch_convert<float, double>(Lv.a32[k], Lv.a64[k], Lv.a_nnz, h->stream)));
    for (int k = 0; k < 3; ++k) {
      PM_LAUNCH((launch_convert<float, double>(Lv.b32[k], Lv.b64[k], Lv.b_nnz, h->stream)));
      PM_LAUNCH((launch_convert<float, double>(Lv.bt32[k], Lv.bt64[k], Lv.bt_nnz, h->stream)));
    }
  }
  PM_TRY(sync(h, "assembly"));
  Lv.asm_theta = sys;
  return PM_OK;
}

pm_status pm_assemble_system_level_device(pm_handle *h, int level, const double *d_cell_h,
                                          const double *d_conv, double nu, double c_mass,
                                          double c_a, double b_scale, double bt_scale) {
  return assemble_impl(h, level, d_cell_h, d_conv, nu, c_mass, c_a, b_scale, bt_scale, true);
}

pm_status pm_assemble_level_device(pm_handle *h, int level, const double *d_cell_h,
                                   const double *d_conv, double nu) {
  return assemble_impl(h, level, d_cell_h, d_conv, nu, 0.0, 1.0, 1.0, 1.0, false);
}

// host inputs into the level's assembly buffers
static pm_status stage_assembly_inputs(pm_handle *h, LevelDev &Lv, const double *cell_h,
                                       const double *conv) {
  if (!Lv.asm_h) PM_TRY(dalloc(h, &Lv.asm_h, (size_t)Lv.ncells * 3));
  if (!Lv.asm_conv) PM_TRY(dalloc(h, &Lv.asm_conv, (size_t)Lv.nu * 3));
  if (cudaMemcpyAsync(Lv.asm_h, cell_h, sizeof(double) * Lv.ncells * 3, cudaMemcpyHostToDevice,
                      h->stream) != cudaSuccess ||
      cudaMemcpyAsync(Lv.asm_conv, conv, sizeof(double) * Lv.nu * 3, cudaMemcpyHostToDevice,
                      h->stream) != cudaSuccess)
    return cuda_fail(h, "assembly inputs");
  return PM_OK;
}

pm_status pm_assemble_system_level(pm_handle *h, int level, const double *cell_h,
                                   const double *conv, double nu, double c_mass, double c_a,
                                   double b_scale, double bt_scale) {
  PM_CHECK_LEVEL(h, level);
  if (!cell_h || !conv) return fail(h, PM_BADARG, "missing cell sizes or convection");
  LevelDev &Lv = h->L[level];
  if (Lv.ncells <= 0) return fail(h, PM_BADARG, "level without cells");
  PM_TRY(stage_assembly_inputs(h, Lv, cell_h, conv));
  return pm_assemble_system_level_device(h, level, Lv.asm_h, Lv.asm_conv, nu, c_mass, c_a,
                                         b_scale, bt_scale);
}

pm_status pm_system_rhs(pm_handle *h, const double *old_rhs, const double *rhs, const double *sol,
                        double c_old, double c_new, double c2, double *out) {
  PM_CHECK_LEVEL(h, 0);
  PM_SINGLE(h);
  if (!old_rhs || !rhs || !sol || !out) return PM_BADARG;
  LevelDev &F = h->L.back();
  if (!F.asm_theta)
    return fail(h, PM_BADARG, "the finest level has no system assembly (Oseen and mass blocks)");
  const size_t n = (size_t)F.ndof;
  // three staging vectors of the level (FP64)
  PM_TRY(h2d(h, F.x64, old_rhs, n));
  PM_TRY(h2d(h, F.y64, rhs, n));
  PM_TRY(h2d(h, F.z64, sol, n));
  double *o = h->xd;  // finest-level sized FP64 buffer of the solver
  PM_LAUNCH(launch_system_rhs(asm_op(F), F.x64, F.y64, F.z64, c_old, c_new, c2, o, h->stream));
  return d2h(h, out, o, n);
}

pm_status pm_system_rhs_device(pm_handle *h, const double *d_old_rhs, const double *d_rhs,
                               const double *d_sol, double c_old, double c_new, double c2,
                               double *d_out) {
  PM_CHECK_LEVEL(h, 0);
  PM_SINGLE(h);
  if (!d_old_rhs || !d_rhs || !d_sol || !d_out) return PM_BADARG;
  if (d_out == d_old_rhs || d_out == d_rhs || d_out == d_sol)
    return fail(h, PM_BADARG, "out aliases an input");
  LevelDev &F = h->L.back();
  if (!F.asm_theta)
    return fail(h, PM_BADARG, "the finest level has no system assembly (Oseen and mass blocks)");
  PM_LAUNCH(launch_system_rhs(asm_op(F), d_old_rhs, d_rhs, d_sol, c_old, c_new, c2, d_out,
                              h->stream));
  return sync(h, "system rhs");
}

// coarse DOF -> fine DOF: corner (fa, fb, fc) in {0, 2}^3 of the fine cell in
// octant (ox, oy, oz) of its parent is the parent's local node
// (ox + fa/2, oy + fb/2, oz + fc/2)
static pm_status build_coarse_nodes(pm_handle *h, int level) {
  LevelDev &F = h->L[level], &Cl = h->L[level - 1];
  if (F.nl != NU_LOC || Cl.nl != NU_LOC)
    return fail(h, PM_BADARG, "coarse-node interpolation: Q2 hexahedral levels only");
  if (F.h_parent.empty() || F.h_child.empty())
    return fail(h, PM_BADARG, "level without cell_parent / cell_child");
  std::vector<int> map((size_t)Cl.nu, -1);
  for (int f = 0; f < F.ncells; ++f) {
    const int p = F.h_parent[f], o = F.h_child[f];
    if (p < 0 || p >= Cl.ncells || o < 0 || o > 7) return fail(h, PM_BADARG, "bad cell_parent");
    const int ox = o & 1, oy = (o >> 1) & 1, oz = (o >> 2) & 1;
    for (int fc = 0; fc <= 2; fc += 2)
      for (int fb = 0; fb <= 2; fb += 2)
        for (int fa = 0; fa <= 2; fa += 2) {
          const int cd = Cl.h_udofs[(size_t)p * NU_LOC + (ox + fa / 2) + 3 * (oy + fb / 2) +
                                    9 * (oz + fc / 2)];
          const int fd = F.h_udofs[(size_t)f * NU_LOC + fa + 3 * fb + 9 * fc];
          if (cd < 0 || cd >= Cl.nu || fd < 0 || fd >= F.nu)
            return fail(h, PM_BADARG, "cell DOF out of range");
          if (map[cd] >= 0 && map[cd] != fd)
            return fail(h, PM_BADARG, "coarse node with two fine DOFs: meshes not nested");
          map[cd] = fd;
        }
  }
  for (int v : map)
    if (v < 0) return fail(h, PM_BADARG, "coarse node not covered by a child cell");
  return upload(h, &F.coarse_nodes, map.data(), map.size());
}

pm_status pm_interpolate_coarse(pm_handle *h, int level, const double *d_fine, double *d_coarse) {
  PM_CHECK_LEVEL(h, level);
  PM_SINGLE(h);
  if (level < 1 || !d_fine || !d_coarse) return PM_BADARG;
  LevelDev &F = h->L[level];
  if (!F.coarse_nodes) PM_TRY(build_coarse_nodes(h, level));
  PM_LAUNCH(launch_interpolate_coarse(F.coarse_nodes, h->L[level - 1].nu, F.nu, d_fine, d_coarse,
                                      h->stream));
  return sync(h, "interpolate coarse");
}

pm_status pm_assemble_level(pm_handle *h, int level, const double *cell_h, const double *conv,
                            double nu) {
  PM_CHECK_LEVEL(h, level);
  if (!cell_h || !conv) return fail(h, PM_BADARG, "missing cell sizes or convection");
  LevelDev &Lv = h->L[level];
  if (Lv.ncells <= 0) return fail(h, PM_BADARG, "level without cells");
  PM_TRY(stage_assembly_inputs(h, Lv, cell_h, conv));
  return pm_assemble_level_device(h, level, Lv.asm_h, Lv.asm_conv, nu);
}

pm_status pm_solve_batch(pm_handle *const *hs, int n, double *const *sols,
                         const double *const *rhss, pm_result *results, int nthreads) {
  if (!hs || !sols || !rhss || n <= 0) return PM_BADARG;
  for (int i = 0; i < n; ++i) {
    if (!hs[i] || !sols[i] || !rhss[i]) return PM_BADARG;
    if (!hs[i]->setup_done) return PM_NOT_SETUP;
    for (int j = 0; j < i; ++j)
      if (hs[j] == hs[i]) return PM_BADARG;  // a handle is not thread-safe
  }
  std::vector<pm_status> st((size_t)n, PM_OK);
  std::atomic<int> next{0};
  auto worker = [&]() {
    for (;;) {
      const int i = next.fetch_add(1);
      if (i >= n) break;
      pm_result r;
      std::memset(&r, 0, sizeof(r));
      if (cudaSetDevice(hs[i]->opt.device) != cudaSuccess) {
        st[(size_t)i] = PM_CUDA_ERROR;
      } else {
        st[(size_t)i] = pm_solve(hs[i], sols[i], rhss[i], &r);
      }
      if (results) results[i] = r;
    }
  };
  const int T = std::max(1, std::min(nthreads > 0 ? nthreads : n, n));
  std::vector<std::thread> pool;
  pool.reserve((size_t)T);
  for (int t = 0; t < T; ++t) pool.emplace_back(worker);
  for (auto &th : pool) th.join();
  for (int i = 0; i < n; ++i)
    if (st[(size_t)i] != PM_OK) return st[(size_t)i];
  return PM_OK;
}

long long pm_kernel_launches(pm_handle *h) { return h ? h->launches : 0; }
long long pm_device_bytes(pm_handle *h) { return h ? h->bytes : 0; }
long long pm_pinned_bytes(pm_handle *h) { return h ? h->pinned_bytes : 0; }

pm_status pm_profile_enable(pm_handle *h, int enable) {
  if (!h) return PM_BADARG;
  h->prof = enable != 0;
  for (int k = 0; k < 2; ++k) {
    h->prof_ms[k] = 0.0;
    h->prof_sum_bytes[k] = 0.0;
    h->prof_launches[k] = 0;
  }
  if (h->prof && h->evpool.empty()) {
    h->evpool.resize(3 << 14);
    for (auto &e : h->evpool) cudaEventCreate(&e);
  }
  return PM_OK;
}

// ------------------------------------------------------ learned smoother --
pm_status pm_mlp_create(pm_mlp **out, int device, unsigned long long seed, int max_batch) {
  if (!out || max_batch <= 0) return PM_BADARG;
  *out = nullptr;
  if (pm_device_count() <= 0) return PM_NO_DEVICE;
  pm_mlp *m = new pm_mlp();
  const cudaError_t e = mlp_create(m->m, device, seed, max_batch);
  if (e != cudaSuccess) {
    cudaGetLastError();
    mlp_destroy(m->m);
    delete m;
    return e == cudaErrorMemoryAllocation ? PM_OOM : PM_CUDA_ERROR;
  }
  *out = m;
  return PM_OK;
}

pm_status pm_mlp_destroy(pm_mlp *m) {
  if (!m) return PM_OK;
  mlp_destroy(m->m);
  delete m;
  return PM_OK;
}

long long pm_mlp_num_params(void) { return kNumParams; }

pm_status pm_mlp_get_params(pm_mlp *m, float *host, long long n) {
  if (!m || !host || n != kNumParams) return PM_BADARG;
  cudaSetDevice(m->m.device);
  if (cudaMemcpyAsync(host, m->m.P, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost,
                      m->m.stream) != cudaSuccess ||
      cudaStreamSynchronize(m->m.stream) != cudaSuccess)
    return PM_CUDA_ERROR;
  return PM_OK;
}

pm_status pm_mlp_set_params(pm_mlp *m, const float *host, long long n) {
  if (!m || !host || n != kNumParams) return PM_BADARG;
  cudaSetDevice(m->m.device);
  if (cudaMemcpyAsync(m->m.P, host, sizeof(float) * kNumParams, cudaMemcpyHostToDevice,
                      m->m.stream) != cudaSuccess ||
      mlp_sync_bf16(m->m, m->m.stream) < 0 || cudaStreamSynchronize(m->m.stream) != cudaSuccess)
    return PM_CUDA_ERROR;
  return PM_OK;
}

// bounded waits of the tcgen05 layers that gave up (flag read and cleared)
static pm_status mlp_err(pm_mlp *m) {
  int e = 0;
  if (cudaMemcpy(&e, m->m.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return PM_CUDA_ERROR;
  if (e) {
    cudaMemset(m->m.err, 0, sizeof(int));
    return PM_TIMEOUT;
  }
  return PM_OK;
}

pm_status pm_mlp_forward(pm_mlp *m, const float *d_X, int M, float *d_Y) {
  if (!m || !d_X || !d_Y || M <= 0 || M > m->m.max_batch) return PM_BADARG;
  cudaSetDevice(m->m.device);
  if (mlp_forward_f32(m->m, d_X, M, d_Y, m->m.stream) < 0 ||
      cudaStreamSynchronize(m->m.stream) != cudaSuccess)
    return PM_CUDA_ERROR;
  return mlp_err(m);
}

pm_status pm_mlp_set_tensor_path(pm_mlp *m, int tcgen05) {
  if (!m) return PM_BADARG;
  m->m.tc = tcgen05 != 0;
  return PM_OK;
}

pm_status pm_mlp_loss_grad(pm_mlp *m, const float *d_X, const float *d_T, int M, double *loss,
                           float *host_grad) {
  if (!m || !d_X || !d_T || M <= 0 || M > m->m.max_batch) return PM_BADARG;
  cudaSetDevice(m->m.device);
  if (mlp_loss_grad(m->m, d_X, d_T, M, m->m.stream) < 0) return PM_CUDA_ERROR;
  double l = 0.0;
  if (cudaMemcpyAsync(&l, m->m.loss, sizeof(double), cudaMemcpyDeviceToHost, m->m.stream) !=
      cudaSuccess)
    return PM_CUDA_ERROR;
  if (host_grad && cudaMemcpyAsync(host_grad, m->m.G, sizeof(float) * kNumParams,
                                   cudaMemcpyDeviceToHost, m->m.stream) != cudaSuccess)
    return PM_CUDA_ERROR;
  if (cudaStreamSynchronize(m->m.stream) != cudaSuccess) return PM_CUDA_ERROR;
  if (loss) *loss = l;
  const pm_status es = mlp_err(m);
  if (es != PM_OK) return es;
  return std::isfinite(l) ? PM_OK : PM_NAN;
}

pm_status pm_mlp_adamw_step(pm_mlp *m, float lr, float beta1, float beta2, float eps, float wd) {
  if (!m) return PM_BADARG;
  cudaSetDevice(m->m.device);
  if (mlp_adamw(m->m, lr, beta1, beta2, eps, wd, m->m.stream) < 0) return PM_CUDA_ERROR;
  return PM_OK;
}

pm_status pm_learned_attach(pm_handle *h, pm_mlp *m, double omega, double fallback_ratio) {
  if (!h) return PM_BADARG;
  PM_SINGLE(h);
  if (!h->setup_done) return PM_NOT_SETUP;
  if (m && m->m.device != h->opt.device) return fail(h, PM_BADARG, "network on another device");
  if (m)
    for (const LevelDev &Lv : h->L)
      if (Lv.nl != NU_LOC)
        return fail(h, PM_BADARG, "learned smoother: Q2 hexahedral levels only (85-DOF cells)");
  drop_graphs(h);  // the captured V-cycles change
  if (!m) {
    h->mlp = nullptr;
    return PM_OK;
  }
  // the network's weights are written on its own stream; make them visible
  if (cudaStreamSynchronize(m->m.stream) != cudaSuccess) return cuda_fail(h, "network sync");
  for (size_t l = 1; l < h->L.size(); ++l) PM_TRY(ensure_learned_buffers(h, h->L[l]));
  if (!h->d_on) PM_TRY(dalloc(h, &h->d_on, 1));
  h->mlp = &m->m;
  h->l_omega = omega;
  h->l_fallback = fallback_ratio;
  h->l_fallbacks = 0;
  PM_TRY(set_learned_flag(h, 1));
  return sync(h, "attach");
}

pm_status pm_learned_status(pm_handle *h, int *enabled, int *fallbacks) {
  if (!h) return PM_BADARG;
  if (enabled) *enabled = h->mlp ? h->l_on_host : 0;
  if (fallbacks) *fallbacks = h->l_fallbacks;
  return PM_OK;
}

pm_status pm_learned_harvest(pm_handle *h, const double *sol_exact, const double *rhs,
                             int n_cycles, float *d_X, float *d_T, long long capacity,
                             long long *n_pairs) {
  PM_CHECK_LEVEL(h, 0);
  PM_SINGLE(h);
  if (!sol_exact || !rhs || !d_X || !d_T || !n_pairs || n_cycles <= 0) return PM_BADARG;
  LevelDev &F = h->L.back();
  if (*n_pairs < 0 || *n_pairs + (long long)n_cycles * F.ncells > capacity)
    return fail(h, PM_BADARG, "harvest capacity exceeded");
  if (h->L.size() < 2) return fail(h, PM_BADARG, "harvest needs at least two levels");
  if (F.nl != NU_LOC) return fail(h, PM_BADARG, "harvest: Q2 hexahedral levels only");
  PM_TRY(ensure_learned_buffers(h, F));
  const int N = F.ndof;
  double *u = h->xd, *b = h->bd, *ue = h->V, *e = h->V + N, *z = h->Z, *r = h->w;
  PM_TRY(h2d(h, b, rhs, N));
  PM_TRY(h2d(h, ue, sol_exact, N));
  PM_LAUNCH(launch_fill<double>(u, 0.0, N, h->stream));
  const int was_on = h->l_on_host;
  if (h->mlp) PM_TRY(set_learned_flag(h, 0));  // pairs of the plain solver
  const DevCells cells = F.cells();
  for (int k = 0; k < n_cycles; ++k) {
    PM_TRY(defect_nse4(h, u, b, r));
    PM_TRY(precondition(h, z, r));
    PM_LAUNCH(launch_axpy<double>(u, 1.0, z, N, h->stream));
    PM_TRY(level_defect<double>(h, F, u, b, r));
    if (cudaMemcpyAsync(e, ue, sizeof(double) * N, cudaMemcpyDeviceToDevice, h->stream) !=
        cudaSuccess)
      return cuda_fail(h, "harvest copy");
    PM_LAUNCH(launch_axpy<double>(e, -1.0, u, N, h->stream));
    PM_TRY(l20<double>(h, e + 3 * F.nu, F.np));
    float *Xrow = d_X + (size_t)(*n_pairs) * kMlpIn;
    float *Trow = d_T + (size_t)(*n_pairs) * kMlpOut;
    PM_LAUNCH(launch_cell_summary<double>(cells, F.nu, r, F.l_summary, nullptr, h->stream));
    PM_LAUNCH(launch_cell_features<double>(cells, F.nu, r, F.l_summary, F.l_nbr, nullptr, Xrow,
                                           F.l_scale, nullptr, h->stream));
    PM_LAUNCH(launch_cell_targets<double>(cells, F.nu, e, F.l_scale, Trow, h->stream));
    *n_pairs += F.ncells;
  }
  if (h->mlp) PM_TRY(set_learned_flag(h, was_on));
  return sync(h, "harvest");
}

pm_status pm_profile_read(pm_handle *h, int kernel, double *ms, long long *launches,
                          double *bytes) {
  if (!h || kernel < 0 || kernel > 1) return PM_BADARG;
  if (ms) *ms = h->prof_ms[kernel];
  if (launches) *launches = h->prof_launches[kernel];
  if (bytes) *bytes = h->prof_sum_bytes[kernel];
  return PM_OK;
}

}  // extern "C"
