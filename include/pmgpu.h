/*
 * pmgpu.h — C ABI of the GB300 (sm_103a) saddle-point multigrid solver for
 * Q2/P1disc Oseen systems (NSTYPE 4: nine velocity blocks A11..A33 sharing one
 * CSR pattern, B1..B3, B1T..B3T).
 *
 * The entry points replace, one for one, the solver objects that ParMooN's
 * NSE3D/TNSE3D programs build when SC_SOLVER_SADDLE=16 (FGMRES),
 * SC_PRECONDITIONER_SADDLE=5 (multigrid) and SC_SMOOTHER_SADDLE=2 (cell Vanka):
 *
 *   pm_create            TNSE_MultiGrid::TNSE_MultiGrid  (include/FE/NSE_MultiGrid.h:193)
 *                        + TFgmresIte ctor parameters    (src/FE/FgmresIte.C:75-176)
 *   pm_add_level         TNSE_MultiGrid::AddLevel        (src/FE/NSE_MultiGrid.C:81-102)
 *                        with the arrays a TNSE_MGLevel4 captures in its ctor
 *                        (src/FE/NSE_MGLevel4.C:119-328)
 *   pm_setup             TNSE_MultiGrid::InitGPU         (src/FE/NSE_MultiGrid.C:105-185)
 *                        (upload, colour, factor all local Vanka blocks once,
 *                        factor the coarse dense system once)
 *   pm_defect            TNSE_MGLevel4::Defect           (src/FE/NSE_MGLevel4.C:465-539)
 *   pm_coupled_defect    Defect_NSE4 / CoupledDefect     (src/FE/MGComponents3D.C:3038-3231)
 *   pm_matvec            MatVect_NSE4 / CoupledMatVect   (src/FE/MGComponents3D.C:2872-3035)
 *   pm_cell_vanka        TNSE_MGLevel4::CellVanka        (src/FE/NSE_MGLevel4.C:1653-2087;
 *                        colour-block semantics of CellVanka_GPU, src/FE/NSE_CellVanka.cu:1748-2555)
 *   pm_restrict          DefectRestriction (vector+scalar) (src/FE/MGComponents3D.C:711-1242)
 *   pm_prolongate        Prolongate (vector+scalar)      (src/FE/MGComponents3D.C:184-708)
 *   pm_solve_exact       TNSE_MGLevel4::SolveExact       (src/FE/NSE_MGLevel4.C:5728-5847)
 *   pm_vcycle            TMultiGridIte::Iterate          (src/FE/MultiGridIte.C:76-132)
 *                        -> TNSE_MultiGrid::Cycle        (src/FE/NSE_MultiGrid.C:434-1779)
 *   pm_solve             TFgmresIte::Iterate (flexible)  (src/FE/FgmresIte.C:250-677)
 *   pm_destroy           destructors
 *
 * All host pointers are plain C arrays in the reference's own layouts:
 * solution/rhs vectors are [u1 | u2 | u3 | p] of length 3*N_U + N_P, CSR
 * arrays are exactly those of TSquareMatrix3D / TMatrix3D.  The *_device
 * variants take device pointers (cudaMalloc'd, same layout) and run without
 * any host<->device copy of the vectors.
 *
 * Errors are returned as pm_status; nothing in the library calls exit().
 * A handle is not thread-safe; it owns one CUDA stream.
 */
#ifndef PMGPU_H
#define PMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PM_OK = 0,
  PM_MAXIT = 1,        /* FGMRES stopped at maxit without meeting the test   */
  PM_DIVERGED = 2,     /* res > SC_DIV_FACTOR * res0 (reference: exit(4711)) */
  PM_NAN = 3,          /* non-finite residual                                */
  PM_TIMEOUT = 4,      /* a bounded device wait ran out                      */
  PM_OOM = 5,          /* device allocation failed                          */
  PM_BADARG = 6,       /* invalid argument / unsupported configuration       */
  PM_CUDA_ERROR = 7,   /* CUDA runtime error                                 */
  PM_NOT_SETUP = 8,    /* pm_setup has not run (or failed)                   */
  PM_NO_DEVICE = 9     /* no CUDA device / extension cannot run              */
} pm_status;

/* Precision of the V-cycle.  FGMRES, Arnoldi, Givens and the coarse direct
 * solve are FP64 in both modes; the local factorisations are stored in the
 * V-cycle precision.  FP64 mode computes them in FP64.  Mixed mode computes
 * the block elimination of decoupled cells in FP32 and the 85x85 LU of
 * coupled cells in FP64 (factor_fp32 = -1, the default); factor_fp32 = 0
 * computes both in FP64, factor_fp32 = 1 both in FP32. */
enum { PM_PREC_FP64 = 0, PM_PREC_MIXED = 1 };

typedef struct {
  int precision;          /* PM_PREC_FP64 | PM_PREC_MIXED                          */
  int factor_fp32;        /* -1 (default) | 0 | 1: see above; 1 mixed only         */
  /* multigrid (TDatabase::ParamDB names) */
  int pre_smooth;         /* SC_PRE_SMOOTH_SADDLE   (default 2)                    */
  int post_smooth;        /* SC_POST_SMOOTH_SADDLE  (default 2)                    */
  double smooth_damp;     /* SC_SMOOTH_DAMP_FACTOR_COARSE_SADDLE (default 1.0)     */
  double alpha;           /* level relaxation al[0] (default 1.0)                 */
  double beta;            /* SC_GMG_DAMP_FACTOR_SADDLE, level al[1] (default 1.0) */
  int project_pressure;   /* INTERNAL_PROJECT_PRESSURE (default 1)                 */
  /* FGMRES */
  int restart;            /* SC_GMRES_RESTART                                      */
  int maxit;              /* SC_LIN_MAXIT_SADDLE                                   */
  int minit;              /* SC_MINIT                                              */
  double red_factor;      /* SC_LIN_RED_FACTOR_SADDLE (relative to res0 of the current restart cycle) */
  double res_norm_min;    /* SC_LIN_RES_NORM_MIN_SADDLE (absolute)                  */
  double div_factor;      /* SC_DIV_FACTOR                                          */
  /* runtime */
  int device;             /* CUDA device ordinal                                    */
  int use_graphs;         /* capture the V-cycle in a CUDA graph (default 1)        */
  int verbose;
  int pin_host;           /* 1: page-lock the caller's matrix value arrays in
                             pm_add_level (cudaHostRegister, as the TNSE_MGLevel4
                             ctor does, src/FE/NSE_MGLevel4.C:168-188); the
                             arrays stay registered until pm_destroy.  Off by
                             default: on Grace-coupled GPUs pageable arrays
                             copy as fast, and copies from registered memory
                             were seen to slow to 5-10 GB/s after sustained
                             GPU load                                        */
  int vanka_inverse;      /* mixed only: store each local block as its FP32
                             inverse (computed from the FP64 LU) so that the
                             sweep applies it as a GEMV; 0 (default) keeps
                             the FP32 LU factors and substitution            */
  int residual_variant;   /* local-residual kernel of the Vanka sweep:
                             0 (default) per level: row groups (8 lanes per
                             CSR row), except the flattened entry stream with
                             segmented sums on FP32 levels that read all
                             nine A blocks (faster there); 1 row groups
                             everywhere; 2 the stream everywhere; -1 time
                             both on every level at pm_setup and keep the
                             faster                                          */
  int apply_variant;      /* LU apply of nine-block levels, factor columns
                             loaded from HBM with register and L2 prefetch:
                             0 (default) per level: two cells per warp (half a
                             warp per cell) in FP64, one cell per warp in
                             FP32 (each measured faster there); 1 (FP32
                             only; FP64 levels use pairs) each cell's factors
                             staged in shared memory by bulk copies; 2 one
                             cell per warp; -1 time them per level at
                             pm_setup.  pm_level_variant reports residual
                             kernel (0 rows, 1 stream) + 2 * apply kernel
                             (0 pairs, 1 bulk, 2 single)                     */
  int upload_mode;        /* how pm_add_level / pm_update_matrices move matrix
                             values: 0 (default) copy-engine copies
                             (cudaMemcpyAsync) then device conversions; 1 the
                             SMs read the caller's arrays directly and write
                             the FP64 and FP32 copies in one pass (needs a
                             device that reads pageable host memory, e.g. a
                             Grace-coupled GPU; PM_BADARG otherwise)         */
  int red_initial;        /* 0 (default, the reference's rule): red_factor
                             applies to res0 of the current restart cycle;
                             1: to the residual at the start of the solve, so
                             that "reduce by red_factor" holds across
                             restarts (e.g. one time step solved to 1e-8)  */
  int decouple;           /* 1 (default): a nine-block level whose
                             off-diagonal blocks A12..A32 are all zero
                             (checked on the device after every upload or
                             assembly) reads only A11, A22, A33 in its
                             defects and sweeps -- only A11 when the three
                             are identical -- and its cells are solved by
                             exact block elimination (the 27x27 inverses and
                             the 4x4 pressure Schur complement) instead of
                             the 85x85 LU: the same local solution;
                             0: the 85x85 LU and all nine blocks on every
                             nine-block level, as the reference's CellVanka
                             (src/FE/NSE_MGLevel4.C:1784-2031)              */
  int wait_limit;         /* polls of the first bounded mbarrier wait of the
                             bulk-copy apply before it gives up (0: the
                             default 2^22; the wait that drains the copies
                             in flight keeps the default); a wait that gives
                             up makes the solve return PM_TIMEOUT           */
  long long max_device_bytes; /* cap on the device memory the handle
                             allocates (0: none); an allocation beyond it
                             fails with PM_OOM, as a failed cudaMalloc does  */
  int learned_levels;     /* levels that run the learned post-smoothing step,
                             counted from the finest: 1 (default) the finest
                             level only, k > 1 the k finest, 0 every
                             smoothed level                                */
} pm_options;

/* One multigrid level in the reference's data layout.  Levels are added
 * coarsest first, as TNSE_MultiGrid::AddLevel is called in
 * TSystemNSE3D::Init (src/System/SystemNSE3D.C:806-876). */
typedef struct {
  int n_udof;            /* N_U: scalar velocity DOFs (rows of A11)             */
  int n_pdof;            /* N_P: pressure DOFs                                   */
  int n_active;          /* N_Active = USpace->GetActiveBound()                  */
  int hanging_bound;     /* HangingNodeBound (== n_active: no hanging nodes)     */
  int n_dirichlet;       /* N_Dirichlet                                          */
  /* velocity blocks: shared pattern (ARowPtr/AKCol, sorted columns) */
  int a_nnz;
  const int *a_rowptr;   /* n_udof+1 */
  const int *a_col;      /* a_nnz    */
  /* A11,A12,A13,A21,A22,A23,A31,A32,A33 entries (NSTYPE 4, TNSE_MGLevel4);
   * or a[0] alone with a[1..8] NULL: one block A shared by the three
   * components and no velocity coupling (NSTYPE 2, TNSE_MGLevel2,
   * src/FE/NSE_MGLevel2.C:54-110), smoothed by the exact block solve of the
   * local system (A^{-1}, 4x4 Schur complement) */
  const double *a[9];
  /* B blocks: N_P x N_U */
  int b_nnz;
  const int *b_rowptr;   /* n_pdof+1 */
  const int *b_col;
  const double *b[3];
  /* BT blocks: N_U x N_P */
  int bt_nnz;
  const int *bt_rowptr;  /* n_udof+1 */
  const int *bt_col;
  const double *bt[3];
  /* cells: local DOF maps (UGlobalNumbers+UBeginIndex[c], PGlobalNumbers+PBeginIndex[c]) */
  int n_cells;
  int n_ulocal;          /* 27 for Q2 hexahedra */
  int n_plocal;          /* 4 for P1disc        */
  const int *cell_udofs; /* n_cells*n_ulocal    */
  const int *cell_pdofs; /* n_cells*n_plocal    */
  /* grid hierarchy (ignored on the coarsest level): parent cell on the next
   * coarser level and child number 0..7 with offset (c&1, (c>>1)&1, (c>>2)&1)
   * in the parent's reference coordinates (regular hexahedral refinement). */
  const int *cell_parent;
  const int *cell_child;
  /* optional cell colouring (no two cells of a colour share a DOF); NULL: the
   * library colours greedily, as TParFEMapper3D::colorCell does. */
  const int *cell_colour;
  /* prolongation from the next coarser level (ignored on the coarsest):
   * scalar CSR with fine rows and coarse columns, for the velocity (applied
   * to each component) and the pressure; restriction is the transpose (as
   * Prolongate / DefectRestriction are transposes in TNSE_MultiGrid).
   * Required when n_ulocal != 27; NULL (nnz 0) for Q2 hexahedra builds them
   * from the regular refinement (GetProlongationMatrix3D). */
  int pu_nnz;
  const int *pu_rowptr;  /* n_udof+1 */
  const int *pu_col;
  const double *pu_val;
  int pp_nnz;
  const int *pp_rowptr;  /* n_pdof+1 */
  const int *pp_col;
  const double *pp_val;
} pm_level_desc;

typedef struct {
  int iterations;        /* FGMRES iterations (return value of Iterate)          */
  double res0;           /* ||b - K x0||                                         */
  double res;            /* final ||b - K x|| estimate (|s[i+1]| or true at restart) */
  double true_res;       /* ||b - K x|| recomputed at exit (FP64)                */
  double setup_ms;       /* factorisation time of the last pm_setup / refactor   */
  double solve_ms;       /* device time of the FGMRES solve                      */
  int vcycles;           /* preconditioner applications                          */
  int status;            /* pm_status of the solve                               */
} pm_result;

typedef struct pm_handle pm_handle;

void        pm_default_options(pm_options *opt);
const char *pm_status_string(int status);
const char *pm_last_error(pm_handle *h);
int         pm_device_count(void);

pm_status pm_create(pm_handle **h, const pm_options *opt);
pm_status pm_add_level(pm_handle *h, const pm_level_desc *lvl);
/* Uploads every level, colours, factors the local blocks and the coarse
 * system.  Host arrays of the level descriptors are read here and may be
 * freed afterwards. */
pm_status pm_setup(pm_handle *h);
/* Replace the matrix values of every level and refactor.  The patterns must
 * be those of pm_add_level: the sizes, every row pointer and a strided
 * sample of the column indices are compared (PM_BADARG on a difference); a
 * change confined to unsampled column indices is not detected. */
pm_status pm_update_matrices(pm_handle *h, const pm_level_desc *levels, int n_levels);
pm_status pm_destroy(pm_handle *h);
/* FGMRES stopping parameters of the next solves (TItMethod::SetMaxit,
 * SetMinit, SetRedFactor, SetResNormMin, SetDivFactor, SetRestart,
 * include/FE/ItMethod.h:118-171); restart at most the value the handle was
 * set up with (PM_BADARG otherwise). */
pm_status pm_set_tolerances(pm_handle *h, int restart, int maxit, int minit, double red_factor,
                            double res_norm_min, double div_factor);
int       pm_n_levels(pm_handle *h);
int       pm_level_ndof(pm_handle *h, int level);
/* velocity blocks of a level: 9 (NSTYPE 4) or 1 (NSTYPE 2); -1 if no such level */
int       pm_level_blocks(pm_handle *h, int level);
/* How a nine-block level runs (pm_options.decouple, decided on the device
 * after every upload or assembly): 0 all nine blocks and the 85x85 LU; 1
 * A12..A32 are zero: A11, A22, A33 read, cells solved by block elimination
 * with three 27x27 inverses; 2 also A11 = A22 = A33: one block read, one
 * inverse per cell (the one-block operator's kernels).  0 for one-block
 * descriptors, -1 if no such level. */
int       pm_level_decoupled(pm_handle *h, int level);
/* kernels a level runs: residual kernel (0 row groups, 1 stream) + 2 * LU
 * apply kernel (0 two cells per warp, 1 bulk-staged, 2 one cell per warp;
 * levels without velocity coupling apply their block elimination instead);
 * -1 if no such level */
int       pm_level_variant(pm_handle *h, int level);

/* Level operators (FP64 on host vectors of length ndof(level)). */
pm_status pm_coupled_defect(pm_handle *h, int level, const double *x, const double *b,
                            double *r, int project_pressure);
pm_status pm_defect(pm_handle *h, int level, const double *u, const double *f,
                    double *d, double *res);
pm_status pm_matvec(pm_handle *h, int level, const double *x, double *y);
/* `sweeps` cell-Vanka sweeps on `level` in the handle's V-cycle precision. */
pm_status pm_cell_vanka(pm_handle *h, int level, double *u, const double *rhs, int sweeps);
/* Coarse rhs of level-1 from the fine defect of `level` (u and p parts). */
pm_status pm_restrict(pm_handle *h, int level, const double *fine, double *coarse);
/* Fine correction on `level` from a coarse vector of level-1. */
pm_status pm_prolongate(pm_handle *h, int level, const double *coarse, double *fine);
pm_status pm_solve_exact(pm_handle *h, const double *rhs, double *u);

/* One preconditioner application z = V-cycle(v) on the finest level. */
pm_status pm_vcycle(pm_handle *h, double *z, const double *v);
/* FGMRES(restart) + V-cycle to the tolerances in the options.
 * sol holds the initial guess on entry, the solution on exit. */
pm_status pm_solve(pm_handle *h, double *sol, const double *rhs, pm_result *out);
/* Same with device pointers (no vector copies); the matrices must be set up. */
pm_status pm_solve_device(pm_handle *h, double *d_sol, const double *d_rhs, pm_result *out);
/* Galerkin Oseen assembly of one level on the device, replacing the level's
 * matrix values (NSType4Galerkin3D, src/FE/NSE3D_FixPo.C:1919-2071, in the
 * cell loop of TAssembleMat3D::Assemble3D, src/System/AssembleMat3D.C:230):
 * A11 = A22 = A33 = nu (grad u, grad v) + ((b . grad) u, v), A12..A32 = 0,
 * B and BT from -(p, div v), Q2/P1disc, 4-point Gauss rule per direction;
 * Dirichlet rows get 1 on the diagonal.  Cells must be axis-aligned boxes:
 * cell_h = (hx, hy, hz) per cell (n_cells x 3), conv = [b1|b2|b3] at the
 * velocity nodes (3 x n_udof).  The level's sparsity pattern is kept; call
 * pm_refactor after assembling the levels. */
pm_status pm_assemble_level(pm_handle *h, int level, const double *cell_h, const double *conv,
                            double nu);
/* Same with device pointers (e.g. the current velocity on the device). */
pm_status pm_assemble_level_device(pm_handle *h, int level, const double *d_cell_h,
                                   const double *d_conv, double nu);
/* Time-dependent system of one level (the theta scheme of
 * TSystemTNSE3D::AssembleSystMat, src/System/SystemTNSE3D.C:1118-1274):
 * velocity blocks c_mass * M + c_a * A with the Q2 mass matrix M and the
 * Oseen block A of pm_assemble_level (A11 = A22 = A33, A12..A32 = 0), B
 * scaled by b_scale and BT by bt_scale; M and A are kept for
 * pm_system_rhs.  The reference's system matrix is c_mass = 1,
 * c_a = tau * theta1, bt_scale = scale (and b_scale = scale * the divergence
 * scaling when that is on).  Call pm_refactor after the levels. */
pm_status pm_assemble_system_level(pm_handle *h, int level, const double *cell_h,
                                   const double *conv, double nu, double c_mass, double c_a,
                                   double b_scale, double bt_scale);
pm_status pm_assemble_system_level_device(pm_handle *h, int level, const double *d_cell_h,
                                          const double *d_conv, double nu, double c_mass,
                                          double c_a, double b_scale, double bt_scale);
/* Working right-hand side of the theta scheme on the finest level (host
 * vectors of its size): out = c_old * old_rhs + c_new * rhs + (M - c2 A) sol
 * on the active velocity rows, rhs on the Dirichlet rows, 0 on the pressure
 * rows; the reference uses c_old = tau theta3, c_new = tau theta4,
 * c2 = tau theta2 (SystemTNSE3D.C:1132-1202).  Needs the finest level
 * assembled by pm_assemble_system_level. */
pm_status pm_system_rhs(pm_handle *h, const double *old_rhs, const double *rhs, const double *sol,
                        double c_old, double c_new, double c2, double *out);
/* Same with device vectors of the finest level's size (out may not alias
 * the inputs). */
pm_status pm_system_rhs_device(pm_handle *h, const double *d_old_rhs, const double *d_rhs,
                               const double *d_sol, double c_old, double c_new, double c2,
                               double *d_out);
/* Nodal values of a velocity field [u1|u2|u3] of `level` at the velocity
 * nodes of level-1 (each coarse node is a node of the nested fine mesh):
 * the convection field of the coarser levels for the assembly entry points,
 * e.g. from the current velocity in a time step.  Device vectors of
 * 3 n_udof(level) and 3 n_udof(level-1); needs cell_parent / cell_child.
 * ParMooN's RestrictFunction (src/FE/MGComponents3D.C:1243-1506) averages
 * child-wise L2 projections instead; both return the coarse function itself
 * when the fine function lies in the coarse space. */
pm_status pm_interpolate_coarse(pm_handle *h, int level, const double *d_fine, double *d_coarse);
/* Batched solves of independent systems (a batch of Oseen systems of uneven
 * size, each in its own set-up handle): pm_solve for every i < n, run
 * concurrently from up to nthreads host threads (0: one per system), so the
 * handles' streams overlap on the GPU.  The handles must be distinct.  Each
 * result equals the one pm_solve gives alone (same kernels, same order on
 * the handle's stream).  results may be NULL; returns the first non-PM_OK
 * status in index order, PM_OK if none. */
pm_status pm_solve_batch(pm_handle *const *hs, int n, double *const *sols,
                         const double *const *rhss, pm_result *results, int nthreads);
/* Fused batch: n_sys independent systems on one mesh (equal sizes on every
 * level; values, convection and viscosity may differ) stacked into one
 * block-diagonal hierarchy, so that every kernel of the V-cycle and of
 * FGMRES covers all of them in one launch.  The reference batches the cells
 * of one colour of one system per launch (CellVanka_GPU,
 * src/FE/NSE_CellVanka.cu:2181-2365; magma_dgesv_batched,
 * src/FE/Magma_Solver.C:38); here one launch covers that colour in all
 * systems.  Call pm_add_level_batch once per level (coarsest first) with the
 * n_sys descriptors of that level, instead of pm_add_level, then pm_setup.
 * Each system keeps its own L^2_0 projection, coarse inverse, Arnoldi
 * process, Givens rotations and stopping test (TFgmresIte::Iterate,
 * src/FE/FgmresIte.C:250-677, per system): results agree with pm_solve of
 * each system alone to rounding (the sums run in another order).  Systems
 * that stop early leave the sweeps.  Entry points of one system
 * (pm_solve, pm_solve_device, pm_solve_exact, pm_update_matrices, the
 * assembly and time-step entry points, the learned smoother) return
 * PM_BADARG on such a handle; the level operators and pm_vcycle act on
 * stacked vectors. */
pm_status pm_add_level_batch(pm_handle *h, const pm_level_desc *descs, int n_sys);
/* sols[s] / rhss[s]: host vectors of system s in its own layout
 * [u1|u2|u3|p]; results[s] per system (may be NULL).  Returns the first
 * non-PM_OK per-system status in index order, PM_OK if none. */
pm_status pm_solve_fused(pm_handle *h, double *const *sols, const double *const *rhss,
                         pm_result *results);
/* systems stacked in the handle (1 for a handle built by pm_add_level) */
int pm_n_systems(pm_handle *h);
/* Re-run the local-block and coarse factorisations on the device (timed into
 * out->setup_ms); used to time factor+solve with inputs resident in HBM. */
pm_status pm_refactor(pm_handle *h, double *ms);

/* Diagnostics: launches of this library's kernels since the handle was
 * created, and device bytes held. */
long long pm_kernel_launches(pm_handle *h);
long long pm_device_bytes(pm_handle *h);
/* Host bytes page-locked by pm_add_level under pin_host (0 if none took). */
long long pm_pinned_bytes(pm_handle *h);
/* Per-kernel timing of the two Vanka sweep kernels while profiling is
 * enabled: CUDA events on the handle's stream bracket every launch (the
 * V-cycle then runs without graph capture).  kernel 0 = local residual,
 * 1 = factor apply + update.  Totals since pm_profile_enable: device time
 * (ms), launches and algorithmic (unique) bytes of those launches. */
pm_status pm_profile_enable(pm_handle *h, int enable);
pm_status pm_profile_read(pm_handle *h, int kernel, double *ms_total, long long *launches,
                          double *bytes_total);

/* ---------------------------------------------------------------------------
 * Learned smoother (no counterpart in the reference: an addition to
 * TNSE_MultiGrid::Cycle's post-smoothing, src/FE/NSE_MultiGrid.C:1608-1742).
 * A per-cell MLP 397 -> 256 -> 256 -> 85 (GELU; BF16 weights/activations,
 * FP32 accumulation on the tensor cores) maps a cell's scaled local residual
 * plus 26 neighbour residual summaries (12 each) to a correction of the
 * cell's 85 DOFs.  Attached to a handle, it runs as one extra post-smoothing
 * step on the pm_options.learned_levels finest levels (default: the finest
 * only; 0: every smoothed level); FGMRES
 * switches it off for the rest of a solve when the residual reduction of an
 * iteration is worse than fallback_ratio and computes that iteration again
 * with the plain V-cycle, so plain cell Vanka is the fallback.
 * Feature vector of cell c (divided by s_c = rms of its 85 local residual
 * entries): [local residual in local DOF order (u1 nodes, u2, u3, p modes)] then,
 * for each neighbour slot n = 0..25 (offsets (dx,dy,dz) in {-1,0,1}^3 \ 0,
 * slot order dx fastest), the neighbour's summary: mean r_u1, r_u2, r_u3
 * over its 27 nodes, rms of each, its 4 pressure residuals, rms of all 85,
 * mean |r_u|.  Targets: the error at the cell's 85 DOFs divided by s_c. */
typedef struct pm_mlp pm_mlp;
enum { PM_MLP_IN = 397, PM_MLP_HIDDEN = 256, PM_MLP_OUT = 85 };

pm_status pm_mlp_create(pm_mlp **m, int device, unsigned long long seed, int max_batch);
pm_status pm_mlp_destroy(pm_mlp *m);
long long pm_mlp_num_params(void);  /* FP32 parameter vector length (padded layout) */
pm_status pm_mlp_get_params(pm_mlp *m, float *host, long long n);
pm_status pm_mlp_set_params(pm_mlp *m, const float *host, long long n);
/* d_X [M x 397] FP32 (device) -> d_Y [M x 85] FP32 (device), BF16 compute */
pm_status pm_mlp_forward(pm_mlp *m, const float *d_X, int M, float *d_Y);
/* The network's GEMMs (forward layers and the training gradients) on the
 * tcgen05 tensor cores (1, default) or on the warp-level mma.sync path (0). */
pm_status pm_mlp_set_tensor_path(pm_mlp *m, int tcgen05);
/* MSE loss of the batch and its gradient (kept in the object; copied to
 * host_grad when non-NULL, length pm_mlp_num_params()) */
pm_status pm_mlp_loss_grad(pm_mlp *m, const float *d_X, const float *d_T, int M, double *loss,
                           float *host_grad);
/* one AdamW step with the last gradient (bias-corrected moments, decoupled
 * weight decay on weights, not biases) */
pm_status pm_mlp_adamw_step(pm_mlp *m, float lr, float beta1, float beta2, float eps,
                            float weight_decay);
/* attach (m != NULL) or detach the network; omega scales the correction */
pm_status pm_learned_attach(pm_handle *h, pm_mlp *m, double omega, double fallback_ratio);
/* Training pairs from the plain solver on the finest level: starting from
 * u = 0 it runs n_cycles iterations u += Vcycle(b - K u) (the post-smoothed
 * state of the cycle) and after each stores every cell's features and
 * scaled error (sol_exact - u) into d_X [.. x 397] / d_T [.. x 85] from row
 * *n_pairs on (capacity rows); *n_pairs is advanced. */
pm_status pm_learned_harvest(pm_handle *h, const double *sol_exact, const double *rhs,
                             int n_cycles, float *d_X, float *d_T, long long capacity,
                             long long *n_pairs);
/* learned step enabled now (1/0) and fallbacks since attach */
pm_status pm_learned_status(pm_handle *h, int *enabled, int *fallbacks);

/* Diagnostic (no counterpart in the reference): the FP64 FMA rate of GPU
 * `device` in flop/s, measured by a kernel of this library (independent FMA
 * chains on every SM, CUDA events, 2 flop per FMA).  It is the compute
 * ceiling of the FP64 factorisations and of FP64 sweeps that do more FP64
 * FMA per byte than the GPU's FP64:HBM balance.  Allocates and frees a
 * small output buffer. */
pm_status pm_measure_fp64_fma(int device, double *flops_per_s);

/* Allocation-free L2_0 projection of a P1disc pressure vector on the device
 * (subtract the mean of the constant modes d_p[0], d_p[4], ...), for callers
 * that cannot allocate device memory where they need it: solvers confined to
 * an application-owned memory pool whose budget is fixed up front, and MPI
 * ranks whose GPU memory is partitioned before the time loop.  No counterpart
 * in the reference (there the projection is host code, IntoL20Vector3D); it
 * computes what pm_coupled_defect's projection computes, without a handle.
 * Its reduction scratch is a 64 KB file-scope device array held by every GPU
 * that loads the library until exit; n_p must be a multiple of 4 and at most
 * 8,388,608 (else PM_BADARG).  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress); make that first call before
 * any stream capture.  Calls share the array: calls that overlap on the GPU
 * race.  stream may be NULL (default stream).  Nothing is allocated. */
pm_status pm_l20_project_noalloc(double *d_p, int n_p, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PMGPU_H */
