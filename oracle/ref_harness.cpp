// ref_harness.cpp — drives the reference's own coupled-system kernels and
// its flexible FGMRES on a level handed over as plain CSR arrays.  TEST
// INFRASTRUCTURE ONLY: it pins the oracle's restatement (oracle.cpp:
// coupled_defect, coupled_matvec, into_l20, oracle_fgmres) against the
// reference code itself, and generates the golden vectors
// tests/golden/ref_defect_*.npz (tests/golden/make_ref_defect_golden.py).
//
// The reference translation units are compiled where they lie in the
// reference tree by oracle/build_oracle.py (build_ref_harness):
//   src/FE/MGComponents3D.C  Defect_NSE4 (:3210), MatVect_NSE4 (:3030),
//                            CoupledDefect (:3038), CoupledMatVect (:2872),
//                            the NSTYPE-2 Defect_NSE2 (:2560), MatVect_NSE2
//                            (:2439), CoupledDefect (:2446), CoupledMatVect
//                            (:2329), and IntoL20Vector3D (:1756)
//   src/FE/FgmresIte.C       TFgmresIte (constructor :75, flexible branch of
//                            Iterate :250-677, Dotprod :857, the plane
//                            rotations and UpdateGmresIterate :199-247)
//   src/FE/ItMethod.C        the TItMethod base
//   src/FE/Matrix.C, SquareMatrix.C, Structure.C, SquareStructure.C
//                            TMatrix / TSquareMatrix / TStructure /
//                            TSquareStructure constructors and accessors
//   src/FE/Blas1.C           Ddot, Daxpy, Dcopy, Dscal
// with -D__3D__ and the MKL declarations of oracle/ref_stubs/ (the MKL calls
// in Matrix.C sit on paths this harness never takes).  The library links
// with -z defs, so every symbol the kept code needs is resolved.
//
// Objects the reference owns:
// * TStructure takes ownership of the row/column arrays it is given
//   (src/FE/Structure.C:40-45, freed in ~TStructure at :90-96), so the
//   harness hands it fresh new[] copies.
// * TMatrix(TStructure*, double*) leaves its MKL members unset
//   (src/FE/Matrix.C:55-59) and ~TMatrix frees them (:126-132).  So the
//   matrices are never destroyed: a harness process builds one level, runs,
//   and exits.
// * The TItMethod constructor initialises no member (src/FE/ItMethod.C:20-24)
//   and its destructor frees the auxiliary arrays, so the FGMRES object and
//   the preconditioner are not destroyed either.
// * FGMRES calls exit(4711) when a residual exceeds div_factor times the
//   residual at the start of its restart cycle (src/FE/FgmresIte.C:564-566).
//   The GMRES residual never grows within a cycle, so a div_factor >= 1
//   keeps that branch closed.  ref_fgmres refuses a smaller one.
// * The active bound of a TSquareStructure is the row count in the
//   array constructor (src/FE/SquareStructure.C:28-32) and is a protected
//   member.  So a derived class sets it to the number of non-Dirichlet rows,
//   which the reference's own structure builder does for its velocity
//   spaces.
#include <chrono>
#include <cstring>
#include <fstream>

#include <Database.h>
#include <FgmresIte.h>
#include <ItMethod.h>
#include <LinAlg.h>
#include <Matrix.h>
#include <SquareMatrix.h>
#include <SquareStructure.h>
#include <Structure.h>

// storage of the static parameter database the kernels read
// (TDatabase::ParamDB->OMPNUMTHREADS, INTERNAL_PROJECT_PRESSURE,
// INTERNAL_PRESSURE_SPACE, the SC_* solver entries) and of the log stream
// the reference's headers name
static TParamDB g_param;
TParamDB *TDatabase::ParamDB = &g_param;
std::ofstream OutFile;
// the smoother timer FgmresIte.C prints (defined in src/FE/NSE_MultiGrid.C,
// which is not compiled here) and the wall clock of src/General/MainUtilities.C
double tSmoother2 = 0.0;
double GetTime() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

namespace {

struct ActiveStructure : public TSquareStructure {
  ActiveStructure(int n, int n_active, int nnz, int *col, int *rowptr)
      : TSquareStructure(n, nnz, col, rowptr) {
    ActiveBound = n_active;
  }
};

template <class T>
T *copy_of(const T *src, long n) {
  T *d = new T[n > 0 ? n : 1];
  if (n > 0) std::memcpy(d, src, sizeof(T) * n);
  return d;
}

struct Level {
  TSquareMatrix *A[9];
  TMatrix *B[6];  // B1, B2, B3 (pressure rows), B1T, B2T, B3T (velocity rows)
};

// n_a = 9 (NSTYPE 4: A11..A33) or 1 (NSTYPE 2: one A for all components)
Level make_level(int n_u, int n_active, int n_p, const int *a_rowptr, const int *a_col,
                 const double *const *a, const int *b_rowptr, const int *b_col,
                 const double *const *b, const int *bt_rowptr, const int *bt_col,
                 const double *const *bt, int n_a = 9) {
  Level L{};
  const int a_nnz = a_rowptr[n_u], b_nnz = b_rowptr[n_p], bt_nnz = bt_rowptr[n_u];
  TSquareStructure *sa = new ActiveStructure(n_u, n_active, a_nnz, copy_of(a_col, a_nnz),
                                             copy_of(a_rowptr, n_u + 1L));
  for (int k = 0; k < n_a; ++k) {
    L.A[k] = new TSquareMatrix(sa);
    std::memcpy(L.A[k]->GetEntries(), a[k], sizeof(double) * a_nnz);
  }
  TStructure *sb = new TStructure(n_p, n_u, b_nnz, copy_of(b_col, b_nnz),
                                  copy_of(b_rowptr, n_p + 1L));
  TStructure *sbt = new TStructure(n_u, n_p, bt_nnz, copy_of(bt_col, bt_nnz),
                                   copy_of(bt_rowptr, n_u + 1L));
  for (int k = 0; k < 3; ++k) {
    L.B[k] = new TMatrix(sb, copy_of(b[k], b_nnz));
    L.B[3 + k] = new TMatrix(sbt, copy_of(bt[k], bt_nnz));
  }
  return L;
}

// A preconditioner given as a C function z = M^{-1} v (z starts at zero, as
// FGMRES clears it before prec->Iterate, src/FE/FgmresIte.C:372-389).
typedef void (*prec_fn)(void *ctx, double *z, const double *v);

struct CallbackPrec : public TItMethod {
  prec_fn fn;
  void *ctx;
  CallbackPrec(prec_fn f, void *c, int n) : TItMethod(nullptr, nullptr, nullptr, 0, n), fn(f), ctx(c) {}
  int Iterate(TSquareMatrix **, TMatrix **, double *sol, double *rhs) override {
    fn(ctx, sol, rhs);
    return 1;
  }
};

void set_params(int threads, int project) {
  std::memset(&g_param, 0, sizeof(g_param));
  g_param.OMPNUMTHREADS = threads > 0 ? threads : 1;
  g_param.INTERNAL_PROJECT_PRESSURE = project;
  g_param.INTERNAL_PRESSURE_SPACE = -11;  // P1disc on hexahedra
}

}  // namespace

extern "C" {

// r = b - K x through Defect_NSE4, with the reference's own pressure
// projection when project != 0.  a[9], b[3], bt[3] are the value arrays of
// the shared A pattern, the B pattern (pressure rows) and the BT pattern
// (velocity rows); Dirichlet velocity rows are the last n_u - n_active.
__attribute__((visibility("default"))) void ref_defect_nse4(
    int n_u, int n_active, int n_p, const int *a_rowptr, const int *a_col,
    const double *const *a, const int *b_rowptr, const int *b_col, const double *const *b,
    const int *bt_rowptr, const int *bt_col, const double *const *bt, const double *x,
    const double *rhs, double *r, int project, int threads) {
  set_params(threads, project);
  Level L = make_level(n_u, n_active, n_p, a_rowptr, a_col, a, b_rowptr, b_col, b, bt_rowptr,
                       bt_col, bt);
  const long n = 3L * n_u + n_p;
  double *xx = copy_of(x, n), *bb = copy_of(rhs, n);
  Defect_NSE4(L.A, L.B, xx, bb, r);
  delete[] xx;
  delete[] bb;
}

// y = K x through MatVect_NSE4
__attribute__((visibility("default"))) void ref_matvec_nse4(
    int n_u, int n_active, int n_p, const int *a_rowptr, const int *a_col,
    const double *const *a, const int *b_rowptr, const int *b_col, const double *const *b,
    const int *bt_rowptr, const int *bt_col, const double *const *bt, const double *x, double *y,
    int threads) {
  set_params(threads, 0);
  Level L = make_level(n_u, n_active, n_p, a_rowptr, a_col, a, b_rowptr, b_col, b, bt_rowptr,
                       bt_col, bt);
  double *xx = copy_of(x, 3L * n_u + n_p);
  MatVect_NSE4(L.A, L.B, xx, y);
  delete[] xx;
}

// The NSTYPE-2 pair: r = b - K x through Defect_NSE2 (projection as above)
// or y = K x through MatVect_NSE2 (when rhs is null), with a[0] the one A
// matrix of all three velocity components.
__attribute__((visibility("default"))) void ref_nse2(
    int n_u, int n_active, int n_p, const int *a_rowptr, const int *a_col,
    const double *const *a, const int *b_rowptr, const int *b_col, const double *const *b,
    const int *bt_rowptr, const int *bt_col, const double *const *bt, const double *x,
    const double *rhs, double *out, int project, int threads) {
  set_params(threads, project);
  Level L = make_level(n_u, n_active, n_p, a_rowptr, a_col, a, b_rowptr, b_col, b, bt_rowptr,
                       bt_col, bt, 1);
  const long n = 3L * n_u + n_p;
  double *xx = copy_of(x, n);
  if (rhs) {
    double *bb = copy_of(rhs, n);
    Defect_NSE2(L.A, L.B, xx, bb, out);
    delete[] bb;
  } else {
    MatVect_NSE2(L.A, L.B, xx, out);
  }
  delete[] xx;
}

// Flexible FGMRES of the reference (TFgmresIte::Iterate) on the level's
// system with the preconditioner prec(ctx, z, v), from the iterate in sol
// (overwritten).  The stopping parameters are those of the SC_* saddle-point
// entries of the parameter database.  Returns the iteration count the
// reference returns, or -1 when div_factor < 1 (refused, see above).
__attribute__((visibility("default"))) int ref_fgmres(
    int n_u, int n_active, int n_p, const int *a_rowptr, const int *a_col,
    const double *const *a, const int *b_rowptr, const int *b_col, const double *const *b,
    const int *bt_rowptr, const int *bt_col, const double *const *bt, double *sol,
    const double *rhs, int restart, int maxit, int minit, double red_factor,
    double res_norm_min, double div_factor, int project, prec_fn prec, void *ctx,
    int threads) {
  if (!(div_factor >= 1.0) || !prec) return -1;
  set_params(threads, project);
  g_param.SC_LIN_RES_NORM_MIN_SADDLE = res_norm_min;
  g_param.SC_LIN_RED_FACTOR_SADDLE = red_factor;
  g_param.SC_LIN_MAXIT_SADDLE = maxit;
  g_param.SC_AMG_PREC_IT = 1;
  g_param.SC_DIV_FACTOR = div_factor;
  g_param.SC_MINIT = minit;
  g_param.SC_GMRES_RESTART = restart;
  g_param.SC_VERBOSE = -1;
  g_param.SC_FLEXIBLE_KRYLOV_SPACE_SOLVER = 1;
  Level L = make_level(n_u, n_active, n_p, a_rowptr, a_col, a, b_rowptr, b_col, b, bt_rowptr,
                       bt_col, bt);
  const int n = 3 * n_u + n_p;
  TItMethod *M = new CallbackPrec(prec, ctx, n);
  TFgmresIte *G = new TFgmresIte(MatVect_NSE4, Defect_NSE4, M, 0, n, 0);
  double *bb = copy_of(rhs, n);
  const int it = G->Iterate(L.A, L.B, sol, bb);
  delete[] bb;
  return it;
}

// in-place IntoL20Vector3D(v, len, order)
__attribute__((visibility("default"))) void ref_into_l20(double *v, int len, int order) {
  IntoL20Vector3D(v, len, order);
}

}  // extern "C"
