// ref_harness.cpp — drives the reference's own coupled-system kernels and
// its flexible FGMRES on a level handed over as plain CSR arrays.  TEST
// INFRASTRUCTURE ONLY: it pins the oracle's restatement (oracle.cpp:
// coupled_defect, coupled_matvec, into_l20, oracle_fgmres) against the
// reference code itself, and generates the golden vectors
// tests/golden/ref_defect_*.npz (tests/golden/make_ref_golden.py).
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
// Lifetimes.  No reference destructor runs here:
// * ~TMatrix frees MKL members that TMatrix(TStructure*, double*) leaves
//   unset (src/FE/Matrix.C:55-59, :126-132).
// * ~TItMethod reads N_Aux, which the TItMethod constructor leaves unset
//   (src/FE/ItMethod.C:20-30).
// * ~TFgmresIte frees new[] arrays with plain delete (src/FE/FgmresIte.C:178-195).
// So the matrices and solver objects are built by placement new in storage
// the harness owns.  The harness frees what they allocated with the matching
// delete[]: the matrices' entry arrays, and FGMRES's work arrays through a
// derived class.  TStructure takes ownership of the row/column arrays it is
// given (src/FE/Structure.C:40-45), and ~TStructure (:90-96) frees them with
// delete[], so the structures are deleted normally.
// Other reference behaviour the harness works around:
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
#include <new>

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

// One level as the reference's matrix objects: A11..A33 on one square
// structure with the active bound, B1..B3 (pressure rows) on one structure,
// B1T..B3T (velocity rows) on another.
struct Level {
  ActiveStructure *sa = nullptr;
  TStructure *sb = nullptr, *sbt = nullptr;
  alignas(TSquareMatrix) unsigned char a_store[9][sizeof(TSquareMatrix)];
  alignas(TMatrix) unsigned char b_store[6][sizeof(TMatrix)];
  TSquareMatrix *A[9] = {};
  TMatrix *B[6] = {};
  int n = 0;
};

// A preconditioner given as a C function z = M^{-1} v (z starts at zero, as
// FGMRES clears it before prec->Iterate, src/FE/FgmresIte.C:372-389).
typedef void (*prec_fn)(void *ctx, double *z, const double *v);

struct CallbackPrec : public TItMethod {
  prec_fn fn;
  void *ctx;
  CallbackPrec(prec_fn f, void *c, int n) : TItMethod(nullptr, nullptr, nullptr, 0, n), fn(f), ctx(c) {
    N_Aux = 0;
    N_DOF = n;
  }
  int Iterate(TSquareMatrix **, TMatrix **, double *sol, double *rhs) override {
    fn(ctx, sol, rhs);
    return 1;
  }
};

// TFgmresIte with its work arrays released by delete[] (their allocation,
// src/FE/FgmresIte.C:135-157); never destroyed through ~TFgmresIte.
struct OwnedFgmres : public TFgmresIte {
  using TFgmresIte::TFgmresIte;
  void release() {
    delete[] s;
    delete[] cosi;
    delete[] sn;
    delete[] H[0];
    delete[] H;
    delete[] v[0];
    delete[] v;
    delete[] zv[0];
    delete[] zv;
    delete[] defect;
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

// Build a level from CSR arrays: a[9], b[3], bt[3] are the value arrays of
// the shared A pattern, the B pattern (pressure rows) and the BT pattern
// (velocity rows); Dirichlet velocity rows are the last n_u - n_active.
// Everything is copied.
__attribute__((visibility("default"))) void *ref_level_create(
    int n_u, int n_active, int n_p, const int *a_rowptr, const int *a_col,
    const double *const *a, const int *b_rowptr, const int *b_col, const double *const *b,
    const int *bt_rowptr, const int *bt_col, const double *const *bt) {
  Level *L = new Level;
  L->n = 3 * n_u + n_p;
  const int a_nnz = a_rowptr[n_u], b_nnz = b_rowptr[n_p], bt_nnz = bt_rowptr[n_u];
  L->sa = new ActiveStructure(n_u, n_active, a_nnz, copy_of(a_col, a_nnz),
                              copy_of(a_rowptr, n_u + 1L));
  for (int k = 0; k < 9; ++k) {
    L->A[k] = new (L->a_store[k]) TSquareMatrix(L->sa);  // allocates its entries
    std::memcpy(L->A[k]->GetEntries(), a[k], sizeof(double) * a_nnz);
  }
  L->sb = new TStructure(n_p, n_u, b_nnz, copy_of(b_col, b_nnz), copy_of(b_rowptr, n_p + 1L));
  L->sbt = new TStructure(n_u, n_p, bt_nnz, copy_of(bt_col, bt_nnz),
                          copy_of(bt_rowptr, n_u + 1L));
  for (int k = 0; k < 3; ++k) {
    L->B[k] = new (L->b_store[k]) TMatrix(L->sb, copy_of(b[k], b_nnz));
    L->B[3 + k] = new (L->b_store[3 + k]) TMatrix(L->sbt, copy_of(bt[k], bt_nnz));
  }
  return L;
}

__attribute__((visibility("default"))) void ref_level_destroy(void *h) {
  Level *L = static_cast<Level *>(h);
  if (!L) return;
  for (int k = 0; k < 9; ++k) delete[] L->A[k]->GetEntries();
  for (int k = 0; k < 6; ++k) delete[] L->B[k]->GetEntries();
  delete L->sa;
  delete L->sb;
  delete L->sbt;
  delete L;
}

// r = b - K x through Defect_NSE4 (nstype 4) or Defect_NSE2 (nstype 2: A11
// as the one A matrix of all three velocity components), with the
// reference's own pressure projection when project != 0.
__attribute__((visibility("default"))) void ref_defect(void *h, int nstype, const double *x,
                                                       const double *rhs, double *r,
                                                       int project, int threads) {
  Level *L = static_cast<Level *>(h);
  set_params(threads, project);
  double *xx = copy_of(x, L->n), *bb = copy_of(rhs, L->n);
  if (nstype == 2)
    Defect_NSE2(L->A, L->B, xx, bb, r);
  else
    Defect_NSE4(L->A, L->B, xx, bb, r);
  delete[] xx;
  delete[] bb;
}

// y = K x through MatVect_NSE4 (nstype 4) or MatVect_NSE2 (nstype 2)
__attribute__((visibility("default"))) void ref_matvec(void *h, int nstype, const double *x,
                                                       double *y, int threads) {
  Level *L = static_cast<Level *>(h);
  set_params(threads, 0);
  double *xx = copy_of(x, L->n);
  if (nstype == 2)
    MatVect_NSE2(L->A, L->B, xx, y);
  else
    MatVect_NSE4(L->A, L->B, xx, y);
  delete[] xx;
}

// Flexible FGMRES of the reference (TFgmresIte::Iterate with Defect_NSE4 /
// MatVect_NSE4) on the level's system with the preconditioner
// prec(ctx, z, v), from the iterate in sol (overwritten).  The stopping
// parameters are those of the SC_* saddle-point entries of the parameter
// database.  Returns the iteration count the reference returns, or -1 when
// div_factor < 1 (refused, see above).
__attribute__((visibility("default"))) int ref_fgmres(void *h, double *sol, const double *rhs,
                                                      int restart, int maxit, int minit,
                                                      double red_factor, double res_norm_min,
                                                      double div_factor, int project,
                                                      prec_fn prec, void *ctx, int threads) {
  if (!(div_factor >= 1.0) || !prec) return -1;
  Level *L = static_cast<Level *>(h);
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
  alignas(CallbackPrec) unsigned char m_store[sizeof(CallbackPrec)];
  alignas(OwnedFgmres) unsigned char g_store[sizeof(OwnedFgmres)];
  CallbackPrec *M = new (m_store) CallbackPrec(prec, ctx, L->n);
  OwnedFgmres *G = new (g_store) OwnedFgmres(MatVect_NSE4, Defect_NSE4, M, 0, L->n, 0);
  double *bb = copy_of(rhs, L->n);
  const int it = G->Iterate(L->A, L->B, sol, bb);
  delete[] bb;
  G->release();
  return it;
}

// in-place IntoL20Vector3D(v, len, order)
__attribute__((visibility("default"))) void ref_into_l20(double *v, int len, int order) {
  IntoL20Vector3D(v, len, order);
}

}  // extern "C"
