// ref_vanka.cpp — runs the reference's own cell Vanka smoother on a level
// handed over as plain arrays.  TEST INFRASTRUCTURE ONLY: it pins the
// oracle's cell_vanka against the reference code itself.
// Linked into oracle/_ref/libref_harness.so with ref_harness.cpp by
// oracle/build_oracle.py (build_ref_harness), with -D__3D__ -D_SEQ (the
// reference's sequential build; the _SEQ cell loop is the one the oracle's
// sequential mode restates), and a second time into
// oracle/_ref/libref_hybrid.so (build_ref_hybrid) with -D_HYBRID instead:
// the reference's colour-parallel CellVanka (src/FE/NSE_MGLevel4.C:603-1651),
// which per colour assembles every cell's local system and right-hand side
// from the current iterate in an OpenMP loop, then solves them and adds the
// damped corrections (cells of one colour share no DOF), colour after
// colour: the ordering of the oracle's colour mode and of the GPU sweeps.
// Its colouring (ptrCellColors / CellReorder, normally from the MPI build's
// TParFEMapper3D) is set by ref_vanka_set_colours; ref_hybrid_mapper.h says
// how the constructor is compiled without that mapper.
//
// Reference code that runs here:
//   src/FE/NSE_MGLevel4.C    TNSE_MGLevel4 constructor (:119-328), the _SEQ
//                            CellVanka (:1653-2087): local 85x85 (or 49x49)
//                            systems from the global matrices, the direct
//                            local solve, the damped update, the relaxation
//                            and the Dirichlet values; and SolveExact
//                            (:5728-5847), the dense coarse solve
//   src/FE/NSE_MGLevel.C     TNSE_MGLevel constructor, SetHangingNodes
//   src/FE/FESpace.C, FESpace3D.C, src/Geometry/Collection.C, src/FE/FE3D.C,
//   SquareStructure3D.C, SquareMatrix3D.C, Matrix3D.C, Structure3D.C
//                            the space, collection, element and matrix
//                            objects the level reads through
//   src/FE/LinAlg.C          SolveLinearSystemLapack (:106-131)
//
// What the harness supplies instead of the mesh and FE machinery:
// * LevelSpace (ref_level_space.h): a TFESpace3D filled from the level's
//   arrays.  The collection's cell array holds null
//   pointers: code on this path reads the array but no cell.
// * TFEDatabase3D::FEs3D: storage for the element table, whose two used
//   entries are registered (RegisterFE3D) as elements with 27 (or 15) and 4
//   local DOFs (TFE3D::GetN_DOF is all the level asks of them).
// * LevelStructure: a TStructure3D built from two spaces on different
//   collections, for which its constructor returns at once
//   (src/FE/Structure3D.C:43-46), then given the B / BT pattern and the
//   level's spaces.
// * dgetrf_ / dgetrs_ (called by SolveLinearSystemLapack): LAPACK's
//   unblocked right-looking LU with partial pivoting (first maximal |a|,
//   multipliers scaled by the reciprocal of the pivot) and the two
//   triangular solves.  The arithmetic is the same as the oracle's
//   lu_factor / lu_solve.  The reference links MKL, whose blocking rounds
//   differently, so the rounding of LAPACK itself is not pinned here (the
//   oracle's LU is checked against scipy's LAPACK instead).
// * DirectSolver, which SolveExact calls, stops the process if reached (it
//   is not).  The Magma_Solver of the level exists only in CUDA builds.
// As in ref_harness.cpp, no reference destructor runs.  The level lives in
// storage the harness owns, and the harness frees what it allocated.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include <Collection.h>
#include <Database.h>
#include <DirectSolver.h>
#include <FE3D.h>
#include <FEDatabase3D.h>
#include <FESpace3D.h>
#include <Matrix3D.h>
#include <NSE_MGLevel2.h>
#include <NSE_MGLevel4.h>  // includes Magma_Solver.h (no include guard)
#include <SquareMatrix3D.h>
#include <SquareStructure3D.h>
#include <Structure3D.h>

#include "ref_level_space.h"

TFE3D *TFEDatabase3D::FEs3D[N_FEs3D] = {nullptr};

void DirectSolver(TSquareMatrix3D *, TSquareMatrix3D *, TSquareMatrix3D *, TSquareMatrix3D *,
                  TSquareMatrix3D *, TSquareMatrix3D *, TSquareMatrix3D *, TSquareMatrix3D *,
                  TSquareMatrix3D *, TMatrix3D *, TMatrix3D *, TMatrix3D *, TMatrix3D *,
                  TMatrix3D *, TMatrix3D *, double *, double *, int) {
  std::fprintf(stderr, "ref_vanka: DirectSolver is not part of the harness\n");
  std::abort();
}

#include "ref_lapack.h"

namespace {

struct FixedElement : public TFE3D {
  explicit FixedElement(int n_dof) : TFE3D() { N_DOF = n_dof; }
};

// element ids the level's spaces name (any two distinct ids serve)
const FE3D kVelocityElement = C_Q2_3D_H_A;
const FE3D kPressureElement = D_P1_3D_H_A;

struct Level : public TNSE_MGLevel4 {
  using TNSE_MGLevel4::TNSE_MGLevel4;
  // the auxiliary vectors of the constructor (src/FE/NSE_MGLevel4.C:274-278);
  // its Magma_Solver is created only in CUDA builds (:305-307)
  void release() {
    delete[] Aux[0];
    delete[] Aux;
  }
#ifdef _HYBRID
  // the colouring the colour-parallel CellVanka walks (the members the
  // constructor takes from TParFEMapper3D, src/FE/NSE_MGLevel4.C:315-324)
  void set_colours(int n_colours, int *colour_ptr, int *cell_order, int max_cells) {
    N_CIntCell = n_colours;
    ptrCellColors = colour_ptr;
    CellReorder = cell_order;
    maxCellsPerColor = max_cells;
  }
#endif
};

// NSTYPE-2 level (src/FE/NSE_MGLevel2.C): one velocity block A for the
// three components; the same auxiliary vectors (:131-135)
struct Level2 : public TNSE_MGLevel2 {
  using TNSE_MGLevel2::TNSE_MGLevel2;
  void release() {
    delete[] Aux[0];
    delete[] Aux;
  }
};

template <class T>
T *copy_of(const T *src, long n) {
  T *d = new T[n > 0 ? n : 1];
  if (n > 0) std::memcpy(d, src, sizeof(T) * n);
  return d;
}

struct VankaLevel {
  int n_u = 0, n_p = 0, n = 0;
  TCollection *coll = nullptr, *other_a = nullptr, *other_b = nullptr;
  int *u_global = nullptr, *u_begin = nullptr, *p_global = nullptr, *p_begin = nullptr;
  FE3D *u_all = nullptr, *p_all = nullptr;
  alignas(LevelSpace) unsigned char us_store[sizeof(LevelSpace)];
  alignas(LevelSpace) unsigned char ps_store[sizeof(LevelSpace)];
  alignas(LevelSpace) unsigned char oa_store[sizeof(LevelSpace)];
  alignas(LevelSpace) unsigned char ob_store[sizeof(LevelSpace)];
  LevelSpace *us = nullptr, *ps = nullptr, *oa = nullptr, *ob = nullptr;
  LevelSquareStructure *sa = nullptr;
  LevelStructure *sb = nullptr, *sbt = nullptr;
  alignas(TSquareMatrix3D) unsigned char a_store[9][sizeof(TSquareMatrix3D)];
  alignas(TMatrix3D) unsigned char b_store[6][sizeof(TMatrix3D)];
  TSquareMatrix3D *A[9] = {};
  TMatrix3D *B[6] = {};
  double *f = nullptr, *u = nullptr, *aux = nullptr;
  double al[2] = {1.0, 1.0};
  alignas(Level) unsigned char level_store[sizeof(Level)];
  Level *level = nullptr;
  alignas(Level2) unsigned char level2_store[sizeof(Level2)];
  Level2 *level2 = nullptr;  // NSTYPE-2 levels (ref_vanka2_create)
  TNSE_MGLevel *base = nullptr;
  int n_blocks = 9;
  int *colour_ptr = nullptr, *cell_order = nullptr;  // colour-parallel build only
  int threads = 1;
};

FixedElement *element_of(int n_dof) {
  static FixedElement e27(27), e15(15), e4(4);
  return n_dof == 27 ? &e27 : n_dof == 15 ? &e15 : &e4;
}

}  // namespace

#ifdef _HYBRID
RefHybridMapper *ref_hybrid_mapper() {
  static RefHybridMapper none;
  return &none;
}
#endif

extern "C" {

// Build the level: n_cells cells of nu_loc (27 or 15) velocity and 4
// pressure DOFs (cell_udofs, cell_pdofs), the CSR arrays as for
// ref_level_create, and the relaxation alpha of the level (al[0] of the
// TNSE_MGLevel4 constructor).  Returns null for an unsupported nu_loc.
}  // extern "C"

namespace {

VankaLevel *make_vanka_level(int n_blocks, int n_u, int n_active, int n_p, int n_cells,
                             int nu_loc, const int *cell_udofs, const int *cell_pdofs,
                             const int *a_rowptr, const int *a_col, const double *const *a,
                             const int *b_rowptr, const int *b_col, const double *const *b,
                             const int *bt_rowptr, const int *bt_col, const double *const *bt,
                             double alpha) {
  if (nu_loc != 27 && nu_loc != 15) return nullptr;
  VankaLevel *V = new VankaLevel;
  V->n_blocks = n_blocks;
  V->n_u = n_u;
  V->n_p = n_p;
  V->n = 3 * n_u + n_p;
  TFEDatabase3D::RegisterFE3D(kVelocityElement, element_of(nu_loc));
  TFEDatabase3D::RegisterFE3D(kPressureElement, element_of(4));
  // a cell array of null pointers: GetCell reads the array, and nothing on
  // this path reads a cell (~TCollection frees the array with delete[])
  V->coll = new TCollection(n_cells, new TBaseCell *[n_cells > 0 ? n_cells : 1]());
  V->other_a = new TCollection(0, nullptr);
  V->other_b = new TCollection(0, nullptr);
  V->u_global = copy_of(cell_udofs, (long)n_cells * nu_loc);
  V->p_global = copy_of(cell_pdofs, 4L * n_cells);
  V->u_begin = new int[n_cells + 1];
  V->p_begin = new int[n_cells + 1];
  V->u_all = new FE3D[n_cells > 0 ? n_cells : 1];
  V->p_all = new FE3D[n_cells > 0 ? n_cells : 1];
  for (int c = 0; c <= n_cells; ++c) {
    V->u_begin[c] = nu_loc * c;
    V->p_begin[c] = 4 * c;
  }
  for (int c = 0; c < n_cells; ++c) {
    V->u_all[c] = kVelocityElement;
    V->p_all[c] = kPressureElement;
  }
  V->us = new (V->us_store)
      LevelSpace(V->coll, n_u, n_active, n_u - n_active, V->u_global, V->u_begin, V->u_all);
  V->ps = new (V->ps_store) LevelSpace(V->coll, n_p, n_p, 0, V->p_global, V->p_begin, V->p_all);
  V->oa = new (V->oa_store) LevelSpace(V->other_a, 0, 0, 0, nullptr, nullptr, nullptr);
  V->ob = new (V->ob_store) LevelSpace(V->other_b, 0, 0, 0, nullptr, nullptr, nullptr);
  const int a_nnz = a_rowptr[n_u], b_nnz = b_rowptr[n_p], bt_nnz = bt_rowptr[n_u];
  V->sa = new LevelSquareStructure(n_u, n_active, a_nnz, copy_of(a_col, a_nnz),
                                   copy_of(a_rowptr, n_u + 1L), V->us);
  V->sb = new LevelStructure(V->oa, V->ob, V->ps, V->us, n_p, n_u, b_nnz, copy_of(b_col, b_nnz),
                             copy_of(b_rowptr, n_p + 1L));
  V->sbt = new LevelStructure(V->oa, V->ob, V->us, V->ps, n_u, n_p, bt_nnz,
                              copy_of(bt_col, bt_nnz), copy_of(bt_rowptr, n_u + 1L));
  for (int k = 0; k < n_blocks; ++k) {
    V->A[k] = new (V->a_store[k]) TSquareMatrix3D(V->sa);  // allocates its entries
    std::memcpy(V->A[k]->GetEntries(), a[k], sizeof(double) * a_nnz);
  }
  for (int k = 0; k < 3; ++k) {
    V->B[k] = new (V->b_store[k]) TMatrix3D(V->sb);
    std::memcpy(V->B[k]->GetEntries(), b[k], sizeof(double) * b_nnz);
    V->B[3 + k] = new (V->b_store[3 + k]) TMatrix3D(V->sbt);
    std::memcpy(V->B[3 + k]->GetEntries(), bt[k], sizeof(double) * bt_nnz);
  }
  V->f = new double[V->n]();
  V->u = new double[V->n]();
  V->aux = new double[V->n]();
  V->al[0] = alpha;
  if (n_blocks == 9) {
    V->level = new (V->level_store)
        Level(0, V->A[0], V->A[1], V->A[2], V->A[3], V->A[4], V->A[5], V->A[6], V->A[7],
              V->A[8], V->B[0], V->B[1], V->B[2], V->B[3], V->B[4], V->B[5], V->f, V->u, 1,
              V->al, 0, 0, V->coll, nullptr);
    V->base = V->level;
  } else {
    V->level2 = new (V->level2_store)
        Level2(0, V->A[0], V->B[0], V->B[1], V->B[2], V->B[3], V->B[4], V->B[5], V->f, V->u, 1,
               V->al, 0, 0, V->coll, nullptr);
    V->base = V->level2;
  }
  return V;
}

}  // namespace

extern "C" {

__attribute__((visibility("default"))) void *ref_vanka_create(
    int n_u, int n_active, int n_p, int n_cells, int nu_loc, const int *cell_udofs,
    const int *cell_pdofs, const int *a_rowptr, const int *a_col, const double *const *a,
    const int *b_rowptr, const int *b_col, const double *const *b, const int *bt_rowptr,
    const int *bt_col, const double *const *bt, double alpha) {
  return make_vanka_level(9, n_u, n_active, n_p, n_cells, nu_loc, cell_udofs, cell_pdofs,
                          a_rowptr, a_col, a, b_rowptr, b_col, b, bt_rowptr, bt_col, bt, alpha);
}

// The same level as NSTYPE 2 (TNSE_MGLevel2, src/FE/NSE_MGLevel2.C:43-146):
// a[0] is the one velocity block of the three components; its CellVanka
// (:336-700) builds the 85x85 (49x49) system with that block on the three
// diagonal positions and solves it as the NSTYPE-4 one does.
__attribute__((visibility("default"))) void *ref_vanka2_create(
    int n_u, int n_active, int n_p, int n_cells, int nu_loc, const int *cell_udofs,
    const int *cell_pdofs, const int *a_rowptr, const int *a_col, const double *const *a,
    const int *b_rowptr, const int *b_col, const double *const *b, const int *bt_rowptr,
    const int *bt_col, const double *const *bt, double alpha) {
  return make_vanka_level(1, n_u, n_active, n_p, n_cells, nu_loc, cell_udofs, cell_pdofs,
                          a_rowptr, a_col, a, b_rowptr, b_col, b, bt_rowptr, bt_col, bt, alpha);
}

__attribute__((visibility("default"))) void ref_vanka_destroy(void *h) {
  VankaLevel *V = static_cast<VankaLevel *>(h);
  if (!V) return;
  if (V->level) V->level->release();
  if (V->level2) V->level2->release();
  for (int k = 0; k < V->n_blocks; ++k) delete[] V->A[k]->GetEntries();
  for (int k = 0; k < 6; ++k) delete[] V->B[k]->GetEntries();
  delete V->sa;
  delete V->sb;
  delete V->sbt;
  for (LevelSpace *s : {V->us, V->ps, V->oa, V->ob}) s->release_names();
  delete[] V->u_global;
  delete[] V->p_global;
  delete[] V->u_begin;
  delete[] V->p_begin;
  delete[] V->u_all;
  delete[] V->p_all;
  delete V->coll;
  delete V->other_a;
  delete V->other_b;
  delete[] V->f;
  delete[] V->u;
  delete[] V->aux;
  delete[] V->colour_ptr;
  delete[] V->cell_order;
  delete V;
}

#ifdef _HYBRID
// The colouring of the colour-parallel CellVanka: colour k holds the cells
// cell_order[colour_ptr[k] .. colour_ptr[k+1]-1] (no two sharing a DOF),
// solved by `threads` OpenMP threads (OMPNUMTHREADS; the result does not
// depend on it).  Returns 0, or -1 for an inconsistent colouring.
__attribute__((visibility("default"))) int ref_vanka_set_colours(void *h, int n_colours,
                                                                 const int *colour_ptr,
                                                                 const int *cell_order,
                                                                 int n_cells, int threads) {
  VankaLevel *V = static_cast<VankaLevel *>(h);
  if (!V->level || n_colours <= 0 || colour_ptr[0] != 0 || colour_ptr[n_colours] != n_cells ||
      threads <= 0)
    return -1;
  int max_cells = 0;
  for (int k = 0; k < n_colours; ++k) {
    const int m = colour_ptr[k + 1] - colour_ptr[k];
    if (m <= 0) return -1;
    if (m > max_cells) max_cells = m;
  }
  delete[] V->colour_ptr;
  delete[] V->cell_order;
  V->colour_ptr = copy_of(colour_ptr, n_colours + 1L);
  V->cell_order = copy_of(cell_order, (long)n_cells);
  V->threads = threads;
  V->level->set_colours(n_colours, V->colour_ptr, V->cell_order, max_cells);
  return 0;
}
#endif

// sweeps x TNSE_MGLevel4::CellVanka(u, rhs, aux, 0, NULL, 2, 1) with the
// damping SC_SMOOTH_DAMP_FACTOR_COARSE_SADDLE = damp and direct local
// solves (SC_LARGEST_DIRECT_SOLVE above the local size); u is updated.
__attribute__((visibility("default"))) void ref_vanka_sweeps(void *h, double *u,
                                                             const double *rhs, int sweeps,
                                                             double damp) {
  VankaLevel *V = static_cast<VankaLevel *>(h);
  TParamDB *db = TDatabase::ParamDB;
  db->SC_SMOOTH_DAMP_FACTOR_COARSE_SADDLE = damp;
  db->SC_LARGEST_DIRECT_SOLVE = 1 << 20;
  db->INTERNAL_LOCAL_DOF = -1;
#ifdef _HYBRID
  if (V->level && !V->colour_ptr) return;  // no colouring set: nothing to sweep
  db->OMPNUMTHREADS = V->threads;
#endif
  double *r = copy_of(rhs, V->n);
  for (int s = 0; s < sweeps; ++s) V->base->CellVanka(u, r, V->aux, 0, nullptr, 2, 1);
  delete[] r;
}

// TNSE_MGLevel4::SolveExact(u, rhs) (src/FE/NSE_MGLevel4.C:5728-5847): the
// level's full system as a dense matrix, solved by SolveLinearSystemLapack;
// u is overwritten.  With pin_pressure (INTERNAL_PROJECT_PRESSURE) the first
// pressure equation becomes p_0 = 0 (:5822-5832), as in the solver's runs.
__attribute__((visibility("default"))) void ref_vanka_solve_exact(void *h, double *u,
                                                                  const double *rhs,
                                                                  int pin_pressure) {
  VankaLevel *V = static_cast<VankaLevel *>(h);
  TDatabase::ParamDB->INTERNAL_PROJECT_PRESSURE = pin_pressure;
  TDatabase::ParamDB->INTERNAL_PRESSURE_SPACE = -11;
  double *r = copy_of(rhs, V->n);
  V->base->SolveExact(u, r);
  delete[] r;
}

}  // extern "C"
