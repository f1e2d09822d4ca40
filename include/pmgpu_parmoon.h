/*
 * pmgpu_parmoon.h — the GB300 solver as a ParMooN iteration method.
 *
 * Compiled inside a ParMooN build (its include/FE on the include path,
 * -D__3D__), linked with libpmgpu.so.  TFgmresIteGPU is a TItMethod
 * (include/FE/ItMethod.h:45-172) with TFgmresIte's constructor signature
 * (include/FE/FgmresIte.h:86-97); it stands for the object TSystemNSE3D
 * builds for SC_SOLVER_SADDLE = 16 (FGMRES) with SC_PRECONDITIONER_SADDLE = 5
 * (TMultiGridIte over TNSE_MultiGrid, cell Vanka), so that
 * TSystemNSE3D::Solve's call (src/System/SystemNSE3D.C:1214-1234)
 *
 *     N_LinIter += Itmethod->Iterate(sqmatrices, matrices, sol, rhs);
 *
 * runs the whole FGMRES + V-cycle on the GPU.  The multigrid levels are
 * handed over once, coarsest first, with the same objects the reference
 * gives each TNSE_MGLevel4 (src/System/SystemNSE3D.C:806-876): the nine
 * velocity blocks (or the one block of NSTYPE 2), B1..B3, B1T..B3T, and
 * the velocity / pressure spaces' cell DOF maps (GlobalNumbers +
 * BeginIndex).  Iterate receives the finest level's matrices in the order
 * TSystemNSE3D passes them (sqmatrices = A11, A12, A13, A21, A22, A23, A31,
 * A32, A33; matrices = B1, B2, B3, B1T, B2T, B3T, the order MatVect_NSE4
 * reads them, src/FE/MGComponents3D.C:3030-3035); a call with different
 * arrays than the finest level holds is refused.
 *
 * Stopping parameters are the TItMethod members, read from
 * TDatabase::ParamDB as TFgmresIte's constructor reads them
 * (src/FE/FgmresIte.C:75-176) and changeable through the TItMethod setters
 * before any Iterate.  The return value is the FGMRES iteration count; a
 * failed solve returns -1 (a diverged one its iterations) and GetStatus()
 * gives the pm_status, where the reference would exit(4711).
 */
#ifndef PMGPU_PARMOON_H
#define PMGPU_PARMOON_H

#include <vector>

#include <Database.h>
#include <ItMethod.h>
#include <Matrix.h>
#include <SquareMatrix.h>

#include "pmgpu_facade.h"

namespace pmgpu {

// One multigrid level in the layout of pmgpu.h, filled from ParMooN's
// objects.  The CSR arrays are the matrices' own (TSquareMatrix /
// TMatrix::GetRowPtr, GetKCol, GetEntries); the cell maps are gathered from
// the spaces' GlobalNumbers / BeginIndex into arrays the level owns.
struct ParmoonLevel {
  pm_level_desc desc = {};
  std::vector<int> cell_udofs, cell_pdofs;
};

// a: the velocity blocks, 9 (A11, A12, A13, A21, A22, A23, A31, A32, A33;
// NSTYPE 4) or 1 (NSTYPE 2); b: B1, B2, B3, B1T, B2T, B3T.  n_active is the
// velocity space's active bound (its Dirichlet DOFs follow), n_ulocal the
// velocity DOFs per cell (27 Q2, 15 P2 + bubbles).  u_global/u_begin and
// p_global/p_begin are TFESpace3D::GetGlobalNumbers / GetBeginIndex of the
// velocity and pressure spaces; cell_parent / cell_child (the cell's parent
// on the next coarser level and its child number; NULL on the coarsest
// level) and cell_colour (NULL: colour greedily) as in pm_level_desc.
inline ParmoonLevel make_level(TSquareMatrix *const *a, int n_a, TMatrix *const *b, int n_active,
                               int n_cells, int n_ulocal, const int *u_global,
                               const int *u_begin, const int *p_global, const int *p_begin,
                               const int *cell_parent = nullptr,
                               const int *cell_child = nullptr,
                               const int *cell_colour = nullptr) {
  ParmoonLevel L;
  pm_level_desc &d = L.desc;
  TSquareMatrix *A = a[0];
  d.n_udof = A->GetN_Rows();
  d.n_pdof = b[0]->GetN_Rows();
  d.n_active = n_active;
  d.hanging_bound = n_active;
  d.n_dirichlet = d.n_udof - n_active;
  d.a_nnz = A->GetN_Entries();
  d.a_rowptr = A->GetRowPtr();
  d.a_col = A->GetKCol();
  for (int k = 0; k < 9; ++k) d.a[k] = (n_a == 9 || k == 0) ? a[n_a == 9 ? k : 0]->GetEntries()
                                                            : nullptr;
  d.b_nnz = b[0]->GetN_Entries();
  d.b_rowptr = b[0]->GetRowPtr();
  d.b_col = b[0]->GetKCol();
  d.bt_nnz = b[3]->GetN_Entries();
  d.bt_rowptr = b[3]->GetRowPtr();
  d.bt_col = b[3]->GetKCol();
  for (int k = 0; k < 3; ++k) {
    d.b[k] = b[k]->GetEntries();
    d.bt[k] = b[3 + k]->GetEntries();
  }
  d.n_cells = n_cells;
  d.n_ulocal = n_ulocal;
  d.n_plocal = 4;
  L.cell_udofs.resize((size_t)n_cells * n_ulocal);
  L.cell_pdofs.resize((size_t)n_cells * 4);
  for (int c = 0; c < n_cells; ++c) {
    for (int j = 0; j < n_ulocal; ++j)
      L.cell_udofs[(size_t)c * n_ulocal + j] = u_global[u_begin[c] + j];
    for (int j = 0; j < 4; ++j) L.cell_pdofs[(size_t)c * 4 + j] = p_global[p_begin[c] + j];
  }
  d.cell_udofs = L.cell_udofs.data();
  d.cell_pdofs = L.cell_pdofs.data();
  d.cell_parent = cell_parent;
  d.cell_child = cell_child;
  d.cell_colour = cell_colour;
  return L;
}

}  // namespace pmgpu

class TFgmresIteGPU : public TItMethod {
 public:
  // TFgmresIte's signature; Prec is not called (the V-cycle runs on the
  // GPU), n_aux is ignored (no host auxiliary arrays).  precision:
  // PM_PREC_FP64 or PM_PREC_MIXED.
  TFgmresIteGPU(MatVecProc *MatVec, DefectProc *Defect, TItMethod *Prec, int n_aux,
                int N_Unknowns, int scalar, int precision = PM_PREC_MIXED, int device = 0)
      : TItMethod(MatVec, Defect, Prec, n_aux, N_Unknowns), core_(options(precision, device)) {
    matvec = MatVec;
    matvecdefect = Defect;
    prec = Prec;
    N_DOF = N_Unknowns;
    N_Aux = 0;  // the base destructor reads it (src/FE/ItMethod.C)
    AuxArray = nullptr;
    defect = nullptr;
    TParamDB *db = TDatabase::ParamDB;
    res_norm_min = scalar ? db->SC_LIN_RES_NORM_MIN_SCALAR : db->SC_LIN_RES_NORM_MIN_SADDLE;
    red_factor = scalar ? db->SC_LIN_RED_FACTOR_SCALAR : db->SC_LIN_RED_FACTOR_SADDLE;
    maxit = scalar ? db->SC_LIN_MAXIT_SCALAR : db->SC_LIN_MAXIT_SADDLE;
    prec_maxit = db->SC_AMG_PREC_IT;
    div_factor = db->SC_DIV_FACTOR;
    minit = db->SC_MINIT;
    restart = db->SC_GMRES_RESTART;
    if (restart > maxit) restart = maxit;
    if (restart <= 0) restart = 10;
  }

  // Coarsest level first, before the first Iterate.
  int AddLevel(const pmgpu::ParmoonLevel &L) {
    levels_.push_back(L);
    // the descriptor points into the copy's own cell arrays
    pmgpu::ParmoonLevel &mine = levels_.back();
    mine.desc.cell_udofs = mine.cell_udofs.data();
    mine.desc.cell_pdofs = mine.cell_pdofs.data();
    return core_.AddLevel(mine.desc);
  }

  // The matrices have not been reassembled since the last Iterate.
  void MatricesUnchanged() { core_.MatricesUnchanged(); }

  int Iterate(TSquareMatrix **A, TMatrix **B, double *sol, double *rhs) override {
    if (levels_.empty()) return fail(PM_NOT_SETUP);
    const pm_level_desc &f = levels_.back().desc;
    if (A[0]->GetEntries() != f.a[0] || A[0]->GetRowPtr() != f.a_rowptr ||
        B[0]->GetEntries() != f.b[0] || B[3]->GetEntries() != f.bt[0])
      return fail(PM_BADARG);
    pmgpu::StopParams p;
    p.restart = restart;
    p.maxit = maxit;
    p.minit = minit;
    p.red_factor = red_factor;
    p.res_norm_min = res_norm_min;
    p.div_factor = div_factor;
    return core_.Iterate(sol, rhs, p);
  }

#ifdef _CUDA
  int IterateGPU(TSquareMatrix **A, TMatrix **B, double *sol, double *rhs,
                 int cycle_index) override {
    (void)cycle_index;
    return Iterate(A, B, sol, rhs);
  }
#endif

  int GetStatus() const { return forced_ != PM_OK ? forced_ : core_.status(); }
  const pm_result &GetResult() const { return core_.result(); }
  pmgpu::FgmresGPU &Core() { return core_; }

 private:
  static pm_options options(int precision, int device) {
    pm_options o;
    pm_default_options(&o);
    o.precision = precision;
    o.device = device;
    TParamDB *db = TDatabase::ParamDB;
    o.pre_smooth = db->SC_PRE_SMOOTH_SADDLE;
    o.post_smooth = db->SC_POST_SMOOTH_SADDLE;
    o.smooth_damp = db->SC_SMOOTH_DAMP_FACTOR_COARSE_SADDLE;
    o.beta = db->SC_GMG_DAMP_FACTOR_SADDLE;
    o.restart = db->SC_GMRES_RESTART > 0 ? db->SC_GMRES_RESTART : 10;
    o.maxit = db->SC_LIN_MAXIT_SADDLE;
    return o;
  }
  int fail(int s) {
    forced_ = s;
    return -1;
  }

  pmgpu::FgmresGPU core_;
  std::vector<pmgpu::ParmoonLevel> levels_;
  int forced_ = PM_OK;
};

#endif  // PMGPU_PARMOON_H
