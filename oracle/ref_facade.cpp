// ref_facade.cpp — compiles the ParMooN-side adapter of the library
// (include/pmgpu_parmoon.h: TFgmresIteGPU, a TItMethod) against the
// reference's own headers and drives it through a TItMethod pointer, as
// TSystemNSE3D::Solve does (src/System/SystemNSE3D.C:1214-1234).  TEST
// INFRASTRUCTURE ONLY (built by oracle/build_oracle.py, build_ref_facade,
// where the reference tree is present; linked with libpmgpu.so).
//
// ref_facade_run builds every level as the reference's matrix objects
// (TSquareMatrix A11..A33 on a square structure with the active bound,
// TMatrix B1..B3 and B1T..B3T, src/FE/SquareMatrix.C, Matrix.C), hands
// them and the cell maps, in the GlobalNumbers / BeginIndex form of
// TFESpace3D, to pmgpu::make_level, checks that the filled descriptors equal
// the ones the levels came from, and calls Iterate(A, B, sol, rhs) of a
// TFgmresIteGPU through TItMethod*.  Without a GPU the library refuses the
// handle and Iterate returns -1 with status PM_NO_DEVICE.
//
// Lifetimes follow ref_harness.cpp: matrices are built by placement new and
// their entry arrays freed with delete[]; TStructure owns its index arrays.
#include <cstring>
#include <fstream>
#include <new>
#include <vector>

#include <Database.h>
#include <ItMethod.h>
#include <Matrix.h>
#include <SquareMatrix.h>
#include <SquareStructure.h>
#include <Structure.h>

#include "pmgpu_parmoon.h"

static TParamDB g_param;
TParamDB *TDatabase::ParamDB = &g_param;
std::ofstream OutFile;

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

struct RefLevel {
  ActiveStructure *sa = nullptr;
  TStructure *sb = nullptr, *sbt = nullptr;
  alignas(TSquareMatrix) unsigned char a_store[9][sizeof(TSquareMatrix)];
  alignas(TMatrix) unsigned char b_store[6][sizeof(TMatrix)];
  TSquareMatrix *A[9] = {};
  TMatrix *B[6] = {};
  std::vector<int> u_global, u_begin, p_global, p_begin;

  explicit RefLevel(const pm_level_desc &d) {
    const int nu = d.n_udof, np = d.n_pdof;
    sa = new ActiveStructure(nu, d.n_active, d.a_nnz, copy_of(d.a_col, d.a_nnz),
                             copy_of(d.a_rowptr, nu + 1L));
    for (int k = 0; k < 9; ++k) {
      A[k] = new (a_store[k]) TSquareMatrix(sa);
      std::memcpy(A[k]->GetEntries(), d.a[k], sizeof(double) * d.a_nnz);
    }
    sb = new TStructure(np, nu, d.b_nnz, copy_of(d.b_col, d.b_nnz), copy_of(d.b_rowptr, np + 1L));
    sbt = new TStructure(nu, np, d.bt_nnz, copy_of(d.bt_col, d.bt_nnz),
                         copy_of(d.bt_rowptr, nu + 1L));
    for (int k = 0; k < 3; ++k) {
      B[k] = new (b_store[k]) TMatrix(sb, copy_of(d.b[k], d.b_nnz));
      B[3 + k] = new (b_store[3 + k]) TMatrix(sbt, copy_of(d.bt[k], d.bt_nnz));
    }
    // the spaces' GlobalNumbers / BeginIndex (cells in order, each cell's
    // DOFs contiguous)
    u_global.assign(d.cell_udofs, d.cell_udofs + (size_t)d.n_cells * d.n_ulocal);
    p_global.assign(d.cell_pdofs, d.cell_pdofs + (size_t)d.n_cells * d.n_plocal);
    u_begin.resize(d.n_cells + 1);
    p_begin.resize(d.n_cells + 1);
    for (int c = 0; c <= d.n_cells; ++c) {
      u_begin[c] = c * d.n_ulocal;
      p_begin[c] = c * d.n_plocal;
    }
  }
  ~RefLevel() {
    for (int k = 0; k < 9; ++k) delete[] A[k]->GetEntries();
    for (int k = 0; k < 6; ++k) delete[] B[k]->GetEntries();
    delete sa;
    delete sb;
    delete sbt;
  }
};

// 0 when the filled descriptor describes the same level as d (same sizes,
// the same CSR patterns and values, cell maps and hierarchy); else the
// number of the first differing field
int compare(const pm_level_desc &f, const pm_level_desc &d) {
  auto same = [](const auto *a, const auto *b, long n) {
    return n <= 0 || (a && b && std::memcmp(a, b, sizeof(*a) * n) == 0);
  };
  if (f.n_udof != d.n_udof || f.n_pdof != d.n_pdof || f.n_active != d.n_active) return 1;
  if (f.hanging_bound != d.hanging_bound || f.n_dirichlet != d.n_dirichlet) return 2;
  if (f.a_nnz != d.a_nnz || !same(f.a_rowptr, d.a_rowptr, d.n_udof + 1L) ||
      !same(f.a_col, d.a_col, d.a_nnz))
    return 3;
  for (int k = 0; k < 9; ++k)
    if (!same(f.a[k], d.a[k], d.a_nnz)) return 4;
  if (f.b_nnz != d.b_nnz || !same(f.b_rowptr, d.b_rowptr, d.n_pdof + 1L) ||
      !same(f.b_col, d.b_col, d.b_nnz) || f.bt_nnz != d.bt_nnz ||
      !same(f.bt_rowptr, d.bt_rowptr, d.n_udof + 1L) || !same(f.bt_col, d.bt_col, d.bt_nnz))
    return 5;
  for (int k = 0; k < 3; ++k)
    if (!same(f.b[k], d.b[k], d.b_nnz) || !same(f.bt[k], d.bt[k], d.bt_nnz)) return 6;
  if (f.n_cells != d.n_cells || f.n_ulocal != d.n_ulocal || f.n_plocal != d.n_plocal) return 7;
  if (!same(f.cell_udofs, d.cell_udofs, (long)d.n_cells * d.n_ulocal) ||
      !same(f.cell_pdofs, d.cell_pdofs, (long)d.n_cells * d.n_plocal))
    return 8;
  if ((d.cell_parent && !same(f.cell_parent, d.cell_parent, d.n_cells)) ||
      (d.cell_child && !same(f.cell_child, d.cell_child, d.n_cells)))
    return 9;
  return 0;
}

}  // namespace

extern "C" {

// Solve the problem given by `levels` (coarsest first) through a
// TFgmresIteGPU held as TItMethod*; the stopping parameters go through
// TDatabase::ParamDB as a ParMooN run sets them.  out[0] = iterations (the
// return value of Iterate), out[1] = status (GetStatus), out[2] = the first
// descriptor mismatch (0: every filled descriptor equals its level).
__attribute__((visibility("default"))) void ref_facade_run(const pm_level_desc *levels,
                                                           int n_levels, int precision,
                                                           int maxit, double res_norm_min,
                                                           double *sol, const double *rhs,
                                                           int *out) {
  std::memset(&g_param, 0, sizeof(g_param));
  g_param.SC_LIN_RES_NORM_MIN_SADDLE = res_norm_min;
  g_param.SC_LIN_RED_FACTOR_SADDLE = 0.0;
  g_param.SC_LIN_MAXIT_SADDLE = maxit;
  g_param.SC_AMG_PREC_IT = 1;
  g_param.SC_DIV_FACTOR = 1e10;
  g_param.SC_MINIT = 0;
  g_param.SC_GMRES_RESTART = 20;
  g_param.SC_PRE_SMOOTH_SADDLE = 2;
  g_param.SC_POST_SMOOTH_SADDLE = 2;
  g_param.SC_SMOOTH_DAMP_FACTOR_COARSE_SADDLE = 1.0;
  g_param.SC_GMG_DAMP_FACTOR_SADDLE = 1.0;
  std::vector<RefLevel *> ref;
  int mismatch = 0;
  const int N = 3 * levels[n_levels - 1].n_udof + levels[n_levels - 1].n_pdof;
  TItMethod *it = new TFgmresIteGPU(nullptr, nullptr, nullptr, 0, N, 0, precision);
  TFgmresIteGPU *gpu = static_cast<TFgmresIteGPU *>(it);
  for (int l = 0; l < n_levels; ++l) {
    const pm_level_desc &d = levels[l];
    RefLevel *R = new RefLevel(d);
    ref.push_back(R);
    pmgpu::ParmoonLevel L = pmgpu::make_level(
        R->A, 9, R->B, d.n_active, d.n_cells, d.n_ulocal, R->u_global.data(), R->u_begin.data(),
        R->p_global.data(), R->p_begin.data(), d.cell_parent, d.cell_child, d.cell_colour);
    if (!mismatch) mismatch = compare(L.desc, d) ? 100 * l + compare(L.desc, d) : 0;
    gpu->AddLevel(L);
  }
  RefLevel *F = ref.back();
  std::vector<double> b(rhs, rhs + N);
  out[0] = it->Iterate(F->A, F->B, sol, b.data());
  out[1] = gpu->GetStatus();
  out[2] = mismatch;
  delete it;
  for (RefLevel *R : ref) delete R;
}

}  // extern "C"
