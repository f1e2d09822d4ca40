/*
 * oracle.h — CPU restatement of ParMooN's saddle-point solver path
 * (TFgmresIte + TNSE_MultiGrid::Cycle + TNSE_MGLevel4 cell Vanka) in FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is compared
 * against and the CPU baseline that bench.py times; it is never linked into
 * or called by the product library.
 *
 * Parity status: the reference cannot be compiled here (icc/MKL/MAGMA/UMFPACK
 * hard requirements), so this restatement is pinned by (a) the reference's
 * known-answer fixture Examples/NSE_3D/AnsatzQuadLin.h (the discrete solution
 * must reproduce the exact Q2 x P1 solution), (b) golden values of the
 * reference's own Q2 and P1disc basis functions compiled from
 * include/FE3D/BF_C_H_Q2_3D.h and BF_D_H_P1_3D.h (oracle/ref_basis_pin.cpp),
 * and (c) scipy's LU on sampled local blocks.  Bit-level agreement with a
 * reference binary is unpinned.
 */
#ifndef PM_ORACLE_H
#define PM_ORACLE_H

#include "pmgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORACLE_VANKA_SEQ = 0,    /* cell loop in collection order, updates immediately (_SEQ) */
  ORACLE_VANKA_COLOUR = 1  /* per colour: all local residuals, solves, then updates
                              (CellVanka_GPU semantics)                              */
};

typedef struct {
  int pre_smooth, post_smooth;
  double smooth_damp, alpha, beta;
  int project_pressure;
  int restart, maxit, minit;
  double red_factor, res_norm_min, div_factor;
  int vanka_mode;          /* ORACLE_VANKA_*                                         */
  int reuse_factors;       /* 1: factor each local block once (diagnostic variant)   */
  int nthreads;            /* OpenMP threads (0 = default)                          */
} oracle_params;

typedef struct oracle oracle;

void    oracle_default_params(oracle_params *p);
oracle *oracle_create(const pm_level_desc *levels, int n_levels, const oracle_params *p);
void    oracle_destroy(oracle *o);
int     oracle_ndof(oracle *o, int level);

void oracle_coupled_defect(oracle *o, int level, const double *x, const double *b, double *r,
                           int project_pressure);
void oracle_matvec(oracle *o, int level, const double *x, double *y);
void oracle_level_defect(oracle *o, int level, const double *u, const double *f, double *d,
                         double *res);
void oracle_cell_vanka(oracle *o, int level, double *u, const double *rhs, int sweeps);
void oracle_restrict(oracle *o, int level, const double *fine, double *coarse);
void oracle_prolongate(oracle *o, int level, const double *coarse, double *fine);
void oracle_solve_exact(oracle *o, const double *rhs, double *u);
void oracle_vcycle(oracle *o, double *z, const double *v);
/* FGMRES; returns iterations, writes res0/res/true residual to out[0..2]. */
int  oracle_fgmres(oracle *o, double *sol, const double *rhs, double *out);
/* Dense LU with partial pivoting of an n x n column-major matrix and solve
 * (dgetrf + dgetrs semantics), exposed for the local-solve pin. */
void oracle_lu_solve(double *a, double *b, int n);
/* Local Vanka system of one cell (column-major, 85x85 for Q2, 49x49 for
 * P2+bubble tetrahedra) and its local rhs; returns the size. */
int  oracle_local_system(oracle *o, int level, int cell, const double *u, const double *rhs,
                         double *system, double *local_rhs);

#ifdef __cplusplus
}
#endif
#endif
