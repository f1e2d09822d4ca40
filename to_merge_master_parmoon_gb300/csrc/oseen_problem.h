/*
 * oseen_problem.h — builds the per-level inputs that ParMooN's TSystemNSE3D
 * hands to its saddle-point solver: a hierarchy of uniformly refined
 * axis-aligned hexahedral meshes, Q2 velocity / P1disc pressure DOF maps
 * (active DOFs first, Dirichlet DOFs last, as TFESpace3D numbers them,
 * src/FE/FESpace3D.C:479-850), and the NSTYPE-4 Galerkin Oseen matrices
 * (NSType4Galerkin3D, src/FE/NSE3D_FixPo.C:1919-2071) in the reference's CSR
 * layout (TSquareStructure3D rows, Dirichlet rows diagonal-only,
 * src/FE/SquareStructure3D.C:104-124; Dirichlet diagonal set to 1,
 * src/FE/Assemble3D.C:466-476).
 *
 * This is the caller side of the solver boundary, not the solver: it only
 * produces inputs for pm_add_level / the oracle.
 */
#ifndef OSEEN_PROBLEM_H
#define OSEEN_PROBLEM_H

#include <stdint.h>
#include "pmgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PMH_EXAMPLE_RANDOM_OSEEN = 0,   /* seeded divergence-free Fourier convection + smooth forcing */
  PMH_EXAMPLE_QUADLIN_STOKES = 1, /* Examples/NSE_3D/AnsatzQuadLin.h, b = 0                     */
  PMH_EXAMPLE_QUADLIN_OSEEN = 2,  /* AnsatzQuadLin with b := exact u (Oseen linearisation)       */
  PMH_EXAMPLE_CHANNEL = 3         /* channel: b = u0 = (1 - eta^2) e_x + seeded divergence-free
                                     perturbation vanishing at the y walls, f = (2 nu (2/Ly)^2, 0, 0)
                                     (holds the parabola in equilibrium), u = 0 on the y walls   */
};

enum { PMH_PERIODIC_X = 1, PMH_PERIODIC_Y = 2, PMH_PERIODIC_Z = 4 };

typedef struct {
  int nx0, ny0, nz0;       /* cells per direction on the coarsest level          */
  int n_levels;            /* number of levels (each a regular refinement)        */
  double x0, x1, y0, y1, z0, z1; /* box                                           */
  double nu;               /* viscosity (coeff[0])                                */
  uint64_t seed;           /* RNG seed of the convection / forcing fields          */
  int example;             /* PMH_EXAMPLE_*                                        */
  int n_modes;             /* Fourier modes of b and f (8)                         */
  int nthreads;            /* OpenMP threads for assembly (0 = default)            */
  int periodic;            /* PMH_PERIODIC_* bits: identified faces, no Dirichlet
                              nodes there (at least 2 cells in such a direction)  */
  double stretch_y;        /* > 0: y nodes at y0 + Ly (1 + tanh(s eta)/tanh(s)) / 2,
                              eta uniform in [-1, 1] on every level; 0: uniform    */
  double perturb;          /* channel: max |perturbation| at the finest nodes      */
  int element;             /* PMH_ELEMENT_*                                        */
} pmh_params;

enum {
  PMH_ELEMENT_HEXA_Q2 = 0, /* hexahedra, Q2 / P1disc (27 + 4 local DOFs)                   */
  PMH_ELEMENT_TETRA_B2 = 1 /* each cube split into 6 Kuhn tetrahedra, P2 + 4 face + 1 cell
                              bubble / P1disc (15 + 4 local DOFs, C_B2_3D_T_A / D_P1_3D_T);
                              no periodic directions, uniform grid                          */
};

typedef struct pmh_problem pmh_problem;

void         pmh_default_params(pmh_params *p);
pmh_problem *pmh_build(const pmh_params *p);
void         pmh_free(pmh_problem *p);
int          pmh_n_levels(const pmh_problem *p);
int          pmh_ndof(const pmh_problem *p, int level);
/* Fill a level descriptor whose pointers stay valid until pmh_free. */
int          pmh_level_desc(const pmh_problem *p, int level, pm_level_desc *out);
/* Right-hand side of the finest level ([f1|f2|f3|0], Dirichlet entries hold
 * the boundary values). */
const double *pmh_rhs(const pmh_problem *p);
/* Interpolant of the exact solution on the finest level (known-answer
 * examples), NULL otherwise. */
const double *pmh_exact(const pmh_problem *p);
/* Q2 reference basis at (xi,eta,zeta): 27 values, and 81 derivatives
 * (d/dxi, d/deta, d/dzeta per function). */
void pmh_q2_basis(double xi, double eta, double zeta, double *values, double *derivs);
/* P2 + 4 face + 1 cell bubble basis on the reference tetrahedron
 * (0,0,0), (1,0,0), (0,1,0), (0,0,1): 15 values and 45 derivatives (the
 * local order of C_T_B2_3D_Funct, include/FE3D/BF_C_T_B2_3D.h); the P1disc
 * basis there: 4 values, 12 derivatives. */
void pmh_b2_basis(double xi, double eta, double zeta, double *values, double *derivs);
void pmh_p1t_basis(double xi, double eta, double zeta, double *values, double *derivs);
double pmh_max_convection(const pmh_problem *p);
/* (hx, hy, hz) of every cell of a level (n_cells x 3); 0 or -1 */
int pmh_cell_sizes(const pmh_problem *p, int level, double *out);
/* the convection field at the level's velocity nodes, [b1|b2|b3]; 0 or -1 */
int pmh_convection_nodal(const pmh_problem *p, int level, double *out);
/* Assemble the matrix values of every level again (the same cell loop as the
 * build, on the build's threads): the host timing of a re-assembly; 0 or -1 */
int pmh_reassemble(pmh_problem *p);

#ifdef __cplusplus
}
#endif
#endif
