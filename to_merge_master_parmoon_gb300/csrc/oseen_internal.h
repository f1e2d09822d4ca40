// oseen_internal.h — shared internals of the caller-side problem builder:
// hexahedral Q2/P1disc levels (oseen_problem.cpp) and tetrahedral
// P2+bubble/P1disc levels (oseen_tet.cpp).  Not an interface of the library.
#ifndef OSEEN_INTERNAL_H
#define OSEEN_INTERNAL_H

#include <vector>

#include "oseen_problem.h"

struct PmhMode {
  double k[3];
  double a[3];
  double phase;
};

struct PMLevelData {
  int nx, ny, nz;                     // cubes per direction
  int n_cells, n_udof, n_pdof, n_active;
  int nu_loc = 27;                    // velocity nodes per cell (27 Q2, 15 P2+bubble)
  std::vector<double> xs, ys, zs;     // cube boundaries
  std::vector<int> grid2dof;          // Q2 node grid -> dof (hexahedra)
  std::vector<int> dof2grid;
  std::vector<int> a_rowptr, a_col;
  std::vector<double> a[9];
  std::vector<int> b_rowptr, b_col;
  std::vector<double> b[3];
  std::vector<int> bt_rowptr, bt_col;
  std::vector<double> bt[3];
  std::vector<int> cell_udofs, cell_pdofs, cell_parent, cell_child, cell_colour;
  // tetrahedra: position of every velocity DOF, the 4 vertices of every cell,
  // and the prolongation from the next coarser level (scalar CSR, fine rows)
  std::vector<double> node_xyz, tet_xyz;
  std::vector<int> pu_rowptr, pu_col, pp_rowptr, pp_col;
  std::vector<double> pu_val, pp_val;
  int gx() const { return 2 * nx + 1; }
  int gy() const { return 2 * ny + 1; }
  int gz() const { return 2 * nz + 1; }
  double node_x(int i) const { return (i & 1) ? 0.5 * (xs[i / 2] + xs[i / 2 + 1]) : xs[i / 2]; }
  double node_y(int j) const { return (j & 1) ? 0.5 * (ys[j / 2] + ys[j / 2 + 1]) : ys[j / 2]; }
  double node_z(int k) const { return (k & 1) ? 0.5 * (zs[k / 2] + zs[k / 2 + 1]) : zs[k / 2]; }
};

struct pmh_problem {
  pmh_params prm;
  std::vector<PMLevelData> levels;
  std::vector<double> rhs;
  std::vector<double> exact;
  bool has_exact = false;
  std::vector<PmhMode> bmodes, fmodes;
  double bscale = 1.0;
  double bmax = 0.0;
};

namespace pmh_detail {
// fields of the examples (oseen_problem.cpp)
void quadlin_u(double x, double y, double z, double *u);
double quadlin_p(double x, double y, double z);
void convection(const pmh_problem &P, double x, double y, double z, double *b);
void forcing(const pmh_problem &P, double x, double y, double z, double *f);
bool boundary_value(const pmh_problem &P, double x, double y, double z, double *u);
// tetrahedral levels (oseen_tet.cpp): structure, assembly, prolongation
void build_tet_levels(pmh_problem &P);
void assemble_tet_level(pmh_problem &P, PMLevelData &L, bool finest);
// P2+bubble basis on the reference tetrahedron: 15 values, 45 derivatives
void b2_basis(double xi, double eta, double zeta, double *val, double *der);
// P1disc basis of the reference tetrahedron (4 values, 12 derivatives)
void p1t_basis(double xi, double eta, double zeta, double *val, double *der);
}  // namespace pmh_detail

#endif
