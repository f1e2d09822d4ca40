// pm_setup_host.h — host-side setup algorithms of libpmgpu (run once per
// pm_setup; no numerical results of the solve are computed here).
#ifndef PM_SETUP_HOST_H
#define PM_SETUP_HOST_H

#include <string>
#include <vector>

#include "pmgpu.h"

namespace pm {

struct HostCsr {
  int rows = 0, cols = 0;
  std::vector<int> rowptr, col;
  std::vector<double> val;
};

// Cells grouped by colour: cells of colour k are order[ptr[k]..ptr[k+1]).
struct Colouring {
  std::vector<int> ptr, order;
  int max_size = 0;
};

// Validate a caller-provided colouring (no velocity or pressure DOF shared
// by two cells of one colour) or, if colour == nullptr, colour greedily in
// cell order (smallest colour unused by any cell sharing a DOF), as
// TParFEMapper3D::colorCell does (src/Parallel/ParFEMapper3D.C:750).
bool make_colouring(int ncells, int nulocal, int nplocal, const int *udofs, const int *pdofs,
                    int nu, int np, const int *colour, Colouring &out, std::string &err);

// Prolongation from the coarse to the fine level, P[i][k] =
// (1/m_i) sum over fine cells containing node i of QQ_child[i_loc][k_loc]
// (Prolongate, src/FE/MGComponents3D.C:468-708, with the multiplicity
// division of :692-707), for Q2 (velocity, continuous) and P1disc
// (pressure).  Restriction is its transpose (DefectRestriction divides by the
// same multiplicity before applying QQ^T, :1036-1235).
bool build_transfers(int nc_cells, const int *c_udofs, const int *c_pdofs, int c_nu, int c_np,
                     int nf_cells, const int *f_udofs, const int *f_pdofs, int f_nu, int f_np,
                     const int *f_parent, const int *f_child, HostCsr &Pu, HostCsr &Ru,
                     HostCsr &Pp, HostCsr &Rp, std::string &err);

HostCsr transpose(const HostCsr &a);

// 26 neighbour slots per cell (-1 = none) for Q2 hexahedra, from the shared
// nodes alone: along each axis the neighbour lies at +1 if all shared nodes
// have local index 2 on that axis, -1 if all have 0, else 0; slot =
// (dx+1) + 3(dy+1) + 9(dz+1) with the centre (13) removed.
void build_neighbours(int ncells, const int *udofs, int nu, std::vector<int> &nbr);
// 1 / (number of cells containing each velocity node)
void node_inverse_multiplicity(int ncells, const int *udofs, int nu, std::vector<float> &inv);

// G level descriptors of one mesh (equal sizes, nnz and local DOF counts;
// values and patterns may differ) stacked into one block-diagonal level:
// velocity DOF i of system s goes to s*na + i if i < na (na = n_active),
// else to G*na + s*(nu - na) + (i - na), pressure DOF j to s*np + j, cell k
// to s*ncells + k.  `coarse` gives the per-system sizes of the next coarser
// stacked level (for parent cells and prolongation columns; ignored for the
// coarsest).  The arrays live in `st`; `out` points into them.
struct StackSizes {
  int nu = 0, na = 0, np = 0, ncells = 0;
};
struct StackedLevel {
  std::vector<int> a_rowptr, a_col, b_rowptr, b_col, bt_rowptr, bt_col;
  std::vector<int> udofs, pdofs, parent, child, colour;
  std::vector<int> pu_rowptr, pu_col, pp_rowptr, pp_col;
  std::vector<double> a[9], b[3], bt[3], pu_val, pp_val;
};
bool stack_levels(const pm_level_desc *d, int G, const StackSizes &coarse, StackedLevel &st,
                  pm_level_desc &out, std::string &err);

}  // namespace pm

#endif
