// ref_transfer.cpp — runs the reference's own grid transfers, and its
// multigrid cycle driver, on nested hexahedral levels handed over as plain
// arrays.  TEST INFRASTRUCTURE ONLY: it pins the oracle's prolongate /
// defect_restriction (and with them the per-child Q2 and P1disc matrices)
// and its V-cycle against the reference code itself.
// Built by oracle/build_oracle.py (build_ref_transfer) into
// oracle/_ref/libref_transfer.so, with -D__3D__ -D_SEQ, from the reference
// sources where they lie.
//
// Reference code that runs here:
//   src/General/Database.C, src/FE/FEDatabase3D.C
//                            the TDatabase and TFEDatabase3D constructors
//                            (shape and refinement descriptors, every
//                            element, basis, nodal functional and reference
//                            transformation registered as in a ParMooN run)
//   src/FE/MGComponents3D.C  Prolongate (vector :468-708, scalar :184-467)
//                            and DefectRestriction (vector :996-1242,
//                            scalar :711-995)
//   src/FE/FEDatabase3D.C    GetProlongationMatrix3D (:1630-1790): the
//                            per-child matrices from the elements' nodal
//                            functionals on the refined reference cell
//   with the geometry, refinement and FE classes they call.
//
// What the harness supplies instead of a ParMooN mesh:
// * cells: reference TGridCell objects without vertices.  A coarse cell
//   carries the regular hexahedral refinement descriptor and its 8 children,
//   a fine cell its parent.  Prolongate and DefectRestriction ask cells for
//   nothing else, and ChangeBF returns at once for Q2 and P1disc (no
//   BF2Change table, src/FE/BaseFunct3D.C:589-595).
// * the children: the reference numbers the children of a regular
//   refinement by its refinement descriptor, each child with its own vertex
//   order.  A child's vertex 0 is a corner of the parent, and its local
//   axes are a rotation or reflection of the parent's.  The level arrays
//   number children by octant, every cell with axis-aligned local DOFs.
//   The harness refines the reference element with the reference's own
//   code, exactly as GetProlongationMatrix3D does
//   (src/FE/FEDatabase3D.C:1721-1727).  From each child's vertices it
//   takes the octant, which links every coarse cell's child slots.  It
//   also takes the child's local frame and hands each fine cell over in it:
//   - the 27 Q2 DOF numbers in the child's local node order;
//   - the P1disc coefficients (basis 1, xi, eta, zeta; the child's local
//     coordinates are a signed permutation of the axis-aligned ones)
//     transformed by that signed permutation on the way in (defects) and
//     on the way out (prolongated functions).
//   The coarse cells have the reference element's own frame, which is the
//   axis-aligned one.
// * spaces: LevelSpace (ref_level_space.h) with C_Q2_3D_H_A velocity and
//   D_P1_3D_H_A pressure elements in every cell.
// * allocation: on this path the reference reads memory that it allocated
//   and did not initialise (TGridCell::Refine of the cell from
//   GenerateRefElement, as GetProlongationMatrix3D itself runs it).  A ParMooN
//   run gets away with this because its heap is fresh, zero pages from the
//   system.  In a process whose heap has been used before, it faults.  So
//   inside this library operator new / new[] return zero-filled memory (the
//   library links with -Bsymbolic, so the reference objects in it call
//   these; no other library does).
// No reference destructor runs; the harness frees what it allocated.
//
// Over more than two levels every cell's frame composes its parent's with
// the reference child's: a child of a cell whose frame is not the
// axis-aligned one is found by its octant in the parent's frame, and its
// local axes are the reference child's axes taken in the parent's frame.
// The node orders this gives are checked against the ones read from the
// refined reference cell's vertices.
//
// Compiled a second time with -D_HYBRID instead of -D_SEQ
// (libref_transfer_hybrid.so), the levels smooth with the reference's
// colour-parallel CellVanka (src/FE/NSE_MGLevel4.C:603-1651, the OpenMP
// colour loop) over colourings set by ref_cycle_set_colours;
// ref_hybrid_mapper.h says how the constructor is compiled without the MPI
// build's TParFEMapper3D.
//
// The same levels also run the reference's multigrid cycle (ref_cycle_*):
// TMultiGridIte::Iterate (src/FE/MultiGridIte.C:76-132), the preconditioner
// call, with TNSE_MultiGrid::Cycle (src/FE/NSE_MultiGrid.C:434-1779) over
// one TNSE_MGLevel4 level (src/FE/NSE_MGLevel4.C) per level, built on the
// levels' spaces and matrices: cell Vanka pre- and post-smoothing (the _SEQ
// cell loop) on every level above the coarsest, the level defects,
// DefectRestriction, SolveExact on the coarsest level, Prolongate,
// CorrectDefect, CorrectNodes and Update.  The cells keep the frames
// described above, so every level's B rows and BT columns of each cell's
// linear pressure modes are transformed by that cell's signed permutation,
// and so are the pressure parts of the finest level's vectors on the way in
// and out; velocity DOFs keep their global numbers.
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <new>
#include <algorithm>
#include <utility>
#include <vector>

#include <BaseCell.h>
#include <BaseFunct3D.h>
#include <Collection.h>
#include <Database.h>
#include <DirectSolver.h>
#include <FE3D.h>
#include <FEDatabase3D.h>
#include <FESpace3D.h>
#include <GridCell.h>
#include <LinAlg.h>
#include <Matrix3D.h>
#include <MultiGrid3D.h>
#include <MultiGridIte.h>
#include <NSE_MGLevel4.h>  // includes Magma_Solver.h (no include guard)
#include <NSE_MultiGrid.h>
#include <RefDesc.h>
#include <SquareMatrix3D.h>
#include <Vertex.h>

#include "ref_lapack.h"
#include "ref_level_space.h"

void *operator new(std::size_t n) {
  void *p = std::calloc(1, n ? n : 1);
  if (!p) throw std::bad_alloc();
  return p;
}
void *operator new[](std::size_t n) {
  void *p = std::calloc(1, n ? n : 1);
  if (!p) throw std::bad_alloc();
  return p;
}
void operator delete(void *p) noexcept { std::free(p); }
void operator delete[](void *p) noexcept { std::free(p); }

namespace {

struct HarnessCell : public TGridCell {
  explicit HarnessCell(TRefDesc *rd) : TGridCell(rd, 0) {}
  void set_children(TBaseCell **c) { Children = c; }
  // the arrays the TBaseCell and TGridCell constructors allocate
  // (src/Geometry/BaseCell.C:16-45, src/Geometry/GridCell.C:22-30)
  void release_arrays() {
    delete[] Children;
    Children = nullptr;
    delete[] Vertices;
    delete[] Joints;
    delete[] Edges;
  }
};

bool g_ready = false;
int g_octant_of_child[8];
// per reference child: axis-aligned local Q2 node of each of its local nodes,
// and for its local coordinate i (xi, eta, zeta) the axis-aligned coordinate
// g_paxis[j][i] and the sign g_psign[j][i] with xi_i = sign * x_axis
int g_uperm[8][27];
int g_paxis[8][3];
double g_psign[8][3];

// A cell's local frame: its local coordinate i (xi, eta, zeta) is
// sign[i] times the axis-aligned coordinate axis[i].  The coarsest cells
// have the identity; a child's frame composes its parent's with the
// reference child's (g_paxis, g_psign).
struct Frame {
  int axis[3] = {0, 1, 2};
  double sign[3] = {1.0, 1.0, 1.0};
};

// the axis-aligned Q2 node of local node t = a + 3b + 9c of a cell in frame
// F: node (a, b, c) lies a, b, c half-edges from the cell's vertex 0 along
// its local axes, and vertex 0 is at the low end of axis[i] where sign[i] > 0
int aligned_node(const Frame &F, int t) {
  const int n[3] = {t % 3, (t / 3) % 3, t / 9};
  int q[3];
  for (int i = 0; i < 3; ++i) q[F.axis[i]] = F.sign[i] > 0 ? n[i] : 2 - n[i];
  return q[0] + 3 * q[1] + 9 * q[2];
}

// octant (bit 0: xi > 0, bit 1: eta > 0, bit 2: zeta > 0, relative to the
// parent's centre) of each child of the regular hexahedral refinement
bool init_databases() {
  if (g_ready) return true;
  new TDatabase();
  new TFEDatabase3D();
  TBaseFunct3D *bf = TFEDatabase3D::GetBaseFunct3D(BF_C_H_Q2_3D);
  TBaseCell *ref = bf->GenerateRefElement();
  double c[3] = {0, 0, 0};
  for (int v = 0; v < 8; ++v) {
    double x, y, z;
    ref->GetVertex(v)->GetCoords(x, y, z);
    c[0] += x / 8;
    c[1] += y / 8;
    c[2] += z / 8;
  }
  ref->SetRefDesc(TDatabase::RefDescDB[N_SHAPES + HexaReg]);
  ref->Refine(0);
  int seen = 0;
  for (int j = 0; j < 8; ++j) {
    TBaseCell *child = ref->GetChild(j);
    double m[3] = {0, 0, 0};
    for (int v = 0; v < 8; ++v) {
      double x, y, z;
      child->GetVertex(v)->GetCoords(x, y, z);
      m[0] += x / 8;
      m[1] += y / 8;
      m[2] += z / 8;
    }
    const int o = (m[0] > c[0]) | ((m[1] > c[1]) << 1) | ((m[2] > c[2]) << 2);
    g_octant_of_child[j] = o;
    seen |= 1 << o;
    // the child's frame: vertex 0 and the edges to vertices 1, 3, 4
    double v[4][3];
    const int vid[4] = {0, 1, 3, 4};
    for (int t = 0; t < 4; ++t) child->GetVertex(vid[t])->GetCoords(v[t][0], v[t][1], v[t][2]);
    double lo[3];  // the child's lower corner
    for (int a = 0; a < 3; ++a) {
      double mn = 1e300;
      for (int vv = 0; vv < 8; ++vv) {
        double x[3];
        child->GetVertex(vv)->GetCoords(x[0], x[1], x[2]);
        if (x[a] < mn) mn = x[a];
      }
      lo[a] = mn;
    }
    for (int i = 0; i < 3; ++i) {
      double e[3];
      for (int a = 0; a < 3; ++a) e[a] = v[i + 1][a] - v[0][a];
      int ax = 0;
      for (int a = 1; a < 3; ++a)
        if (std::fabs(e[a]) > std::fabs(e[ax])) ax = a;
      g_paxis[j][i] = ax;
      g_psign[j][i] = e[ax] > 0 ? 1.0 : -1.0;
    }
    const double h = std::fabs(v[1][g_paxis[j][0]] - v[0][g_paxis[j][0]]);  // child edge
    for (int cc = 0; cc < 3; ++cc)
      for (int b = 0; b < 3; ++b)
        for (int a = 0; a < 3; ++a) {
          double pos[3];
          for (int d = 0; d < 3; ++d)
            pos[d] = v[0][d] + 0.5 * a * (v[1][d] - v[0][d]) + 0.5 * b * (v[2][d] - v[0][d]) +
                     0.5 * cc * (v[3][d] - v[0][d]);
          int q[3];
          for (int d = 0; d < 3; ++d) q[d] = (int)std::lround(2.0 * (pos[d] - lo[d]) / h);
          g_uperm[j][a + 3 * b + 9 * cc] = q[0] + 3 * q[1] + 9 * q[2];
        }
  }
  ref->Derefine();
  if (seen != 0xff) {
    std::fprintf(stderr, "ref_transfer: the refined reference cell has no child per octant\n");
    return false;
  }
  // the node orders taken from the children's vertices are the ones their
  // frames give (what composing frames over several levels relies on)
  for (int j = 0; j < 8; ++j) {
    Frame F;
    for (int i = 0; i < 3; ++i) {
      F.axis[i] = g_paxis[j][i];
      F.sign[i] = g_psign[j][i];
    }
    for (int t = 0; t < 27; ++t)
      if (aligned_node(F, t) != g_uperm[j][t]) {
        std::fprintf(stderr, "ref_transfer: child %d's node order is not its frame's\n", j);
        return false;
      }
  }
  g_ready = true;
  return true;
}

struct Side {
  int n_cells = 0, n_u = 0, n_p = 0;
  std::vector<HarnessCell *> cells;
  TBaseCell **cell_array = nullptr;
  TCollection *coll = nullptr;
  int *ug = nullptr, *ub = nullptr, *pg = nullptr, *pb = nullptr;
  FE3D *ua = nullptr, *pa = nullptr;
  alignas(LevelSpace) unsigned char us_store[sizeof(LevelSpace)];
  alignas(LevelSpace) unsigned char ps_store[sizeof(LevelSpace)];
  LevelSpace *us = nullptr, *ps = nullptr;
};

void make_side(Side &S, int n_cells, int n_u, int n_active, int n_p, const int *udofs,
               const int *pdofs, TRefDesc *rd) {
  S.n_cells = n_cells;
  S.n_u = n_u;
  S.n_p = n_p;
  S.cell_array = new TBaseCell *[n_cells > 0 ? n_cells : 1];
  for (int c = 0; c < n_cells; ++c) {
    S.cells.push_back(new HarnessCell(rd));
    S.cell_array[c] = S.cells.back();
  }
  S.coll = new TCollection(n_cells, S.cell_array);
  S.ug = new int[(size_t)27 * n_cells + 1];
  S.pg = new int[(size_t)4 * n_cells + 1];
  std::memcpy(S.ug, udofs, sizeof(int) * 27 * (size_t)n_cells);
  std::memcpy(S.pg, pdofs, sizeof(int) * 4 * (size_t)n_cells);
  S.ub = new int[n_cells + 1];
  S.pb = new int[n_cells + 1];
  S.ua = new FE3D[n_cells + 1];
  S.pa = new FE3D[n_cells + 1];
  for (int c = 0; c <= n_cells; ++c) {
    S.ub[c] = 27 * c;
    S.pb[c] = 4 * c;
    S.ua[c] = C_Q2_3D_H_A;
    S.pa[c] = D_P1_3D_H_A;
  }
  S.us = new (S.us_store) LevelSpace(S.coll, n_u, n_active, n_u - n_active, S.ug, S.ub, S.ua);
  S.ps = new (S.ps_store) LevelSpace(S.coll, n_p, n_p, 0, S.pg, S.pb, S.pa);
}

void free_side(Side &S) {
  for (HarnessCell *c : S.cells) {
    c->release_arrays();
    ::operator delete(static_cast<void *>(c));  // storage only: no reference destructor
  }
  S.us->release_names();
  S.ps->release_names();
  delete S.coll;  // frees cell_array (delete[], src/Geometry/Collection.C:57-62)
  delete[] S.ug;
  delete[] S.pg;
  delete[] S.ub;
  delete[] S.pb;
  delete[] S.ua;
  delete[] S.pa;
}

// Nested levels, level 0 the coarsest: every cell of level l > 0 is a child
// of a cell of level l - 1 and is handed to the reference in its frame.
struct Hier {
  std::vector<Side *> sides;
  std::vector<std::vector<Frame>> frames;  // per level and cell
};

// The levels as plain arrays (per level: cells, DOFs, active velocity DOFs,
// pressure DOFs, 27 + 4 DOFs per cell in the axis-aligned local order; for
// l > 0 each cell's parent on level l - 1 and its octant there, bit 0 x,
// bit 1 y, bit 2 z).  Null when a parent has not exactly one child per
// octant.
Hier *build_hier(int L, const int *n_cells, const int *n_u, const int *n_active, const int *n_p,
                 const int *const *udofs, const int *const *pdofs, const int *const *parent,
                 const int *const *child) {
  if (L < 2 || !init_databases()) return nullptr;
  std::vector<std::vector<int>> slot(L);
  for (int l = 1; l < L; ++l) {
    slot[l].assign((size_t)8 * n_cells[l - 1], -1);
    for (int f = 0; f < n_cells[l]; ++f) {
      const int p = parent[l][f], o = child[l][f];
      if (p < 0 || p >= n_cells[l - 1] || o < 0 || o > 7 || slot[l][(size_t)8 * p + o] >= 0)
        return nullptr;
      slot[l][(size_t)8 * p + o] = f;
    }
    for (int sl : slot[l])
      if (sl < 0) return nullptr;
  }
  Hier *H = new Hier;
  H->frames.resize(L);
  for (int l = 0; l < L; ++l) {
    H->sides.push_back(new Side);
    make_side(*H->sides.back(), n_cells[l], n_u[l], n_active[l], n_p[l], udofs[l], pdofs[l],
              TDatabase::RefDescDB[l + 1 < L ? N_SHAPES + HexaReg : Hexahedron]);
    H->frames[l].assign(n_cells[l], Frame());
  }
  for (int l = 1; l < L; ++l) {
    Side &C = *H->sides[l - 1], &F = *H->sides[l];
    for (int c = 0; c < C.n_cells; ++c) {
      const Frame &P = H->frames[l - 1][c];
      TBaseCell **ch = new TBaseCell *[8];
      for (int j = 0; j < 8; ++j) {
        // child j's octant in the parent's frame, then axis-aligned
        const int lo = g_octant_of_child[j];
        int o = 0;
        for (int i = 0; i < 3; ++i) o |= (((lo >> i) & 1) ^ (P.sign[i] < 0 ? 1 : 0)) << P.axis[i];
        const int f = slot[l][(size_t)8 * c + o];
        ch[j] = F.cells[f];
        ch[j]->SetParent(C.cells[c]);
        Frame &Fr = H->frames[l][f];
        for (int i = 0; i < 3; ++i) {
          Fr.axis[i] = P.axis[g_paxis[j][i]];
          Fr.sign[i] = P.sign[g_paxis[j][i]] * g_psign[j][i];
        }
        for (int t = 0; t < 27; ++t)  // the fine cell's DOFs in its frame's node order
          F.ug[(size_t)27 * f + t] = udofs[l][(size_t)27 * f + aligned_node(Fr, t)];
      }
      C.cells[c]->set_children(ch);
    }
  }
  return H;
}

void free_hier(Hier *H) {
  for (Side *S : H->sides) {
    free_side(*S);
    delete S;
  }
  delete H;
}

// pressure coefficients of every cell of level S between the axis-aligned
// frame and the cell's frame (to_child: xi_i coefficient = sign_i *
// coefficient of axis(i); the inverse otherwise)
void convert_pressure(const Side &S, const std::vector<Frame> &fr, double *fp, bool to_child) {
  for (int f = 0; f < S.n_cells; ++f) {
    const Frame &F = fr[f];
    const int *dof = S.pg + 4 * (size_t)f;
    double in[3], out[3];
    for (int i = 0; i < 3; ++i) in[i] = fp[dof[1 + i]];
    for (int i = 0; i < 3; ++i) {
      if (to_child)
        out[i] = F.sign[i] * in[F.axis[i]];
      else
        out[F.axis[i]] = F.sign[i] * in[i];
    }
    for (int i = 0; i < 3; ++i) fp[dof[1 + i]] = out[i];
  }
}

}  // namespace

extern "C" {

// Two nested Q2/P1disc hexahedral levels: per cell 27 velocity and 4
// pressure DOFs; fine cell f is child number fine_child[f] (its octant:
// bit 0 x, bit 1 y, bit 2 z) of coarse cell fine_parent[f].  Returns null
// when a coarse cell has not exactly one child per octant.
__attribute__((visibility("default"))) void *ref_transfer_create(
    int nc_cells, int nc_u, int nc_active, int nc_p, const int *c_udofs, const int *c_pdofs,
    int nf_cells, int nf_u, int nf_active, int nf_p, const int *f_udofs, const int *f_pdofs,
    const int *fine_parent, const int *fine_child) {
  const int n_cells[2] = {nc_cells, nf_cells}, n_u[2] = {nc_u, nf_u},
            n_active[2] = {nc_active, nf_active}, n_p[2] = {nc_p, nf_p};
  const int *udofs[2] = {c_udofs, f_udofs}, *pdofs[2] = {c_pdofs, f_pdofs};
  const int *parent[2] = {nullptr, fine_parent}, *child[2] = {nullptr, fine_child};
  return build_hier(2, n_cells, n_u, n_active, n_p, udofs, pdofs, parent, child);
}

__attribute__((visibility("default"))) void ref_transfer_destroy(void *h) {
  if (h) free_hier(static_cast<Hier *>(h));
}

// fine = the reference's prolongation of coarse: Prolongate over the three
// velocity components (N_Functions = 3) and the scalar Prolongate for the
// pressure; vectors are [u1|u2|u3|p] of each level.
__attribute__((visibility("default"))) void ref_transfer_prolongate(void *h, const double *coarse,
                                                                    double *fine) {
  Hier *H = static_cast<Hier *>(h);
  const Side &C = *H->sides[0], &F = *H->sides[1];
  std::vector<double> cu(coarse, coarse + 3 * (size_t)C.n_u + C.n_p), aux(F.n_u + F.n_p + 1);
  Prolongate(C.us, F.us, 3, cu.data(), fine, aux.data());
  Prolongate(C.ps, F.ps, cu.data() + 3 * (size_t)C.n_u, fine + 3 * (size_t)F.n_u, aux.data());
  convert_pressure(F, H->frames[1], fine + 3 * (size_t)F.n_u, false);
}

// coarse = the reference's defect restriction of fine (DefectRestriction
// over the velocity components, then the scalar one for the pressure)
__attribute__((visibility("default"))) void ref_transfer_restrict(void *h, const double *fine,
                                                                  double *coarse) {
  Hier *H = static_cast<Hier *>(h);
  const Side &C = *H->sides[0], &F = *H->sides[1];
  std::vector<double> fu(fine, fine + 3 * (size_t)F.n_u + F.n_p), aux(F.n_u + F.n_p + 1);
  convert_pressure(F, H->frames[1], fu.data() + 3 * (size_t)F.n_u, true);
  DefectRestriction(C.us, F.us, 3, coarse, fu.data(), aux.data());
  DefectRestriction(C.ps, F.ps, coarse + 3 * (size_t)C.n_u, fu.data() + 3 * (size_t)F.n_u,
                    aux.data());
}


// ================================================================ cycle ====
}  // extern "C"

void DirectSolver(TSquareMatrix3D *, TSquareMatrix3D *, TSquareMatrix3D *, TSquareMatrix3D *,
                  TSquareMatrix3D *, TSquareMatrix3D *, TSquareMatrix3D *, TSquareMatrix3D *,
                  TSquareMatrix3D *, TMatrix3D *, TMatrix3D *, TMatrix3D *, TMatrix3D *,
                  TMatrix3D *, TMatrix3D *, double *, double *, int) {
  std::fprintf(stderr, "ref_cycle: DirectSolver is not part of the harness\n");
  std::abort();
}

namespace {

struct CycleLevel : public TNSE_MGLevel4 {
  using TNSE_MGLevel4::TNSE_MGLevel4;
  // the auxiliary vectors of the constructor (src/FE/NSE_MGLevel4.C:274-278)
  void release() {
    delete[] Aux[0];
    delete[] Aux;
  }
#ifdef _HYBRID
  // the colouring of the colour-parallel CellVanka (the members the
  // constructor takes from TParFEMapper3D, src/FE/NSE_MGLevel4.C:315-324)
  void set_colours(int n_colours, int *colour_ptr, int *cell_order, int max_cells) {
    N_CIntCell = n_colours;
    ptrCellColors = colour_ptr;
    CellReorder = cell_order;
    maxCellsPerColor = max_cells;
  }
#endif
};

#ifdef _HYBRID
}  // namespace
RefHybridMapper *ref_hybrid_mapper() {
  static RefHybridMapper none;
  return &none;
}
namespace {
#endif

// One level's matrices, vectors and TNSE_MGLevel4 over a Side's spaces
struct MGLevelStore {
  alignas(LevelSpace) unsigned char oa_store[sizeof(LevelSpace)];
  alignas(LevelSpace) unsigned char ob_store[sizeof(LevelSpace)];
  LevelSpace *oa = nullptr, *ob = nullptr;
  TCollection *other_a = nullptr, *other_b = nullptr;
  LevelSquareStructure *sa = nullptr;
  LevelStructure *sb = nullptr, *sbt = nullptr;
  alignas(TSquareMatrix3D) unsigned char a_store[9][sizeof(TSquareMatrix3D)];
  alignas(TMatrix3D) unsigned char b_store[6][sizeof(TMatrix3D)];
  TSquareMatrix3D *A[9] = {};
  TMatrix3D *B[6] = {};
  double *f = nullptr, *u = nullptr;
  double al[2] = {1.0, 1.0};
  alignas(CycleLevel) unsigned char level_store[sizeof(CycleLevel)];
  CycleLevel *level = nullptr;
  int *colour_ptr = nullptr, *cell_order = nullptr;  // colour-parallel build only
};

int *copy_ints(const int *src, long n) {
  int *d = new int[n > 0 ? n : 1];
  if (n > 0) std::memcpy(d, src, sizeof(int) * n);
  return d;
}

// B (pressure rows) and BT (pressure columns) of level S with the linear
// pressure modes of every cell c taken in its frame fr[c]: row / column of
// mode i is sign_i times the one of axis mode axis(i)
void frame_pressure(const Side &S, const std::vector<Frame> &fr, int n_u, const int *b_rowptr,
                    const int *b_col, const double *const *b, const int *bt_rowptr,
                    const int *bt_col, const double *const *bt, std::vector<int> &brp,
                    std::vector<int> &bc, std::vector<double> (&bv)[3], std::vector<int> &btc,
                    std::vector<double> (&btv)[3]) {
  const int n_p = S.n_p;
  // per pressure DOF: the source row and its sign (B); per source column its
  // new column and sign (BT)
  std::vector<int> src(n_p), dst(n_p);
  std::vector<double> sg(n_p, 1.0), dsg(n_p, 1.0);
  for (int q = 0; q < n_p; ++q) src[q] = dst[q] = q;
  for (int c = 0; c < S.n_cells; ++c) {
    const Frame &F = fr[c];
    const int *dof = S.pg + 4 * (size_t)c;
    for (int i = 0; i < 3; ++i) {
      src[dof[1 + i]] = dof[1 + F.axis[i]];
      sg[dof[1 + i]] = F.sign[i];
      dst[dof[1 + F.axis[i]]] = dof[1 + i];
      dsg[dof[1 + F.axis[i]]] = F.sign[i];
    }
  }
  brp.assign(n_p + 1, 0);
  bc.clear();
  for (int k = 0; k < 3; ++k) bv[k].clear();
  for (int q = 0; q < n_p; ++q) {
    const int r = src[q];
    for (int e = b_rowptr[r]; e < b_rowptr[r + 1]; ++e) {
      bc.push_back(b_col[e]);
      for (int k = 0; k < 3; ++k) bv[k].push_back(sg[q] * b[k][e]);
    }
    brp[q + 1] = (int)bc.size();
  }
  btc.assign(bt_col, bt_col + bt_rowptr[n_u]);
  for (int k = 0; k < 3; ++k) btv[k].assign(bt[k], bt[k] + bt_rowptr[n_u]);
  for (int i = 0; i < n_u; ++i) {
    const int e0 = bt_rowptr[i], e1 = bt_rowptr[i + 1];
    std::vector<std::pair<int, int>> order;  // (new column, entry)
    for (int e = e0; e < e1; ++e) order.emplace_back(dst[bt_col[e]], e);
    std::sort(order.begin(), order.end());
    for (int t = 0; t < e1 - e0; ++t) {
      const int e = order[(size_t)t].second;
      btc[(size_t)e0 + t] = order[(size_t)t].first;
      for (int k = 0; k < 3; ++k) btv[k][(size_t)e0 + t] = dsg[bt_col[e]] * bt[k][e];
    }
  }
}

void make_mg_level(MGLevelStore &M, Side &S, int level, int n_active, int n_blocks,
                   const int *a_rowptr, const int *a_col, const double *const *a,
                   const std::vector<int> &brp, const std::vector<int> &bc,
                   const std::vector<double> (&bv)[3], const int *bt_rowptr,
                   const std::vector<int> &btc, const std::vector<double> (&btv)[3],
                   double alpha, double beta) {
  const int n_u = S.n_u, n_p = S.n_p, n = 3 * n_u + n_p;
  M.other_a = new TCollection(0, nullptr);
  M.other_b = new TCollection(0, nullptr);
  M.oa = new (M.oa_store) LevelSpace(M.other_a, 0, 0, 0, nullptr, nullptr, nullptr);
  M.ob = new (M.ob_store) LevelSpace(M.other_b, 0, 0, 0, nullptr, nullptr, nullptr);
  const int a_nnz = a_rowptr[n_u], b_nnz = brp[n_p], bt_nnz = bt_rowptr[n_u];
  M.sa = new LevelSquareStructure(n_u, n_active, a_nnz, copy_ints(a_col, a_nnz),
                                  copy_ints(a_rowptr, n_u + 1L), S.us);
  M.sb = new LevelStructure(M.oa, M.ob, S.ps, S.us, n_p, n_u, b_nnz,
                            copy_ints(bc.data(), b_nnz), copy_ints(brp.data(), n_p + 1L));
  M.sbt = new LevelStructure(M.oa, M.ob, S.us, S.ps, n_u, n_p, bt_nnz,
                             copy_ints(btc.data(), bt_nnz), copy_ints(bt_rowptr, n_u + 1L));
  for (int k = 0; k < 9; ++k) {
    M.A[k] = new (M.a_store[k]) TSquareMatrix3D(M.sa);  // allocates its entries
    // one-block levels: A11 = A22 = A33 = a[0], A12..A32 = 0
    const double *src = n_blocks == 9 ? a[k] : (k % 4 == 0 ? a[0] : nullptr);
    if (src)
      std::memcpy(M.A[k]->GetEntries(), src, sizeof(double) * a_nnz);
    else
      std::memset(M.A[k]->GetEntries(), 0, sizeof(double) * a_nnz);
  }
  for (int k = 0; k < 3; ++k) {
    M.B[k] = new (M.b_store[k]) TMatrix3D(M.sb);
    std::memcpy(M.B[k]->GetEntries(), bv[k].data(), sizeof(double) * b_nnz);
    M.B[3 + k] = new (M.b_store[3 + k]) TMatrix3D(M.sbt);
    std::memcpy(M.B[3 + k]->GetEntries(), btv[k].data(), sizeof(double) * bt_nnz);
  }
  M.f = new double[n]();
  M.u = new double[n]();
  M.al[0] = alpha;  // CellVanka's relaxation
  M.al[1] = beta;   // the coarse-grid correction's damping (TNSE_MGLevel::Update)
  // four auxiliary vectors, as TSystemNSE3D creates its levels; velocity
  // space 2 (Q2) and pressure space -11 (P1disc: the L2_0 projections of
  // CorrectNodes, CorrectDefect and Defect act on the constant modes)
  M.level = new (M.level_store)
      CycleLevel(level, M.A[0], M.A[1], M.A[2], M.A[3], M.A[4], M.A[5], M.A[6], M.A[7], M.A[8],
                 M.B[0], M.B[1], M.B[2], M.B[3], M.B[4], M.B[5], M.f, M.u, 4, M.al, 2, -11,
                 S.coll, nullptr);
}

void free_mg_level(MGLevelStore &M) {
  M.level->release();
  for (int k = 0; k < 9; ++k) delete[] M.A[k]->GetEntries();
  for (int k = 0; k < 6; ++k) delete[] M.B[k]->GetEntries();
  // the structures' destructors free their column and row-pointer copies
  delete M.sa;
  delete M.sb;
  delete M.sbt;
  M.oa->release_names();
  M.ob->release_names();
  delete M.other_a;
  delete M.other_b;
  delete[] M.f;
  delete[] M.u;
  delete[] M.colour_ptr;
  delete[] M.cell_order;
}

struct CycleChain {
  int pre = 2, post = 2, threads = 1;
  double damp = 1.0;
  Hier *H = nullptr;
  std::vector<MGLevelStore *> lev;
  TNSE_MultiGrid *mg = nullptr;
  alignas(TMultiGridIte) unsigned char ite_store[sizeof(TMultiGridIte)];
  TMultiGridIte *ite = nullptr;
};

}  // namespace

extern "C" {

// Nested levels as in build_hier (n_levels >= 2, level 0 the coarsest) with
// their matrices (per level, A: nine blocks a[9l..9l+8], or a[9l] alone for
// one-block levels; B: n_p x n_u, BT: n_u x n_p, three blocks each at 3l) as
// the solver's level descriptors hold them, the level relaxation alpha and
// the coarse-grid correction damping beta (al[0] and al[1] of every
// TNSE_MGLevel4, SC_GMG_DAMP_FACTOR_SADDLE).  Returns null when the levels
// are not a regular refinement.
__attribute__((visibility("default"))) void *ref_cycle_create(
    int n_levels, const int *n_cells, const int *n_u, const int *n_active, const int *n_p,
    const int *const *udofs, const int *const *pdofs, const int *const *parent,
    const int *const *child, int n_blocks, const int *const *a_rowptr, const int *const *a_col,
    const double *const *a, const int *const *b_rowptr, const int *const *b_col,
    const double *const *b, const int *const *bt_rowptr, const int *const *bt_col,
    const double *const *bt, double alpha, double beta) {
  Hier *H = build_hier(n_levels, n_cells, n_u, n_active, n_p, udofs, pdofs, parent, child);
  if (!H) return nullptr;
  CycleChain *Y = new CycleChain;
  Y->H = H;
  Y->mg = new TNSE_MultiGrid(1, 0, nullptr);
  for (int l = 0; l < n_levels; ++l) {
    Side &S = *H->sides[l];
    std::vector<int> brp, bc, btc;
    std::vector<double> bv[3], btv[3];
    frame_pressure(S, H->frames[l], S.n_u, b_rowptr[l], b_col[l], b + 3 * l, bt_rowptr[l],
                   bt_col[l], bt + 3 * l, brp, bc, bv, btc, btv);
    Y->lev.push_back(new MGLevelStore);
    make_mg_level(*Y->lev.back(), S, l, n_active[l], n_blocks, a_rowptr[l], a_col[l], a + 9 * l,
                  brp, bc, bv, bt_rowptr[l], btc, btv, alpha, beta);
    Y->mg->AddLevel(Y->lev.back()->level);
  }
  const int top = n_levels - 1, n_fine = 3 * n_u[top] + n_p[top];
  Y->ite = new (Y->ite_store) TMultiGridIte(nullptr, nullptr, nullptr, 0, n_fine, Y->mg, 1);
  return Y;
}

__attribute__((visibility("default"))) void ref_cycle_destroy(void *h) {
  CycleChain *Y = static_cast<CycleChain *>(h);
  if (!Y) return;
  // TItMethod's constructor allocates no vector for n_aux = 0
  for (MGLevelStore *M : Y->lev) {
    free_mg_level(*M);
    delete M;
  }
  ::operator delete(static_cast<void *>(Y->mg));  // storage only: no reference destructor
  free_hier(Y->H);
  delete Y;
}

// z = one V(pre, post) cycle from zero on v (finest level, [u1|u2|u3|p] with
// the pressure in the axis-aligned frame): TMultiGridIte::Iterate with cell
// Vanka on every level above the coarsest (SC_SMOOTHER_SADDLE 2, damping
// `damp`, direct local solves), the coarsest level solved exactly
// (SC_COARSE_SMOOTHER_SADDLE 17, first pressure equation pinned), no
// step-length control.
__attribute__((visibility("default"))) void ref_cycle_vcycle(void *h, const double *v, double *z,
                                                             int pre, int post, double damp) {
  CycleChain *Y = static_cast<CycleChain *>(h);
  TParamDB *db = TDatabase::ParamDB;
  db->SC_SMOOTHER_SADDLE = 2;
  db->SC_COARSE_SMOOTHER_SADDLE = 17;
  db->SC_PRE_SMOOTH_SADDLE = pre;
  db->SC_POST_SMOOTH_SADDLE = post;
  db->SC_SMOOTH_DAMP_FACTOR_SADDLE = damp;
  db->SC_SMOOTH_DAMP_FACTOR_COARSE_SADDLE = damp;
  db->SC_SMOOTH_DAMP_FACTOR_FINE_SADDLE = damp;
  db->SC_MG_CYCLE_SADDLE = 1;
  db->SC_STEP_LENGTH_CONTROL_ALL_SADDLE = 0;
  db->SC_STEP_LENGTH_CONTROL_FINE_SADDLE = 0;
  db->SC_LARGEST_DIRECT_SOLVE = 1 << 20;
  db->INTERNAL_LOCAL_DOF = -1;
  db->INTERNAL_PROJECT_PRESSURE = 1;
  db->INTERNAL_PRESSURE_SPACE = -11;
  db->SC_VERBOSE = 0;
  db->MG_DEBUG = 0;
#ifdef _HYBRID
  db->OMPNUMTHREADS = Y->threads;
#endif
  const int top = (int)Y->H->sides.size() - 1;
  const Side &F = *Y->H->sides[top];
  const int n = 3 * F.n_u + F.n_p;
  std::vector<double> rhs(v, v + n);
  convert_pressure(F, Y->H->frames[top], rhs.data() + 3 * (size_t)F.n_u, true);
  Y->ite->Iterate(nullptr, nullptr, z, rhs.data());
  convert_pressure(F, Y->H->frames[top], z + 3 * (size_t)F.n_u, false);
}

#ifdef _HYBRID
// The colour-parallel build: the colouring of level `level` (colour k holds
// the cells cell_order[colour_ptr[k] .. colour_ptr[k+1]-1], no two sharing a
// DOF) and the OpenMP threads of the colour loops (OMPNUMTHREADS; the result
// does not depend on it).  Every smoothed level needs one before a cycle.
// Returns 0, or -1 for an inconsistent colouring.
__attribute__((visibility("default"))) int ref_cycle_set_colours(void *h, int level,
                                                                 int n_colours,
                                                                 const int *colour_ptr,
                                                                 const int *cell_order,
                                                                 int n_cells, int threads) {
  CycleChain *Y = static_cast<CycleChain *>(h);
  if (level < 0 || level >= (int)Y->lev.size() || n_cells != Y->H->sides[level]->n_cells ||
      n_colours <= 0 || colour_ptr[0] != 0 || colour_ptr[n_colours] != n_cells || threads <= 0)
    return -1;
  int max_cells = 0;
  for (int k = 0; k < n_colours; ++k) {
    const int m = colour_ptr[k + 1] - colour_ptr[k];
    if (m <= 0) return -1;
    max_cells = std::max(max_cells, m);
  }
  MGLevelStore &M = *Y->lev[level];
  delete[] M.colour_ptr;
  delete[] M.cell_order;
  M.colour_ptr = copy_ints(colour_ptr, n_colours + 1L);
  M.cell_order = copy_ints(cell_order, n_cells);
  M.level->set_colours(n_colours, M.colour_ptr, M.cell_order, max_cells);
  Y->threads = threads;
  return 0;
}
#endif

// The smoothing counts and damping of ref_cycle_precond (V(2,2) with
// damping 1 until set).
__attribute__((visibility("default"))) void ref_cycle_configure(void *h, int pre, int post,
                                                                double damp) {
  CycleChain *Y = static_cast<CycleChain *>(h);
  Y->pre = pre;
  Y->post = post;
  Y->damp = damp;
}

// The cycle as a preconditioner callback z = M(v), the signature ref_fgmres
// of oracle/ref_harness.cpp takes.
__attribute__((visibility("default"))) void ref_cycle_precond(void *h, double *z, const double *v) {
  CycleChain *Y = static_cast<CycleChain *>(h);
  ref_cycle_vcycle(h, v, z, Y->pre, Y->post, Y->damp);
}

}  // extern "C"
