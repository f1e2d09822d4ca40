// oseen_tet.cpp — tetrahedral levels of the caller-side problem builder:
// every cube of the hexahedral hierarchy split into 6 Kuhn tetrahedra (all
// sharing the cube's main diagonal; the split of a refined cube refines the
// split of its parent, so the levels are nested), P2 velocity enriched by 4
// face and 1 cell bubble (15 nodes, ParMooN's C_B2_3D_T_A,
// include/FE3D/BF_C_T_B2_3D.h, the stable partner of P1disc,
// src/General/MainUtilities.C:2711-2716) and P1disc pressure
// (include/FE3D/BF_D_T_P1_3D.h).  Local block 3 * 15 + 4 = 49.
//
// Nodal functionals are point values at the reference points of
// include/FE3D/NF_C_T_B2_3D.h: vertices 0, 2, 5, 9, edge midpoints 1, 3, 4,
// 6, 7, 8, face barycentres 10-13, cell barycentre 14.  The basis is the
// Lagrange basis of P2 + {l_a l_b l_c} + {l0 l1 l2 l3} at those points,
// obtained by inverting the nodal matrix of that spanning set.
//
// Galerkin Oseen forms as on the hexahedra (NSType4Galerkin3D,
// src/FE/NSE3D_FixPo.C:1919-2071) with b the nodal interpolant of the
// convection field; quadrature: a Duffy-mapped Gauss-Legendre rule with 7
// points per direction (exact to degree 11, the degree of
// phi_i (b . grad phi_j) for b in the same space).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oseen_internal.h"

namespace pmh_detail {
namespace {

constexpr int NT = 15;  // velocity nodes per tetrahedron
constexpr int NQ1 = 7;  // Gauss points per direction of the Duffy rule
constexpr int NQ = NQ1 * NQ1 * NQ1;

// reference points of the 15 nodal functionals
const double kNode[NT][3] = {{0, 0, 0},     {0.5, 0, 0},   {1, 0, 0},     {0, 0.5, 0},
                             {0.5, 0.5, 0}, {0, 1, 0},     {0, 0, 0.5},   {0.5, 0, 0.5},
                             {0, 0.5, 0.5}, {0, 0, 1},     {1.0 / 3, 1.0 / 3, 0},
                             {1.0 / 3, 0, 1.0 / 3},        {1.0 / 3, 1.0 / 3, 1.0 / 3},
                             {0, 1.0 / 3, 1.0 / 3},        {0.25, 0.25, 0.25}};
// vertices (0..3) of the edge / face nodes
const int kEdge[6][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}};  // nodes 1,3,4,6,7,8
const int kEdgeNode[6] = {1, 3, 4, 6, 7, 8};
const int kFace[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};      // nodes 10..13
const int kVertexNode[4] = {0, 2, 5, 9};

// spanning set: 4 vertex and 6 edge P2 functions, 4 face cubics, 1 quartic
void spanning(double xi, double eta, double zeta, double *v, double *d) {
  const double l[4] = {1.0 - xi - eta - zeta, xi, eta, zeta};
  const double g[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  int k = 0;
  for (int i = 0; i < 4; ++i, ++k) {
    v[k] = l[i] * (2.0 * l[i] - 1.0);
    for (int c = 0; c < 3; ++c) d[3 * k + c] = (4.0 * l[i] - 1.0) * g[i][c];
  }
  for (int e = 0; e < 6; ++e, ++k) {
    const int a = kEdge[e][0], b = kEdge[e][1];
    v[k] = 4.0 * l[a] * l[b];
    for (int c = 0; c < 3; ++c) d[3 * k + c] = 4.0 * (g[a][c] * l[b] + l[a] * g[b][c]);
  }
  for (int f = 0; f < 4; ++f, ++k) {
    const int a = kFace[f][0], b = kFace[f][1], e = kFace[f][2];
    v[k] = l[a] * l[b] * l[e];
    for (int c = 0; c < 3; ++c)
      d[3 * k + c] = g[a][c] * l[b] * l[e] + l[a] * g[b][c] * l[e] + l[a] * l[b] * g[e][c];
  }
  v[k] = l[0] * l[1] * l[2] * l[3];
  for (int c = 0; c < 3; ++c)
    d[3 * k + c] = g[0][c] * l[1] * l[2] * l[3] + l[0] * g[1][c] * l[2] * l[3] +
                   l[0] * l[1] * g[2][c] * l[3] + l[0] * l[1] * l[2] * g[3][c];
}

// inverse of a small dense matrix (Gauss-Jordan, partial pivoting)
void invert(int n, double *a, double *inv) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) inv[i * n + j] = i == j ? 1.0 : 0.0;
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r * n + c]) > std::fabs(a[p * n + c])) p = r;
    for (int j = 0; j < n; ++j) {
      std::swap(a[c * n + j], a[p * n + j]);
      std::swap(inv[c * n + j], inv[p * n + j]);
    }
    const double s = 1.0 / a[c * n + c];
    for (int j = 0; j < n; ++j) {
      a[c * n + j] *= s;
      inv[c * n + j] *= s;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = a[r * n + c];
      if (f == 0.0) continue;
      for (int j = 0; j < n; ++j) {
        a[r * n + j] -= f * a[c * n + j];
        inv[r * n + j] -= f * inv[c * n + j];
      }
    }
  }
}

// coefficients A (phi_i = sum_k A[i][k] psi_k): A = Psi^{-1}, Psi[k][p] = psi_k(x_p)
struct B2Coef {
  double A[NT][NT];
  B2Coef() {
    double Psi[NT * NT], v[NT], d[3 * NT];
    for (int p = 0; p < NT; ++p) {
      spanning(kNode[p][0], kNode[p][1], kNode[p][2], v, d);
      for (int k = 0; k < NT; ++k) Psi[k * NT + p] = v[k];
    }
    invert(NT, Psi, &A[0][0]);
  }
};
const B2Coef &b2_coef() {
  static B2Coef c;
  return c;
}

// Gauss-Legendre points and weights on [0, 1] (Newton iteration on the
// three-term recurrence of the Legendre polynomials)
void gauss_legendre01(int n, double *x, double *w) {
  for (int i = 0; i < n; ++i) {
    double t = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = t;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (t * p1 - p0) / (t * t - 1.0);
      const double dt = p1 / dp;
      t -= dt;
      if (std::fabs(dt) < 1e-16) break;
    }
    x[i] = 0.5 * (1.0 - t);
    w[i] = 1.0 / ((1.0 - t * t) * dp * dp);  // 2 / ((1-t^2) p'^2) / 2
  }
}

// reference tables at the quadrature points and reference integrals
struct TetTables {
  double w[NQ], pt[NQ][3];
  double phi[NQ][NT], dphi[NQ][NT][3], psi[NQ][4];
  double S[3][3][NT][NT];  // sum_q w dphi_i,a dphi_j,b
  double Bref[3][4][NT];   // sum_q w psi_m dphi_j,a
  double Mp[4][4];         // psi_m at the reference vertices: [vertex][mode]
  TetTables() {
    double gx[NQ1], gw[NQ1];
    gauss_legendre01(NQ1, gx, gw);
    int q = 0;
    for (int a = 0; a < NQ1; ++a)
      for (int b = 0; b < NQ1; ++b)
        for (int c = 0; c < NQ1; ++c, ++q) {
          const double u = gx[a], v = gx[b], t = gx[c];
          pt[q][0] = u;
          pt[q][1] = v * (1.0 - u);
          pt[q][2] = t * (1.0 - u) * (1.0 - v);
          w[q] = gw[a] * gw[b] * gw[c] * (1.0 - u) * (1.0 - u) * (1.0 - v);
          double der[3 * NT], pd[12];
          b2_basis(pt[q][0], pt[q][1], pt[q][2], phi[q], der);
          for (int i = 0; i < NT; ++i)
            for (int e = 0; e < 3; ++e) dphi[q][i][e] = der[3 * i + e];
          p1t_basis(pt[q][0], pt[q][1], pt[q][2], psi[q], pd);
        }
    std::memset(S, 0, sizeof(S));
    std::memset(Bref, 0, sizeof(Bref));
    for (q = 0; q < NQ; ++q)
      for (int a = 0; a < 3; ++a) {
        for (int b = 0; b < 3; ++b)
          for (int i = 0; i < NT; ++i)
            for (int j = 0; j < NT; ++j) S[a][b][i][j] += w[q] * dphi[q][i][a] * dphi[q][j][b];
        for (int m = 0; m < 4; ++m)
          for (int j = 0; j < NT; ++j) Bref[a][m][j] += w[q] * psi[q][m] * dphi[q][j][a];
      }
    const double rv[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 4; ++i) {
      double pd[12];
      p1t_basis(rv[i][0], rv[i][1], rv[i][2], Mp[i], pd);
    }
  }
};
const TetTables &tet_tables() {
  static TetTables t;
  return t;
}

// Kuhn tetrahedron p of a cube: vertex offsets (0,0,0), e_a, e_a + e_b, (1,1,1)
const int kPerm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
void kuhn_vertices(int p, int off[4][3]) {
  for (int c = 0; c < 3; ++c) off[0][c] = 0, off[3][c] = 1;
  for (int c = 0; c < 3; ++c) off[1][c] = (c == kPerm[p][0]) ? 1 : 0;
  for (int c = 0; c < 3; ++c) off[2][c] = off[1][c] + ((c == kPerm[p][1]) ? 1 : 0);
}

struct Affine {
  double v0[3], J[3][3], Ji[3][3], det;  // x = v0 + J xi
};
Affine affine(const double *xyz) {  // 4 vertices, 12 doubles
  Affine f;
  for (int c = 0; c < 3; ++c) {
    f.v0[c] = xyz[c];
    for (int k = 0; k < 3; ++k) f.J[c][k] = xyz[3 * (k + 1) + c] - xyz[c];
  }
  const double(*J)[3] = f.J;
  f.det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
          J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  const double id = 1.0 / f.det;
  f.Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
  f.Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
  f.Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  f.Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
  f.Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  f.Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
  f.Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
  f.Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
  f.Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  return f;
}
void to_ref(const Affine &f, const double *x, double *xi) {
  const double d[3] = {x[0] - f.v0[0], x[1] - f.v0[1], x[2] - f.v0[2]};
  for (int k = 0; k < 3; ++k) xi[k] = f.Ji[k][0] * d[0] + f.Ji[k][1] * d[1] + f.Ji[k][2] * d[2];
}

int find_col(const int *cols, int n, int key) {
  const int *p = std::lower_bound(cols, cols + n, key);
  return (p != cols + n && *p == key) ? (int)(p - cols) : -1;
}

// structure of one level: DOFs, cells, patterns, colours
void build_structure(PMLevelData &L) {
  const int gx = L.gx(), gy = L.gy(), gz = L.gz();
  const int ncube = L.nx * L.ny * L.nz;
  L.nu_loc = NT;
  L.n_cells = 6 * ncube;
  L.n_pdof = 4 * L.n_cells;
  auto gidx = [&](int i, int j, int k) { return i + gx * (j + gy * k); };
  auto on_bd = [&](int i, int j, int k) {
    return i == 0 || j == 0 || k == 0 || i == gx - 1 || j == gy - 1 || k == gz - 1;
  };
  // local nodes of every tetrahedron: grid nodes (0..9) and face keys (10..13)
  std::vector<int> loc_grid((size_t)L.n_cells * 10);
  std::vector<long long> face_key((size_t)L.n_cells * 4);
  std::vector<unsigned char> face_bd((size_t)L.n_cells * 4);
  L.cell_colour.resize(L.n_cells);
  L.tet_xyz.resize((size_t)L.n_cells * 12);
  for (int cz = 0; cz < L.nz; ++cz)
    for (int cy = 0; cy < L.ny; ++cy)
      for (int cx = 0; cx < L.nx; ++cx) {
        const int cube = cx + L.nx * (cy + L.ny * cz);
        for (int p = 0; p < 6; ++p) {
          const int t = 6 * cube + p;
          int off[4][3], V[4][3];
          kuhn_vertices(p, off);
          for (int v = 0; v < 4; ++v) {
            V[v][0] = 2 * (cx + off[v][0]);
            V[v][1] = 2 * (cy + off[v][1]);
            V[v][2] = 2 * (cz + off[v][2]);
            L.tet_xyz[(size_t)t * 12 + 3 * v + 0] = L.node_x(V[v][0]);
            L.tet_xyz[(size_t)t * 12 + 3 * v + 1] = L.node_y(V[v][1]);
            L.tet_xyz[(size_t)t * 12 + 3 * v + 2] = L.node_z(V[v][2]);
          }
          int *g = &loc_grid[(size_t)t * 10];
          for (int v = 0; v < 4; ++v) g[kVertexNode[v]] = gidx(V[v][0], V[v][1], V[v][2]);
          for (int e = 0; e < 6; ++e) {
            const int a = kEdge[e][0], b = kEdge[e][1];
            g[kEdgeNode[e]] = gidx((V[a][0] + V[b][0]) / 2, (V[a][1] + V[b][1]) / 2,
                                   (V[a][2] + V[b][2]) / 2);
          }
          for (int f = 0; f < 4; ++f) {
            long long k3[3];
            for (int c = 0; c < 3; ++c) {
              const int *P = V[kFace[f][c]];
              k3[c] = gidx(P[0], P[1], P[2]);
            }
            std::sort(k3, k3 + 3);
            const long long ng = (long long)gx * gy * gz;
            face_key[(size_t)t * 4 + f] = (k3[0] * ng + k3[1]) * ng + k3[2];
            // boundary face: its three vertices share an extreme coordinate
            bool b = false;
            const int gmax[3] = {gx - 1, gy - 1, gz - 1};
            for (int c = 0; c < 3 && !b; ++c)
              for (int side = 0; side < 2 && !b; ++side) {
                const int val = side ? gmax[c] : 0;
                b = V[kFace[f][0]][c] == val && V[kFace[f][1]][c] == val &&
                    V[kFace[f][2]][c] == val;
              }
            face_bd[(size_t)t * 4 + f] = b ? 1 : 0;
          }
          L.cell_colour[t] = (cx & 1) + 2 * (cy & 1) + 4 * (cz & 1) + 8 * p;
        }
      }
  // faces: first appearance in cell order
  std::unordered_map<long long, int> face_id;
  face_id.reserve((size_t)L.n_cells * 2);
  std::vector<int> tface((size_t)L.n_cells * 4);
  std::vector<unsigned char> fbd;
  for (size_t k = 0; k < face_key.size(); ++k) {
    auto it = face_id.find(face_key[k]);
    if (it == face_id.end()) {
      const int id = (int)fbd.size();
      face_id.emplace(face_key[k], id);
      fbd.push_back(face_bd[k]);
      tface[k] = id;
    } else {
      tface[k] = it->second;
    }
  }
  const int nface = (int)fbd.size(), ngrid = gx * gy * gz;
  // numbering: active grid nodes, active faces, cells; then Dirichlet grid
  // nodes and faces
  std::vector<int> gdof(ngrid, -1), fdof(nface, -1);
  int next = 0;
  for (int k = 0; k < gz; ++k)
    for (int j = 0; j < gy; ++j)
      for (int i = 0; i < gx; ++i)
        if (!on_bd(i, j, k)) gdof[gidx(i, j, k)] = next++;
  for (int f = 0; f < nface; ++f)
    if (!fbd[f]) fdof[f] = next++;
  const int cell0 = next;
  next += L.n_cells;
  L.n_active = next;
  for (int k = 0; k < gz; ++k)
    for (int j = 0; j < gy; ++j)
      for (int i = 0; i < gx; ++i)
        if (on_bd(i, j, k)) gdof[gidx(i, j, k)] = next++;
  for (int f = 0; f < nface; ++f)
    if (fbd[f]) fdof[f] = next++;
  L.n_udof = next;
  L.cell_udofs.resize((size_t)L.n_cells * NT);
  L.cell_pdofs.resize((size_t)L.n_cells * 4);
  L.node_xyz.assign((size_t)3 * L.n_udof, 0.0);
  for (int t = 0; t < L.n_cells; ++t) {
    int *ud = &L.cell_udofs[(size_t)t * NT];
    for (int k = 0; k < 10; ++k) ud[k] = gdof[loc_grid[(size_t)t * 10 + k]];
    for (int f = 0; f < 4; ++f) ud[10 + f] = fdof[tface[(size_t)t * 4 + f]];
    ud[14] = cell0 + t;
    for (int m = 0; m < 4; ++m) L.cell_pdofs[(size_t)t * 4 + m] = 4 * t + m;
    // DOF positions: the nodes of the affine image of the reference points
    const Affine A = affine(&L.tet_xyz[(size_t)t * 12]);
    for (int k = 0; k < NT; ++k) {
      double *x = &L.node_xyz[(size_t)3 * ud[k]];
      for (int c = 0; c < 3; ++c)
        x[c] = A.v0[c] + A.J[c][0] * kNode[k][0] + A.J[c][1] * kNode[k][1] +
               A.J[c][2] * kNode[k][2];
    }
  }
  // DOF -> cells incidence
  std::vector<int> iptr(L.n_udof + 1, 0), ient((size_t)L.n_cells * NT);
  for (size_t k = 0; k < L.cell_udofs.size(); ++k) iptr[L.cell_udofs[k] + 1]++;
  for (int r = 0; r < L.n_udof; ++r) iptr[r + 1] += iptr[r];
  {
    std::vector<int> fill(iptr.begin(), iptr.end() - 1);
    for (int t = 0; t < L.n_cells; ++t)
      for (int k = 0; k < NT; ++k) ient[fill[L.cell_udofs[(size_t)t * NT + k]]++] = t;
  }
  const int nu = L.n_udof;
  auto a_row = [&](int r, std::vector<int> &out) {
    out.clear();
    for (int e = iptr[r]; e < iptr[r + 1]; ++e)
      for (int k = 0; k < NT; ++k) out.push_back(L.cell_udofs[(size_t)ient[e] * NT + k]);
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
  };
  L.a_rowptr.assign(nu + 1, 0);
#pragma omp parallel
  {
    std::vector<int> buf;
#pragma omp for schedule(static)
    for (int r = 0; r < nu; ++r) {
      if (r >= L.n_active) {
        L.a_rowptr[r + 1] = 1;
        continue;
      }
      a_row(r, buf);
      L.a_rowptr[r + 1] = (int)buf.size();
    }
  }
  for (int r = 0; r < nu; ++r) L.a_rowptr[r + 1] += L.a_rowptr[r];
  L.a_col.resize(L.a_rowptr[nu]);
#pragma omp parallel
  {
    std::vector<int> buf;
#pragma omp for schedule(static)
    for (int r = 0; r < nu; ++r) {
      if (r >= L.n_active) {
        L.a_col[L.a_rowptr[r]] = r;
        continue;
      }
      a_row(r, buf);
      std::copy(buf.begin(), buf.end(), L.a_col.begin() + L.a_rowptr[r]);
    }
  }
  for (int b = 0; b < 9; ++b) L.a[b].assign(L.a_col.size(), 0.0);
  // B: row 4t+m -> the cell's 15 velocity DOFs, sorted
  L.b_rowptr.resize(L.n_pdof + 1);
  for (int p = 0; p <= L.n_pdof; ++p) L.b_rowptr[p] = NT * p;
  L.b_col.resize((size_t)NT * L.n_pdof);
  for (int t = 0; t < L.n_cells; ++t) {
    int sorted[NT];
    std::memcpy(sorted, &L.cell_udofs[(size_t)t * NT], sizeof(sorted));
    std::sort(sorted, sorted + NT);
    for (int m = 0; m < 4; ++m) std::memcpy(&L.b_col[(size_t)(4 * t + m) * NT], sorted, sizeof(sorted));
  }
  for (int b = 0; b < 3; ++b) L.b[b].assign(L.b_col.size(), 0.0);
  // BT: row r -> the pressure DOFs of the cells containing r, sorted
  L.bt_rowptr.assign(nu + 1, 0);
  for (int r = 0; r < nu; ++r) L.bt_rowptr[r + 1] = 4 * (iptr[r + 1] - iptr[r]);
  for (int r = 0; r < nu; ++r) L.bt_rowptr[r + 1] += L.bt_rowptr[r];
  L.bt_col.resize(L.bt_rowptr[nu]);
  for (int r = 0; r < nu; ++r) {
    int *out = L.bt_col.data() + L.bt_rowptr[r];
    int n = 0;
    for (int e = iptr[r]; e < iptr[r + 1]; ++e)
      for (int m = 0; m < 4; ++m) out[n++] = 4 * ient[e] + m;
    std::sort(out, out + n);
  }
  for (int b = 0; b < 3; ++b) L.bt[b].assign(L.bt_col.size(), 0.0);
}

// P (fine x coarse) by nodal interpolation of the coarse functions at the
// fine nodes; pressure: the fine P1disc representation of the coarse linear
// function on each fine cell
void build_prolongation(const PMLevelData &C, PMLevelData &F) {
  const TetTables &T = tet_tables();
  F.cell_parent.assign(F.n_cells, -1);
  F.cell_child.assign(F.n_cells, -1);
  std::vector<std::vector<std::pair<int, double>>> rows(F.n_udof);
  std::vector<unsigned char> done(F.n_udof, 0);
  F.pp_rowptr.assign(F.n_pdof + 1, 0);
  F.pp_col.assign((size_t)F.n_pdof * 4, 0);
  F.pp_val.assign((size_t)F.n_pdof * 4, 0.0);
  double Mpinv[16], Mp[16];
  for (int i = 0; i < 4; ++i)
    for (int m = 0; m < 4; ++m) Mp[i * 4 + m] = T.Mp[i][m];
  invert(4, Mp, Mpinv);  // [mode][vertex]
  std::vector<int> nchild(C.n_cells, 0);
  for (int t = 0; t < F.n_cells; ++t) {
    const int cube = t / 6;
    const int fx = cube % F.nx, fy = (cube / F.nx) % F.ny, fz = cube / (F.nx * F.ny);
    const int ccube = fx / 2 + C.nx * (fy / 2 + C.ny * (fz / 2));
    const double *xt = &F.tet_xyz[(size_t)t * 12];
    const double cen[3] = {0.25 * (xt[0] + xt[3] + xt[6] + xt[9]),
                           0.25 * (xt[1] + xt[4] + xt[7] + xt[10]),
                           0.25 * (xt[2] + xt[5] + xt[8] + xt[11])};
    int parent = -1;
    Affine Ac{};
    for (int p = 0; p < 6 && parent < 0; ++p) {
      const int tc = 6 * ccube + p;
      Ac = affine(&C.tet_xyz[(size_t)tc * 12]);
      double xi[3];
      to_ref(Ac, cen, xi);
      if (xi[0] > -1e-12 && xi[1] > -1e-12 && xi[2] > -1e-12 && xi[0] + xi[1] + xi[2] < 1 + 1e-12)
        parent = tc;
    }
    F.cell_parent[t] = parent;
    F.cell_child[t] = parent >= 0 ? nchild[parent]++ : -1;
    if (parent < 0) {  // cannot happen for nested Kuhn splits; keep the CSR consistent
      for (int m = 0; m < 4; ++m) F.pp_rowptr[4 * t + m + 1] = 4;
      continue;
    }
    const int *cud = &C.cell_udofs[(size_t)parent * NT];
    const int *fud = &F.cell_udofs[(size_t)t * NT];
    for (int k = 0; k < NT; ++k) {
      const int r = fud[k];
      if (done[r]) continue;
      done[r] = 1;
      double xi[3], v[NT];
      to_ref(Ac, &F.node_xyz[(size_t)3 * r], xi);
      b2_basis(xi[0], xi[1], xi[2], v, nullptr);
      for (int j = 0; j < NT; ++j)
        if (std::fabs(v[j]) > 1e-14) rows[r].emplace_back(cud[j], v[j]);
    }
    // pressure: E[i][n] = psi_n(coarse reference coordinates of fine vertex i)
    double E[4][4];
    for (int i = 0; i < 4; ++i) {
      double xi[3], pd[12];
      to_ref(Ac, xt + 3 * i, xi);
      p1t_basis(xi[0], xi[1], xi[2], E[i], pd);
    }
    for (int m = 0; m < 4; ++m) {
      const int row = 4 * t + m;
      for (int n = 0; n < 4; ++n) {
        double s = 0.0;
        for (int i = 0; i < 4; ++i) s += Mpinv[m * 4 + i] * E[i][n];
        F.pp_col[(size_t)row * 4 + n] = 4 * parent + n;
        F.pp_val[(size_t)row * 4 + n] = s;
      }
      F.pp_rowptr[row + 1] = 4;
    }
  }
  for (int r = 0; r < F.n_pdof; ++r) F.pp_rowptr[r + 1] += F.pp_rowptr[r];
  F.pu_rowptr.assign(F.n_udof + 1, 0);
  for (int r = 0; r < F.n_udof; ++r) {
    std::sort(rows[r].begin(), rows[r].end());
    F.pu_rowptr[r + 1] = F.pu_rowptr[r] + (int)rows[r].size();
  }
  F.pu_col.resize(F.pu_rowptr[F.n_udof]);
  F.pu_val.resize(F.pu_rowptr[F.n_udof]);
  for (int r = 0; r < F.n_udof; ++r) {
    int o = F.pu_rowptr[r];
    for (auto &e : rows[r]) {
      F.pu_col[o] = e.first;
      F.pu_val[o++] = e.second;
    }
  }
}

}  // namespace

void b2_basis(double xi, double eta, double zeta, double *val, double *der) {
  const B2Coef &c = b2_coef();
  double v[NT], d[3 * NT];
  spanning(xi, eta, zeta, v, d);
  for (int i = 0; i < NT; ++i) {
    double s = 0.0, s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = 0; k < NT; ++k) {
      s += c.A[i][k] * v[k];
      s0 += c.A[i][k] * d[3 * k];
      s1 += c.A[i][k] * d[3 * k + 1];
      s2 += c.A[i][k] * d[3 * k + 2];
    }
    if (val) val[i] = s;
    if (der) {
      der[3 * i] = s0;
      der[3 * i + 1] = s1;
      der[3 * i + 2] = s2;
    }
  }
}

// D_T_P1_3D: the constant 6 (unit integral on the reference tetrahedron) and
// three linear modes with zero mean; kept as the reference defines them so
// that pressure DOF values mean the same
void p1t_basis(double xi, double eta, double zeta, double *val, double *der) {
  val[0] = 6.0;
  val[1] = -1.0 + 2.0 * xi + eta + zeta;
  val[2] = -1.0 + xi + 2.0 * eta + zeta;
  val[3] = -1.0 + xi + eta + 2.0 * zeta;
  if (der) {
    const double d[12] = {0, 0, 0, 2, 1, 1, 1, 2, 1, 1, 1, 2};
    std::memcpy(der, d, sizeof(d));
  }
}

void assemble_tet_level(pmh_problem &P, PMLevelData &L, bool finest) {
  const TetTables &T = tet_tables();
  const double nu = P.prm.nu;
  // convection at the velocity DOFs (the nodal interpolant is the FE field)
  std::vector<double> bnod((size_t)3 * L.n_udof);
#pragma omp parallel for schedule(static)
  for (int r = 0; r < L.n_udof; ++r)
    convection(P, L.node_xyz[3 * r], L.node_xyz[3 * r + 1], L.node_xyz[3 * r + 2],
               &bnod[(size_t)3 * r]);
  if (finest) P.rhs.assign((size_t)3 * L.n_udof + L.n_pdof, 0.0);
  const int ncol = 48;
  for (int colour = 0; colour < ncol; ++colour) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int t = 0; t < L.n_cells; ++t) {
      if (L.cell_colour[t] != colour) continue;
      const Affine A = affine(&L.tet_xyz[(size_t)t * 12]);
      const double det = std::fabs(A.det);
      const int *ud = &L.cell_udofs[(size_t)t * NT];
      // G = Ji Ji^T (reference metric of the gradients)
      double G[3][3];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          G[a][b] = A.Ji[a][0] * A.Ji[b][0] + A.Ji[a][1] * A.Ji[b][1] + A.Ji[a][2] * A.Ji[b][2];
      double Aloc[NT][NT];
      for (int i = 0; i < NT; ++i)
        for (int j = 0; j < NT; ++j) {
          double s = 0.0;
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) s += G[a][b] * T.S[a][b][i][j];
          Aloc[i][j] = nu * det * s;
        }
      double bl[NT][3];
      for (int k = 0; k < NT; ++k)
        for (int c = 0; c < 3; ++c) bl[k][c] = bnod[(size_t)3 * ud[k] + c];
      double floc[3][NT];
      std::memset(floc, 0, sizeof(floc));
      for (int q = 0; q < NQ; ++q) {
        double bq[3] = {0, 0, 0};
        for (int k = 0; k < NT; ++k)
          for (int c = 0; c < 3; ++c) bq[c] += bl[k][c] * T.phi[q][k];
        // b . grad = (Ji b) . grad_ref
        double br[3];
        for (int a = 0; a < 3; ++a) br[a] = A.Ji[a][0] * bq[0] + A.Ji[a][1] * bq[1] + A.Ji[a][2] * bq[2];
        double g[NT];
        for (int j = 0; j < NT; ++j)
          g[j] = br[0] * T.dphi[q][j][0] + br[1] * T.dphi[q][j][1] + br[2] * T.dphi[q][j][2];
        const double wq = T.w[q] * det;
        for (int i = 0; i < NT; ++i) {
          const double wi = wq * T.phi[q][i];
          for (int j = 0; j < NT; ++j) Aloc[i][j] += wi * g[j];
        }
        if (finest) {
          double x[3], f[3];
          for (int c = 0; c < 3; ++c)
            x[c] = A.v0[c] + A.J[c][0] * T.pt[q][0] + A.J[c][1] * T.pt[q][1] +
                   A.J[c][2] * T.pt[q][2];
          forcing(P, x[0], x[1], x[2], f);
          for (int i = 0; i < NT; ++i)
            for (int c = 0; c < 3; ++c) floc[c][i] += wq * f[c] * T.phi[q][i];
        }
      }
      // B_d[m][j] = -int psi_m d_d phi_j = -det sum_a Ji[a][d] Bref_a[m][j]
      double Bloc[3][4][NT];
      for (int d = 0; d < 3; ++d)
        for (int m = 0; m < 4; ++m)
          for (int j = 0; j < NT; ++j)
            Bloc[d][m][j] = -det * (A.Ji[0][d] * T.Bref[0][m][j] + A.Ji[1][d] * T.Bref[1][m][j] +
                                    A.Ji[2][d] * T.Bref[2][m][j]);
      for (int i = 0; i < NT; ++i) {
        const int r = ud[i];
        if (r >= L.n_active) continue;
        const int rs = L.a_rowptr[r], rn = L.a_rowptr[r + 1] - rs;
        for (int j = 0; j < NT; ++j) {
          const int pos = find_col(&L.a_col[rs], rn, ud[j]);
          if (pos < 0) continue;
          L.a[0][rs + pos] += Aloc[i][j];
          L.a[4][rs + pos] += Aloc[i][j];
          L.a[8][rs + pos] += Aloc[i][j];
        }
        const int bs = L.bt_rowptr[r], bn = L.bt_rowptr[r + 1] - bs;
        for (int m = 0; m < 4; ++m) {
          const int pos = find_col(&L.bt_col[bs], bn, 4 * t + m);
          if (pos < 0) continue;
          for (int d = 0; d < 3; ++d) L.bt[d][bs + pos] += Bloc[d][m][i];
        }
        if (finest)
          for (int d = 0; d < 3; ++d) P.rhs[(size_t)d * L.n_udof + r] += floc[d][i];
      }
      for (int m = 0; m < 4; ++m) {
        const int p = 4 * t + m, bs = L.b_rowptr[p];
        for (int j = 0; j < NT; ++j) {
          const int pos = find_col(&L.b_col[bs], NT, ud[j]);
          for (int d = 0; d < 3; ++d) L.b[d][bs + pos] += Bloc[d][m][j];
        }
      }
    }
  }
  for (int r = L.n_active; r < L.n_udof; ++r) {
    const int pos = L.a_rowptr[r];
    for (int b = 0; b < 9; ++b) L.a[b][pos] = 1.0;
  }
  if (finest)
    for (int r = L.n_active; r < L.n_udof; ++r) {
      double u[3];
      boundary_value(P, L.node_xyz[3 * r], L.node_xyz[3 * r + 1], L.node_xyz[3 * r + 2], u);
      for (int d = 0; d < 3; ++d) P.rhs[(size_t)d * L.n_udof + r] = u[d];
    }
}

void build_tet_levels(pmh_problem &P) {
  const int nl = (int)P.levels.size();
  for (int l = 0; l < nl; ++l) build_structure(P.levels[l]);
  for (int l = 1; l < nl; ++l) build_prolongation(P.levels[l - 1], P.levels[l]);
}

}  // namespace pmh_detail
