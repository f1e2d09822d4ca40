// oracle.cpp — FP64 CPU restatement of ParMooN's FGMRES + GMG + cell-Vanka
// path for NSTYPE-4 Q2/P1disc systems.  TEST INFRASTRUCTURE: the checker for
// the GPU library and the CPU baseline timed by bench.py; never part of the
// product.  Each function cites the reference code it restates.
#include "oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const int NU_LOC = 27;  // Q2 local DOFs (hexahedral transfer tables)
const int NP_LOC = 4;   // P1disc local DOFs
const int NLOC_MAX = 3 * NU_LOC + NP_LOC;  // 85: the largest local block

struct OLevel {
  pm_level_desc d;
  int nu = 0, np = 0, ndof = 0;
  int nl = 27, nloc = 85;  // velocity nodes per cell, local block size (27/85 or 15/49)
  std::vector<double> sol, rhs, aux0, aux1;
  // children[parent*8 + childnumber] = fine cell (stored on the fine level)
  std::vector<int> children;
  std::vector<int> colour_ptr, colour_cells;
  std::vector<std::vector<double>> fac;  // reuse_factors variant
  std::vector<std::vector<int>> piv;
};

// Q2 basis on [-1,1]^3, local function a+3b+9c (C_H_Q2_3D_Funct order).
void q2_values(double xi, double eta, double zeta, double *v) {
  auto L = [](double t, double *o) {
    o[0] = 0.5 * t * (t - 1.0);
    o[1] = 1.0 - t * t;
    o[2] = 0.5 * t * (t + 1.0);
  };
  double vx[3], vy[3], vz[3];
  L(xi, vx);
  L(eta, vy);
  L(zeta, vz);
  for (int c = 0; c < 3; ++c)
    for (int b = 0; b < 3; ++b)
      for (int a = 0; a < 3; ++a) v[a + 3 * b + 9 * c] = vx[a] * vy[b] * vz[c];
}

}  // namespace

struct oracle {
  oracle_params p;
  std::vector<OLevel> L;
  // prolongation matrices per child, QQ[k][l]: coarse basis l evaluated by
  // the fine element's nodal functional k (GetProlongationMatrix3D,
  // src/FE/FEDatabase3D.C:1630-1790)
  double qq_u[8][NU_LOC][NU_LOC];
  double qq_p[8][NP_LOC][NP_LOC];
};

namespace {

// child j sits at offset ((j&1),(j>>1)&1,(j>>2)&1) of its parent: parent
// reference coordinate = (child coordinate + o)/2 with o = -1 or +1.
void build_prolongation_tables(oracle *o) {
  for (int j = 0; j < 8; ++j) {
    const double ox = (j & 1) ? 1.0 : -1.0, oy = (j & 2) ? 1.0 : -1.0, oz = (j & 4) ? 1.0 : -1.0;
    // Q2: nodal functionals are point values at the 27 Lagrange nodes
    for (int c = 0; c < 3; ++c)
      for (int b = 0; b < 3; ++b)
        for (int a = 0; a < 3; ++a) {
          int k = a + 3 * b + 9 * c;
          double v[27];
          q2_values(0.5 * ((a - 1.0) + ox), 0.5 * ((b - 1.0) + oy), 0.5 * ((c - 1.0) + oz), v);
          for (int l = 0; l < 27; ++l) o->qq_u[j][k][l] = v[l];
        }
    // P1disc: functionals of NF_D_H_P1_3D (8 points +-1/sqrt(3); mean and
    // 0.375 * first moments, include/FE3D/NF_D_H_P1_3D.h)
    const double g = 0.5773502691896257645091489;
    double pts[8][3];
    for (int i = 0; i < 8; ++i) {
      pts[i][0] = (i & 1) ? g : -g;
      pts[i][1] = (i & 2) ? g : -g;
      pts[i][2] = (i & 4) ? g : -g;
    }
    for (int l = 0; l < 4; ++l) {
      double pv[8];
      for (int i = 0; i < 8; ++i) {
        double X = 0.5 * (pts[i][0] + ox), Y = 0.5 * (pts[i][1] + oy), Z = 0.5 * (pts[i][2] + oz);
        const double basis[4] = {1.0, X, Y, Z};
        pv[i] = basis[l];
      }
      double f0 = 0, f1 = 0, f2 = 0, f3 = 0;
      for (int i = 0; i < 8; ++i) {
        f0 += pv[i];
        f1 += pv[i] * pts[i][0];
        f2 += pv[i] * pts[i][1];
        f3 += pv[i] * pts[i][2];
      }
      o->qq_p[j][0][l] = f0 * 0.125;
      o->qq_p[j][1][l] = f1 * 0.375;
      o->qq_p[j][2][l] = f2 * 0.375;
      o->qq_p[j][3][l] = f3 * 0.375;
    }
  }
}

// dgetrf-style right-looking LU with partial pivoting (first maximal |a|),
// column-major, Golub & Van Loan Alg. 3.4.1; ipiv[k] = row swapped with k.
void lu_factor(double *a, int n, int *ipiv) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    double amax = std::fabs(a[k + k * n]);
    for (int i = k + 1; i < n; ++i) {
      double v = std::fabs(a[i + k * n]);
      if (v > amax) {
        amax = v;
        p = i;
      }
    }
    ipiv[k] = p;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(a[k + j * n], a[p + j * n]);
    const double piv = a[k + k * n];
    if (piv != 0.0) {
      const double r = 1.0 / piv;
      for (int i = k + 1; i < n; ++i) a[i + k * n] *= r;
    }
    for (int j = k + 1; j < n; ++j) {
      const double ukj = a[k + j * n];
      if (ukj == 0.0) continue;
      double *col = a + j * n;
      const double *lk = a + k * n;
      for (int i = k + 1; i < n; ++i) col[i] -= lk[i] * ukj;
    }
  }
}

// dgetrs 'N' with nrhs = 1
void lu_solve(const double *a, int n, const int *ipiv, double *b) {
  for (int k = 0; k < n; ++k)
    if (ipiv[k] != k) std::swap(b[k], b[ipiv[k]]);
  for (int j = 0; j < n; ++j) {
    const double bj = b[j];
    if (bj != 0.0)
      for (int i = j + 1; i < n; ++i) b[i] -= a[i + j * n] * bj;
  }
  for (int j = n - 1; j >= 0; --j) {
    b[j] /= a[j + j * n];
    const double bj = b[j];
    if (bj != 0.0)
      for (int i = 0; i < j; ++i) b[i] -= a[i + j * n] * bj;
  }
}

// CoupledDefect NSTYPE 4 (src/FE/MGComponents3D.C:3038-3209) without the
// projection; r = b - K x.
void coupled_defect(const OLevel &L, const double *x, const double *b, double *r) {
  const pm_level_desc &d = L.d;
  const int nu = L.nu, np = L.np, na = d.n_active;
  const double *u1 = x, *u2 = x + nu, *u3 = x + 2 * nu, *p = x + 3 * nu;
  const double *v1 = b, *v2 = b + nu, *v3 = b + 2 * nu, *q = b + 3 * nu;
  double *r1 = r, *r2 = r + nu, *r3 = r + 2 * nu, *r4 = r + 3 * nu;
#pragma omp parallel
  {
#pragma omp for
    for (int i = 0; i < na; ++i) {
      double s = v1[i], t = v2[i], u = v3[i];
      for (int j = d.a_rowptr[i]; j < d.a_rowptr[i + 1]; ++j) {
        const int idx = d.a_col[j];
        const double x1 = u1[idx], x2 = u2[idx], x3 = u3[idx];
        s -= d.a[0][j] * x1 + d.a[1][j] * x2 + d.a[2][j] * x3;
        t -= d.a[3][j] * x1 + d.a[4][j] * x2 + d.a[5][j] * x3;
        u -= d.a[6][j] * x1 + d.a[7][j] * x2 + d.a[8][j] * x3;
      }
      r1[i] = s;
      r2[i] = t;
      r3[i] = u;
    }
#pragma omp for
    for (int i = na; i < nu; ++i) {
      double s = v1[i], t = v2[i], u = v3[i];
      for (int j = d.a_rowptr[i]; j < d.a_rowptr[i + 1]; ++j) {
        const int idx = d.a_col[j];
        s -= d.a[0][j] * u1[idx];
        t -= d.a[4][j] * u2[idx];
        u -= d.a[8][j] * u3[idx];
      }
      r1[i] = s;
      r2[i] = t;
      r3[i] = u;
    }
#pragma omp for
    for (int i = 0; i < np; ++i) {
      double s = q[i];
      for (int j = d.b_rowptr[i]; j < d.b_rowptr[i + 1]; ++j) {
        const int idx = d.b_col[j];
        s -= d.b[0][j] * u1[idx] + d.b[1][j] * u2[idx] + d.b[2][j] * u3[idx];
      }
      r4[i] = s;
    }
#pragma omp for
    for (int i = 0; i < na; ++i) {
      double s = 0, t = 0, u = 0;
      for (int j = d.bt_rowptr[i]; j < d.bt_rowptr[i + 1]; ++j) {
        const double v = p[d.bt_col[j]];
        s += d.bt[0][j] * v;
        t += d.bt[1][j] * v;
        u += d.bt[2][j] * v;
      }
      r1[i] -= s;
      r2[i] -= t;
      r3[i] -= u;
    }
  }
}

// CoupledMatVect NSTYPE 4 (src/FE/MGComponents3D.C:2872-3029)
void coupled_matvec(const OLevel &L, const double *x, double *y) {
  const pm_level_desc &d = L.d;
  const int nu = L.nu, np = L.np, na = d.n_active;
  const double *u1 = x, *u2 = x + nu, *u3 = x + 2 * nu, *p = x + 3 * nu;
  double *v1 = y, *v2 = y + nu, *v3 = y + 2 * nu, *q = y + 3 * nu;
#pragma omp parallel
  {
#pragma omp for
    for (int i = 0; i < na; ++i) {
      double s = 0, t = 0, u = 0;
      for (int j = d.a_rowptr[i]; j < d.a_rowptr[i + 1]; ++j) {
        const int idx = d.a_col[j];
        const double x1 = u1[idx], x2 = u2[idx], x3 = u3[idx];
        s += d.a[0][j] * x1 + d.a[1][j] * x2 + d.a[2][j] * x3;
        t += d.a[3][j] * x1 + d.a[4][j] * x2 + d.a[5][j] * x3;
        u += d.a[6][j] * x1 + d.a[7][j] * x2 + d.a[8][j] * x3;
      }
      double bs = 0, bt = 0, bu = 0;
      for (int j = d.bt_rowptr[i]; j < d.bt_rowptr[i + 1]; ++j) {
        const double v = p[d.bt_col[j]];
        bs += d.bt[0][j] * v;
        bt += d.bt[1][j] * v;
        bu += d.bt[2][j] * v;
      }
      v1[i] = s + bs;
      v2[i] = t + bt;
      v3[i] = u + bu;
    }
#pragma omp for
    for (int i = na; i < nu; ++i) {
      double s = 0, t = 0, u = 0;
      for (int j = d.a_rowptr[i]; j < d.a_rowptr[i + 1]; ++j) {
        const int idx = d.a_col[j];
        s += d.a[0][j] * u1[idx];
        t += d.a[4][j] * u2[idx];
        u += d.a[8][j] * u3[idx];
      }
      v1[i] = s;
      v2[i] = t;
      v3[i] = u;
    }
#pragma omp for
    for (int i = 0; i < np; ++i) {
      double s = 0;
      for (int j = d.b_rowptr[i]; j < d.b_rowptr[i + 1]; ++j) {
        const int idx = d.b_col[j];
        s += d.b[0][j] * u1[idx] + d.b[1][j] * u2[idx] + d.b[2][j] * u3[idx];
      }
      q[i] = s;
    }
  }
}

// IntoL20Vector3D, case -11 (P1disc on hexahedra): subtract the mean of the
// constant modes (src/FE/MGComponents3D.C:1756-1786)
void into_l20(double *v, int len) {
  double s = 0;
  for (int i = 0; i < len; i += 4) s += v[i];
  s /= len;
  s *= 4;
  for (int i = 0; i < len; i += 4) v[i] -= s;
}

double dot(const double *a, const double *b, int n) {
  double s = 0;
#pragma omp parallel for reduction(+ : s)
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

// Ddot (src/FE/Blas1.C:14-31): one sequential sum, the order of the
// reference's TFgmresIte::Dotprod without MPI (src/FE/FgmresIte.C:857-926)
double ddot(const double *a, const double *b, int n) {
  double s = 0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

// TNSE_MGLevel4::Defect (src/FE/NSE_MGLevel4.C:465-539)
void level_defect(const oracle *o, const OLevel &L, const double *u, const double *f, double *d,
                  double *res) {
  coupled_defect(L, u, f, d);
  if (o->p.project_pressure) into_l20(d + 3 * L.nu, L.np);
  for (int c = 0; c < 3; ++c)
    std::memset(d + c * L.nu + L.d.n_active, 0, sizeof(double) * (L.nu - L.d.n_active));
  if (res) *res = std::sqrt(dot(d, d, L.ndof));
}

// TNSE_MGLevel4::CorrectNodes (src/FE/NSE_MGLevel4.C:542-601); no hanging nodes
void correct_nodes(const OLevel &L, double *u) {
  for (int c = 0; c < 3; ++c)
    std::memset(u + c * L.nu + L.d.hanging_bound, 0, sizeof(double) * L.d.n_dirichlet);
}
// TNSE_MultiGrid::SetDirichletNodes (src/FE/NSE_MultiGrid.C:1781-1802)
void set_dirichlet(const OLevel &L, double *u, const double *rhs) {
  for (int c = 0; c < 3; ++c)
    std::memcpy(u + c * L.nu + L.d.hanging_bound, rhs + c * L.nu + L.d.hanging_bound,
                sizeof(double) * L.d.n_dirichlet);
}
// TNSE_MGLevel::CorrectDefect (src/FE/NSE_MGLevel.C:202-278)
void correct_defect(const oracle *o, const OLevel &L, double *v) {
  for (int c = 0; c < 3; ++c)
    std::memset(v + c * L.nu + L.d.n_active, 0, sizeof(double) * (L.nu - L.d.n_active));
  if (o->p.project_pressure) into_l20(v + 3 * L.nu, L.np);
}

// Local 85x85 system (column-major System[col*85+row]) and local residual of
// one cell, as assembled in the _SEQ CellVanka (src/FE/NSE_MGLevel4.C:1810-1960).
void local_system(const OLevel &L, int cell, const double *u, const double *rhs, double *System,
                  double *Rhs) {
  const pm_level_desc &d = L.d;
  const int nu = L.nu, N = L.nloc, active = d.n_active, NU_LOC = L.nl;
  const double *u1 = u, *u2 = u + nu, *u3 = u + 2 * nu, *p = u + 3 * nu;
  const int *UDOFs = d.cell_udofs + (size_t)cell * NU_LOC;
  const int *PDOFs = d.cell_pdofs + (size_t)cell * NP_LOC;
  std::memset(System, 0, sizeof(double) * N * N);
  for (int j = 0; j < NU_LOC; ++j) {
    const int j1 = j, j2 = j + NU_LOC, j3 = j + 2 * NU_LOC;
    const int UDOF = UDOFs[j];
    Rhs[j1] = rhs[UDOF];
    Rhs[j2] = rhs[nu + UDOF];
    Rhs[j3] = rhs[2 * nu + UDOF];
    for (int k = d.a_rowptr[UDOF]; k < d.a_rowptr[UDOF + 1]; ++k) {
      const int l = d.a_col[k];
      double v11 = d.a[0][k], v12 = d.a[1][k], v13 = d.a[2][k];
      double v21 = d.a[3][k], v22 = d.a[4][k], v23 = d.a[5][k];
      double v31 = d.a[6][k], v32 = d.a[7][k], v33 = d.a[8][k];
      if (UDOF >= active) v12 = v13 = v21 = v23 = v31 = v32 = 0;
      Rhs[j1] -= v11 * u1[l] + v12 * u2[l] + v13 * u3[l];
      Rhs[j2] -= v21 * u1[l] + v22 * u2[l] + v23 * u3[l];
      Rhs[j3] -= v31 * u1[l] + v32 * u2[l] + v33 * u3[l];
      for (int m = 0; m < NU_LOC; ++m)
        if (UDOFs[m] == l) {
          const int k1 = m * N, k2 = (m + NU_LOC) * N, k3 = (m + 2 * NU_LOC) * N;
          System[k1 + j1] = v11;
          System[k2 + j1] = v12;
          System[k3 + j1] = v13;
          System[k1 + j2] = v21;
          System[k2 + j2] = v22;
          System[k3 + j2] = v23;
          System[k1 + j3] = v31;
          System[k2 + j3] = v32;
          System[k3 + j3] = v33;
          break;
        }
    }
    if (UDOF < active) {
      for (int k = d.bt_rowptr[UDOF]; k < d.bt_rowptr[UDOF + 1]; ++k) {
        const int l = d.bt_col[k];
        const double w1 = d.bt[0][k], w2 = d.bt[1][k], w3 = d.bt[2][k], val = p[l];
        Rhs[j1] -= w1 * val;
        Rhs[j2] -= w2 * val;
        Rhs[j3] -= w3 * val;
        for (int m = 0; m < NP_LOC; ++m)
          if (PDOFs[m] == l) {
            const int k1 = (m + 3 * NU_LOC) * N;
            System[k1 + j1] = w1;
            System[k1 + j2] = w2;
            System[k1 + j3] = w3;
            break;
          }
      }
    }
  }
  for (int j = 0; j < NP_LOC; ++j) {
    const int j1 = j + 3 * NU_LOC;
    const int PDOF = PDOFs[j];
    Rhs[j1] = rhs[3 * nu + PDOF];
    for (int k = d.b_rowptr[PDOF]; k < d.b_rowptr[PDOF + 1]; ++k) {
      const int l = d.b_col[k];
      const double w1 = d.b[0][k], w2 = d.b[1][k], w3 = d.b[2][k];
      Rhs[j1] -= w1 * u1[l];
      Rhs[j1] -= w2 * u2[l];
      Rhs[j1] -= w3 * u3[l];
      for (int m = 0; m < NU_LOC; ++m)
        if (UDOFs[m] == l) {
          System[m * N + j1] = w1;
          System[(m + NU_LOC) * N + j1] = w2;
          System[(m + 2 * NU_LOC) * N + j1] = w3;
          break;
        }
    }
  }
}

void add_local(const OLevel &L, int cell, double *u, const double *sol, double damp) {
  const int nu = L.nu, NU_LOC = L.nl;
  const int *UDOFs = L.d.cell_udofs + (size_t)cell * NU_LOC;
  const int *PDOFs = L.d.cell_pdofs + (size_t)cell * NP_LOC;
  for (int j = 0; j < NU_LOC; ++j) {
    const int l = UDOFs[j];
    u[l] += damp * sol[j];
    u[nu + l] += damp * sol[j + NU_LOC];
    u[2 * nu + l] += damp * sol[j + 2 * NU_LOC];
  }
  for (int j = 0; j < NP_LOC; ++j) u[3 * nu + PDOFs[j]] += damp * sol[j + 3 * NU_LOC];
}

void solve_local(oracle *o, OLevel &L, int cell, double *System, double *Rhs) {
  const int NLOC = L.nloc;
  if (o->p.reuse_factors) {
    // the per-cell slots exist (cell_vanka sizes them before any parallel
    // loop); each cell is factored by the one thread that owns it
    if (L.fac[cell].empty()) {
      L.fac[cell].assign(System, System + NLOC * NLOC);
      L.piv[cell].assign(NLOC, 0);
      lu_factor(L.fac[cell].data(), NLOC, L.piv[cell].data());
    }
    lu_solve(L.fac[cell].data(), NLOC, L.piv[cell].data(), Rhs);
    return;
  }
  int ipiv[NLOC_MAX];
  lu_factor(System, NLOC, ipiv);  // SolveLinearSystemLapack, src/FE/LinAlg.C:106-131
  lu_solve(System, NLOC, ipiv, Rhs);
}

// TNSE_MGLevel4::CellVanka (src/FE/NSE_MGLevel4.C:1653-2087): one sweep.
void cell_vanka(oracle *o, OLevel &L, double *u, const double *rhs) {
  const double damp = o->p.smooth_damp;
  const int NLOC = L.nloc;
  const int ncell = L.d.n_cells;
  set_dirichlet(L, u, rhs);
  std::vector<double> uold(u, u + L.ndof);
  if (o->p.reuse_factors && L.fac.size() != (size_t)ncell) {
    L.fac.assign(ncell, {});
    L.piv.assign(ncell, {});
  }
  if (o->p.vanka_mode == ORACLE_VANKA_SEQ) {
    std::vector<double> System(NLOC * NLOC), Rhs(NLOC);
    for (int c = 0; c < ncell; ++c) {
      local_system(L, c, u, rhs, System.data(), Rhs.data());
      solve_local(o, L, c, System.data(), Rhs.data());
      add_local(L, c, u, Rhs.data(), damp);
    }
  } else {
    // colour-block: residuals of one colour from the state before the
    // colour, batched solves, then the (disjoint) updates (the OpenMP colour
    // loop of the colour-parallel CellVanka, src/FE/NSE_MGLevel4.C:603-1651,
    // and CellVanka_GPU, src/FE/NSE_CellVanka.cu:2181-2365)
    const int ncol = (int)L.colour_ptr.size() - 1;
    std::vector<double> sols;
    for (int col = 0; col < ncol; ++col) {
      const int b = L.colour_ptr[col], e = L.colour_ptr[col + 1];
      sols.assign((size_t)(e - b) * NLOC, 0.0);
#pragma omp parallel
      {
        std::vector<double> System(NLOC * NLOC);
#pragma omp for schedule(dynamic, 4)
        for (int t = b; t < e; ++t) {
          const int c = L.colour_cells[t];
          double *R = &sols[(size_t)(t - b) * NLOC];
          local_system(L, c, u, rhs, System.data(), R);
          solve_local(o, L, c, System.data(), R);
        }
      }
#pragma omp parallel for schedule(static)
      for (int t = b; t < e; ++t) add_local(L, L.colour_cells[t], u, &sols[(size_t)(t - b) * NLOC], damp);
    }
  }
  if (std::fabs(1.0 - o->p.alpha) > 1e-3)
    for (int j = 0; j < L.ndof; ++j) u[j] = uold[j] + o->p.alpha * (u[j] - uold[j]);
  set_dirichlet(L, u, rhs);
}

// Prolongate (vector src/FE/MGComponents3D.C:468-708, scalar :184-467)
void prolongate(const oracle *o, const OLevel &C, const OLevel &F, const double *coarse,
                double *fine) {
  if (F.d.pu_rowptr) {  // handed-over prolongation (non-hexahedral cells)
    for (int comp = 0; comp < 3; ++comp)
      for (int i = 0; i < F.nu; ++i) {
        double s = 0.0;
        for (int e = F.d.pu_rowptr[i]; e < F.d.pu_rowptr[i + 1]; ++e)
          s += F.d.pu_val[e] * coarse[comp * C.nu + F.d.pu_col[e]];
        fine[comp * F.nu + i] = s;
      }
    for (int i = 0; i < F.np; ++i) {
      double s = 0.0;
      for (int e = F.d.pp_rowptr[i]; e < F.d.pp_rowptr[i + 1]; ++e)
        s += F.d.pp_val[e] * coarse[3 * C.nu + F.d.pp_col[e]];
      fine[3 * F.nu + i] = s;
    }
    return;
  }
  std::vector<double> aux(F.nu, 0.0);
  std::memset(fine, 0, sizeof(double) * F.ndof);
  const int ncc = C.d.n_cells;
  for (int pc = 0; pc < ncc; ++pc) {
    const int *CDOF = C.d.cell_udofs + (size_t)pc * NU_LOC;
    for (int j = 0; j < 8; ++j) {
      const int fc = F.children[pc * 8 + j];
      if (fc < 0) continue;
      const int *FDOF = F.d.cell_udofs + (size_t)fc * NU_LOC;
      for (int comp = 0; comp < 3; ++comp) {
        double Val[NU_LOC];
        for (int l = 0; l < NU_LOC; ++l) Val[l] = coarse[comp * C.nu + CDOF[l]];
        for (int k = 0; k < NU_LOC; ++k) {
          double s = 0;
          for (int l = 0; l < NU_LOC; ++l) s += o->qq_u[j][k][l] * Val[l];
          fine[comp * F.nu + FDOF[k]] += s;
          aux[FDOF[k]] += 1;
        }
      }
    }
  }
  for (int i = 0; i < F.nu; ++i) aux[i] *= 1.0 / 3.0;
  for (int comp = 0; comp < 3; ++comp)
    for (int i = 0; i < F.nu; ++i)
      if (aux[i] != 0.0) fine[comp * F.nu + i] /= aux[i];
  // pressure (scalar, discontinuous)
  std::vector<double> auxp(F.np, 0.0);
  const double *cp = coarse + 3 * C.nu;
  double *fp = fine + 3 * F.nu;
  for (int pc = 0; pc < ncc; ++pc) {
    const int *CDOF = C.d.cell_pdofs + (size_t)pc * NP_LOC;
    for (int j = 0; j < 8; ++j) {
      const int fc = F.children[pc * 8 + j];
      if (fc < 0) continue;
      const int *FDOF = F.d.cell_pdofs + (size_t)fc * NP_LOC;
      for (int k = 0; k < NP_LOC; ++k) {
        double s = 0;
        for (int l = 0; l < NP_LOC; ++l) s += o->qq_p[j][k][l] * cp[CDOF[l]];
        fp[FDOF[k]] += s;
        auxp[FDOF[k]] += 1;
      }
    }
  }
  for (int i = 0; i < F.np; ++i)
    if (auxp[i] != 0.0) fp[i] /= auxp[i];
}

// DefectRestriction (vector src/FE/MGComponents3D.C:996-1242, scalar :711-995)
void defect_restriction(const oracle *o, const OLevel &C, const OLevel &F, double *coarse,
                        const double *fine_in) {
  std::memset(coarse, 0, sizeof(double) * C.ndof);
  if (F.d.pu_rowptr) {  // the transpose of the handed-over prolongation
    for (int comp = 0; comp < 3; ++comp)
      for (int i = 0; i < F.nu; ++i)
        for (int e = F.d.pu_rowptr[i]; e < F.d.pu_rowptr[i + 1]; ++e)
          coarse[comp * C.nu + F.d.pu_col[e]] += F.d.pu_val[e] * fine_in[comp * F.nu + i];
    for (int i = 0; i < F.np; ++i)
      for (int e = F.d.pp_rowptr[i]; e < F.d.pp_rowptr[i + 1]; ++e)
        coarse[3 * C.nu + F.d.pp_col[e]] += F.d.pp_val[e] * fine_in[3 * F.nu + i];
    return;
  }
  std::vector<double> fine(fine_in, fine_in + F.ndof);
  std::vector<double> aux(F.nu, 0.0), auxp(F.np, 0.0);
  for (int c = 0; c < F.d.n_cells; ++c) {
    for (int j = 0; j < NU_LOC; ++j) aux[F.d.cell_udofs[(size_t)c * NU_LOC + j]] += 1;
    for (int j = 0; j < NP_LOC; ++j) auxp[F.d.cell_pdofs[(size_t)c * NP_LOC + j]] += 1;
  }
  for (int comp = 0; comp < 3; ++comp)
    for (int i = 0; i < F.nu; ++i) fine[comp * F.nu + i] /= aux[i];
  for (int i = 0; i < F.np; ++i) fine[3 * F.nu + i] /= auxp[i];
  for (int pc = 0; pc < C.d.n_cells; ++pc) {
    const int *CDOF = C.d.cell_udofs + (size_t)pc * NU_LOC;
    const int *CPDOF = C.d.cell_pdofs + (size_t)pc * NP_LOC;
    for (int j = 0; j < 8; ++j) {
      const int fc = F.children[pc * 8 + j];
      if (fc < 0) continue;
      const int *FDOF = F.d.cell_udofs + (size_t)fc * NU_LOC;
      for (int comp = 0; comp < 3; ++comp) {
        double Val[NU_LOC];
        for (int l = 0; l < NU_LOC; ++l) Val[l] = fine[comp * F.nu + FDOF[l]];
        for (int k = 0; k < NU_LOC; ++k) {
          double s = 0;
          for (int l = 0; l < NU_LOC; ++l) s += o->qq_u[j][l][k] * Val[l];
          coarse[comp * C.nu + CDOF[k]] += s;
        }
      }
      const int *FPDOF = F.d.cell_pdofs + (size_t)fc * NP_LOC;
      for (int k = 0; k < NP_LOC; ++k) {
        double s = 0;
        for (int l = 0; l < NP_LOC; ++l) s += o->qq_p[j][l][k] * fine[3 * F.nu + FPDOF[l]];
        coarse[3 * C.nu + CPDOF[k]] += s;
      }
    }
  }
}

// TNSE_MGLevel4::SolveExact (src/FE/NSE_MGLevel4.C:5728-5847)
void solve_exact(const oracle *o, const OLevel &L, double *u1, const double *rhs1) {
  const pm_level_desc &d = L.d;
  const int N = L.ndof, nu = L.nu, nu2 = 2 * nu, nug = 3 * nu;
  std::vector<double> a((size_t)N * N, 0.0), b(rhs1, rhs1 + N);
  for (int i = 0; i < d.n_active; ++i)
    for (int j = d.a_rowptr[i]; j < d.a_rowptr[i + 1]; ++j) {
      const size_t idx = d.a_col[j];
      a[idx * N + i] = d.a[0][j];
      a[(idx + nu) * N + i] = d.a[1][j];
      a[idx * N + i + nu] = d.a[3][j];
      a[(idx + nu) * N + i + nu] = d.a[4][j];
      a[(idx + nu2) * N + i] = d.a[2][j];
      a[(idx + nu2) * N + i + nu] = d.a[5][j];
      a[idx * N + i + nu2] = d.a[6][j];
      a[(idx + nu) * N + i + nu2] = d.a[7][j];
      a[(idx + nu2) * N + i + nu2] = d.a[8][j];
    }
  for (int i = d.n_active; i < nu; ++i)
    for (int j = d.a_rowptr[i]; j < d.a_rowptr[i + 1]; ++j) {
      const size_t idx = d.a_col[j];
      a[i + N * idx] = d.a[0][j];
      a[(idx + nu) * N + i + nu] = d.a[4][j];
      a[(idx + nu2) * N + i + nu2] = d.a[8][j];
    }
  for (int i = 0; i < d.n_active; ++i)
    for (int j = d.bt_rowptr[i]; j < d.bt_rowptr[i + 1]; ++j) {
      const size_t l = ((size_t)d.bt_col[j] + nug) * N;
      a[l + i] = d.bt[0][j];
      a[l + i + nu] = d.bt[1][j];
      a[l + i + 2 * nu] = d.bt[2][j];
    }
  for (int i = 0; i < L.np; ++i)
    for (int j = d.b_rowptr[i]; j < d.b_rowptr[i + 1]; ++j) {
      const size_t idx = d.b_col[j];
      a[idx * N + i + nug] = d.b[0][j];
      a[(idx + nu) * N + i + nug] = d.b[1][j];
      a[(idx + nu2) * N + i + nug] = d.b[2][j];
    }
  if (o->p.project_pressure) {
    for (int i = 0; i < N; ++i) a[(size_t)i * N + nug] = 0;
    a[(size_t)nug * N + nug] = 1;
    b[nug] = 0;
  }
  std::vector<int> ipiv(N);
  lu_factor(a.data(), N, ipiv.data());
  lu_solve(a.data(), N, ipiv.data(), b.data());
  std::memcpy(u1, b.data(), sizeof(double) * N);
}

// TNSE_MultiGrid::Cycle, V-cycle, smoother 2 (src/FE/NSE_MultiGrid.C:434-1779).
// Defects that only feed log output are not computed (they do not change
// any state the cycle reads later).
void cycle(oracle *o, int i) {
  OLevel &Cur = o->L[i];
  double *u = Cur.sol.data(), *rhs = Cur.rhs.data();
  correct_nodes(Cur, u);
  set_dirichlet(Cur, u, rhs);
  if (i == 0) {
    solve_exact(o, Cur, u, rhs);  // case 17
    return;
  }
  OLevel &Crs = o->L[i - 1];
  for (int s = 0; s < o->p.pre_smooth; ++s) cell_vanka(o, Cur, u, rhs);
  correct_nodes(Cur, u);
  double res;
  level_defect(o, Cur, u, rhs, Cur.aux0.data(), &res);
  defect_restriction(o, Crs, Cur, Crs.rhs.data(), Cur.aux0.data());
  correct_defect(o, Crs, Crs.rhs.data());
  std::fill(Crs.sol.begin(), Crs.sol.end(), 0.0);
  cycle(o, i - 1);
  prolongate(o, Crs, Cur, Crs.sol.data(), Cur.aux0.data());
  correct_nodes(Cur, Cur.aux0.data());
  for (int j = 0; j < Cur.ndof; ++j) u[j] += o->p.beta * Cur.aux0[j];  // TNSE_MGLevel::Update
  correct_nodes(Cur, u);
  for (int s = 0; s < o->p.post_smooth; ++s) cell_vanka(o, Cur, u, rhs);
}

// TMultiGridIte::Iterate (src/FE/MultiGridIte.C:76-132), zero start
void vcycle(oracle *o, double *sol, const double *rhs) {
  OLevel &F = o->L.back();
  std::fill(F.sol.begin(), F.sol.end(), 0.0);
  std::memcpy(F.rhs.data(), rhs, sizeof(double) * F.ndof);
  set_dirichlet(F, F.sol.data(), F.rhs.data());
  cycle(o, (int)o->L.size() - 1);
  std::memcpy(sol, F.sol.data(), sizeof(double) * F.ndof);
}

void defect_nse4(oracle *o, const double *x, const double *b, double *r) {
  const OLevel &F = o->L.back();
  coupled_defect(F, x, b, r);  // Defect_NSE4 (src/FE/MGComponents3D.C:3210-3231)
  if (o->p.project_pressure) into_l20(r + 3 * F.nu, F.np);
}

// GeneratePlaneRotation / ApplyPlaneRotation / UpdateGmresIterate
// (src/FE/FgmresIte.C:199-247)
void gen_rot(double dx, double dy, double *cs, double *sn) {
  if (dy == 0.0) {
    *cs = 1.0;
    *sn = 0.0;
  } else if (std::fabs(dy) > std::fabs(dx)) {
    double t = dx / dy;
    *sn = 1.0 / std::sqrt(1.0 + t * t);
    *cs = t * *sn;
  } else {
    double t = dy / dx;
    *cs = 1.0 / std::sqrt(1.0 + t * t);
    *sn = t * *cs;
  }
}
void apply_rot(double *dx, double *dy, double cs, double sn) {
  double t = cs * *dx + sn * *dy;
  *dy = -sn * *dx + cs * *dy;
  *dx = t;
}

// UpdateGmresIterate's sum z_0 y_0 + ... + z_k y_k, formed in a zeroed vector
// and then added to the iterate with Daxpy (src/FE/FgmresIte.C:229-247,
// :480-490, :574-577): the same rounding as the reference
void add_update(double *sol, const std::vector<std::vector<double>> &zv,
                const std::vector<double> &y, int k, int N) {
  std::vector<double> w(N, 0.0);
  for (int j = 0; j <= k; ++j)
    for (int t = 0; t < N; ++t) w[t] += zv[j][t] * y[j];
  for (int t = 0; t < N; ++t) sol[t] += 1.0 * w[t];
}

}  // namespace

extern "C" {

void oracle_default_params(oracle_params *p) {
  std::memset(p, 0, sizeof(*p));
  p->pre_smooth = 2;
  p->post_smooth = 2;
  p->smooth_damp = 1.0;
  p->alpha = 1.0;
  p->beta = 1.0;
  p->project_pressure = 1;
  p->restart = 20;
  p->maxit = 100;
  p->minit = 0;
  p->red_factor = 0.0;
  p->res_norm_min = 1e-10;
  p->div_factor = 1e10;
  p->vanka_mode = ORACLE_VANKA_COLOUR;
  p->reuse_factors = 0;
  p->nthreads = 0;
}

oracle *oracle_create(const pm_level_desc *levels, int n_levels, const oracle_params *p) {
  oracle *o = new oracle();
  o->p = *p;
#ifdef _OPENMP
  if (p->nthreads > 0) omp_set_num_threads(p->nthreads);
#endif
  build_prolongation_tables(o);
  o->L.resize(n_levels);
  for (int l = 0; l < n_levels; ++l) {
    OLevel &L = o->L[l];
    L.d = levels[l];
    L.nu = L.d.n_udof;
    L.np = L.d.n_pdof;
    L.ndof = 3 * L.nu + L.np;
    L.nl = L.d.n_ulocal > 0 ? L.d.n_ulocal : NU_LOC;
    L.nloc = 3 * L.nl + NP_LOC;
    L.sol.assign(L.ndof, 0.0);
    L.rhs.assign(L.ndof, 0.0);
    L.aux0.assign(L.ndof, 0.0);
    L.aux1.assign(L.ndof, 0.0);
    if (l > 0 && L.d.cell_child && !L.d.pu_rowptr) {
      L.children.assign((size_t)levels[l - 1].n_cells * 8, -1);
      for (int c = 0; c < L.d.n_cells; ++c)
        L.children[(size_t)L.d.cell_parent[c] * 8 + L.d.cell_child[c]] = c;
    }
    // colour lists in increasing colour, cells in increasing index
    int ncol = 0;
    for (int c = 0; c < L.d.n_cells; ++c) ncol = std::max(ncol, L.d.cell_colour ? L.d.cell_colour[c] + 1 : 1);
    L.colour_ptr.assign(ncol + 1, 0);
    for (int c = 0; c < L.d.n_cells; ++c) L.colour_ptr[(L.d.cell_colour ? L.d.cell_colour[c] : 0) + 1]++;
    for (int k = 0; k < ncol; ++k) L.colour_ptr[k + 1] += L.colour_ptr[k];
    L.colour_cells.resize(L.d.n_cells);
    std::vector<int> fill(L.colour_ptr.begin(), L.colour_ptr.end() - 1);
    for (int c = 0; c < L.d.n_cells; ++c) L.colour_cells[fill[L.d.cell_colour ? L.d.cell_colour[c] : 0]++] = c;
  }
  return o;
}

void oracle_destroy(oracle *o) { delete o; }
int oracle_ndof(oracle *o, int level) { return o->L[level].ndof; }

void oracle_coupled_defect(oracle *o, int level, const double *x, const double *b, double *r,
                           int project) {
  const OLevel &L = o->L[level];
  coupled_defect(L, x, b, r);
  if (project) into_l20(r + 3 * L.nu, L.np);
}
void oracle_matvec(oracle *o, int level, const double *x, double *y) { coupled_matvec(o->L[level], x, y); }
void oracle_level_defect(oracle *o, int level, const double *u, const double *f, double *d,
                         double *res) {
  level_defect(o, o->L[level], u, f, d, res);
}
void oracle_cell_vanka(oracle *o, int level, double *u, const double *rhs, int sweeps) {
  for (int s = 0; s < sweeps; ++s) cell_vanka(o, o->L[level], u, rhs);
}
void oracle_restrict(oracle *o, int level, const double *fine, double *coarse) {
  defect_restriction(o, o->L[level - 1], o->L[level], coarse, fine);
}
void oracle_prolongate(oracle *o, int level, const double *coarse, double *fine) {
  prolongate(o, o->L[level - 1], o->L[level], coarse, fine);
}
void oracle_solve_exact(oracle *o, const double *rhs, double *u) { solve_exact(o, o->L[0], u, rhs); }
void oracle_vcycle(oracle *o, double *z, const double *v) { vcycle(o, z, v); }

void oracle_lu_solve(double *a, double *b, int n) {
  std::vector<int> ipiv(n);
  lu_factor(a, n, ipiv.data());
  lu_solve(a, n, ipiv.data(), b);
}

int oracle_local_system(oracle *o, int level, int cell, const double *u, const double *rhs,
                        double *system, double *local_rhs) {
  local_system(o->L[level], cell, u, rhs, system, local_rhs);
  return o->L[level].nloc;
}

// TFgmresIte::Iterate, flexible branch (src/FE/FgmresIte.C:250-677)
int oracle_fgmres(oracle *o, double *sol, const double *rhs, double *out) {
  const OLevel &F = o->L.back();
  const int N = F.ndof;
  int restart = o->p.restart;
  const int maxit = o->p.maxit, minit = o->p.minit;
  if (restart > maxit) restart = maxit;
  if (restart <= 0) restart = 10;
  const double red = o->p.red_factor, resmin = o->p.res_norm_min, divf = o->p.div_factor;
  std::vector<double> s(restart + 1), cs(restart + 1), sn(restart + 1);
  std::vector<double> H((size_t)(restart + 1) * restart, 0.0);
  auto h = [&](int r, int c) -> double & { return H[(size_t)r * restart + c]; };
  std::vector<std::vector<double>> v(restart + 1, std::vector<double>(N)), zv(restart + 1, std::vector<double>(N));
  std::vector<double> defect(N);

  defect_nse4(o, sol, rhs, v[0].data());
  double res = std::sqrt(ddot(v[0].data(), v[0].data(), N));
  double res0 = res, beta = res;
  if (out) out[0] = res0;
  int maxite = maxit;
  if (beta <= resmin) {
    if (minit == 0 || beta < 1e-20) {
      if (out) {
        out[1] = res;
        out[2] = res;
      }
      return 0;
    }
    maxite = minit;
  }
  int j = 1;
  int status_div = 0;
  while (j <= maxite) {
    for (int t = 0; t < N; ++t) v[0][t] *= 1.0 / beta;
    std::fill(s.begin(), s.end(), 0.0);
    s[0] = beta;
    int i;
    for (i = 0; i < restart && j <= maxite; i++, j++) {
      std::fill(zv[i].begin(), zv[i].end(), 0.0);
      vcycle(o, zv[i].data(), v[i].data());
      coupled_matvec(F, zv[i].data(), defect.data());
      for (int k = 0; k <= i; ++k) {
        h(k, i) = ddot(defect.data(), v[k].data(), N);
        const double hk = h(k, i);
        for (int t = 0; t < N; ++t) defect[t] -= hk * v[k][t];
      }
      h(i + 1, i) = std::sqrt(ddot(defect.data(), defect.data(), N));
      v[i + 1] = defect;
      if (h(i + 1, i) != 0)
        for (int t = 0; t < N; ++t) v[i + 1][t] *= 1.0 / h(i + 1, i);
      for (int k = 0; k < i; ++k) apply_rot(&h(k, i), &h(k + 1, i), cs[k], sn[k]);
      gen_rot(h(i, i), h(i + 1, i), &cs[i], &sn[i]);
      apply_rot(&h(i, i), &h(i + 1, i), cs[i], sn[i]);
      apply_rot(&s[i], &s[i + 1], cs[i], sn[i]);
      res = std::fabs(s[i + 1]);
      if (j >= minit && (res < resmin || res < red * res0)) {
        std::vector<double> y(s.begin(), s.end());
        for (int r = i; r >= 0; --r) {
          y[r] /= h(r, r);
          for (int q = r - 1; q >= 0; --q) y[q] -= h(q, r) * y[r];
        }
        add_update(sol, zv, y, i, N);
        if (out) {
          out[1] = res;
          std::vector<double> r(N);
          defect_nse4(o, sol, rhs, r.data());
          out[2] = std::sqrt(ddot(r.data(), r.data(), N));
        }
        return j;
      }
      if (res > divf * res0) {
        status_div = 1;
        break;
      }
    }
    if (status_div) break;
    {
      // the reference always back-solves with restart-1 columns
      // (src/FE/FgmresIte.C:575); when the loop ended early at maxit only
      // the first i columns of H belong to this cycle, so use those.
      std::vector<double> y(s.begin(), s.end());
      const int k = i - 1;
      for (int r = k; r >= 0; --r) {
        y[r] /= h(r, r);
        for (int q = r - 1; q >= 0; --q) y[q] -= h(q, r) * y[r];
      }
      add_update(sol, zv, y, k, N);
    }
    defect_nse4(o, sol, rhs, v[0].data());
    res = std::sqrt(ddot(v[0].data(), v[0].data(), N));
    res0 = res;
    beta = res;
  }
  if (j > maxite) j = maxite;
  if (out) {
    out[1] = res;
    std::vector<double> r(N);
    defect_nse4(o, sol, rhs, r.data());
    out[2] = std::sqrt(ddot(r.data(), r.data(), N));
  }
  return status_div ? -j : j;
}

}  // extern "C"
