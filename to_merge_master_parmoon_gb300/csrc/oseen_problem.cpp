// oseen_problem.cpp — caller-side builder of Q2/P1disc Oseen systems on a
// hierarchy of uniformly refined axis-aligned hexahedral meshes.
//
// Layout decisions mirror ParMooN so that the arrays can be handed to the
// solver exactly as TNSE_MGLevel4 would see them:
//  * velocity DOFs: active (inner) nodes first, Dirichlet nodes last
//    (TFESpace3D numbering classes, src/FE/FESpace3D.C:479-850);
//  * pressure DOFs: P1disc, 4 per cell, cell-major, mode 0 the constant
//    (IntoL20Vector3D relies on that stride, src/FE/MGComponents3D.C:1768-1786);
//  * A rows: active rows hold all couplings, Dirichlet rows only the diagonal
//    (src/FE/SquareStructure3D.C:104-124) with value 1 in every square block
//    (src/FE/Assemble3D.C:466-476); columns sorted ascending;
//  * B: P test x U ansatz, all columns; BT: U test x P ansatz, Dirichlet rows
//    present in the structure with zero values (rectangular assembly skips
//    non-active test rows, src/FE/Assemble3D.C:548-580);
//  * local forms: NSType4Galerkin3D (src/FE/NSE3D_FixPo.C:1919-2071) with
//    4-point Gauss per direction (Gauss4Hexa, src/FE/FEDatabase3D.C:1015).
#include "oseen_problem.h"
#include "oseen_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ------------------------------------------------------------------ RNG ----
// SplitMix64 (Steele, Lea, Flood 2014) -> uniform doubles -> Box-Muller.
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double normal() {
    double u1 = 1.0 - uniform();  // (0,1]
    double u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
  }
};


// --------------------------------------------------------------- basis -----
inline void lagrange2(double t, double *v, double *d) {
  v[0] = 0.5 * t * (t - 1.0);
  v[1] = 1.0 - t * t;
  v[2] = 0.5 * t * (t + 1.0);
  d[0] = t - 0.5;
  d[1] = -2.0 * t;
  d[2] = t + 0.5;
}

// Local Q2 numbering: node (a,b,c) in {0,1,2}^3 at reference point
// (-1+a, -1+b, -1+c) is local function a + 3b + 9c (xi fastest), the order of
// C_H_Q2_3D_Funct (include/FE3D/BF_C_H_Q2_3D.h).
void q2_basis(double xi, double eta, double zeta, double *val, double *der) {
  double vx[3], vy[3], vz[3], dx[3], dy[3], dz[3];
  lagrange2(xi, vx, dx);
  lagrange2(eta, vy, dy);
  lagrange2(zeta, vz, dz);
  for (int c = 0; c < 3; ++c)
    for (int b = 0; b < 3; ++b)
      for (int a = 0; a < 3; ++a) {
        int i = a + 3 * b + 9 * c;
        if (val) val[i] = vx[a] * vy[b] * vz[c];
        if (der) {
          der[3 * i + 0] = dx[a] * vy[b] * vz[c];
          der[3 * i + 1] = vx[a] * dy[b] * vz[c];
          der[3 * i + 2] = vx[a] * vy[b] * dz[c];
        }
      }
}

const double kGauss4Pt[4] = {-0.86113631159405257522, -0.33998104358485626480,
                             0.33998104358485626480, 0.86113631159405257522};
const double kGauss4Wt[4] = {0.34785484513745385737, 0.65214515486254614263,
                             0.65214515486254614263, 0.34785484513745385737};

struct RefTables {
  double w[64];
  double pt[64][3];
  double phi[64][27];
  double dphi[64][27][3];
  double psi[64][4];
  double K[3][27][27];  // sum_q w dphi_i,d dphi_j,d
  double B[3][4][27];   // sum_q w psi_m dphi_j,d
  RefTables() {
    for (int qc = 0; qc < 4; ++qc)
      for (int qb = 0; qb < 4; ++qb)
        for (int qa = 0; qa < 4; ++qa) {
          int q = qa + 4 * qb + 16 * qc;
          w[q] = kGauss4Wt[qa] * kGauss4Wt[qb] * kGauss4Wt[qc];
          pt[q][0] = kGauss4Pt[qa];
          pt[q][1] = kGauss4Pt[qb];
          pt[q][2] = kGauss4Pt[qc];
          double der[81];
          q2_basis(pt[q][0], pt[q][1], pt[q][2], phi[q], der);
          for (int i = 0; i < 27; ++i)
            for (int d = 0; d < 3; ++d) dphi[q][i][d] = der[3 * i + d];
          psi[q][0] = 1.0;
          psi[q][1] = pt[q][0];
          psi[q][2] = pt[q][1];
          psi[q][3] = pt[q][2];
        }
    std::memset(K, 0, sizeof(K));
    std::memset(B, 0, sizeof(B));
    for (int q = 0; q < 64; ++q)
      for (int d = 0; d < 3; ++d) {
        for (int i = 0; i < 27; ++i)
          for (int j = 0; j < 27; ++j) K[d][i][j] += w[q] * dphi[q][i][d] * dphi[q][j][d];
        for (int m = 0; m < 4; ++m)
          for (int j = 0; j < 27; ++j) B[d][m][j] += w[q] * psi[q][m] * dphi[q][j][d];
      }
  }
};

const RefTables &ref_tables() {
  static RefTables t;
  return t;
}

}  // namespace

// ------------------------------------------------------------ problem ------
// PMLevelData and pmh_problem: oseen_internal.h

namespace pmh_detail {

// Exact solution of Examples/NSE_3D/AnsatzQuadLin.h:15-44.
void quadlin_u(double x, double y, double z, double *u) {
  u[0] = x * x + y * y + z * z;
  u[1] = x * x + 2 * x * z + 13;
  u[2] = -2 * x * z + 5 * y * y;
}
double quadlin_p(double x, double y, double z) { return 3 * x - 2 * y + 7 * z - 4; }
void quadlin_grad(double x, double y, double z, double g[3][3]) {
  // g[k][d] = d u_k / d x_d
  g[0][0] = 2 * x; g[0][1] = 2 * y; g[0][2] = 2 * z;
  g[1][0] = 2 * x + 2 * z; g[1][1] = 0; g[1][2] = 2 * x;
  g[2][0] = -2 * z; g[2][1] = 10 * y; g[2][2] = -2 * x;
}

// Channel perturbation: sum_m curl(a_m sin(theta_m) w(y)) with the wall
// factor w = (1 - eta^2)^2 (w = w' = 0 at the walls), wavenumbers that are
// periodic in x and z: curl(a s w) = w cos(theta) (k x a) + s w' (e_y x a).
void channel_perturbation(const pmh_problem &P, double x, double y, double z, double *p) {
  const pmh_params &q = P.prm;
  const double Lx = q.x1 - q.x0, Ly = q.y1 - q.y0, Lz = q.z1 - q.z0;
  const double eta = (2.0 * y - q.y0 - q.y1) / Ly, e2 = 1.0 - eta * eta;
  const double w = e2 * e2, dw = -4.0 * eta * e2 * (2.0 / Ly);
  p[0] = p[1] = p[2] = 0.0;
  for (const PmhMode &m : P.bmodes) {
    const double kx = 2.0 * M_PI * m.k[0] / Lx, ky = M_PI * m.k[1] / Ly,
                 kz = 2.0 * M_PI * m.k[2] / Lz;
    const double th = kx * (x - q.x0) + ky * (y - q.y0) + kz * (z - q.z0) + m.phase;
    const double c = w * std::cos(th), sn = dw * std::sin(th);
    p[0] += c * (ky * m.a[2] - kz * m.a[1]) + sn * m.a[2];
    p[1] += c * (kz * m.a[0] - kx * m.a[2]);
    p[2] += c * (kx * m.a[1] - ky * m.a[0]) - sn * m.a[0];
  }
}

void convection(const pmh_problem &P, double x, double y, double z, double *b) {
  b[0] = b[1] = b[2] = 0.0;
  if (P.prm.example == PMH_EXAMPLE_QUADLIN_STOKES) return;
  if (P.prm.example == PMH_EXAMPLE_CHANNEL) {
    const double eta = (2.0 * y - P.prm.y0 - P.prm.y1) / (P.prm.y1 - P.prm.y0);
    double p[3];
    channel_perturbation(P, x, y, z, p);
    b[0] = (1.0 - eta * eta) + P.bscale * p[0];
    b[1] = P.bscale * p[1];
    b[2] = P.bscale * p[2];
    return;
  }
  if (P.prm.example == PMH_EXAMPLE_QUADLIN_OSEEN) {
    quadlin_u(x, y, z, b);
    return;
  }
  // b = sum_m curl(a_m sin(2 pi k_m.x + phi_m)) = sum_m 2 pi cos(theta_m) (k_m x a_m)
  for (const PmhMode &m : P.bmodes) {
    double th = 2.0 * M_PI * (m.k[0] * x + m.k[1] * y + m.k[2] * z) + m.phase;
    double c = 2.0 * M_PI * std::cos(th);
    b[0] += c * (m.k[1] * m.a[2] - m.k[2] * m.a[1]);
    b[1] += c * (m.k[2] * m.a[0] - m.k[0] * m.a[2]);
    b[2] += c * (m.k[0] * m.a[1] - m.k[1] * m.a[0]);
  }
  b[0] *= P.bscale;
  b[1] *= P.bscale;
  b[2] *= P.bscale;
}

void forcing(const pmh_problem &P, double x, double y, double z, double *f) {
  const double nu = P.prm.nu;
  if (P.prm.example == PMH_EXAMPLE_QUADLIN_STOKES) {
    f[0] = -6 * nu + 3;
    f[1] = -2 * nu - 2;
    f[2] = -10 * nu + 7;
    return;
  }
  if (P.prm.example == PMH_EXAMPLE_QUADLIN_OSEEN) {
    double u[3], g[3][3];
    quadlin_u(x, y, z, u);
    quadlin_grad(x, y, z, g);
    const double lap[3] = {6, 2, 10}, gp[3] = {3, -2, 7};
    for (int k = 0; k < 3; ++k)
      f[k] = -nu * lap[k] + u[0] * g[k][0] + u[1] * g[k][1] + u[2] * g[k][2] + gp[k];
    return;
  }
  if (P.prm.example == PMH_EXAMPLE_CHANNEL) {
    const double s = 2.0 / (P.prm.y1 - P.prm.y0);
    f[0] = 2.0 * nu * s * s;  // -nu d2/dy2 (1 - eta^2)
    f[1] = f[2] = 0.0;
    return;
  }
  f[0] = f[1] = f[2] = 0.0;
  for (const PmhMode &m : P.fmodes) {
    double s = std::sin(2.0 * M_PI * (m.k[0] * x + m.k[1] * y + m.k[2] * z) + m.phase);
    f[0] += m.a[0] * s;
    f[1] += m.a[1] * s;
    f[2] += m.a[2] * s;
  }
}

bool boundary_value(const pmh_problem &P, double x, double y, double z, double *u) {
  if (P.prm.example == PMH_EXAMPLE_RANDOM_OSEEN || P.prm.example == PMH_EXAMPLE_CHANNEL) {
    u[0] = u[1] = u[2] = 0.0;
    return false;
  }
  quadlin_u(x, y, z, u);
  return true;
}

}  // namespace pmh_detail

namespace {
using namespace pmh_detail;

// per-dimension coupling lists of a Q2 node index i on a line of g = 2n + 1
// grid nodes (the nodes of all cells that contain it); a periodic direction
// identifies node 2n with node 0, so indices wrap modulo 2n (duplicates, for
// n = 2, are removed by the caller)
inline int node_list(int i, int g, bool per, int *out) {
  const int lo = (i & 1) ? i - 1 : i - 2, hi = (i & 1) ? i + 1 : i + 2;
  int n = 0;
  if (per) {
    const int m = g - 1;
    for (int t = lo; t <= hi; ++t) out[n++] = ((t % m) + m) % m;
  } else {
    for (int t = std::max(lo, 0); t <= std::min(hi, g - 1); ++t) out[n++] = t;
  }
  return n;
}
// cells (per direction) that contain node i; nc cells on the line
inline int cell_list(int i, int nc, bool per, int *out) {
  const int lo = (i & 1) ? (i - 1) / 2 : i / 2 - 1, hi = (i & 1) ? (i - 1) / 2 : i / 2;
  int n = 0;
  for (int t = lo; t <= hi; ++t) {
    if (per)
      out[n++] = ((t % nc) + nc) % nc;
    else if (t >= 0 && t < nc)
      out[n++] = t;
  }
  return n;
}

void build_level_structure(PMLevelData &L, int periodic) {
  const bool px = periodic & PMH_PERIODIC_X, py = periodic & PMH_PERIODIC_Y,
             pz = periodic & PMH_PERIODIC_Z;
  const int gx = L.gx(), gy = L.gy(), gz = L.gz();
  const int ng = gx * gy * gz;
  // canonical grid node: the last node of a periodic direction is the first
  auto canon = [&](int i, int j, int k) {
    if (px && i == gx - 1) i = 0;
    if (py && j == gy - 1) j = 0;
    if (pz && k == gz - 1) k = 0;
    return i + gx * (j + gy * k);
  };
  auto dirichlet = [&](int i, int j, int k) {
    return (!px && (i == 0 || i == gx - 1)) || (!py && (j == 0 || j == gy - 1)) ||
           (!pz && (k == 0 || k == gz - 1));
  };
  L.n_cells = L.nx * L.ny * L.nz;
  L.n_pdof = 4 * L.n_cells;
  L.grid2dof.assign(ng, -1);
  int next = 0;
  for (int pass = 0; pass < 2; ++pass) {  // active nodes first, then Dirichlet
    for (int k = 0; k < gz; ++k)
      for (int j = 0; j < gy; ++j)
        for (int i = 0; i < gx; ++i) {
          const int g = i + gx * (j + gy * k);
          if (canon(i, j, k) != g || dirichlet(i, j, k) != (pass == 1)) continue;
          L.grid2dof[g] = next++;
        }
    if (pass == 0) L.n_active = next;
  }
  L.n_udof = next;
  L.dof2grid.assign(next, -1);
  for (int k = 0; k < gz; ++k)
    for (int j = 0; j < gy; ++j)
      for (int i = 0; i < gx; ++i) {
        const int g = i + gx * (j + gy * k), c = canon(i, j, k);
        if (c == g) L.dof2grid[L.grid2dof[g]] = g;
        else L.grid2dof[g] = L.grid2dof[c];
      }

  // cells
  L.cell_udofs.resize((size_t)L.n_cells * 27);
  L.cell_pdofs.resize((size_t)L.n_cells * 4);
  L.cell_colour.resize(L.n_cells);
  for (int cz = 0; cz < L.nz; ++cz)
    for (int cy = 0; cy < L.ny; ++cy)
      for (int cx = 0; cx < L.nx; ++cx) {
        int c = cx + L.nx * (cy + L.ny * cz);
        for (int lc = 0; lc < 3; ++lc)
          for (int lb = 0; lb < 3; ++lb)
            for (int la = 0; la < 3; ++la)
              L.cell_udofs[(size_t)c * 27 + la + 3 * lb + 9 * lc] =
                  L.grid2dof[(2 * cx + la) + gx * ((2 * cy + lb) + gy * (2 * cz + lc))];
        for (int m = 0; m < 4; ++m) L.cell_pdofs[(size_t)c * 4 + m] = 4 * c + m;
        L.cell_colour[c] = (cx & 1) + 2 * (cy & 1) + 4 * (cz & 1);
      }

  // A pattern: active rows hold the nodes of all cells containing the node
  const int nu = L.n_udof;
  auto a_row = [&](int r, int *out) {
    const int g = L.dof2grid[r];
    const int i = g % gx, j = (g / gx) % gy, k = g / (gx * gy);
    int li[5], lj[5], lk[5];
    const int ni = node_list(i, gx, px, li), nj = node_list(j, gy, py, lj),
              nk = node_list(k, gz, pz, lk);
    int n = 0;
    for (int c = 0; c < nk; ++c)
      for (int b = 0; b < nj; ++b)
        for (int a = 0; a < ni; ++a) out[n++] = L.grid2dof[li[a] + gx * (lj[b] + gy * lk[c])];
    std::sort(out, out + n);
    return (int)(std::unique(out, out + n) - out);
  };
  L.a_rowptr.assign(nu + 1, 0);
#pragma omp parallel for schedule(static)
  for (int r = 0; r < nu; ++r) {
    int buf[125];
    L.a_rowptr[r + 1] = r >= L.n_active ? 1 : a_row(r, buf);
  }
  for (int r = 0; r < nu; ++r) L.a_rowptr[r + 1] += L.a_rowptr[r];
  L.a_col.resize(L.a_rowptr[nu]);
#pragma omp parallel for schedule(static)
  for (int r = 0; r < nu; ++r) {
    int *out = L.a_col.data() + L.a_rowptr[r];
    if (r >= L.n_active) {
      out[0] = r;
      continue;
    }
    int buf[125];
    const int n = a_row(r, buf);
    std::memcpy(out, buf, sizeof(int) * n);
  }
  for (int b = 0; b < 9; ++b) L.a[b].assign(L.a_col.size(), 0.0);

  // B pattern: row 4c+m -> the cell's 27 nodes, sorted
  L.b_rowptr.resize(L.n_pdof + 1);
  for (int p = 0; p <= L.n_pdof; ++p) L.b_rowptr[p] = 27 * p;
  L.b_col.resize((size_t)27 * L.n_pdof);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < L.n_cells; ++c) {
    int sorted[27];
    std::memcpy(sorted, &L.cell_udofs[(size_t)c * 27], sizeof(sorted));
    std::sort(sorted, sorted + 27);
    for (int m = 0; m < 4; ++m) std::memcpy(&L.b_col[(size_t)(4 * c + m) * 27], sorted, sizeof(sorted));
  }
  for (int b = 0; b < 3; ++b) L.b[b].assign(L.b_col.size(), 0.0);

  // BT pattern: row r -> P dofs of all cells containing node r (sorted)
  auto bt_row = [&](int r, int *out) {
    const int g = L.dof2grid[r];
    const int i = g % gx, j = (g / gx) % gy, k = g / (gx * gy);
    int li[2], lj[2], lk[2];
    const int ni = cell_list(i, L.nx, px, li), nj = cell_list(j, L.ny, py, lj),
              nk = cell_list(k, L.nz, pz, lk);
    int n = 0;
    for (int c = 0; c < nk; ++c)
      for (int b = 0; b < nj; ++b)
        for (int a = 0; a < ni; ++a) {
          const int cell = li[a] + L.nx * (lj[b] + L.ny * lk[c]);
          for (int m = 0; m < 4; ++m) out[n++] = 4 * cell + m;
        }
    std::sort(out, out + n);
    return (int)(std::unique(out, out + n) - out);
  };
  L.bt_rowptr.assign(nu + 1, 0);
#pragma omp parallel for schedule(static)
  for (int r = 0; r < nu; ++r) {
    int buf[32];
    L.bt_rowptr[r + 1] = bt_row(r, buf);
  }
  for (int r = 0; r < nu; ++r) L.bt_rowptr[r + 1] += L.bt_rowptr[r];
  L.bt_col.resize(L.bt_rowptr[nu]);
#pragma omp parallel for schedule(static)
  for (int r = 0; r < nu; ++r) {
    int buf[32];
    const int n = bt_row(r, buf);
    std::memcpy(L.bt_col.data() + L.bt_rowptr[r], buf, sizeof(int) * n);
  }
  for (int b = 0; b < 3; ++b) L.bt[b].assign(L.bt_col.size(), 0.0);
}

inline int find_col(const int *cols, int n, int key) {
  const int *p = std::lower_bound(cols, cols + n, key);
  return (p != cols + n && *p == key) ? (int)(p - cols) : -1;
}

void assemble_level(pmh_problem &P, PMLevelData &L, bool finest) {
  const RefTables &T = ref_tables();
  const double nu = P.prm.nu;
  const int gx = L.gx(), gy = L.gy();

  // convection field at the Q2 nodes (its interpolant is the FE parameter)
  std::vector<double> bnod((size_t)3 * L.n_udof);
#pragma omp parallel for schedule(static)
  for (int r = 0; r < L.n_udof; ++r) {
    int g = L.dof2grid[r];
    int i = g % gx, j = (g / gx) % gy, k = g / (gx * gy);
    convection(P, L.node_x(i), L.node_y(j), L.node_z(k), &bnod[(size_t)3 * r]);
  }

  if (finest) {
    P.rhs.assign((size_t)3 * L.n_udof + L.n_pdof, 0.0);
  }

  for (int colour = 0; colour < 8; ++colour) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int c = 0; c < L.n_cells; ++c) {
      if (L.cell_colour[c] != colour) continue;
      const int cx = c % L.nx, cy = (c / L.nx) % L.ny, cz = c / (L.nx * L.ny);
      const double hx = L.xs[cx + 1] - L.xs[cx], hy = L.ys[cy + 1] - L.ys[cy],
                   hz = L.zs[cz + 1] - L.zs[cz];
      const double xc = 0.5 * (L.xs[cx] + L.xs[cx + 1]), yc = 0.5 * (L.ys[cy] + L.ys[cy + 1]),
                   zc = 0.5 * (L.zs[cz] + L.zs[cz + 1]);
      const double detJ = hx * hy * hz / 8.0;
      const double s[3] = {2.0 / hx, 2.0 / hy, 2.0 / hz};
      const int *ud = &L.cell_udofs[(size_t)c * 27];

      double Aloc[27][27];
      for (int i = 0; i < 27; ++i)
        for (int j = 0; j < 27; ++j)
          Aloc[i][j] = nu * detJ *
                       (s[0] * s[0] * T.K[0][i][j] + s[1] * s[1] * T.K[1][i][j] +
                        s[2] * s[2] * T.K[2][i][j]);
      double bl[27][3];
      for (int i = 0; i < 27; ++i)
        for (int d = 0; d < 3; ++d) bl[i][d] = bnod[(size_t)3 * ud[i] + d];
      double floc[3][27];
      std::memset(floc, 0, sizeof(floc));
      for (int q = 0; q < 64; ++q) {
        double bq[3] = {0, 0, 0};
        for (int i = 0; i < 27; ++i)
          for (int d = 0; d < 3; ++d) bq[d] += bl[i][d] * T.phi[q][i];
        double g[27];
        for (int j = 0; j < 27; ++j)
          g[j] = bq[0] * s[0] * T.dphi[q][j][0] + bq[1] * s[1] * T.dphi[q][j][1] +
                 bq[2] * s[2] * T.dphi[q][j][2];
        const double wq = T.w[q] * detJ;
        for (int i = 0; i < 27; ++i) {
          double wi = wq * T.phi[q][i];
          for (int j = 0; j < 27; ++j) Aloc[i][j] += wi * g[j];
        }
        if (finest) {
          double f[3];
          forcing(P, xc + 0.5 * hx * T.pt[q][0], yc + 0.5 * hy * T.pt[q][1],
                  zc + 0.5 * hz * T.pt[q][2], f);
          for (int i = 0; i < 27; ++i)
            for (int d = 0; d < 3; ++d) floc[d][i] += wq * f[d] * T.phi[q][i];
        }
      }
      // B_d[m][j] = -int psi_m d_d phi_j
      double Bloc[3][4][27];
      for (int d = 0; d < 3; ++d)
        for (int m = 0; m < 4; ++m)
          for (int j = 0; j < 27; ++j) Bloc[d][m][j] = -detJ * s[d] * T.B[d][m][j];

      // scatter A (active rows only; Dirichlet rows are set afterwards)
      for (int i = 0; i < 27; ++i) {
        const int r = ud[i];
        if (r >= L.n_active) continue;
        const int rs = L.a_rowptr[r], rn = L.a_rowptr[r + 1] - rs;
        for (int j = 0; j < 27; ++j) {
          int pos = find_col(&L.a_col[rs], rn, ud[j]);
          if (pos < 0) continue;  // cannot happen for the Q2 pattern
          L.a[0][rs + pos] += Aloc[i][j];
          L.a[4][rs + pos] += Aloc[i][j];
          L.a[8][rs + pos] += Aloc[i][j];
        }
        // BT row r, columns 4c+m
        const int bs = L.bt_rowptr[r], bn = L.bt_rowptr[r + 1] - bs;
        for (int m = 0; m < 4; ++m) {
          int pos = find_col(&L.bt_col[bs], bn, 4 * c + m);
          if (pos < 0) continue;
          for (int d = 0; d < 3; ++d) L.bt[d][bs + pos] += Bloc[d][m][i];
        }
        if (finest)
          for (int d = 0; d < 3; ++d) P.rhs[(size_t)d * L.n_udof + r] += floc[d][i];
      }
      // B rows of this cell (exclusive)
      for (int m = 0; m < 4; ++m) {
        const int p = 4 * c + m;
        const int bs = L.b_rowptr[p];
        for (int j = 0; j < 27; ++j) {
          int pos = find_col(&L.b_col[bs], 27, ud[j]);
          for (int d = 0; d < 3; ++d) L.b[d][bs + pos] += Bloc[d][m][j];
        }
      }
    }
  }
  // Dirichlet rows: diagonal 1 in every square block
  for (int r = L.n_active; r < L.n_udof; ++r) {
    const int pos = L.a_rowptr[r];
    for (int b = 0; b < 9; ++b) L.a[b][pos] = 1.0;
  }
  if (finest) {
    for (int r = L.n_active; r < L.n_udof; ++r) {
      int g = L.dof2grid[r];
      int i = g % gx, j = (g / gx) % gy, k = g / (gx * gy);
      double u[3];
      boundary_value(P, L.node_x(i), L.node_y(j), L.node_z(k), u);
      for (int d = 0; d < 3; ++d) P.rhs[(size_t)d * L.n_udof + r] = u[d];
    }
  }
}

}  // namespace

extern "C" {

void pmh_default_params(pmh_params *p) {
  std::memset(p, 0, sizeof(*p));
  p->nx0 = p->ny0 = p->nz0 = 2;
  p->n_levels = 4;
  p->x0 = p->y0 = p->z0 = 0.0;
  p->x1 = p->y1 = p->z1 = 1.0;
  p->nu = 1e-2;
  p->seed = 0;
  p->example = PMH_EXAMPLE_RANDOM_OSEEN;
  p->n_modes = 8;
  p->nthreads = 0;
  p->periodic = 0;
  p->stretch_y = 0.0;
  p->perturb = 0.05;
  p->element = PMH_ELEMENT_HEXA_Q2;
}

void pmh_q2_basis(double xi, double eta, double zeta, double *values, double *derivs) {
  q2_basis(xi, eta, zeta, values, derivs);
}

void pmh_b2_basis(double xi, double eta, double zeta, double *values, double *derivs) {
  b2_basis(xi, eta, zeta, values, derivs);
}

void pmh_p1t_basis(double xi, double eta, double zeta, double *values, double *derivs) {
  p1t_basis(xi, eta, zeta, values, derivs);
}

pmh_problem *pmh_build(const pmh_params *prm) {
  if (!prm || prm->n_levels < 1 || prm->nx0 < 1 || prm->ny0 < 1 || prm->nz0 < 1) return nullptr;
  // a periodic direction needs an even number of cells (>= 2): the parity
  // colouring must separate the cells on both sides of the identified faces
  if (((prm->periodic & PMH_PERIODIC_X) && (prm->nx0 < 2 || (prm->nx0 & 1))) ||
      ((prm->periodic & PMH_PERIODIC_Y) && (prm->ny0 < 2 || (prm->ny0 & 1))) ||
      ((prm->periodic & PMH_PERIODIC_Z) && (prm->nz0 < 2 || (prm->nz0 & 1))) ||
      prm->stretch_y < 0.0)
    return nullptr;
  if (prm->element != PMH_ELEMENT_HEXA_Q2 &&
      (prm->element != PMH_ELEMENT_TETRA_B2 || prm->periodic != 0 || prm->stretch_y != 0.0 ||
       prm->example == PMH_EXAMPLE_CHANNEL))
    return nullptr;
#ifdef _OPENMP
  if (prm->nthreads > 0) omp_set_num_threads(prm->nthreads);
#endif
  pmh_problem *P = new pmh_problem();
  P->prm = *prm;
  SplitMix64 rng(prm->seed);
  for (int m = 0; m < prm->n_modes; ++m) {
    PmhMode md;
    for (int d = 0; d < 3; ++d) md.k[d] = 1.0 + std::floor(4.0 * rng.uniform());
    for (int d = 0; d < 3; ++d) md.a[d] = rng.normal();
    md.phase = 2.0 * M_PI * rng.uniform();
    P->bmodes.push_back(md);
  }
  for (int m = 0; m < prm->n_modes; ++m) {
    PmhMode md;
    for (int d = 0; d < 3; ++d) md.k[d] = 1.0 + std::floor(4.0 * rng.uniform());
    for (int d = 0; d < 3; ++d) md.a[d] = rng.normal();
    md.phase = 2.0 * M_PI * rng.uniform();
    P->fmodes.push_back(md);
  }
  P->levels.resize(prm->n_levels);
  for (int l = 0; l < prm->n_levels; ++l) {
    PMLevelData &L = P->levels[l];
    L.nx = prm->nx0 << l;
    L.ny = prm->ny0 << l;
    L.nz = prm->nz0 << l;
    L.xs.resize(L.nx + 1);
    L.ys.resize(L.ny + 1);
    L.zs.resize(L.nz + 1);
    for (int i = 0; i <= L.nx; ++i) L.xs[i] = prm->x0 + (prm->x1 - prm->x0) * i / L.nx;
    for (int i = 0; i <= L.ny; ++i) {
      if (prm->stretch_y > 0.0) {
        const double eta = -1.0 + 2.0 * i / L.ny;
        const double t = std::tanh(prm->stretch_y * eta) / std::tanh(prm->stretch_y);
        L.ys[i] = prm->y0 + (prm->y1 - prm->y0) * 0.5 * (1.0 + t);
      } else {
        L.ys[i] = prm->y0 + (prm->y1 - prm->y0) * i / L.ny;
      }
    }
    for (int i = 0; i <= L.nz; ++i) L.zs[i] = prm->z0 + (prm->z1 - prm->z0) * i / L.nz;
    if (prm->element == PMH_ELEMENT_HEXA_Q2) build_level_structure(L, prm->periodic);
    if (prm->element != PMH_ELEMENT_HEXA_Q2) continue;
    L.cell_parent.assign(L.n_cells, -1);
    L.cell_child.assign(L.n_cells, -1);
    if (l > 0) {
      for (int cz = 0; cz < L.nz; ++cz)
        for (int cy = 0; cy < L.ny; ++cy)
          for (int cx = 0; cx < L.nx; ++cx) {
            int c = cx + L.nx * (cy + L.ny * cz);
            int pnx = L.nx / 2, pny = L.ny / 2;
            L.cell_parent[c] = (cx / 2) + pnx * ((cy / 2) + pny * (cz / 2));
            L.cell_child[c] = (cx & 1) + 2 * (cy & 1) + 4 * (cz & 1);
          }
    }
  }
  if (prm->element == PMH_ELEMENT_TETRA_B2) {
    build_tet_levels(*P);
    // normalise b: max |b| = 1 over the finest grid nodes (the P2 nodes)
    if (prm->example == PMH_EXAMPLE_RANDOM_OSEEN) {
      const PMLevelData &F = P->levels.back();
      double bmax = 0.0;
      P->bscale = 1.0;
      const int gx = F.gx(), gy = F.gy(), gz = F.gz();
#pragma omp parallel for reduction(max : bmax) schedule(static)
      for (int g = 0; g < gx * gy * gz; ++g) {
        const int i = g % gx, j = (g / gx) % gy, k = g / (gx * gy);
        double b[3];
        convection(*P, F.node_x(i), F.node_y(j), F.node_z(k), b);
        bmax = std::max(bmax, std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]));
      }
      P->bscale = bmax > 0 ? 1.0 / bmax : 1.0;
      P->bmax = 1.0;
    }
    for (int l = 0; l < prm->n_levels; ++l)
      assemble_tet_level(*P, P->levels[l], l == prm->n_levels - 1);
    if (prm->example == PMH_EXAMPLE_QUADLIN_STOKES || prm->example == PMH_EXAMPLE_QUADLIN_OSEEN) {
      const PMLevelData &F = P->levels.back();
      P->has_exact = true;
      P->exact.assign((size_t)3 * F.n_udof + F.n_pdof, 0.0);
      for (int r = 0; r < F.n_udof; ++r) {
        double u[3];
        quadlin_u(F.node_xyz[3 * r], F.node_xyz[3 * r + 1], F.node_xyz[3 * r + 2], u);
        for (int d = 0; d < 3; ++d) P->exact[(size_t)d * F.n_udof + r] = u[d];
      }
      // P1disc coefficients: p at the 4 vertices = sum_m c_m psi_m(vertex)
      for (int t = 0; t < F.n_cells; ++t) {
        const double *x = &F.tet_xyz[(size_t)t * 12];
        double pv[4];
        for (int i = 0; i < 4; ++i) pv[i] = quadlin_p(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
        // psi at the reference vertices: (6, -1, -1, -1), (6, 1, 0, 0), (6, 0, 1, 0),
        // (6, 0, 0, 1), so p_k - p_0 = c_k + s (k = 1..3) with s = c_1 + c_2 + c_3
        double *c = &P->exact[(size_t)3 * F.n_udof + 4 * t];
        const double s4 = (pv[1] + pv[2] + pv[3] - 3.0 * pv[0]) / 4.0;
        c[1] = pv[1] - pv[0] - s4;
        c[2] = pv[2] - pv[0] - s4;
        c[3] = pv[3] - pv[0] - s4;
        c[0] = (pv[1] - c[1]) / 6.0;
      }
    }
    return P;
  }
  // normalise b: max over the finest level's Q2 nodes of |b| = 1
  if (prm->example == PMH_EXAMPLE_RANDOM_OSEEN) {
    const PMLevelData &F = P->levels.back();
    double bmax = 0.0;
    P->bscale = 1.0;
#pragma omp parallel for reduction(max : bmax) schedule(static)
    for (int g = 0; g < F.n_udof; ++g) {
      int i = g % F.gx(), j = (g / F.gx()) % F.gy(), k = g / (F.gx() * F.gy());
      double b[3];
      convection(*P, F.node_x(i), F.node_y(j), F.node_z(k), b);
      double n = std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
      bmax = std::max(bmax, n);
    }
    P->bscale = bmax > 0 ? 1.0 / bmax : 1.0;
    P->bmax = 1.0;
  }
  // channel: perturbation scaled to max |p| = perturb at the finest nodes
  if (prm->example == PMH_EXAMPLE_CHANNEL) {
    const PMLevelData &F = P->levels.back();
    double pmax = 0.0;
#pragma omp parallel for reduction(max : pmax) schedule(static)
    for (int r = 0; r < F.n_udof; ++r) {
      const int g = F.dof2grid[r];
      const int i = g % F.gx(), j = (g / F.gx()) % F.gy(), k = g / (F.gx() * F.gy());
      double p[3];
      channel_perturbation(*P, F.node_x(i), F.node_y(j), F.node_z(k), p);
      pmax = std::max(pmax, std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]));
    }
    P->bscale = pmax > 0 ? prm->perturb / pmax : 0.0;
    double bmax = 0.0;
#pragma omp parallel for reduction(max : bmax) schedule(static)
    for (int r = 0; r < F.n_udof; ++r) {
      const int g = F.dof2grid[r];
      const int i = g % F.gx(), j = (g / F.gx()) % F.gy(), k = g / (F.gx() * F.gy());
      double b[3];
      convection(*P, F.node_x(i), F.node_y(j), F.node_z(k), b);
      bmax = std::max(bmax, std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]));
    }
    P->bmax = bmax;
  }
  for (int l = 0; l < prm->n_levels; ++l) assemble_level(*P, P->levels[l], l == prm->n_levels - 1);

  if (prm->example == PMH_EXAMPLE_QUADLIN_STOKES || prm->example == PMH_EXAMPLE_QUADLIN_OSEEN) {
    const PMLevelData &F = P->levels.back();
    P->has_exact = true;
    P->exact.assign((size_t)3 * F.n_udof + F.n_pdof, 0.0);
    for (int r = 0; r < F.n_udof; ++r) {
      int g = F.dof2grid[r];
      int i = g % F.gx(), j = (g / F.gx()) % F.gy(), k = g / (F.gx() * F.gy());
      double u[3];
      quadlin_u(F.node_x(i), F.node_y(j), F.node_z(k), u);
      for (int d = 0; d < 3; ++d) P->exact[(size_t)d * F.n_udof + r] = u[d];
    }
    for (int c = 0; c < F.n_cells; ++c) {
      const int cx = c % F.nx, cy = (c / F.nx) % F.ny, cz = c / (F.nx * F.ny);
      double hx = F.xs[cx + 1] - F.xs[cx], hy = F.ys[cy + 1] - F.ys[cy], hz = F.zs[cz + 1] - F.zs[cz];
      double xc = 0.5 * (F.xs[cx] + F.xs[cx + 1]), yc = 0.5 * (F.ys[cy] + F.ys[cy + 1]),
             zc = 0.5 * (F.zs[cz] + F.zs[cz + 1]);
      double *p = &P->exact[(size_t)3 * F.n_udof + 4 * c];
      p[0] = quadlin_p(xc, yc, zc);
      p[1] = 3.0 * 0.5 * hx;
      p[2] = -2.0 * 0.5 * hy;
      p[3] = 7.0 * 0.5 * hz;
    }
  }
  return P;
}

void pmh_free(pmh_problem *p) { delete p; }
int pmh_n_levels(const pmh_problem *p) { return p ? (int)p->levels.size() : 0; }
int pmh_ndof(const pmh_problem *p, int level) {
  if (!p || level < 0 || level >= (int)p->levels.size()) return -1;
  return 3 * p->levels[level].n_udof + p->levels[level].n_pdof;
}
double pmh_max_convection(const pmh_problem *p) { return p ? p->bmax : 0.0; }

int pmh_cell_sizes(const pmh_problem *p, int level, double *out) {
  if (!p || level < 0 || level >= (int)p->levels.size() || !out) return -1;
  const PMLevelData &L = p->levels[level];
  if (L.nu_loc != 27) return -1;  // boxes only
  for (int c = 0; c < L.n_cells; ++c) {
    const int cx = c % L.nx, cy = (c / L.nx) % L.ny, cz = c / (L.nx * L.ny);
    out[3 * c] = L.xs[cx + 1] - L.xs[cx];
    out[3 * c + 1] = L.ys[cy + 1] - L.ys[cy];
    out[3 * c + 2] = L.zs[cz + 1] - L.zs[cz];
  }
  return 0;
}

int pmh_convection_nodal(const pmh_problem *p, int level, double *out) {
  if (!p || level < 0 || level >= (int)p->levels.size() || !out) return -1;
  const PMLevelData &L = p->levels[level];
  if (!L.node_xyz.empty()) {
    for (int r = 0; r < L.n_udof; ++r) {
      double b[3];
      convection(*p, L.node_xyz[3 * r], L.node_xyz[3 * r + 1], L.node_xyz[3 * r + 2], b);
      for (int d = 0; d < 3; ++d) out[(size_t)d * L.n_udof + r] = b[d];
    }
    return 0;
  }
  const int gx = L.gx(), gy = L.gy();
  for (int r = 0; r < L.n_udof; ++r) {
    const int g = L.dof2grid[r];
    const int i = g % gx, j = (g / gx) % gy, k = g / (gx * gy);
    double b[3];
    convection(*p, L.node_x(i), L.node_y(j), L.node_z(k), b);
    for (int d = 0; d < 3; ++d) out[(size_t)d * L.n_udof + r] = b[d];
  }
  return 0;
}

int pmh_reassemble(pmh_problem *p) {
  if (!p) return -1;
  const int n = (int)p->levels.size();
  for (int l = 0; l < n; ++l) {
    PMLevelData &L = p->levels[l];
    for (auto &v : L.a) std::fill(v.begin(), v.end(), 0.0);
    for (auto &v : L.b) std::fill(v.begin(), v.end(), 0.0);
    for (auto &v : L.bt) std::fill(v.begin(), v.end(), 0.0);
    if (p->prm.element == PMH_ELEMENT_TETRA_B2)
      assemble_tet_level(*p, L, l == n - 1);
    else
      assemble_level(*p, L, l == n - 1);
  }
  return 0;
}

int pmh_level_desc(const pmh_problem *p, int level, pm_level_desc *o) {
  if (!p || !o || level < 0 || level >= (int)p->levels.size()) return -1;
  const PMLevelData &L = p->levels[level];
  std::memset(o, 0, sizeof(*o));
  o->n_udof = L.n_udof;
  o->n_pdof = L.n_pdof;
  o->n_active = L.n_active;
  o->hanging_bound = L.n_active;
  o->n_dirichlet = L.n_udof - L.n_active;
  o->a_nnz = (int)L.a_col.size();
  o->a_rowptr = L.a_rowptr.data();
  o->a_col = L.a_col.data();
  for (int b = 0; b < 9; ++b) o->a[b] = L.a[b].data();
  o->b_nnz = (int)L.b_col.size();
  o->b_rowptr = L.b_rowptr.data();
  o->b_col = L.b_col.data();
  for (int b = 0; b < 3; ++b) o->b[b] = L.b[b].data();
  o->bt_nnz = (int)L.bt_col.size();
  o->bt_rowptr = L.bt_rowptr.data();
  o->bt_col = L.bt_col.data();
  for (int b = 0; b < 3; ++b) o->bt[b] = L.bt[b].data();
  o->n_cells = L.n_cells;
  o->n_ulocal = L.nu_loc;
  o->n_plocal = 4;
  o->cell_udofs = L.cell_udofs.data();
  o->cell_pdofs = L.cell_pdofs.data();
  o->cell_parent = level > 0 ? L.cell_parent.data() : nullptr;
  o->cell_child = level > 0 && L.nu_loc == 27 ? L.cell_child.data() : nullptr;
  o->cell_colour = L.cell_colour.data();
  if (level > 0 && !L.pu_rowptr.empty()) {
    o->pu_nnz = (int)L.pu_col.size();
    o->pu_rowptr = L.pu_rowptr.data();
    o->pu_col = L.pu_col.data();
    o->pu_val = L.pu_val.data();
    o->pp_nnz = (int)L.pp_col.size();
    o->pp_rowptr = L.pp_rowptr.data();
    o->pp_col = L.pp_col.data();
    o->pp_val = L.pp_val.data();
  }
  return 0;
}

const double *pmh_rhs(const pmh_problem *p) { return p ? p->rhs.data() : nullptr; }
const double *pmh_exact(const pmh_problem *p) { return (p && p->has_exact) ? p->exact.data() : nullptr; }

}  // extern "C"
