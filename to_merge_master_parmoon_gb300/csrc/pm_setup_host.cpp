// pm_setup_host.cpp — colouring and grid-transfer construction for libpmgpu.
#include "pm_setup_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <string>
#include <utility>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace pm {

namespace {

// Q2 Lagrange basis on [-1,1]^3, local function a+3b+9c (xi fastest).
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

struct Tables {
  double qu[8][27][27];  // coarse Q2 basis l at fine node k of child j
  double qp[8][4][4];    // P1disc: coefficients of the restricted coarse mode
  Tables() {
    for (int j = 0; j < 8; ++j) {
      const double o[3] = {(j & 1) ? 1.0 : -1.0, (j & 2) ? 1.0 : -1.0, (j & 4) ? 1.0 : -1.0};
      for (int c = 0; c < 3; ++c)
        for (int b = 0; b < 3; ++b)
          for (int a = 0; a < 3; ++a)
            q2_values(0.5 * (a - 1.0 + o[0]), 0.5 * (b - 1.0 + o[1]), 0.5 * (c - 1.0 + o[2]),
                      qu[j][a + 3 * b + 9 * c]);
      // coarse mode (1, X, Y, Z) with X = (x' + o_x)/2 in child coordinates
      std::memset(qp[j], 0, sizeof(qp[j]));
      qp[j][0][0] = 1.0;
      for (int d = 0; d < 3; ++d) {
        qp[j][0][1 + d] = 0.5 * o[d];
        qp[j][1 + d][1 + d] = 0.5;
      }
    }
  }
};

const Tables &tables() {
  static Tables t;
  return t;
}

// dof -> list of (cell, local index)
void incidence(int ncells, int nloc, const int *dofs, int ndof, std::vector<int> &ptr,
               std::vector<int> &ent) {
  ptr.assign(ndof + 1, 0);
  for (long long t = 0; t < (long long)ncells * nloc; ++t) ptr[dofs[t] + 1]++;
  for (int i = 0; i < ndof; ++i) ptr[i + 1] += ptr[i];
  ent.resize((size_t)ptr[ndof]);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int c = 0; c < ncells; ++c)
    for (int k = 0; k < nloc; ++k) ent[fill[dofs[(size_t)c * nloc + k]]++] = c * nloc + k;
}

bool build_one(int nf_cells, int nloc, const int *f_dofs, int f_n, const int *c_dofs, int c_n,
               const int *f_parent, const int *f_child, bool velocity, HostCsr &P,
               std::string &err) {
  const Tables &T = tables();
  std::vector<int> ptr, ent;
  incidence(nf_cells, nloc, f_dofs, f_n, ptr, ent);
  P.rows = f_n;
  P.cols = c_n;
  P.rowptr.assign(f_n + 1, 0);
  std::vector<std::vector<std::pair<int, double>>> rows(f_n);
  bool bad = false;
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < f_n; ++i) {
    auto &row = rows[i];
    const int m = ptr[i + 1] - ptr[i];
    if (m == 0) continue;
    for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
      const int fc = ent[e] / nloc, k = ent[e] % nloc;
      const int pc = f_parent[fc], j = f_child[fc];
      if (pc < 0 || j < 0 || j > 7) {
        bad = true;
        continue;
      }
      for (int l = 0; l < nloc; ++l) {
        const double v = velocity ? T.qu[j][k][l] : T.qp[j][k][l];
        if (v == 0.0) continue;
        const int K = c_dofs[(size_t)pc * nloc + l];
        auto it = std::find_if(row.begin(), row.end(),
                               [K](const std::pair<int, double> &q) { return q.first == K; });
        if (it == row.end())
          row.emplace_back(K, v);
        else
          it->second += v;
      }
    }
    const double inv = 1.0 / (double)m;
    for (auto &q : row) q.second *= inv;
    std::sort(row.begin(), row.end());
  }
  if (bad) {
    err = "cell_parent/cell_child out of range";
    return false;
  }
  for (int i = 0; i < f_n; ++i) P.rowptr[i + 1] = P.rowptr[i] + (int)rows[i].size();
  P.col.resize(P.rowptr[f_n]);
  P.val.resize(P.rowptr[f_n]);
  for (int i = 0; i < f_n; ++i) {
    int o = P.rowptr[i];
    for (auto &q : rows[i]) {
      P.col[o] = q.first;
      P.val[o] = q.second;
      ++o;
    }
  }
  return true;
}

}  // namespace

void build_neighbours(int ncells, const int *udofs, int nu, std::vector<int> &nbr) {
  std::vector<int> ptr, ent;
  incidence(ncells, 27, udofs, nu, ptr, ent);
  nbr.assign((size_t)ncells * 26, -1);
#pragma omp parallel for schedule(dynamic, 256)
  for (int c = 0; c < ncells; ++c) {
    // neighbour cell -> bitmask of c's local nodes it shares
    int cand[64];
    unsigned int mask[64];
    int nc = 0;
    for (int k = 0; k < 27; ++k) {
      const int d = udofs[(size_t)c * 27 + k];
      for (int e = ptr[d]; e < ptr[d + 1]; ++e) {
        const int o = ent[e] / 27;
        if (o == c) continue;
        int q = 0;
        while (q < nc && cand[q] != o) ++q;
        if (q == nc) {
          if (nc == 64) continue;
          cand[nc] = o;
          mask[nc] = 0;
          ++nc;
        }
        mask[q] |= 1u << k;
      }
    }
    for (int q = 0; q < nc; ++q) {
      int off[3];
      for (int axis = 0; axis < 3; ++axis) {
        bool all0 = true, all2 = true;
        for (int k = 0; k < 27; ++k)
          if (mask[q] & (1u << k)) {
            const int idx = axis == 0 ? k % 3 : (axis == 1 ? (k / 3) % 3 : k / 9);
            all0 = all0 && idx == 0;
            all2 = all2 && idx == 2;
          }
        off[axis] = all2 ? 1 : (all0 ? -1 : 0);
      }
      int slot = (off[0] + 1) + 3 * (off[1] + 1) + 9 * (off[2] + 1);
      if (slot == 13) continue;
      if (slot > 13) --slot;
      nbr[(size_t)c * 26 + slot] = cand[q];
    }
  }
}

void node_inverse_multiplicity(int ncells, const int *udofs, int nu, std::vector<float> &inv) {
  std::vector<int> cnt(nu, 0);
  for (long long t = 0; t < (long long)ncells * 27; ++t) cnt[udofs[t]]++;
  inv.resize(nu);
  for (int i = 0; i < nu; ++i) inv[i] = cnt[i] > 0 ? 1.0f / (float)cnt[i] : 0.0f;
}

HostCsr transpose(const HostCsr &a) {
  HostCsr t;
  t.rows = a.cols;
  t.cols = a.rows;
  t.rowptr.assign(t.rows + 1, 0);
  for (int c : a.col) t.rowptr[c + 1]++;
  for (int i = 0; i < t.rows; ++i) t.rowptr[i + 1] += t.rowptr[i];
  t.col.resize(a.col.size());
  t.val.resize(a.val.size());
  std::vector<int> fill(t.rowptr.begin(), t.rowptr.end() - 1);
  for (int i = 0; i < a.rows; ++i)
    for (int j = a.rowptr[i]; j < a.rowptr[i + 1]; ++j) {
      const int o = fill[a.col[j]]++;
      t.col[o] = i;
      t.val[o] = a.val[j];
    }
  return t;
}

bool build_transfers(int nc_cells, const int *c_udofs, const int *c_pdofs, int c_nu, int c_np,
                     int nf_cells, const int *f_udofs, const int *f_pdofs, int f_nu, int f_np,
                     const int *f_parent, const int *f_child, HostCsr &Pu, HostCsr &Ru,
                     HostCsr &Pp, HostCsr &Rp, std::string &err) {
  (void)nc_cells;
  if (!f_parent || !f_child) {
    err = "fine level without cell_parent/cell_child";
    return false;
  }
  for (int c = 0; c < nf_cells; ++c)
    if (f_parent[c] < 0 || f_parent[c] >= nc_cells) {
      err = "cell_parent out of range";
      return false;
    }
  if (!build_one(nf_cells, 27, f_udofs, f_nu, c_udofs, c_nu, f_parent, f_child, true, Pu, err))
    return false;
  if (!build_one(nf_cells, 4, f_pdofs, f_np, c_pdofs, c_np, f_parent, f_child, false, Pp, err))
    return false;
  Ru = transpose(Pu);
  Rp = transpose(Pp);
  return true;
}

bool make_colouring(int ncells, int nulocal, int nplocal, const int *udofs, const int *pdofs,
                    int nu, int np, const int *colour, Colouring &out, std::string &err) {
  std::vector<int> col(ncells, -1);
  if (colour) {
    for (int c = 0; c < ncells; ++c) {
      if (colour[c] < 0 || colour[c] > 4095) {
        err = "cell_colour out of range";
        return false;
      }
      col[c] = colour[c];
    }
  } else {
    std::vector<int> uptr, uent;
    incidence(ncells, nulocal, udofs, nu, uptr, uent);
    std::vector<int> stamp(4096, -1);
    for (int c = 0; c < ncells; ++c) {
      for (int k = 0; k < nulocal; ++k) {
        const int d = udofs[(size_t)c * nulocal + k];
        for (int e = uptr[d]; e < uptr[d + 1]; ++e) {
          const int o = uent[e] / nulocal;
          if (col[o] >= 0) stamp[col[o]] = c;
        }
      }
      int k = 0;
      while (stamp[k] == c) ++k;
      col[c] = k;
    }
  }
  int ncol = 0;
  for (int c = 0; c < ncells; ++c) ncol = std::max(ncol, col[c] + 1);
  out.ptr.assign(ncol + 1, 0);
  for (int c = 0; c < ncells; ++c) out.ptr[col[c] + 1]++;
  for (int k = 0; k < ncol; ++k) out.ptr[k + 1] += out.ptr[k];
  out.order.resize(ncells);
  std::vector<int> fill(out.ptr.begin(), out.ptr.end() - 1);
  for (int c = 0; c < ncells; ++c) out.order[fill[col[c]]++] = c;
  out.max_size = 0;
  for (int k = 0; k < ncol; ++k) out.max_size = std::max(out.max_size, out.ptr[k + 1] - out.ptr[k]);
  // conflict check: no DOF twice within one colour
  std::vector<int> su(nu, -1), sp(np, -1);
  for (int k = 0; k < ncol; ++k)
    for (int t = out.ptr[k]; t < out.ptr[k + 1]; ++t) {
      const int c = out.order[t];
      for (int q = 0; q < nulocal; ++q) {
        const int d = udofs[(size_t)c * nulocal + q];
        if (d < 0 || d >= nu) {
          err = "cell_udofs out of range";
          return false;
        }
        if (su[d] == k) {
          err = "colouring conflict: two cells of one colour share a velocity DOF";
          return false;
        }
        su[d] = k;
      }
      for (int q = 0; q < nplocal; ++q) {
        const int d = pdofs[(size_t)c * nplocal + q];
        if (d < 0 || d >= np) {
          err = "cell_pdofs out of range";
          return false;
        }
        if (sp[d] == k) {
          err = "colouring conflict: two cells of one colour share a pressure DOF";
          return false;
        }
        sp[d] = k;
      }
    }
  return true;
}

}  // namespace pm

namespace pm {

namespace {

// stacked index of velocity DOF i of system s (n_active-first per component)
inline int vmap(int G, int nu, int na, int s, int i) {
  return i < na ? s * na + i : G * na + s * (nu - na) + (i - na);
}

// CSR rows in stacked order (rows_of(s, i) for stacked row R), columns mapped
void stack_csr(int G, int rows_sys, const std::vector<std::pair<int, int>> &order,
               const pm_level_desc *d, const int *pm_level_desc::*rp, const int *pm_level_desc::*cp,
               int nnz_sys, const std::function<int(int, int)> &colmap, std::vector<int> &rowptr,
               std::vector<int> &col, std::vector<long long> &src) {
  (void)rows_sys;
  rowptr.assign(order.size() + 1, 0);
  col.clear();
  col.reserve((size_t)G * nnz_sys);
  src.clear();
  src.reserve((size_t)G * nnz_sys);
  for (size_t R = 0; R < order.size(); ++R) {
    const int s = order[R].first, i = order[R].second;
    const int *rowp = d[s].*rp;
    const int *colp = d[s].*cp;
    for (int j = rowp[i]; j < rowp[i + 1]; ++j) {
      col.push_back(colmap(s, colp[j]));
      src.push_back((long long)s * nnz_sys + j);
    }
    rowptr[R + 1] = (int)col.size();
  }
}

void gather_vals(int G, const std::vector<long long> &src, const double *const *per_sys,
                 int nnz_sys, std::vector<double> &out) {
  (void)G;
  out.resize(src.size());
  for (size_t k = 0; k < src.size(); ++k) {
    const long long q = src[k];
    out[k] = per_sys[q / nnz_sys][q % nnz_sys];
  }
}

}  // namespace

bool stack_levels(const pm_level_desc *d, int G, const StackSizes &coarse, StackedLevel &st,
                  pm_level_desc &out, std::string &err) {
  const pm_level_desc &d0 = d[0];
  for (int s = 1; s < G; ++s) {
    const pm_level_desc &e = d[s];
    if (e.n_udof != d0.n_udof || e.n_pdof != d0.n_pdof || e.n_active != d0.n_active ||
        e.n_dirichlet != d0.n_dirichlet || e.hanging_bound != d0.hanging_bound ||
        e.a_nnz != d0.a_nnz || e.b_nnz != d0.b_nnz || e.bt_nnz != d0.bt_nnz ||
        e.n_cells != d0.n_cells || e.n_ulocal != d0.n_ulocal || e.n_plocal != d0.n_plocal ||
        e.pu_nnz != d0.pu_nnz || e.pp_nnz != d0.pp_nnz) {
      err = "stacked systems must have equal sizes on every level (system " +
            std::to_string(s) + " differs)";
      return false;
    }
    for (int k = 0; k < 9; ++k)
      if ((e.a[k] != nullptr) != (d0.a[k] != nullptr)) {
        err = "stacked systems must give the same A blocks";
        return false;
      }
    if ((e.cell_colour != nullptr) != (d0.cell_colour != nullptr) ||
        (e.cell_parent != nullptr) != (d0.cell_parent != nullptr) ||
        (e.pu_rowptr != nullptr) != (d0.pu_rowptr != nullptr)) {
      err = "stacked systems must give the same optional arrays";
      return false;
    }
  }
  const int nu = d0.n_udof, na = d0.n_active, np = d0.n_pdof, nc = d0.n_cells;
  const int nl = d0.n_ulocal, npl = d0.n_plocal;
  if ((long long)G * (3LL * nu + np) > 2000000000LL || (long long)G * d0.a_nnz > 2000000000LL) {
    err = "stacked level too large for 32-bit indices";
    return false;
  }
  // stacked velocity rows: the G systems' active rows, then their Dirichlet rows
  std::vector<std::pair<int, int>> vrows;
  vrows.reserve((size_t)G * nu);
  for (int s = 0; s < G; ++s)
    for (int i = 0; i < na; ++i) vrows.emplace_back(s, i);
  for (int s = 0; s < G; ++s)
    for (int i = na; i < nu; ++i) vrows.emplace_back(s, i);
  std::vector<std::pair<int, int>> prows;
  prows.reserve((size_t)G * np);
  for (int s = 0; s < G; ++s)
    for (int i = 0; i < np; ++i) prows.emplace_back(s, i);
  auto vcol = [&](int s, int c) { return vmap(G, nu, na, s, c); };
  auto pcol = [&](int s, int c) { return s * np + c; };
  std::vector<long long> src;
  std::vector<const double *> per((size_t)G);
  stack_csr(G, nu, vrows, d, &pm_level_desc::a_rowptr, &pm_level_desc::a_col, d0.a_nnz, vcol,
            st.a_rowptr, st.a_col, src);
  for (int k = 0; k < 9; ++k) {
    st.a[k].clear();
    if (!d0.a[k]) continue;
    for (int s = 0; s < G; ++s) per[(size_t)s] = d[s].a[k];
    gather_vals(G, src, per.data(), d0.a_nnz, st.a[k]);
  }
  stack_csr(G, np, prows, d, &pm_level_desc::b_rowptr, &pm_level_desc::b_col, d0.b_nnz, vcol,
            st.b_rowptr, st.b_col, src);
  for (int k = 0; k < 3; ++k) {
    for (int s = 0; s < G; ++s) per[(size_t)s] = d[s].b[k];
    gather_vals(G, src, per.data(), d0.b_nnz, st.b[k]);
  }
  stack_csr(G, nu, vrows, d, &pm_level_desc::bt_rowptr, &pm_level_desc::bt_col, d0.bt_nnz, pcol,
            st.bt_rowptr, st.bt_col, src);
  for (int k = 0; k < 3; ++k) {
    for (int s = 0; s < G; ++s) per[(size_t)s] = d[s].bt[k];
    gather_vals(G, src, per.data(), d0.bt_nnz, st.bt[k]);
  }
  // cells, system after system
  st.udofs.resize((size_t)G * nc * nl);
  st.pdofs.resize((size_t)G * nc * npl);
  for (int s = 0; s < G; ++s) {
    for (size_t k = 0; k < (size_t)nc * nl; ++k)
      st.udofs[(size_t)s * nc * nl + k] = vcol(s, d[s].cell_udofs[k]);
    for (size_t k = 0; k < (size_t)nc * npl; ++k)
      st.pdofs[(size_t)s * nc * npl + k] = pcol(s, d[s].cell_pdofs[k]);
  }
  st.parent.clear();
  st.child.clear();
  if (d0.cell_parent && d0.cell_child) {
    st.parent.resize((size_t)G * nc);
    st.child.resize((size_t)G * nc);
    for (int s = 0; s < G; ++s)
      for (int k = 0; k < nc; ++k) {
        st.parent[(size_t)s * nc + k] = s * coarse.ncells + d[s].cell_parent[k];
        st.child[(size_t)s * nc + k] = d[s].cell_child[k];
      }
  }
  st.colour.clear();
  if (d0.cell_colour) {
    st.colour.resize((size_t)G * nc);
    for (int s = 0; s < G; ++s)
      std::memcpy(st.colour.data() + (size_t)s * nc, d[s].cell_colour, sizeof(int) * nc);
  }
  if (d0.pu_rowptr) {
    auto cvcol = [&](int s, int c) { return vmap(G, coarse.nu, coarse.na, s, c); };
    auto cpcol = [&](int s, int c) { return s * coarse.np + c; };
    stack_csr(G, nu, vrows, d, &pm_level_desc::pu_rowptr, &pm_level_desc::pu_col, d0.pu_nnz,
              cvcol, st.pu_rowptr, st.pu_col, src);
    for (int s = 0; s < G; ++s) per[(size_t)s] = d[s].pu_val;
    gather_vals(G, src, per.data(), d0.pu_nnz, st.pu_val);
    stack_csr(G, np, prows, d, &pm_level_desc::pp_rowptr, &pm_level_desc::pp_col, d0.pp_nnz,
              cpcol, st.pp_rowptr, st.pp_col, src);
    for (int s = 0; s < G; ++s) per[(size_t)s] = d[s].pp_val;
    gather_vals(G, src, per.data(), d0.pp_nnz, st.pp_val);
  }
  std::memset(&out, 0, sizeof(out));
  out.n_udof = G * nu;
  out.n_pdof = G * np;
  out.n_active = G * na;
  out.hanging_bound = G * na;
  out.n_dirichlet = G * (nu - na);
  out.a_nnz = (int)st.a_col.size();
  out.a_rowptr = st.a_rowptr.data();
  out.a_col = st.a_col.data();
  for (int k = 0; k < 9; ++k) out.a[k] = st.a[k].empty() ? nullptr : st.a[k].data();
  out.b_nnz = (int)st.b_col.size();
  out.b_rowptr = st.b_rowptr.data();
  out.b_col = st.b_col.data();
  out.bt_nnz = (int)st.bt_col.size();
  out.bt_rowptr = st.bt_rowptr.data();
  out.bt_col = st.bt_col.data();
  for (int k = 0; k < 3; ++k) {
    out.b[k] = st.b[k].data();
    out.bt[k] = st.bt[k].data();
  }
  out.n_cells = G * nc;
  out.n_ulocal = nl;
  out.n_plocal = npl;
  out.cell_udofs = st.udofs.data();
  out.cell_pdofs = st.pdofs.data();
  out.cell_parent = st.parent.empty() ? nullptr : st.parent.data();
  out.cell_child = st.child.empty() ? nullptr : st.child.data();
  out.cell_colour = st.colour.empty() ? nullptr : st.colour.data();
  if (d0.pu_rowptr) {
    out.pu_nnz = (int)st.pu_col.size();
    out.pu_rowptr = st.pu_rowptr.data();
    out.pu_col = st.pu_col.data();
    out.pu_val = st.pu_val.data();
    out.pp_nnz = (int)st.pp_col.size();
    out.pp_rowptr = st.pp_rowptr.data();
    out.pp_col = st.pp_col.data();
    out.pp_val = st.pp_val.data();
  }
  return true;
}

}  // namespace pm
