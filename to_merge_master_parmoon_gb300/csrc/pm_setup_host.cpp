// pm_setup_host.cpp — colouring and grid-transfer construction for libpmgpu.
#include "pm_setup_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
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
