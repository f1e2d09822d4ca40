// facade_driver.cpp — GPU check of the ParMooN-side solver object's core
// (include/pmgpu_facade.h, pmgpu::FgmresGPU), built and run by
// tests/test_facade.py.  Prints one JSON line.
//
// A 3-level Oseen problem (8^3 cells, nu = 1e-2, seed 0) from the host
// builder; its levels go to FgmresGPU as ParMooN's levels go to
// TNSE_MultiGrid, and Iterate runs FGMRES(20) + V(2,2) to 1e-10 of the
// projected right-hand side.  The oracle's FGMRES (liboracle, the CPU
// restatement of src/FE/FgmresIte.C:250-677) on the same system is the
// answer.  Then B and BT of every level are doubled in place, as a caller
// reassembling its matrices between solves would change them: the next
// Iterate uploads them again, and its solution (the same velocity, half the
// pressure) is compared with the oracle's on the changed system.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "oracle.h"
#include "oseen_problem.h"
#include "pmgpu_facade.h"

namespace {

double rel_diff(const std::vector<double> &x, const std::vector<double> &y, int nu3) {
  // pressures compared after the same L2_0 normalisation (constant P1disc modes)
  auto mean = [&](const std::vector<double> &v) {
    double s = 0.0;
    int n = 0;
    for (size_t i = nu3; i < v.size(); i += 4, ++n) s += v[i];
    return n ? s / n : 0.0;
  };
  const double mx = mean(x), my = mean(y);
  double num = 0.0, den = 0.0;
  for (size_t i = 0; i < x.size(); ++i) {
    const bool mode0 = i >= (size_t)nu3 && (i - nu3) % 4 == 0;
    const double a = x[i] - (mode0 ? mx : 0.0), b = y[i] - (mode0 ? my : 0.0);
    num += (a - b) * (a - b);
    den += b * b;
  }
  return std::sqrt(num / den);
}

}  // namespace

int main(int argc, char **argv) {
  const int precision = argc > 1 ? std::atoi(argv[1]) : PM_PREC_FP64;
  pmh_params pp;
  pmh_default_params(&pp);
  pp.n_levels = 3;
  pp.nu = 1e-2;
  pp.seed = 0;
  pmh_problem *P = pmh_build(&pp);
  if (!P) return 2;
  const int L = pmh_n_levels(P);
  std::vector<pm_level_desc> d(L);
  for (int l = 0; l < L; ++l) pmh_level_desc(P, l, &d[l]);
  const int N = pmh_ndof(P, L - 1), nu3 = 3 * d[L - 1].n_udof;
  std::vector<double> rhs(pmh_rhs(P), pmh_rhs(P) + N);
  double r0 = 0.0, pm = 0.0;
  for (int i = nu3; i < N; i += 4) pm += rhs[i];
  pm /= (N - nu3) / 4;
  for (int i = 0; i < N; ++i) {
    const double v = rhs[i] - ((i >= nu3 && (i - nu3) % 4 == 0) ? pm : 0.0);
    r0 += v * v;
  }
  r0 = std::sqrt(r0);
  const double tol = 1e-10 * r0;

  auto oracle_solve = [&](std::vector<double> &x) {
    oracle_params op;
    oracle_default_params(&op);
    op.restart = 20;
    op.maxit = 80;
    op.res_norm_min = tol;
    oracle *O = oracle_create(d.data(), L, &op);
    double out[3];
    x.assign(N, 0.0);
    const int it = oracle_fgmres(O, x.data(), rhs.data(), out);
    oracle_destroy(O);
    return it;
  };

  pm_options o;
  pm_default_options(&o);
  o.precision = precision;
  pmgpu::FgmresGPU F(o);
  for (int l = 0; l < L; ++l) F.AddLevel(d[l]);
  pmgpu::StopParams sp;
  sp.maxit = 80;
  sp.res_norm_min = tol;

  std::vector<double> xo, x(N, 0.0);
  const int io = oracle_solve(xo);
  const int it = F.Iterate(x.data(), rhs.data(), sp);
  const double e1 = rel_diff(x, xo, nu3);
  const double res1 = F.result().true_res / r0;
  const int st1 = F.status();

  // the caller changes its matrices in place: B and BT doubled on every level
  for (int l = 0; l < L; ++l)
    for (int k = 0; k < 3; ++k) {
      double *b = const_cast<double *>(d[l].b[k]), *bt = const_cast<double *>(d[l].bt[k]);
      for (int j = 0; j < d[l].b_nnz; ++j) b[j] *= 2.0;
      for (int j = 0; j < d[l].bt_nnz; ++j) bt[j] *= 2.0;
    }
  std::vector<double> xo2, x2(N, 0.0);
  const int io2 = oracle_solve(xo2);
  const int it2 = F.Iterate(x2.data(), rhs.data(), sp);
  const double e2 = rel_diff(x2, xo2, nu3);
  // the changed system has the same velocity and half the pressure
  std::vector<double> half(x);
  for (int i = nu3; i < N; ++i) half[i] *= 0.5;
  const double e_half = rel_diff(x2, half, nu3);
  std::printf(
      "{\"precision\": %d, \"iterations\": %d, \"oracle_iterations\": %d, \"status\": %d, "
      "\"rel_res\": %.3e, \"error_vs_oracle\": %.3e, \"iterations_after_update\": %d, "
      "\"oracle_iterations_after_update\": %d, \"status_after_update\": %d, "
      "\"error_vs_oracle_after_update\": %.3e, \"error_vs_half_pressure\": %.3e}\n",
      precision, it, io, st1, res1, e1, it2, io2, (int)F.status(), e2, e_half);
  pmh_free(P);
  return 0;
}
