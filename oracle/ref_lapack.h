// ref_lapack.h — the two LAPACK routines SolveLinearSystemLapack calls
// (src/FE/LinAlg.C:106-131), for the reference harnesses (ref_vanka.cpp,
// ref_transfer.cpp).  TEST INFRASTRUCTURE ONLY.  dgetrf_: LAPACK's unblocked
// right-looking LU with partial pivoting (first maximal |a|, multipliers
// scaled by the reciprocal of the pivot); dgetrs_: the two triangular solves
// after the row interchanges.  The arithmetic is the oracle's lu_factor /
// lu_solve.  Include it in exactly one translation unit of a library.
#ifndef REF_LAPACK_H
#define REF_LAPACK_H

#include <cmath>
#include <cstddef>

extern "C" {
void dgetrf_(int *m, int *n, double *a, int *lda, int *ipiv, int *info) {
  const int N = *n, ld = *lda;
  *info = 0;
  if (*m != N) {
    *info = -1;
    return;
  }
  for (int k = 0; k < N; ++k) {
    int p = k;
    double amax = std::fabs(a[k + k * ld]);
    for (int i = k + 1; i < N; ++i) {
      const double v = std::fabs(a[i + k * ld]);
      if (v > amax) {
        amax = v;
        p = i;
      }
    }
    ipiv[k] = p + 1;
    if (p != k)
      for (int j = 0; j < N; ++j) {
        const double t = a[k + j * ld];
        a[k + j * ld] = a[p + j * ld];
        a[p + j * ld] = t;
      }
    const double piv = a[k + k * ld];
    if (piv != 0.0) {
      const double r = 1.0 / piv;
      for (int i = k + 1; i < N; ++i) a[i + k * ld] *= r;
    } else if (*info == 0) {
      *info = k + 1;
    }
    for (int j = k + 1; j < N; ++j) {
      const double ukj = a[k + j * ld];
      if (ukj == 0.0) continue;
      for (int i = k + 1; i < N; ++i) a[i + j * ld] -= a[i + k * ld] * ukj;
    }
  }
}

void dgetrs_(char *trans, int *n, int *nrhs, double *a, int *lda, int *ipiv, double *b, int *ldb,
             int *info) {
  const int N = *n, ld = *lda;
  *info = (*trans == 'n' || *trans == 'N') ? 0 : -1;
  if (*info) return;
  for (int r = 0; r < *nrhs; ++r) {
    double *x = b + (size_t)r * *ldb;
    for (int k = 0; k < N; ++k)
      if (ipiv[k] - 1 != k) {
        const double t = x[k];
        x[k] = x[ipiv[k] - 1];
        x[ipiv[k] - 1] = t;
      }
    for (int j = 0; j < N; ++j) {
      const double xj = x[j];
      if (xj != 0.0)
        for (int i = j + 1; i < N; ++i) x[i] -= a[i + j * ld] * xj;
    }
    for (int j = N - 1; j >= 0; --j) {
      x[j] /= a[j + j * ld];
      const double xj = x[j];
      if (xj != 0.0)
        for (int i = 0; i < j; ++i) x[i] -= a[i + j * ld] * xj;
    }
  }
}
}  // extern "C"

#endif
