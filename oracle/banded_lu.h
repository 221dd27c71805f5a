/*
 * banded_lu.h -- TEST INFRASTRUCTURE (oracle). Direct banded LU without pivoting.
 *
 * The reference solves M f = R each step with Eigen::SparseLU<SpMat, COLAMDOrdering<int>>
 * (Sayram-2D source/Solver.h:35; analyzePattern at source/Solver.cc:54, factorize and solve at
 * Solver.cc:277-278). Eigen is a third-party dependency that is not vendored in the reference
 * (no pinned version; the reference's README.md:69-77 lists it by home page only), so the
 * oracle restates "a direct LU solve of M" instead:
 *   Gaussian elimination without pivoting on the band of M (lower/upper bandwidth p/q).
 * M is a column-diagonally-dominant M-matrix (its columns sum to G*dx*dy/dt*(1+dt/tau) plus
 * Dirichlet face terms, because every inner face adds +A to a diagonal and -A to the same
 * column, Solver.cc:135-138), and elimination without pivoting is backward stable for
 * column-diagonally-dominant matrices.  The solution therefore equals Eigen's up to
 * rounding (~1e-14 relative for these systems).
 *
 * Only tests, smoke() and bench.py's CPU baseline may use this file.
 */
#ifndef SAYRAM_ORACLE_BANDED_LU_H
#define SAYRAM_ORACLE_BANDED_LU_H

#include <stddef.h>

/* Band storage: row r holds columns r-p .. r+q at band[r*(p+q+1) + (c - r + p)]. */
static inline size_t blu_idx(long r, long c, long p, long q) {
  return (size_t)r * (size_t)(p + q + 1) + (size_t)(c - r + p);
}

/* In-place LU (no pivoting). Returns 0 on success, -1 on a zero pivot. */
static inline int blu_factor(double* band, long n, long p, long q) {
  for (long k = 0; k < n; ++k) {
    const double piv = band[blu_idx(k, k, p, q)];
    if (piv == 0.0) return -1;
    const long iend = (k + p < n - 1) ? k + p : n - 1;
    const long jend = (k + q < n - 1) ? k + q : n - 1;
    for (long i = k + 1; i <= iend; ++i) {
      double* lik_p = &band[blu_idx(i, k, p, q)];
      if (*lik_p == 0.0) continue;
      const double lik = *lik_p / piv;
      *lik_p = lik;
      const double* urow = &band[blu_idx(k, k, p, q)];
      double* irow = &band[blu_idx(i, k, p, q)];
      for (long j = k + 1; j <= jend; ++j) irow[j - k] -= lik * urow[j - k];
    }
  }
  return 0;
}

/* Solve with the factors from blu_factor; x may alias b. */
static inline void blu_solve(const double* band, long n, long p, long q, const double* b, double* x) {
  if (x != b)
    for (long i = 0; i < n; ++i) x[i] = b[i];
  for (long i = 0; i < n; ++i) {
    const long k0 = (i - p > 0) ? i - p : 0;
    double s = x[i];
    for (long k = k0; k < i; ++k) s -= band[blu_idx(i, k, p, q)] * x[k];
    x[i] = s;
  }
  for (long i = n - 1; i >= 0; --i) {
    const long jend = (i + q < n - 1) ? i + q : n - 1;
    double s = x[i];
    for (long j = i + 1; j <= jend; ++j) s -= band[blu_idx(i, j, p, q)] * x[j];
    x[i] = s / band[blu_idx(i, i, p, q)];
  }
}

#endif
