/* Oracle (test infrastructure): the banded sweeps and the Chebyshev derivative recurrence of
 * oracle/linalg.py and oracle/spectral.py in C, with the same floating-point operations in the
 * same order (built with -ffp-contract=off, so the results equal the NumPy restatement's bit for
 * bit).  They restate pypde's Fortran kernels: fdma.f90:1-38 (solve), :135-141 (LU sweep),
 * tdma.f90:56-107 (offset-k tridiagonal), twodma.f90:2-62, differentiate_cheby.f90:28-53.
 *
 * Arrays are row-major n x m: the sweep runs over rows (axis 0), the m columns are independent
 * right-hand sides.  Coefficient arrays are shared by all columns (cs = 0: one value a row) or
 * hold one system per column (cs = 1: n_rows x m, the stacked systems of the Poisson solve). */
#include <stddef.h>

#define CO(a, r, j) (a)[cs ? (size_t)(r) * (size_t)m + (size_t)(j) : (size_t)(r)]

/* Plan_fdma.FDMA_LU / init_fdma's sweep, per column of a stack of m systems (in place). */
void ok_fdma_lu(double* l, double* d, double* u1, double* u2, int n, int m) {
  const int cs = 1;
  for (int i = 2; i < n; ++i)
    for (int j = 0; j < m; ++j) {
      CO(l, i - 2, j) = CO(l, i - 2, j) / CO(d, i - 2, j);
      CO(d, i, j) = CO(d, i, j) - CO(l, i - 2, j) * CO(u1, i - 2, j);
      if (i < n - 2) CO(u1, i, j) = CO(u1, i, j) - CO(l, i - 2, j) * CO(u2, i - 2, j);
    }
}

/* solve_fdma_1d / _2d along axis 0, in place on x. */
void ok_fdma_solve(const double* l, const double* d, const double* u1, const double* u2, int cs, double* x,
                   int n, int m) {
  for (int i = 2; i < n; ++i) {
    double* xi = x + (size_t)i * m;
    const double* xp = x + (size_t)(i - 2) * m;
    for (int j = 0; j < m; ++j) xi[j] -= CO(l, i - 2, j) * xp[j];
  }
  for (int j = 0; j < m; ++j) {
    x[(size_t)(n - 1) * m + j] = x[(size_t)(n - 1) * m + j] / CO(d, n - 1, j);
    x[(size_t)(n - 2) * m + j] = x[(size_t)(n - 2) * m + j] / CO(d, n - 2, j);
    x[(size_t)(n - 3) * m + j] =
        (x[(size_t)(n - 3) * m + j] - CO(u1, n - 3, j) * x[(size_t)(n - 1) * m + j]) / CO(d, n - 3, j);
    x[(size_t)(n - 4) * m + j] =
        (x[(size_t)(n - 4) * m + j] - CO(u1, n - 4, j) * x[(size_t)(n - 2) * m + j]) / CO(d, n - 4, j);
  }
  for (int i = n - 5; i >= 0; --i) {
    double* xi = x + (size_t)i * m;
    const double* x2 = x + (size_t)(i + 2) * m;
    const double* x4 = x + (size_t)(i + 4) * m;
    for (int j = 0; j < m; ++j) xi[j] = (xi[j] - CO(u1, i, j) * x2[j] - CO(u2, i, j) * x4[j]) / CO(d, i, j);
  }
}

/* solve_twodma_1d / _2d along axis 0, in place on x. */
void ok_twodma_solve(const double* d, const double* u, double* x, int n, int m) {
  for (int j = 0; j < m; ++j) {
    x[(size_t)(n - 1) * m + j] = x[(size_t)(n - 1) * m + j] / d[n - 1];
    x[(size_t)(n - 2) * m + j] = x[(size_t)(n - 2) * m + j] / d[n - 2];
  }
  for (int i = n - 3; i >= 0; --i) {
    double* xi = x + (size_t)i * m;
    const double* x2 = x + (size_t)(i + 2) * m;
    for (int j = 0; j < m; ++j) xi[j] = (xi[j] - u[i] * x2[j]) / d[i];
  }
}

/* solve_tdma_2d: A x = d with A at offsets -k, 0, +k (a: n-k, b: n, c: n-k); w is scratch (n-k). */
void ok_tdma_offset(const double* a, const double* b, const double* c, const double* d, double* x, double* g,
                    double* w, int n, int m, int k) {
  for (int i = 0; i < n - k; ++i) w[i] = i < k ? c[i] / b[i] : c[i] / (b[i] - a[i - k] * w[i - k]);
  for (int i = 0; i < n; ++i) {
    double* gi = g + (size_t)i * m;
    const double* di = d + (size_t)i * m;
    if (i < k) {
      for (int j = 0; j < m; ++j) gi[j] = di[j] / b[i];
    } else {
      const double* gp = g + (size_t)(i - k) * m;
      const double den = b[i] - a[i - k] * w[i - k];
      for (int j = 0; j < m; ++j) gi[j] = (di[j] - a[i - k] * gp[j]) / den;
    }
  }
  for (int i = n - k - 1; i < n; ++i)
    for (int j = 0; j < m; ++j) x[(size_t)i * m + j] = g[(size_t)i * m + j];
  for (int i = n - k - 1; i >= 0; --i) {
    double* xi = x + (size_t)i * m;
    const double* gi = g + (size_t)i * m;
    const double* xk = x + (size_t)(i + k) * m;
    for (int j = 0; j < m; ++j) xi[j] = gi[j] - w[i] * xk[j];
  }
}

/* One Chebyshev derivative along axis 0: dc (zeroed by the caller) from c. */
void ok_cheb_diff1(const double* c, double* dc, int n, int m) {
  const double f = 2.0 * (n - 1);
  for (int j = 0; j < m; ++j) dc[(size_t)(n - 2) * m + j] = f * c[(size_t)(n - 1) * m + j];
  for (int i = n - 3; i > 0; --i) {
    const double fi = 2.0 * (i + 1);
    double* di = dc + (size_t)i * m;
    const double* d2 = dc + (size_t)(i + 2) * m;
    const double* c1 = c + (size_t)(i + 1) * m;
    for (int j = 0; j < m; ++j) di[j] = d2[j] + fi * c1[j];
  }
  for (int j = 0; j < m; ++j) dc[j] = dc[(size_t)2 * m + j] / 2.0 + c[(size_t)m + j];
}
