// tridiag.cpp -- lowest eigenpair of a symmetric tridiagonal matrix, the role LAPACK dstev_
// plays in the reference Lanczos loops (sml/LANCZOS_SYM.c:158, sml/LANCZOS_SLOW_SYM.c:137,
// dmrg/DMRG_LANCZOS_SLOW_OBC.c:110), where only the lowest eigenvalue Lap_D[0] and its
// eigenvector (first column of Lap_V) are ever used.
//
// Methods (written from the published descriptions):
//  * eigenvalue: Sturm-sequence bisection (Barth, Martin & Wilkinson, Numer. Math. 9 (1967)
//    386-393) with Kahan's guarded pivots: the count of negative pivots of the LDL^T
//    factorisation of T - x I equals the number of eigenvalues below x.  The lowest
//    eigenvalue lies in [Gershgorin lower bound, min_i d_i]; a previous estimate that is an
//    upper bound (Cauchy interlacing for a growing Lanczos matrix) narrows the bracket.
//  * eigenvector: inverse iteration on T - lambda I with the tridiagonal LU factorisation
//    with partial pivoting (Peters & Wilkinson, "The calculation of specified eigenvectors
//    by inverse iteration", Handbook for Automatic Computation II/18, 1971), two sweeps.
#include "tridiag.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

namespace dg {

namespace {

// Number of eigenvalues of T strictly below x.
int sturm_count(const double *d, const double *e2, int n, double x, double pivmin) {
  int count = 0;
  double q = d[0] - x;
  if (std::fabs(q) < pivmin) q = -pivmin;
  if (q < 0) ++count;
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - e2[i - 1] / q;
    if (std::fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++count;
  }
  return count;
}

}  // namespace

double tridiag_lowest_eigenvalue(const double *d, const double *e, int n, double upper_hint) {
  if (n == 1) return d[0];
  std::vector<double> e2(n - 1);
  double emax2 = 0.0, lo = d[0], hi = d[0], anorm = 0.0;
  for (int i = 0; i < n; ++i) {
    double left = (i > 0) ? std::fabs(e[i - 1]) : 0.0;
    double right = (i < n - 1) ? std::fabs(e[i]) : 0.0;
    lo = std::min(lo, d[i] - left - right);
    hi = std::min(hi, d[i]);
    anorm = std::max(anorm, std::fabs(d[i]) + left + right);
    if (i < n - 1) {
      e2[i] = e[i] * e[i];
      emax2 = std::max(emax2, e2[i]);
    }
  }
  const double pivmin = std::max(DBL_MIN, DBL_MIN * emax2);
  if (std::isfinite(upper_hint) && upper_hint < hi) {
    // The hint is an upper bound only if at least one eigenvalue lies at or below it.
    if (sturm_count(d, e2.data(), n, upper_hint, pivmin) >= 1) hi = upper_hint;
  }
  // Expand hi slightly so that an eigenvalue equal to hi is strictly below it.
  const double tol_abs = 2.0 * DBL_EPSILON * std::max(anorm, DBL_MIN);
  hi += tol_abs;
  lo -= tol_abs;
  // Narrow a wide bracket from the top first: near convergence the lowest eigenvalue sits
  // just below the hint, so probe hi - delta with growing delta.
  double delta = std::max(tol_abs, 1e-12 * std::fabs(hi));
  while (hi - delta > lo) {
    double x = hi - delta;
    if (sturm_count(d, e2.data(), n, x, pivmin) >= 1) {
      hi = x;
      delta *= 16.0;
    } else {
      lo = x;
      break;
    }
  }
  // Bisect down to adjacent floating-point numbers: the Lanczos convergence test compares
  // successive eigenvalues to an absolute 1e-14, about one ulp at |E| ~ 50, so the
  // eigenvalue must be resolved to the last bit.
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (sturm_count(d, e2.data(), n, mid, pivmin) >= 1)
      hi = mid;
    else
      lo = mid;
  }
  return 0.5 * (lo + hi);
}

void tridiag_eigenvector(const double *d, const double *e, int n, double lambda, double *z) {
  if (n == 1) {
    z[0] = 1.0;
    return;
  }
  double anorm = 0.0;
  for (int i = 0; i < n; ++i) {
    double s = std::fabs(d[i]) + (i > 0 ? std::fabs(e[i - 1]) : 0.0) + (i < n - 1 ? std::fabs(e[i]) : 0.0);
    anorm = std::max(anorm, s);
  }
  const double eps_piv = DBL_EPSILON * std::max(anorm, DBL_MIN);
  // LU with partial pivoting of (T - lambda I): rows i may swap with i+1.  U has up to two
  // super-diagonals (u0 diag, u1, u2); l holds the multipliers; piv records swaps.
  std::vector<double> u0(n), u1(n), u2(n), l(n);
  std::vector<char> piv(n, 0);
  double a = d[0] - lambda;            // current pivot-row diagonal
  double b = (n > 1) ? e[0] : 0.0;     // current pivot-row super-diagonal
  double c = 0.0;                      // current pivot-row second super-diagonal
  for (int i = 0; i < n - 1; ++i) {
    const double sub = e[i];                  // T[i+1][i]
    const double nd = d[i + 1] - lambda;      // T[i+1][i+1]
    const double ns = (i + 1 < n - 1) ? e[i + 1] : 0.0;  // T[i+1][i+2]
    if (std::fabs(sub) > std::fabs(a)) {
      // swap rows i and i+1
      piv[i] = 1;
      const double m = a / sub;
      l[i] = m;
      u0[i] = sub;
      u1[i] = nd;
      u2[i] = ns;
      a = b - m * nd;
      b = c - m * ns;
      c = 0.0;
    } else {
      if (a == 0.0) a = eps_piv;
      const double m = sub / a;
      l[i] = m;
      u0[i] = a;
      u1[i] = b;
      u2[i] = c;
      a = nd - m * b;
      b = ns - m * c;
      c = 0.0;
    }
  }
  if (a == 0.0) a = eps_piv;
  u0[n - 1] = a;
  u1[n - 1] = 0.0;
  u2[n - 1] = 0.0;
  for (int i = 0; i < n; ++i)
    if (std::fabs(u0[i]) < eps_piv) u0[i] = std::copysign(eps_piv, u0[i] == 0.0 ? 1.0 : u0[i]);

  // First sweep solves U z = (1,...,1) directly (Wilkinson's choice of starting vector);
  // subsequent sweeps apply L^{-1} P first.
  for (int i = 0; i < n; ++i) z[i] = 1.0;
  for (int sweep = 0; sweep < 3; ++sweep) {
    if (sweep > 0) {
      for (int i = 0; i < n - 1; ++i) {
        if (piv[i]) std::swap(z[i], z[i + 1]);
        z[i + 1] -= l[i] * z[i];
      }
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = z[i];
      if (i + 1 < n) s -= u1[i] * z[i + 1];
      if (i + 2 < n) s -= u2[i] * z[i + 2];
      z[i] = s / u0[i];
    }
    double nrm = 0.0, big = 0.0;
    for (int i = 0; i < n; ++i) big = std::max(big, std::fabs(z[i]));
    if (big == 0.0 || !std::isfinite(big)) {
      for (int i = 0; i < n; ++i) z[i] = (i == 0) ? 1.0 : 0.0;
      return;
    }
    for (int i = 0; i < n; ++i) {
      z[i] /= big;
      nrm += z[i] * z[i];
    }
    nrm = 1.0 / std::sqrt(nrm);
    for (int i = 0; i < n; ++i) z[i] *= nrm;
  }
  // Sign convention: largest-magnitude component positive.
  int imax = 0;
  for (int i = 1; i < n; ++i)
    if (std::fabs(z[i]) > std::fabs(z[imax])) imax = i;
  if (z[imax] < 0)
    for (int i = 0; i < n; ++i) z[i] = -z[i];
}

}  // namespace dg
