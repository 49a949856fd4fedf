// tridiag.h -- lowest eigenpair of a symmetric tridiagonal matrix (host side).
#pragma once

#include <limits>

namespace dg {

// Lowest eigenvalue of T = tridiag(e, d, e) of order n (d[0..n-1], e[0..n-2]).
// upper_hint, when finite, is a value known to be >= the lowest eigenvalue (for a growing
// Lanczos matrix: the previous step's lowest Ritz value); it only narrows the bracket.
double tridiag_lowest_eigenvalue(const double *d, const double *e, int n,
                                 double upper_hint = std::numeric_limits<double>::infinity());

// Unit eigenvector of T for the eigenvalue lambda, written to z[0..n-1]; the component of
// largest magnitude is made positive.
void tridiag_eigenvector(const double *d, const double *e, int n, double lambda, double *z);

}  // namespace dg
