/* TEST INFRASTRUCTURE: plain-loop CBLAS level-1 routines (dot, scal,
 * axpy, nrm2, asum; double precision) for building the reference's
 * PCG_SOLVER / VECTOR code into a checking tool.  Sums run in index order;
 * nrm2 is the square root of the sum of squares (no scaling: the checked
 * vectors are far from overflow). */
#include <math.h>

double cblas_ddot(int n, const double *x, int incx, const double *y, int incy) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += x[(long)i * incx] * y[(long)i * incy];
  return s;
}

void cblas_dscal(int n, double alpha, double *x, int incx) {
  for (int i = 0; i < n; ++i) x[(long)i * incx] *= alpha;
}

void cblas_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy) {
  for (int i = 0; i < n; ++i) y[(long)i * incy] += alpha * x[(long)i * incx];
}

double cblas_dnrm2(int n, const double *x, int incx) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += x[(long)i * incx] * x[(long)i * incx];
  return sqrt(s);
}

double cblas_dasum(int n, const double *x, int incx) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += fabs(x[(long)i * incx]);
  return s;
}
