/* TEST INFRASTRUCTURE: the CBLAS level-1 routines that the reference's
 * VECTOR class (src/rschol/linearalgebra/VECTOR_FAST.cpp) calls, declared
 * with the standard CBLAS signatures; cblas_level1.c defines them as plain
 * loops.  Used only to build the reference's PCG_SOLVER into a checking
 * tool under oracle/_ref/. */
#ifndef RSCHOL_REF_SHIM_CBLAS_H
#define RSCHOL_REF_SHIM_CBLAS_H
#ifdef __cplusplus
extern "C" {
#endif
double cblas_ddot(int n, const double *x, int incx, const double *y, int incy);
float cblas_sdot(int n, const float *x, int incx, const float *y, int incy);
void cblas_dscal(int n, double alpha, double *x, int incx);
void cblas_sscal(int n, float alpha, float *x, int incx);
void cblas_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy);
void cblas_saxpy(int n, float alpha, const float *x, int incx, float *y, int incy);
double cblas_dnrm2(int n, const double *x, int incx);
float cblas_snrm2(int n, const float *x, int incx);
double cblas_dasum(int n, const double *x, int incx);
float cblas_sasum(int n, const float *x, int incx);
#ifdef __cplusplus
}
#endif
#endif
