/* Minimal stand-in for the CBLAS declarations the reference's lll.c uses
 * (plain loops in refshim.c; oracle test infrastructure). */
#ifndef QG_REFSHIM_CBLAS_H
#define QG_REFSHIM_CBLAS_H
void cblas_daxpy(const int n, const double alpha, const double *x, const int incx, double *y, const int incy);
double cblas_ddot(const int n, const double *x, const int incx, const double *y, const int incy);
void cblas_dswap(const int n, double *x, const int incx, double *y, const int incy);
#endif
