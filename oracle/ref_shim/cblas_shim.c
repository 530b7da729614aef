/* Test-infrastructure shim: forwards the CBLAS names to scipy's OpenBLAS. */
#include "cblas.h"

double scipy_cblas_dnrm2(int n, const double *x, int incx);
double scipy_cblas_ddot(int n, const double *x, int incx, const double *y, int incy);
void scipy_cblas_dgemv(CBLAS_ORDER, CBLAS_TRANSPOSE, int, int, double, const double *, int,
                       const double *, int, double, double *, int);
void scipy_cblas_dgemm(CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int, int, int, double,
                       const double *, int, const double *, int, double, double *, int);
void scipy_cblas_dtrsm(CBLAS_ORDER, CBLAS_SIDE, CBLAS_UPLO, CBLAS_TRANSPOSE, CBLAS_DIAG, int,
                       int, double, const double *, int, double *, int);
void scipy_openblas_set_num_threads(int);

double cblas_dnrm2(int n, const double *x, int incx) { return scipy_cblas_dnrm2(n, x, incx); }
double cblas_ddot(int n, const double *x, int incx, const double *y, int incy)
{ return scipy_cblas_ddot(n, x, incx, y, incy); }
void cblas_dgemv(CBLAS_ORDER o, CBLAS_TRANSPOSE t, int m, int n, double al, const double *a,
                 int lda, const double *x, int incx, double be, double *y, int incy)
{ scipy_cblas_dgemv(o, t, m, n, al, a, lda, x, incx, be, y, incy); }
void cblas_dgemm(CBLAS_ORDER o, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n, int k,
                 double al, const double *a, int lda, const double *b, int ldb, double be,
                 double *c, int ldc)
{ scipy_cblas_dgemm(o, ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc); }
void cblas_dtrsm(CBLAS_ORDER o, CBLAS_SIDE s, CBLAS_UPLO u, CBLAS_TRANSPOSE t, CBLAS_DIAG d,
                 int m, int n, double al, const double *a, int lda, double *b, int ldb)
{ scipy_cblas_dtrsm(o, s, u, t, d, m, n, al, a, lda, b, ldb); }
void openblas_set_num_threads(int n) { scipy_openblas_set_num_threads(n); }
