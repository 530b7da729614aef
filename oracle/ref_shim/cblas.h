/*
 * Test-infrastructure shim: the five CBLAS routines the reference calls
 * (dnrm2, ddot, dgemv, dgemm, dtrsm; H2P-ERI src/H2ERI_config.h:30-47),
 * forwarded to the OpenBLAS build bundled with scipy (scipy_cblas_*).
 * Only used to compile the reference sources into the oracle library.
 */
#ifndef ORACLE_CBLAS_SHIM_H
#define ORACLE_CBLAS_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_ORDER;
typedef CBLAS_ORDER CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef enum { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;

double cblas_dnrm2(int n, const double *x, int incx);
double cblas_ddot(int n, const double *x, int incx, const double *y, int incy);
void cblas_dgemv(CBLAS_ORDER order, CBLAS_TRANSPOSE trans, int m, int n, double alpha,
                 const double *a, int lda, const double *x, int incx, double beta,
                 double *y, int incy);
void cblas_dgemm(CBLAS_ORDER order, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n, int k,
                 double alpha, const double *a, int lda, const double *b, int ldb,
                 double beta, double *c, int ldc);
void cblas_dtrsm(CBLAS_ORDER order, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE ta,
                 CBLAS_DIAG diag, int m, int n, double alpha, const double *a, int lda,
                 double *b, int ldb);
void openblas_set_num_threads(int n);

#ifdef __cplusplus
}
#endif

#endif
