/*
 * Oracle-only compatibility header (test infrastructure, never shipped).
 *
 * Lets the reference HCORE sources compile, unmodified, against the OpenBLAS
 * that SciPy bundles (every symbol carries a "scipy_" prefix there).  Only the
 * CBLAS names the reference's kernels and tests use are mapped.  Enum values
 * follow the CBLAS standard, which the reference relies on
 * (src/include/hcore.h:30-44 uses the same numbers).
 */
#ifndef ORACLE_COMPAT_CBLAS_H
#define ORACLE_COMPAT_CBLAS_H
#include <stddef.h>
#include <stdlib.h>
#include <stdint.h>

enum CBLAS_ORDER     { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO      { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG      { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE      { CblasLeft = 141, CblasRight = 142 };
typedef enum CBLAS_TRANSPOSE CBLAS_TRANSPOSE;

#define ORACLE_CB(name) scipy_cblas_##name
#define cblas_dgemm ORACLE_CB(dgemm)
#define cblas_sgemm ORACLE_CB(sgemm)
#define cblas_dcopy ORACLE_CB(dcopy)
#define cblas_scopy ORACLE_CB(scopy)
#define cblas_dscal ORACLE_CB(dscal)
#define cblas_sscal ORACLE_CB(sscal)
#define cblas_dtrmm ORACLE_CB(dtrmm)
#define cblas_strmm ORACLE_CB(strmm)
#define cblas_dtrsm ORACLE_CB(dtrsm)
#define cblas_strsm ORACLE_CB(strsm)
#define cblas_dsyrk ORACLE_CB(dsyrk)
#define cblas_dgemv ORACLE_CB(dgemv)
#define cblas_dnrm2 ORACLE_CB(dnrm2)

void cblas_dgemm(int order, int ta, int tb, int m, int n, int k, double alpha,
                 const double *a, int lda, const double *b, int ldb,
                 double beta, double *c, int ldc);
void cblas_sgemm(int order, int ta, int tb, int m, int n, int k, float alpha,
                 const float *a, int lda, const float *b, int ldb,
                 float beta, float *c, int ldc);
void cblas_dcopy(int n, const double *x, int incx, double *y, int incy);
void cblas_scopy(int n, const float *x, int incx, float *y, int incy);
void cblas_dscal(int n, double alpha, double *x, int incx);
void cblas_sscal(int n, float alpha, float *x, int incx);
void cblas_dtrmm(int order, int side, int uplo, int ta, int diag, int m, int n,
                 double alpha, const double *a, int lda, double *b, int ldb);
void cblas_strmm(int order, int side, int uplo, int ta, int diag, int m, int n,
                 float alpha, const float *a, int lda, float *b, int ldb);
void cblas_dtrsm(int order, int side, int uplo, int ta, int diag, int m, int n,
                 double alpha, const double *a, int lda, double *b, int ldb);
void cblas_strsm(int order, int side, int uplo, int ta, int diag, int m, int n,
                 float alpha, const float *a, int lda, float *b, int ldb);
void cblas_dsyrk(int order, int uplo, int trans, int n, int k, double alpha,
                 const double *a, int lda, double beta, double *c, int ldc);
void cblas_dgemv(int order, int ta, int m, int n, double alpha, const double *a,
                 int lda, const double *x, int incx, double beta, double *y, int incy);
double cblas_dnrm2(int n, const double *x, int incx);

/* complex (hcore_zgemm.c): scalars by address, as CBLAS specifies */
#define cblas_zgemm ORACLE_CB(zgemm)
#define cblas_zcopy ORACLE_CB(zcopy)
#define cblas_zscal ORACLE_CB(zscal)
#define cblas_ztrmm ORACLE_CB(ztrmm)
void cblas_zgemm(int order, int ta, int tb, int m, int n, int k, const void *alpha,
                 const void *a, int lda, const void *b, int ldb, const void *beta, void *c,
                 int ldc);
void cblas_zcopy(int n, const void *x, int incx, void *y, int incy);
void cblas_zscal(int n, const void *alpha, void *x, int incx);
void cblas_ztrmm(int order, int side, int uplo, int ta, int diag, int m, int n,
                 const void *alpha, const void *a, int lda, void *b, int ldb);
#endif
