/* Minimal CBLAS declarations written for this project.  The matching
 * definitions are the naive loops in oracle/ref_shim.c; only the level-1/2/3
 * names the reference's numerics sources call are declared. */
#ifndef ORACLE_STUB_CBLAS_H
#define ORACLE_STUB_CBLAS_H
#include "openblas_config.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_ORDER;
typedef enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113, CblasConjNoTrans = 114 } CBLAS_TRANSPOSE;
typedef enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;
typedef CBLAS_ORDER CBLAS_LAYOUT;
double cblas_dnrm2(const blasint n, const double *x, const blasint incx);
double cblas_ddot(const blasint n, const double *x, const blasint incx, const double *y, const blasint incy);
void cblas_dcopy(const blasint n, const double *x, const blasint incx, double *y, const blasint incy);
void cblas_daxpy(const blasint n, const double alpha, const double *x, const blasint incx, double *y, const blasint incy);
void cblas_dscal(const blasint n, const double alpha, double *x, const blasint incx);
size_t cblas_idamax(const blasint n, const double *x, const blasint incx);
double cblas_dasum(const blasint n, const double *x, const blasint incx);
void cblas_dswap(const blasint n, double *x, const blasint incx, double *y, const blasint incy);
void cblas_dgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE trans, const blasint m, const blasint n,
                 const double alpha, const double *a, const blasint lda, const double *x, const blasint incx,
                 const double beta, double *y, const blasint incy);
void cblas_dgemm(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TransA, const enum CBLAS_TRANSPOSE TransB,
                 const blasint M, const blasint N, const blasint K, const double alpha, const double *A,
                 const blasint lda, const double *B, const blasint ldb, const double beta, double *C, const blasint ldc);
void cblas_dger(const enum CBLAS_ORDER order, const blasint M, const blasint N, const double alpha, const double *X,
                const blasint incX, const double *Y, const blasint incY, double *A, const blasint lda);
void cblas_dtrsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
                 const enum CBLAS_DIAG Diag, const blasint N, const double *A, const blasint lda, double *X,
                 const blasint incX);
#ifdef __cplusplus
}
#endif
#endif
