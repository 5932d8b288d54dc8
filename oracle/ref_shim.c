/* Naive CBLAS loops written for this project, linked into oracle/_ref so the
 * reference's numerics sources run without a system BLAS.  Test
 * infrastructure only.  dnrm2 is a plain sum of squares followed by sqrt
 * (reference BLAS scales to avoid overflow; the results differ only in the
 * last ulps).  The CPU restatement in fc3d_oracle.c uses the same loop, so
 * the two agree bit for bit. */
#include <math.h>
#include <stddef.h>
#include "cblas.h"

double cblas_dnrm2(const blasint n, const double *x, const blasint incx) {
  double s = 0.0;
  for (blasint i = 0; i < n; i++) s += x[(size_t)i * incx] * x[(size_t)i * incx];
  return sqrt(s);
}
double cblas_ddot(const blasint n, const double *x, const blasint incx, const double *y, const blasint incy) {
  double s = 0.0;
  for (blasint i = 0; i < n; i++) s += x[(size_t)i * incx] * y[(size_t)i * incy];
  return s;
}
void cblas_dcopy(const blasint n, const double *x, const blasint incx, double *y, const blasint incy) {
  for (blasint i = 0; i < n; i++) y[(size_t)i * incy] = x[(size_t)i * incx];
}
void cblas_daxpy(const blasint n, const double alpha, const double *x, const blasint incx, double *y,
                 const blasint incy) {
  for (blasint i = 0; i < n; i++) y[(size_t)i * incy] += alpha * x[(size_t)i * incx];
}
void cblas_dscal(const blasint n, const double alpha, double *x, const blasint incx) {
  for (blasint i = 0; i < n; i++) x[(size_t)i * incx] *= alpha;
}
size_t cblas_idamax(const blasint n, const double *x, const blasint incx) {
  size_t best = 0;
  double bv = -1.0;
  for (blasint i = 0; i < n; i++) {
    double v = fabs(x[(size_t)i * incx]);
    if (v > bv) { bv = v; best = (size_t)i; }
  }
  return best;
}
double cblas_dasum(const blasint n, const double *x, const blasint incx) {
  double s = 0.0;
  for (blasint i = 0; i < n; i++) s += fabs(x[(size_t)i * incx]);
  return s;
}
void cblas_dswap(const blasint n, double *x, const blasint incx, double *y, const blasint incy) {
  for (blasint i = 0; i < n; i++) {
    double t = x[(size_t)i * incx];
    x[(size_t)i * incx] = y[(size_t)i * incy];
    y[(size_t)i * incy] = t;
  }
}
/* element (i,j) of a matrix stored with the given order and leading dimension */
static inline double at(enum CBLAS_ORDER o, const double *a, blasint lda, blasint i, blasint j) {
  return o == CblasColMajor ? a[(size_t)j * lda + i] : a[(size_t)i * lda + j];
}
void cblas_dgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE trans, const blasint m, const blasint n,
                 const double alpha, const double *a, const blasint lda, const double *x, const blasint incx,
                 const double beta, double *y, const blasint incy) {
  int tr = (trans != CblasNoTrans);
  blasint ny = tr ? n : m, nx = tr ? m : n;
  for (blasint i = 0; i < ny; i++) {
    double s = 0.0;
    for (blasint k = 0; k < nx; k++) s += (tr ? at(order, a, lda, k, i) : at(order, a, lda, i, k)) * x[(size_t)k * incx];
    y[(size_t)i * incy] = (beta == 0.0 ? 0.0 : beta * y[(size_t)i * incy]) + alpha * s;
  }
}
void cblas_dgemm(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TransA, const enum CBLAS_TRANSPOSE TransB,
                 const blasint M, const blasint N, const blasint K, const double alpha, const double *A,
                 const blasint lda, const double *B, const blasint ldb, const double beta, double *C,
                 const blasint ldc) {
  for (blasint i = 0; i < M; i++)
    for (blasint j = 0; j < N; j++) {
      double s = 0.0;
      for (blasint k = 0; k < K; k++) {
        double av = TransA == CblasNoTrans ? at(Order, A, lda, i, k) : at(Order, A, lda, k, i);
        double bv = TransB == CblasNoTrans ? at(Order, B, ldb, k, j) : at(Order, B, ldb, j, k);
        s += av * bv;
      }
      double *c = Order == CblasColMajor ? &C[(size_t)j * ldc + i] : &C[(size_t)i * ldc + j];
      *c = (beta == 0.0 ? 0.0 : beta * *c) + alpha * s;
    }
}
void cblas_dger(const enum CBLAS_ORDER order, const blasint M, const blasint N, const double alpha, const double *X,
                const blasint incX, const double *Y, const blasint incY, double *A, const blasint lda) {
  for (blasint i = 0; i < M; i++)
    for (blasint j = 0; j < N; j++) {
      double *c = order == CblasColMajor ? &A[(size_t)j * lda + i] : &A[(size_t)i * lda + j];
      *c += alpha * X[(size_t)i * incX] * Y[(size_t)j * incY];
    }
}
void cblas_dtrsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
                 const enum CBLAS_DIAG Diag, const blasint N, const double *A, const blasint lda, double *X,
                 const blasint incX) {
  int upper = (Uplo == CblasUpper) ^ (TransA != CblasNoTrans);
  for (blasint s = 0; s < N; s++) {
    blasint i = upper ? N - 1 - s : s;
    double v = X[(size_t)i * incX];
    for (blasint k = 0; k < N; k++) {
      if ((upper && k > i) || (!upper && k < i)) {
        double a = TransA == CblasNoTrans ? at(order, A, lda, i, k) : at(order, A, lda, k, i);
        v -= a * X[(size_t)k * incX];
      }
    }
    if (Diag == CblasNonUnit) v /= (TransA == CblasNoTrans ? at(order, A, lda, i, i) : at(order, A, lda, i, i));
    X[(size_t)i * incX] = v;
  }
}
