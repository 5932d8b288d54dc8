/* Naive CBLAS loops written for this project, linked into oracle/_ref so the
 * reference's numerics sources run without a system BLAS.  Test
 * infrastructure only.  dnrm2 is a plain sum of squares followed by sqrt
 * (reference BLAS scales to avoid overflow; the results differ only in the
 * last ulps).  The CPU restatement in fc3d_oracle.c uses the same loop, so
 * the two agree bit for bit. */
#include <math.h>
#include <stddef.h>
#include "cblas.h"
#include "lapacke.h"

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

/* Dense LU for the reference's NM_LU_factorize / NM_LU_solve on NM_DENSE
 * matrices (NumericsMatrix.c:3543-3590, :3699-3735), column-major only:
 * unblocked right-looking elimination, first largest pivot, multipliers by
 * division; on an exactly zero pivot the column is skipped and info records
 * it.  dgetrs applies the row swaps in order, then the unit-lower forward
 * substitution (ascending columns) and the upper back substitution
 * (descending columns, then the division by the pivot).  The CPU restatement
 * in gfc3d_oracle.c factorises and solves in the same order. */
lapack_int LAPACKE_dgetrf(int layout, lapack_int m, lapack_int n, double *a, lapack_int lda, lapack_int *ipiv) {
  lapack_int info = 0;
  if (layout != LAPACK_COL_MAJOR) return -1;
  lapack_int mn = m < n ? m : n;
  for (lapack_int j = 0; j < mn; j++) {
    lapack_int p = j;
    double best = -1.0;
    for (lapack_int i = j; i < m; i++)
      if (fabs(a[(size_t)j * lda + i]) > best) {
        best = fabs(a[(size_t)j * lda + i]);
        p = i;
      }
    ipiv[j] = p + 1;
    if (a[(size_t)j * lda + p] == 0.0) {
      if (!info) info = j + 1;
      continue;
    }
    if (p != j)
      for (lapack_int k = 0; k < n; k++) {
        double t = a[(size_t)k * lda + j];
        a[(size_t)k * lda + j] = a[(size_t)k * lda + p];
        a[(size_t)k * lda + p] = t;
      }
    for (lapack_int i = j + 1; i < m; i++) a[(size_t)j * lda + i] = a[(size_t)j * lda + i] / a[(size_t)j * lda + j];
    for (lapack_int k = j + 1; k < n; k++)
      for (lapack_int i = j + 1; i < m; i++)
        a[(size_t)k * lda + i] = a[(size_t)k * lda + i] - a[(size_t)j * lda + i] * a[(size_t)k * lda + j];
  }
  return info;
}

lapack_int LAPACKE_dgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const double *a, lapack_int lda,
                          const lapack_int *ipiv, double *b, lapack_int ldb) {
  if (layout != LAPACK_COL_MAJOR || (trans != 'N' && trans != 'n')) return -1;
  for (lapack_int c = 0; c < nrhs; c++) {
    double *x = b + (size_t)c * ldb;
    for (lapack_int i = 0; i < n; i++) {
      lapack_int p = ipiv[i] - 1;
      if (p != i) {
        double t = x[i];
        x[i] = x[p];
        x[p] = t;
      }
    }
    for (lapack_int i = 0; i < n; i++) {
      double v = x[i];
      for (lapack_int k = 0; k < i; k++) v = v - a[(size_t)k * lda + i] * x[k];
      x[i] = v;
    }
    for (lapack_int i = n - 1; i >= 0; i--) {
      double v = x[i];
      for (lapack_int k = n - 1; k > i; k--) v = v - a[(size_t)k * lda + i] * x[k];
      x[i] = v / a[(size_t)i * lda + i];
    }
  }
  return 0;
}
