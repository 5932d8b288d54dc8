/* Minimal stand-in written for this project: the reference's LAPACK wrapper
 * headers name lapack_int and the LAPACKE_* entry points.  dgetrf and dgetrs
 * (the dense LU of NM_LU_solve, reached by the global FC3D NSGS) are
 * implemented in oracle/ref_shim.c; every other one is off the paths the
 * oracle runs, and the oracle build turns each into an aborting stub. */
#ifndef ORACLE_STUB_LAPACKE_H
#define ORACLE_STUB_LAPACKE_H
#ifndef lapack_int
#define lapack_int int
#endif
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
lapack_int LAPACKE_dgetrf(int layout, lapack_int m, lapack_int n, double *a, lapack_int lda, lapack_int *ipiv);
lapack_int LAPACKE_dgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const double *a, lapack_int lda,
                          const lapack_int *ipiv, double *b, lapack_int ldb);
#endif
