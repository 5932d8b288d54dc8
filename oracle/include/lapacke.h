/* Minimal stand-in written for this project: the reference's LAPACK wrapper
 * headers name lapack_int and the LAPACKE_* entry points; none of them is
 * reached on the SBM NSGS path, and the oracle build turns each into an
 * aborting stub. */
#ifndef ORACLE_STUB_LAPACKE_H
#define ORACLE_STUB_LAPACKE_H
#ifndef lapack_int
#define lapack_int int
#endif
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
#endif
