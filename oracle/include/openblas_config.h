/* Minimal stand-in written for this project: the reference's safe_casts.h
 * checks sizeof(blasint) against SIZEOF_BLASINT; the project's cblas shim
 * uses 32-bit integers. */
#ifndef ORACLE_STUB_OPENBLAS_CONFIG_H
#define ORACLE_STUB_OPENBLAS_CONFIG_H
typedef int blasint;
#define SIZEOF_BLASINT 4
#endif
