/* Minimal stand-in for the CXSparse header, written for this project so the
 * reference's numerics sources compile without SuiteSparse.  Only the type
 * names and the struct shape that the reference's headers name are given
 * (CSparseMatrix.h:52-64 describes them); no CXSparse routine is provided,
 * and none is reached on the SBM NSGS path. */
#ifndef ORACLE_STUB_CS_H
#define ORACLE_STUB_CS_H
#include <stddef.h>
#include <stdint.h>
#include <limits.h>
#define CS_INT int64_t
#define CS_INT_MAX INT64_MAX
#define CS_ENTRY double
#define CS_NAME(nm) cs_dl##nm
#define CS_ID "%ld"
typedef int64_t cs_long_t;
typedef struct cs_dl_sparse {
  int64_t nzmax;
  int64_t m;
  int64_t n;
  int64_t *p;
  int64_t *i;
  double *x;
  int64_t nz;
} cs_dl;
typedef struct cs_dl_symbolic {
  int64_t *pinv, *q, *parent, *cp, *leftmost;
  int64_t m2;
  double lnz, unz;
} cs_dls;
typedef struct cs_dl_numeric {
  cs_dl *L, *U;
  int64_t *pinv;
  double *B;
} cs_dln;
typedef struct cs_dl_dmperm_results {
  int64_t *p, *q, *r, *s;
  int64_t nb;
  int64_t rr[5], cc[5];
} cs_dld;
/* CS_LONG short names */
typedef cs_dl cs;
typedef cs_dls css;
typedef cs_dln csn;
typedef cs_dld csd;
typedef int64_t csi;
#define CS_CSC(A) (A && (A->nz == -1))
#define CS_TRIPLET(A) (A && (A->nz >= 0))
#define CS_MAX(a, b) (((a) > (b)) ? (a) : (b))
#define CS_MIN(a, b) (((a) < (b)) ? (a) : (b))
#define CS_FLIP(i) (-(i)-2)
#define CS_UNFLIP(i) (((i) < 0) ? CS_FLIP(i) : (i))
#define CS_MARKED(w, j) (w[j] < 0)
#define CS_MARK(w, j) { w[j] = CS_FLIP(w[j]); }
#define CS_VER 3
#define CS_SUBVER 2
#define CS_SUBSUB 0
#define CS_DATE "stub"
#define CS_COPYRIGHT "stub"
#ifdef __cplusplus
extern "C" {
#endif
cs_dl *cs_dl_spalloc(int64_t m, int64_t n, int64_t nzmax, int64_t values, int64_t triplet);
cs_dl *cs_dl_spfree(cs_dl *A);
int64_t cs_dl_sprealloc(cs_dl *A, int64_t nzmax);
int64_t cs_dl_entry(cs_dl *T, int64_t i, int64_t j, double x);
cs_dl *cs_dl_compress(const cs_dl *T);
cs_dl *cs_dl_transpose(const cs_dl *A, int64_t values);
cs_dl *cs_dl_multiply(const cs_dl *A, const cs_dl *B);
cs_dl *cs_dl_add(const cs_dl *A, const cs_dl *B, double alpha, double beta);
int64_t cs_dl_gaxpy(const cs_dl *A, const double *x, double *y);
int64_t cs_dl_print(const cs_dl *A, int64_t brief);
int64_t cs_dl_dupl(cs_dl *A);
int64_t cs_dl_fkeep(cs_dl *A, int64_t (*fkeep)(int64_t, int64_t, double, void *), void *other);
int64_t cs_dl_droptol(cs_dl *A, double tol);
int64_t cs_dl_dropzeros(cs_dl *A);
double cs_dl_norm(const cs_dl *A);
void *cs_dl_malloc(int64_t n, size_t size);
void *cs_dl_calloc(int64_t n, size_t size);
void *cs_dl_realloc(void *p, int64_t n, size_t size, int64_t *ok);
void *cs_dl_free(void *p);
cs_dls *cs_dl_sqr(int64_t order, const cs_dl *A, int64_t qr);
cs_dln *cs_dl_lu(const cs_dl *A, const cs_dls *S, double tol);
cs_dln *cs_dl_chol(const cs_dl *A, const cs_dls *S);
cs_dln *cs_dl_qr(const cs_dl *A, const cs_dls *S);
cs_dls *cs_dl_sfree(cs_dls *S);
cs_dln *cs_dl_nfree(cs_dln *N);
cs_dld *cs_dl_dfree(cs_dld *D);
int64_t cs_dl_lsolve(const cs_dl *L, double *x);
int64_t cs_dl_usolve(const cs_dl *U, double *x);
int64_t cs_dl_ltsolve(const cs_dl *L, double *x);
int64_t cs_dl_utsolve(const cs_dl *U, double *x);
int64_t cs_dl_ipvec(const int64_t *p, const double *b, double *x, int64_t n);
int64_t cs_dl_pvec(const int64_t *p, const double *b, double *x, int64_t n);
int64_t cs_dl_lusol(int64_t order, const cs_dl *A, double *b, double tol);
int64_t cs_dl_cholsol(int64_t order, const cs_dl *A, double *b);
int64_t cs_dl_qrsol(int64_t order, const cs_dl *A, double *b);
int64_t *cs_dl_pinv(int64_t const *p, int64_t n);
cs_dl *cs_dl_permute(const cs_dl *A, const int64_t *pinv, const int64_t *q, int64_t values);
cs_dl *cs_dl_symperm(const cs_dl *A, const int64_t *pinv, int64_t values);
int64_t *cs_dl_amd(int64_t order, const cs_dl *A);
cs_dl *cs_dl_done(cs_dl *C, void *w, void *x, int64_t ok);
int64_t cs_dl_scatter(const cs_dl *A, int64_t j, double beta, int64_t *w, double *x, int64_t mark, cs_dl *C, int64_t nz);
double cs_dl_cumsum(int64_t *p, int64_t *c, int64_t n);
#ifdef __cplusplus
}
#endif
#endif
