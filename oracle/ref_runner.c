/* Array-in/array-out wrappers around the reference's own numerics entry
 * points, compiled into oracle/_ref by oracle/build_ref.py.  Test
 * infrastructure only: these let Python tests and the golden-fixture script
 * run the unmodified reference fc3d_driver (SICONOS_FRICTION_3D_NSGS,
 * fc3d_nsgs.c:560) and fc3d_compute_error (fc3d_compute_error.c:70) on
 * problems given as block-CSR arrays, and read the reference's .dat
 * fixtures with its own reader (FrictionContactProblem.c:103).  The global
 * problem (gfc3d_driver, SICONOS_GLOBAL_FRICTION_3D_NSGS, gfc3d_nsgs.c:62)
 * runs on dense M and H. */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "FrictionContactProblem.h"
#include "FrictionContact_options.h"
#include "NonSmoothDrivers.h"
#include "NumericsMatrix.h"
#include "SolverOptions.h"
#include "SparseBlockMatrix.h"
#include "fc2d_Solvers.h"
#include "fc2d_compute_error.h"
#include "fc3d_Solvers.h"
#include "fc3d_compute_error.h"
#include "numerics_verbose.h"
#include "op3x3.h"
#include "op5x5.h"
#include "RollingFrictionContactProblem.h"
#include "RollingFrictionContact_options.h"
#include "rolling_fc_Solvers.h"
#include "rolling_friction_3d_compute_error.h"
#include "projectionOnCone.h"
#include "GlobalFrictionContactProblem.h"
#include "gfc3d_compute_error.h"
#include "SiconosBlas.h"

/* Build a 3x3-block SBM that points into caller-owned arrays.  blocks holds
 * nnzb column-major 3x3 blocks in row order, rowptr/colidx the block-CSR
 * structure. */
static NumericsMatrix *make_sbm_d(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                                  int d) {
  SparseBlockStructuredMatrix *m = SBM_new();
  size_t nnzb = (size_t)rowptr[nc];
  m->nbblocks = nnzb;
  m->blocknumber0 = (size_t)nc;
  m->blocknumber1 = (size_t)nc;
  m->blocksize0 = (size_t *)malloc(sizeof(size_t) * (size_t)nc);
  m->blocksize1 = (size_t *)malloc(sizeof(size_t) * (size_t)nc);
  for (int i = 0; i < nc; i++) m->blocksize0[i] = m->blocksize1[i] = (size_t)d * (size_t)(i + 1);
  m->filled1 = (size_t)nc + 1;
  m->filled2 = nnzb;
  m->index1_data = (size_t *)malloc(sizeof(size_t) * ((size_t)nc + 1));
  m->index2_data = (size_t *)malloc(sizeof(size_t) * (nnzb ? nnzb : 1));
  m->block = (double **)malloc(sizeof(double *) * (nnzb ? nnzb : 1));
  for (int i = 0; i <= nc; i++) m->index1_data[i] = (size_t)rowptr[i];
  for (size_t k = 0; k < nnzb; k++) {
    m->index2_data[k] = (size_t)colidx[k];
    m->block[k] = (double *)&blocks[(size_t)(d * d) * k];
  }
  return NM_create_from_data(NM_SPARSE_BLOCK, d * nc, d * nc, m);
}

static NumericsMatrix *make_sbm(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks) {
  return make_sbm_d(nc, rowptr, colidx, blocks, 3);
}

static void free_sbm(NumericsMatrix *M) {
  SparseBlockStructuredMatrix *m = M->matrix1;
  free(m->blocksize0);
  free(m->blocksize1);
  free(m->index1_data);
  free(m->index2_data);
  free(m->block);
  free(m->diagonal_blocks);
  free(m);
  M->matrix1 = NULL;
  if (M->internalData) {
    free(M->internalData->iWork);
    free(M->internalData->dWork);
    free(M->internalData);
  }
  free(M);
}

typedef struct {
  double *buf;
  int cap;
  int len;
} Trace;

static void trace_cb(void *env, size_t size, double *reaction, double *velocity, double error, void *extra) {
  (void)size;
  (void)reaction;
  (void)velocity;
  (void)extra;
  Trace *t = (Trace *)env;
  if (t->len < t->cap) t->buf[t->len] = error;
  t->len++;
}

/* Run the reference's fc3d_driver with SICONOS_FRICTION_3D_NSGS default
 * options (solver_options_create) and the given tolerance and iteration
 * cap.  r holds the warm start on entry.  trace (optional) receives the
 * per-iteration error the reference reports through its callback. */
int ref_fc3d_nsgs(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks, const double *q,
                  const double *mu, double *r, double *u, double tol, int maxiter, int *iters, double *err,
                  double *trace, int trace_cap, int *trace_len) {
  NumericsMatrix *M = make_sbm(nc, rowptr, colidx, blocks);
  FrictionContactProblem P;
  memset(&P, 0, sizeof(P));
  P.dimension = 3;
  P.numberOfContacts = nc;
  P.M = M;
  P.q = (double *)q;
  P.mu = (double *)mu;
  SolverOptions *opt = solver_options_create(SICONOS_FRICTION_3D_NSGS);
  opt->iparam[SICONOS_IPARAM_MAX_ITER] = maxiter;
  opt->dparam[SICONOS_DPARAM_TOL] = tol;
  Trace t = {trace, trace_cap, 0};
  Callback cb = {&t, trace_cb};
  if (trace) opt->callback = &cb;
  int info = fc3d_driver(&P, r, u, opt);
  if (iters) *iters = opt->iparam[SICONOS_IPARAM_ITER_DONE];
  if (err) *err = opt->dparam[SICONOS_DPARAM_RESIDU];
  if (trace_len) *trace_len = t.len;
  opt->callback = NULL;
  solver_options_delete(opt);
  free_sbm(M);
  return info;
}

/* ref_fc3d_nsgs with NSGS options beyond the defaults: opts6 = {error
 * evaluation (iparam 13), its frequency (iparam 14), local tolerance
 * strategy (iparam 2), relaxation (iparam 10), filter (iparam 16), freezing
 * (iparam 15)},
 * dopts2 = {INTERNAL_ERROR_RATIO (dparam 11), RELAXATION_VALUE (dparam 10)}. */
int ref_fc3d_nsgs_opts(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks, const double *q,
                       const double *mu, double *r, double *u, double tol, int maxiter, const int32_t *opts6,
                       const double *dopts2, int *iters, double *err, double *trace, int trace_cap,
                       int *trace_len) {
  NumericsMatrix *M = make_sbm(nc, rowptr, colidx, blocks);
  FrictionContactProblem P;
  memset(&P, 0, sizeof(P));
  P.dimension = 3;
  P.numberOfContacts = nc;
  P.M = M;
  P.q = (double *)q;
  P.mu = (double *)mu;
  SolverOptions *opt = solver_options_create(SICONOS_FRICTION_3D_NSGS);
  opt->iparam[SICONOS_IPARAM_MAX_ITER] = maxiter;
  opt->dparam[SICONOS_DPARAM_TOL] = tol;
  opt->iparam[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION] = opts6[0];
  opt->iparam[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION_FREQUENCY] = opts6[1];
  opt->iparam[SICONOS_FRICTION_3D_IPARAM_INTERNAL_ERROR_STRATEGY] = opts6[2];
  opt->iparam[SICONOS_FRICTION_3D_NSGS_RELAXATION] = opts6[3];
  opt->iparam[SICONOS_FRICTION_3D_NSGS_FILTER_LOCAL_SOLUTION] = opts6[4];
  opt->iparam[SICONOS_FRICTION_3D_NSGS_FREEZING_CONTACT] = opts6[5];
  opt->dparam[SICONOS_FRICTION_3D_DPARAM_INTERNAL_ERROR_RATIO] = dopts2[0];
  opt->dparam[SICONOS_FRICTION_3D_NSGS_RELAXATION_VALUE] = dopts2[1];
  Trace t = {trace, trace_cap, 0};
  Callback cb = {&t, trace_cb};
  if (trace) opt->callback = &cb;
  int info = fc3d_driver(&P, r, u, opt);
  if (iters) *iters = opt->iparam[SICONOS_IPARAM_ITER_DONE];
  if (err) *err = opt->dparam[SICONOS_DPARAM_RESIDU];
  if (trace_len) *trace_len = t.len;
  opt->callback = NULL;
  solver_options_delete(opt);
  free_sbm(M);
  return info;
}

/* The reference's 2D NSGS (fc2d_driver with SICONOS_FRICTION_2D_NSGS and its
 * defaults, tolerance and iteration budget set) on a block-CSR W of 2x2
 * blocks. */
int ref_fc2d_nsgs(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks, const double *q,
                  const double *mu, double *r, double *u, double tol, int maxiter, int *iters, double *err) {
  NumericsMatrix *M = make_sbm_d(nc, rowptr, colidx, blocks, 2);
  FrictionContactProblem P;
  memset(&P, 0, sizeof(P));
  P.dimension = 2;
  P.numberOfContacts = nc;
  P.M = M;
  P.q = (double *)q;
  P.mu = (double *)mu;
  SolverOptions *opt = solver_options_create(SICONOS_FRICTION_2D_NSGS);
  opt->iparam[SICONOS_IPARAM_MAX_ITER] = maxiter;
  opt->dparam[SICONOS_DPARAM_TOL] = tol;
  int info = fc2d_driver(&P, r, u, opt);
  if (iters) *iters = opt->iparam[SICONOS_IPARAM_ITER_DONE];
  if (err) *err = opt->dparam[SICONOS_DPARAM_RESIDU];
  solver_options_delete(opt);
  free_sbm(M);
  return info;
}

/* The reference's fc2d_compute_error on the given r; u receives q + W r. */
double ref_fc2d_compute_error(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                              const double *q, const double *mu, const double *r, double *u) {
  NumericsMatrix *M = make_sbm_d(nc, rowptr, colidx, blocks, 2);
  FrictionContactProblem P;
  memset(&P, 0, sizeof(P));
  P.dimension = 2;
  P.numberOfContacts = nc;
  P.M = M;
  P.q = (double *)q;
  P.mu = (double *)mu;
  double norm_q = cblas_dnrm2(2 * nc, q, 1);
  double e = 0.0;
  fc2d_compute_error(&P, (double *)r, u, 1e-300, norm_q, &e);
  free_sbm(M);
  return e;
}

/* The reference's fc3d_compute_error on the given r; u receives q + W r. */
double ref_fc3d_compute_error(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                              const double *q, const double *mu, const double *r, double *u) {
  NumericsMatrix *M = make_sbm(nc, rowptr, colidx, blocks);
  FrictionContactProblem P;
  memset(&P, 0, sizeof(P));
  P.dimension = 3;
  P.numberOfContacts = nc;
  P.M = M;
  P.q = (double *)q;
  P.mu = (double *)mu;
  double norm_q = cblas_dnrm2(3 * nc, q, 1);
  double e = 0.0;
  fc3d_compute_error(&P, (double *)r, u, 1e-300, NULL, norm_q, &e);
  free_sbm(M);
  return e;
}

/* .dat fixtures through the reference's own reader. */
typedef struct {
  FrictionContactProblem *P;
} DatHandle;

void *ref_dat_open(const char *fname, int *nc, int64_t *nnzb, int *storage, int *dim) {
  FrictionContactProblem *P = frictionContact_new_from_filename(fname);
  if (!P) return NULL;
  DatHandle *h = (DatHandle *)malloc(sizeof(DatHandle));
  h->P = P;
  *nc = P->numberOfContacts;
  *dim = P->dimension;
  *storage = (int)P->M->storageType;
  if (P->M->storageType == NM_SPARSE_BLOCK)
    *nnzb = (int64_t)P->M->matrix1->nbblocks;
  else if (P->M->storageType == NM_DENSE) {
    /* dense: every d x d block with a nonzero entry becomes a block */
    int n = P->numberOfContacts, d = P->dimension;
    int64_t cnt = 0;
    for (int bi = 0; bi < n; bi++)
      for (int bj = 0; bj < n; bj++) {
        int nz = (bi == bj);
        for (int a = 0; a < d && !nz; a++)
          for (int b = 0; b < d && !nz; b++)
            nz = P->M->matrix0[(size_t)(d * bj + b) * (size_t)(d * n) + (size_t)(d * bi + a)] != 0.0;
        cnt += nz;
      }
    *nnzb = cnt;
  } else
    *nnzb = -1;
  return h;
}

int ref_dat_get(void *hv, int64_t *rowptr, int64_t *colidx, double *blocks, double *q, double *mu) {
  DatHandle *h = (DatHandle *)hv;
  FrictionContactProblem *P = h->P;
  int n = P->numberOfContacts, d = P->dimension;
  memcpy(q, P->q, sizeof(double) * (size_t)d * (size_t)n);
  memcpy(mu, P->mu, sizeof(double) * (size_t)n);
  if (P->M->storageType == NM_SPARSE_BLOCK) {
    SparseBlockStructuredMatrix *m = P->M->matrix1;
    if (m->filled1 != (size_t)n + 1) {
      /* trailing empty rows: pad the row pointer */
      for (int i = 0; i <= n; i++) rowptr[i] = (int64_t)(i < (int)m->filled1 ? m->index1_data[i] : m->index1_data[m->filled1 - 1]);
    } else
      for (int i = 0; i <= n; i++) rowptr[i] = (int64_t)m->index1_data[i];
    for (size_t k = 0; k < m->nbblocks; k++) {
      colidx[k] = (int64_t)m->index2_data[k];
      memcpy(&blocks[(size_t)(d * d) * k], m->block[k], (size_t)(d * d) * sizeof(double));
    }
    return 0;
  }
  if (P->M->storageType == NM_DENSE) {
    int64_t k = 0;
    const double *A = P->M->matrix0;
    for (int bi = 0; bi < n; bi++) {
      rowptr[bi] = k;
      for (int bj = 0; bj < n; bj++) {
        int nz = (bi == bj);
        for (int a = 0; a < d && !nz; a++)
          for (int b = 0; b < d && !nz; b++) nz = A[(size_t)(d * bj + b) * (size_t)(d * n) + (size_t)(d * bi + a)] != 0.0;
        if (!nz) continue;
        colidx[k] = bj;
        for (int b = 0; b < d; b++)
          for (int a = 0; a < d; a++)
            blocks[(int64_t)(d * d) * k + d * b + a] = A[(size_t)(d * bj + b) * (size_t)(d * n) + (size_t)(d * bi + a)];
        k++;
      }
    }
    rowptr[n] = k;
    return 0;
  }
  return -1;
}

void ref_dat_close(void *hv) {
  DatHandle *h = (DatHandle *)hv;
  frictionContactProblem_free(h->P);
  free(h);
}

/* Write a problem with the reference's own writer (frictionContact_printInFilename):
 * W as a sparse-block matrix, or (dense != 0) as a dense one. */
int ref_dat_write(const char *fname, int dim, int nc, const int64_t *rowptr, const int64_t *colidx,
                  const double *blocks, const double *q, const double *mu, int dense) {
  const int d = dim, n = dim * nc;
  const int64_t nb = rowptr[nc];
  NumericsMatrix *M = NULL;
  if (dense) {
    M = NM_create(NM_DENSE, n, n);
    memset(M->matrix0, 0, sizeof(double) * (size_t)n * (size_t)n);
    for (int i = 0; i < nc; i++)
      for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++)
        for (int b = 0; b < d; b++)
          for (int a = 0; a < d; a++)
            M->matrix0[(size_t)(d * colidx[k] + b) * (size_t)n + (size_t)(d * i + a)] = blocks[(int64_t)(d * d) * k + d * b + a];
  } else {
    SparseBlockStructuredMatrix *m = SBM_new();
    m->nbblocks = (size_t)nb;
    m->blocknumber0 = m->blocknumber1 = (size_t)nc;
    m->blocksize0 = (size_t *)malloc(sizeof(size_t) * (size_t)nc);
    m->blocksize1 = (size_t *)malloc(sizeof(size_t) * (size_t)nc);
    for (int i = 0; i < nc; i++) m->blocksize0[i] = m->blocksize1[i] = (size_t)(d * (i + 1));
    m->filled1 = (size_t)nc + 1;
    m->filled2 = (size_t)nb;
    m->index1_data = (size_t *)malloc(sizeof(size_t) * ((size_t)nc + 1));
    m->index2_data = (size_t *)malloc(sizeof(size_t) * (size_t)nb);
    m->block = (double **)malloc(sizeof(double *) * (size_t)nb);
    for (int i = 0; i <= nc; i++) m->index1_data[i] = (size_t)rowptr[i];
    for (int64_t k = 0; k < nb; k++) {
      m->index2_data[k] = (size_t)colidx[k];
      m->block[k] = (double *)malloc((size_t)(d * d) * sizeof(double));
      memcpy(m->block[k], &blocks[(int64_t)(d * d) * k], (size_t)(d * d) * sizeof(double));
    }
    M = NM_new();
    NM_fill(M, NM_SPARSE_BLOCK, n, n, m);
  }
  double *qq = (double *)malloc(sizeof(double) * (size_t)n);
  double *mm = (double *)malloc(sizeof(double) * (size_t)nc);
  memcpy(qq, q, sizeof(double) * (size_t)n);
  memcpy(mm, mu, sizeof(double) * (size_t)nc);
  FrictionContactProblem *P = frictionContactProblem_new_with_data(d, (size_t)nc, M, qq, mm);
  int rc = frictionContact_printInFilename(P, (char *)fname);
  frictionContactProblem_free(P);
  return rc;
}

/* Exported wrappers around static inline helpers of op3x3.h and the
 * reference's cone projection, for known-answer tests. */
int ref_solve_3x3_gepp(const double *a, double *b) { return solve_3x3_gepp(a, b); }
unsigned ref_projection_on_cone(double *r, double mu) { return projectionOnCone(r, mu); }
void ref_set_verbose(int v) { numerics_set_verbose(v); }

/* ---- 3D rolling friction (dimension 5) ---------------------------------- */

/* The reference's rolling-friction NSGS extracts diagonal blocks of dense
 * or CSparse storage only (its sparse-block branch asserts,
 * NumericsMatrix.c:1870), so W goes to it as a dense column-major matrix. */
static NumericsMatrix *make_dense_d(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                                    int d) {
  const size_t n = (size_t)d * (size_t)nc;
  double *A = (double *)calloc(n * n, sizeof(double));
  for (int i = 0; i < nc; i++)
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++)
      for (int b = 0; b < d; b++)
        for (int a = 0; a < d; a++)
          A[((size_t)d * (size_t)colidx[k] + (size_t)b) * n + (size_t)d * (size_t)i + (size_t)a] =
              blocks[(size_t)(d * d) * (size_t)k + (size_t)(d * b + a)];
  return NM_create_from_data(NM_DENSE, (int)n, (int)n, A);
}

static void free_dense(NumericsMatrix *M) {
  free(M->matrix0);
  M->matrix0 = NULL;
  NM_clear(M);
  free(M);
}

/* The reference's rolling_friction_3d_driver with SICONOS_ROLLING_FRICTION_3D_NSGS
 * default options, tolerance and iteration budget set, on a block-CSR W of
 * 5x5 blocks (passed as a dense matrix).  r holds the warm start. */
int ref_rfc3d_nsgs(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks, const double *q,
                   const double *mu, const double *mur, double *r, double *u, double tol, int maxiter, int *iters,
                   double *err, double *trace, int trace_cap, int *trace_len) {
  NumericsMatrix *M = make_dense_d(nc, rowptr, colidx, blocks, 5);
  RollingFrictionContactProblem P;
  memset(&P, 0, sizeof(P));
  P.dimension = 5;
  P.numberOfContacts = nc;
  P.M = M;
  P.q = (double *)q;
  P.mu = (double *)mu;
  P.mu_r = (double *)mur;
  SolverOptions *opt = solver_options_create(SICONOS_ROLLING_FRICTION_3D_NSGS);
  opt->iparam[SICONOS_IPARAM_MAX_ITER] = maxiter;
  opt->dparam[SICONOS_DPARAM_TOL] = tol;
  Trace t = {trace, trace_cap, 0};
  Callback cb = {&t, trace_cb};
  if (trace) opt->callback = &cb;
  int info = rolling_friction_3d_driver(&P, r, u, opt);
  if (iters) *iters = opt->iparam[SICONOS_IPARAM_ITER_DONE];
  if (err) *err = opt->dparam[SICONOS_DPARAM_RESIDU];
  if (trace_len) *trace_len = t.len;
  opt->callback = NULL;
  solver_options_delete(opt);
  free_dense(M);
  return info;
}

/* The reference's rolling_friction_3d_compute_error on r; u receives q + W r. */
double ref_rfc3d_compute_error(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                               const double *q, const double *mu, const double *mur, const double *r, double *u) {
  NumericsMatrix *M = make_dense_d(nc, rowptr, colidx, blocks, 5);
  RollingFrictionContactProblem P;
  memset(&P, 0, sizeof(P));
  P.dimension = 5;
  P.numberOfContacts = nc;
  P.M = M;
  P.q = (double *)q;
  P.mu = (double *)mu;
  P.mu_r = (double *)mur;
  double norm_q = cblas_dnrm2(5 * nc, q, 1);
  double e = 0.0;
  rolling_friction_3d_compute_error(&P, (double *)r, u, 1e-300, NULL, norm_q, &e);
  free_dense(M);
  return e;
}

/* Largest eigenvalue by the reference's 5x5 symmetric eigenvalue routine. */
double ref_rfc3d_max_eig(const double *a) {
  double ev[5];
  eigvals_sym5x5_for_loop(a, ev);
  return ev[4];
}

/* A rolling-friction problem read by the reference's reader
 * (rollingFrictionContact_new_from_filename), W given back as block-CSR of
 * 5x5 blocks: sparse-block storage as stored, dense storage as every block
 * holding a nonzero entry plus the diagonal. */
typedef struct {
  RollingFrictionContactProblem *P;
} RDatHandle;

void *ref_rfc3d_dat_open(const char *fname, int *nc, int64_t *nnzb, int *storage) {
  RollingFrictionContactProblem *P = rollingFrictionContact_new_from_filename(fname);
  if (!P) return NULL;
  if (P->dimension != 5) {
    rollingFrictionContactProblem_free(P);
    return NULL;
  }
  RDatHandle *h = (RDatHandle *)malloc(sizeof(RDatHandle));
  h->P = P;
  *nc = P->numberOfContacts;
  *storage = (int)P->M->storageType;
  const int n = P->numberOfContacts, d = 5;
  if (P->M->storageType == NM_SPARSE_BLOCK)
    *nnzb = (int64_t)P->M->matrix1->nbblocks;
  else if (P->M->storageType == NM_DENSE) {
    int64_t cnt = 0;
    for (int bi = 0; bi < n; bi++)
      for (int bj = 0; bj < n; bj++) {
        int nz = (bi == bj);
        for (int a = 0; a < d && !nz; a++)
          for (int b = 0; b < d && !nz; b++)
            nz = P->M->matrix0[(size_t)(d * bj + b) * (size_t)(d * n) + (size_t)(d * bi + a)] != 0.0;
        cnt += nz;
      }
    *nnzb = cnt;
  } else
    *nnzb = -1;
  return h;
}

int ref_rfc3d_dat_get(void *hv, int64_t *rowptr, int64_t *colidx, double *blocks, double *q, double *mu,
                      double *mur) {
  RDatHandle *h = (RDatHandle *)hv;
  RollingFrictionContactProblem *P = h->P;
  const int n = P->numberOfContacts, d = 5;
  memcpy(q, P->q, sizeof(double) * (size_t)d * (size_t)n);
  memcpy(mu, P->mu, sizeof(double) * (size_t)n);
  memcpy(mur, P->mu_r, sizeof(double) * (size_t)n);
  if (P->M->storageType == NM_SPARSE_BLOCK) {
    SparseBlockStructuredMatrix *m = P->M->matrix1;
    for (int i = 0; i <= n; i++)
      rowptr[i] = (int64_t)(i < (int)m->filled1 ? m->index1_data[i] : m->index1_data[m->filled1 - 1]);
    for (size_t k = 0; k < m->nbblocks; k++) {
      colidx[k] = (int64_t)m->index2_data[k];
      memcpy(&blocks[(size_t)(d * d) * k], m->block[k], (size_t)(d * d) * sizeof(double));
    }
    return 0;
  }
  if (P->M->storageType == NM_DENSE) {
    int64_t k = 0;
    const double *A = P->M->matrix0;
    for (int bi = 0; bi < n; bi++) {
      rowptr[bi] = k;
      for (int bj = 0; bj < n; bj++) {
        int nz = (bi == bj);
        for (int a = 0; a < d && !nz; a++)
          for (int b = 0; b < d && !nz; b++) nz = A[(size_t)(d * bj + b) * (size_t)(d * n) + (size_t)(d * bi + a)] != 0.0;
        if (!nz) continue;
        colidx[k] = bj;
        for (int b = 0; b < d; b++)
          for (int a = 0; a < d; a++)
            blocks[(size_t)(d * d) * (size_t)k + (size_t)(d * b + a)] =
                A[(size_t)(d * bj + b) * (size_t)(d * n) + (size_t)(d * bi + a)];
        k++;
      }
    }
    rowptr[n] = k;
    return 0;
  }
  return -1;
}

void ref_rfc3d_dat_close(void *hv) {
  RDatHandle *h = (RDatHandle *)hv;
  rollingFrictionContactProblem_free(h->P);
  free(h);
}


/* ---------------- global FC3D (M v = q + H r, u = H^T v + b) ---------------- */

typedef struct {
  GlobalFrictionContactProblem *P;
} GDatHandle;

/* A GFC3D .dat fixture through the reference's reader
 * (GlobalFrictionContactProblem.c:118); M and H are then read entry by entry
 * (NM_get_value), whatever their storage. */
void *ref_gfc3d_dat_open(const char *fname, int *n, int *nc, int *mstorage, int *hstorage) {
  GlobalFrictionContactProblem *P = globalFrictionContact_new_from_filename(fname);
  if (!P) return NULL;
  GDatHandle *h = (GDatHandle *)malloc(sizeof(GDatHandle));
  h->P = P;
  *n = P->M->size0;
  *nc = P->numberOfContacts;
  *mstorage = (int)P->M->storageType;
  *hstorage = (int)P->H->storageType;
  return h;
}

/* M (n x n) and H (n x 3nc) column-major, q, b, mu. */
int ref_gfc3d_dat_get(void *hv, double *M, double *H, double *q, double *b, double *mu) {
  GlobalFrictionContactProblem *P = ((GDatHandle *)hv)->P;
  const int n = P->M->size0, m = 3 * P->numberOfContacts;
  if (P->dimension != 3 || P->H->size0 != n || P->H->size1 != m) return -1;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) M[(size_t)j * n + i] = NM_get_value(P->M, i, j);
  for (int j = 0; j < m; j++)
    for (int i = 0; i < n; i++) H[(size_t)j * n + i] = NM_get_value(P->H, i, j);
  memcpy(q, P->q, sizeof(double) * (size_t)n);
  memcpy(b, P->b, sizeof(double) * (size_t)m);
  memcpy(mu, P->mu, sizeof(double) * (size_t)P->numberOfContacts);
  return 0;
}

void ref_gfc3d_dat_close(void *hv) {
  GDatHandle *h = (GDatHandle *)hv;
  globalFrictionContact_free(h->P);
  free(h);
}

static GlobalFrictionContactProblem *make_gfc3d(int n, int nc, const double *M, const double *H, const double *q,
                                                const double *b, const double *mu) {
  GlobalFrictionContactProblem *P = globalFrictionContactProblem_new();
  const int m = 3 * nc;
  P->dimension = 3;
  P->numberOfContacts = nc;
  P->M = NM_create(NM_DENSE, n, n);
  memcpy(P->M->matrix0, M, sizeof(double) * (size_t)n * (size_t)n);
  /* the dense LU factors go to a copy of M, not into M itself (by default
     NM_LU_factorize factorises in place, NumericsMatrix.c:89, :3547, and
     gfc3d_compute_error would then multiply by the packed factors) */
  NM_preserve(P->M);
  P->H = NM_create(NM_DENSE, n, m);
  memcpy(P->H->matrix0, H, sizeof(double) * (size_t)n * (size_t)(m > 0 ? m : 0));
  P->q = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  P->b = (double *)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
  P->mu = (double *)malloc(sizeof(double) * (size_t)(nc > 0 ? nc : 1));
  memcpy(P->q, q, sizeof(double) * (size_t)n);
  memcpy(P->b, b, sizeof(double) * (size_t)m);
  memcpy(P->mu, mu, sizeof(double) * (size_t)nc);
  return P;
}

/* gfc3d_driver with SICONOS_GLOBAL_FRICTION_3D_NSGS (defaults of
 * solver_options_create, then max_iter, tol and the error-evaluation
 * frequency); r, u, v in/out.  Returns info; *error = dparam[1]. */
int ref_gfc3d_nsgs(int n, int nc, const double *M, const double *H, const double *q, const double *b,
                   const double *mu, double *r, double *u, double *v, double tol, int maxiter, int freq,
                   double *error) {
  GlobalFrictionContactProblem *P = make_gfc3d(n, nc, M, H, q, b, mu);
  SolverOptions *o = solver_options_create(SICONOS_GLOBAL_FRICTION_3D_NSGS);
  o->iparam[SICONOS_IPARAM_MAX_ITER] = maxiter;
  o->dparam[SICONOS_DPARAM_TOL] = tol;
  o->iparam[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION_FREQUENCY] = freq;
  int info = gfc3d_driver(P, r, u, v, o);
  *error = o->dparam[SICONOS_DPARAM_RESIDU];
  solver_options_delete(o);
  globalFrictionContact_free(P);
  return info;
}

/* gfc3d_compute_error (gfc3d_compute_error.c:38) of (r, v); writes u. */
double ref_gfc3d_compute_error(int n, int nc, const double *M, const double *H, const double *q, const double *b,
                               const double *mu, const double *r, const double *v, double *u) {
  GlobalFrictionContactProblem *P = make_gfc3d(n, nc, M, H, q, b, mu);
  SolverOptions *o = solver_options_create(SICONOS_GLOBAL_FRICTION_3D_NSGS);
  double e = 0.0;
  const int m = 3 * nc;
  gfc3d_compute_error(P, (double *)r, u, (double *)v, 1e-300, o, cblas_dnrm2(n, P->q, 1), cblas_dnrm2(m, P->b, 1),
                      &e);
  solver_options_delete(o);
  globalFrictionContact_free(P);
  return e;
}
