/* Host side of the GPU solver for the global 3D friction-contact problem, in
 * C: the registry-facing solve, init, free and set_default functions, the
 * driver's checks and no-contact case, and the conversion of the caller's
 * NumericsMatrix storage of M and H into the CSR arrays of the device
 * context (gfc3dgpu.cu).
 *
 * Reference behaviour mirrored here:
 *   gfc3d_driver checks, no-contact case   gfc3d_driver.c:77-120
 *   gfc3d_nsgs outputs (info, dparam[0..1])  gfc3d_nsgs.c:62-198
 *   gfc3d_nsgs_set_default                 gfc3d_nsgs.c:200-208
 *   registry defaults (1000, 1e-4)         gfc3d_nsgs.c:232-237 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fc3dgpu_bcsr.h"
#include "gfc3dgpu.h"

#define GFC3DGPU_CACHE_MAGIC 0x47464333u

typedef struct {
  unsigned magic;
  gfc3dgpu_ctx *ctx;
} gfc3dgpu_cache;

/* A matrix as CSR with ascending columns per row. */
typedef struct {
  int64_t rows;
  int64_t *p, *i;
  double *x;
} Csr;

static void csr_free(Csr *c) {
  free(c->p);
  free(c->i);
  free(c->x);
  memset(c, 0, sizeof(*c));
}

typedef struct {
  int64_t col;
  double val;
} Entry;

static int cmp_entry(const void *a, const void *b) {
  int64_t x = ((const Entry *)a)->col, y = ((const Entry *)b)->col;
  return (x > y) - (x < y);
}

/* Dense (column-major, the reference's matrix0) or sparse-block storage to
 * CSR.  Dense storage keeps the nonzero entries; sparse-block storage keeps
 * every entry of its stored blocks.  Returns 0 or a NUMERICS_ERR_* code. */
static int csr_of(const NumericsMatrix *A, const char *name, Csr *out) {
  memset(out, 0, sizeof(*out));
  const int64_t rows = A->size0, cols = A->size1;
  out->rows = rows;
  out->p = (int64_t *)calloc((size_t)rows + 1, sizeof(int64_t));
  if (!out->p) {
    fc3dgpu_set_error("host allocation failed");
    return NUMERICS_ERR_MEMORY;
  }
  if (A->storageType == NM_DENSE) {
    if (!A->matrix0 && rows * cols > 0) {
      fc3dgpu_set_error("%s: dense storage without data", name);
      return NUMERICS_ERR_NULL_POINTER;
    }
    int64_t nnz = 0;
    for (int64_t j = 0; j < cols; j++)
      for (int64_t r = 0; r < rows; r++)
        if (A->matrix0[j * rows + r] != 0.0) {
          out->p[r + 1]++;
          nnz++;
        }
    for (int64_t r = 0; r < rows; r++) out->p[r + 1] += out->p[r];
    out->i = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nnz ? nnz : 1));
    out->x = (double *)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(rows ? rows : 1));
    if (!out->i || !out->x || !fill) {
      free(fill);
      fc3dgpu_set_error("host allocation failed");
      return NUMERICS_ERR_MEMORY;
    }
    memcpy(fill, out->p, sizeof(int64_t) * (size_t)rows);
    for (int64_t j = 0; j < cols; j++) /* column by column: rows' entries come out ascending */
      for (int64_t r = 0; r < rows; r++) {
        const double v = A->matrix0[j * rows + r];
        if (v != 0.0) {
          out->i[fill[r]] = j;
          out->x[fill[r]++] = v;
        }
      }
    free(fill);
    return 0;
  }
  if (A->storageType != NM_SPARSE_BLOCK) {
    fc3dgpu_set_error("%s: only dense and sparse-block storage are supported (storage %d)", name,
                      (int)A->storageType);
    return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  const SparseBlockStructuredMatrix *S = A->matrix1;
  if (!S || (S->nbblocks && (!S->block || !S->index2_data)) || !S->blocksize0 || !S->blocksize1 ||
      !S->index1_data) {
    fc3dgpu_set_error("%s: sparse-block storage without data", name);
    return NUMERICS_ERR_NULL_POINTER;
  }
  if (S->blocknumber0 < 1 || S->blocknumber1 < 1 || (int64_t)S->blocksize0[S->blocknumber0 - 1] != rows ||
      (int64_t)S->blocksize1[S->blocknumber1 - 1] != cols) {
    fc3dgpu_set_error("%s: block sizes do not add up to %lld x %lld", name, (long long)rows, (long long)cols);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  const size_t nbr = S->filled1 ? S->filled1 - 1 : 0; /* block rows with a pointer entry */
  int64_t nnz = 0;
  for (size_t bi = 0; bi < nbr && bi < S->blocknumber0; bi++) {
    const int64_t r0 = bi ? (int64_t)S->blocksize0[bi - 1] : 0, r1 = (int64_t)S->blocksize0[bi];
    for (size_t k = S->index1_data[bi]; k < S->index1_data[bi + 1]; k++) {
      const size_t bj = S->index2_data[k];
      if (bj >= S->blocknumber1 || !S->block[k]) {
        fc3dgpu_set_error("%s: block %zu is out of range or has no data", name, k);
        return NUMERICS_ERR_INVALID_ARGUMENT;
      }
      const int64_t c0 = bj ? (int64_t)S->blocksize1[bj - 1] : 0, c1 = (int64_t)S->blocksize1[bj];
      for (int64_t r = r0; r < r1; r++) out->p[r + 1] += c1 - c0;
      nnz += (r1 - r0) * (c1 - c0);
    }
  }
  for (int64_t r = 0; r < rows; r++) out->p[r + 1] += out->p[r];
  out->i = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nnz ? nnz : 1));
  out->x = (double *)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
  Entry *row = (Entry *)malloc(sizeof(Entry) * (size_t)(cols ? cols : 1));
  int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(rows ? rows : 1));
  if (!out->i || !out->x || !row || !fill) {
    free(row);
    free(fill);
    fc3dgpu_set_error("host allocation failed");
    return NUMERICS_ERR_MEMORY;
  }
  memcpy(fill, out->p, sizeof(int64_t) * (size_t)rows);
  for (size_t bi = 0; bi < nbr && bi < S->blocknumber0; bi++) {
    const int64_t r0 = bi ? (int64_t)S->blocksize0[bi - 1] : 0, r1 = (int64_t)S->blocksize0[bi];
    for (size_t k = S->index1_data[bi]; k < S->index1_data[bi + 1]; k++) {
      const size_t bj = S->index2_data[k];
      const int64_t c0 = bj ? (int64_t)S->blocksize1[bj - 1] : 0, c1 = (int64_t)S->blocksize1[bj];
      const int64_t rs = r1 - r0;
      for (int64_t r = r0; r < r1; r++)
        for (int64_t c = c0; c < c1; c++) {
          out->i[fill[r]] = c;
          out->x[fill[r]++] = S->block[k][(c - c0) * rs + (r - r0)];
        }
    }
  }
  /* blocks of a row in any order: sort each row by column */
  for (int64_t r = 0; r < rows; r++) {
    const int64_t a = out->p[r], n = out->p[r + 1] - a;
    int sorted = 1;
    for (int64_t k = a + 1; k < a + n && sorted; k++) sorted = out->i[k] > out->i[k - 1];
    if (sorted) continue;
    for (int64_t k = 0; k < n; k++) {
      row[k].col = out->i[a + k];
      row[k].val = out->x[a + k];
    }
    qsort(row, (size_t)n, sizeof(Entry), cmp_entry);
    for (int64_t k = 0; k < n; k++) {
      if (k && row[k].col == row[k - 1].col) {
        free(row);
        free(fill);
        fc3dgpu_set_error("%s: two blocks overlap in row %lld", name, (long long)r);
        return NUMERICS_ERR_INVALID_ARGUMENT;
      }
      out->i[a + k] = row[k].col;
      out->x[a + k] = row[k].val;
    }
  }
  free(row);
  free(fill);
  return 0;
}

static int check_problem(const GlobalFrictionContactProblem *P, int need_contacts) {
  if (!P || !P->M || !P->q) {
    fc3dgpu_set_error("null problem, M or q");
    return NUMERICS_ERR_NULL_POINTER;
  }
  if (P->dimension != 3) {
    fc3dgpu_set_error("Invalid dimension: expected 3, got %d", P->dimension);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (P->M->size0 <= 0 || P->M->size0 != P->M->size1) {
    fc3dgpu_set_error("M is %d x %d, expected a square matrix", P->M->size0, P->M->size1);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (P->numberOfContacts < 0) {
    fc3dgpu_set_error("negative number of contacts");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (need_contacts) {
    if (!P->H || !P->b || !P->mu) {
      fc3dgpu_set_error("null H, b or mu");
      return NUMERICS_ERR_NULL_POINTER;
    }
    if (P->H->size0 != P->M->size0 || P->H->size1 != 3 * P->numberOfContacts) {
      fc3dgpu_set_error("H is %d x %d, expected %d x %d", P->H->size0, P->H->size1, P->M->size0,
                        3 * P->numberOfContacts);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
  }
  return 0;
}

static int check_options(const SolverOptions *o) {
  if (!o || !o->iparam || !o->dparam || o->iSize < OPTIONS_PARAM_SIZE || o->dSize < OPTIONS_PARAM_SIZE) {
    fc3dgpu_set_error("options are not set");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  return 0;
}

void gfc3dgpu_nsgs_set_default(SolverOptions *options) { fc3dgpu_nsgs_set_default(options); }

SolverOptions *gfc3dgpu_options_create(void) {
  SolverOptions *o = fc3dgpu_options_alloc(SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU, 1000, 1e-4);
  if (!o) return NULL;
  gfc3dgpu_nsgs_set_default(o);
  return o;
}

static gfc3dgpu_ctx *cached_ctx(SolverOptions *o, int *rc) {
  gfc3dgpu_cache *c = (gfc3dgpu_cache *)o->solverData;
  if (c && c->magic != GFC3DGPU_CACHE_MAGIC) {
    fc3dgpu_set_error("options->solverData holds foreign data");
    *rc = NUMERICS_ERR_INVALID_OPTION;
    return NULL;
  }
  if (!c) {
    c = (gfc3dgpu_cache *)calloc(1, sizeof(gfc3dgpu_cache));
    if (!c) {
      fc3dgpu_set_error("host allocation failed");
      *rc = NUMERICS_ERR_MEMORY;
      return NULL;
    }
    c->magic = GFC3DGPU_CACHE_MAGIC;
    o->solverData = c;
  }
  if (!c->ctx) c->ctx = gfc3dgpu_ctx_create(0);
  if (!c->ctx) *rc = NUMERICS_ERR_NOT_IMPLEMENTED; /* no CUDA device: no CPU fallback */
  return c->ctx;
}

/* Upload M, H, q, b, mu into ctx. */
static int upload(gfc3dgpu_ctx *ctx, const GlobalFrictionContactProblem *P) {
  Csr M, H;
  memset(&H, 0, sizeof(H));
  int rc = csr_of(P->M, "M", &M);
  if (!rc && P->numberOfContacts > 0) rc = csr_of(P->H, "H", &H);
  if (!rc)
    rc = gfc3dgpu_ctx_set_problem(ctx, P->M->size0, P->numberOfContacts, M.p, M.i, M.x, H.p, H.i, H.x, P->q,
                                  P->b, P->mu);
  csr_free(&M);
  csr_free(&H);
  return rc;
}

int gfc3dgpu_nsgs(GlobalFrictionContactProblem *problem, double *reaction, double *velocity, double *globalVelocity,
                  SolverOptions *options) {
  int rc = check_problem(problem, 1);
  if (rc) return rc;
  if (!reaction || !velocity || !globalVelocity) {
    fc3dgpu_set_error("null reaction, velocity or globalVelocity");
    return NUMERICS_ERR_NULL_POINTER;
  }
  rc = check_options(options);
  if (rc) return rc;
  if (problem->numberOfContacts == 0) {
    fc3dgpu_set_error("gfc3dgpu_nsgs: no contact (gfc3dgpu_driver handles that case)");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  gfc3dgpu_ctx *ctx = cached_ctx(options, &rc);
  if (!ctx) return rc;
  rc = upload(ctx, problem);
  if (!rc) rc = gfc3dgpu_ctx_set_arithmetic(ctx, options->iparam[FC3DGPU_IPARAM_PRECISION] == 2);
  if (!rc) rc = gfc3dgpu_ctx_set_start(ctx, reaction, globalVelocity);
  if (rc) return rc;
  const double tol = options->dparam[SICONOS_DPARAM_TOL];
  int iters = 0, info = -1;
  double error = 1.0, ms = 0.0;
  rc = gfc3dgpu_ctx_solve(ctx, tol, options->iparam[SICONOS_IPARAM_MAX_ITER],
                          options->iparam[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION_FREQUENCY], &iters, &error,
                          &info, &ms);
  if (!rc) rc = gfc3dgpu_ctx_get(ctx, reaction, velocity, globalVelocity);
  if (rc) return rc;
  options->dparam[SICONOS_DPARAM_TOL] = tol;
  options->dparam[SICONOS_DPARAM_RESIDU] = error;
  options->dparam[FC3DGPU_DPARAM_MS_SOLVE] = ms;
  return info;
}

int gfc3dgpu_driver(GlobalFrictionContactProblem *problem, double *reaction, double *velocity,
                    double *globalVelocity, SolverOptions *options) {
  if (!problem || !globalVelocity || !problem->M || !problem->q) {
    fc3dgpu_set_error("null problem, globalVelocity, M or q");
    return NUMERICS_ERR_NULL_POINTER;
  }
  int rc = check_options(options);
  if (rc) return rc;
  if (!problem->H) {
    fc3dgpu_set_error("null H");
    return NUMERICS_ERR_NULL_POINTER;
  }
  rc = check_problem(problem, 0);
  if (rc) return rc;
  if (problem->H->size1 == 0) {
    /* no contact: globalVelocity = M^-1 q (gfc3d_driver.c:107-114) */
    gfc3dgpu_ctx *ctx = cached_ctx(options, &rc);
    if (!ctx) return rc;
    GlobalFrictionContactProblem P0 = *problem;
    P0.numberOfContacts = 0;
    rc = upload(ctx, &P0);
    int iters, info;
    double err;
    if (!rc) rc = gfc3dgpu_ctx_solve(ctx, 0.0, 0, 0, &iters, &err, &info, NULL);
    if (!rc) rc = gfc3dgpu_ctx_get(ctx, NULL, NULL, globalVelocity);
    return rc;
  }
  if (!reaction || !velocity || !problem->b) {
    fc3dgpu_set_error("null reaction, velocity or b");
    return NUMERICS_ERR_NULL_POINTER;
  }
  if (options->solverId != SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU) {
    fc3dgpu_set_error("gfc3d_driver: solver ID %d is not the GPU global NSGS (%d)", options->solverId,
                      SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU);
    return NUMERICS_ERR_INVALID_SOLVER;
  }
  return gfc3dgpu_nsgs(problem, reaction, velocity, globalVelocity, options);
}

int gfc3dgpu_nsgs_solve_wrap(void *problem, double *reaction, double *velocity, double *globalVelocity,
                             SolverOptions *options) {
  return gfc3dgpu_nsgs((GlobalFrictionContactProblem *)problem, reaction, velocity, globalVelocity, options);
}

/* as gfc3d_nsgs_init_wrap (gfc3d_nsgs.c:210-215): set_default already ran */
int gfc3dgpu_nsgs_init_wrap(void *problem, SolverOptions *options) {
  (void)problem;
  (void)options;
  return NUMERICS_OK;
}

/* the device context lives until the options are released */
void gfc3dgpu_nsgs_free_wrap(void *problem, SolverOptions *options) {
  (void)problem;
  (void)options;
}

void gfc3dgpu_release(SolverOptions *options) {
  if (!options || !options->solverData) return;
  gfc3dgpu_cache *c = (gfc3dgpu_cache *)options->solverData;
  if (c->magic != GFC3DGPU_CACHE_MAGIC) return;
  gfc3dgpu_ctx_destroy(c->ctx);
  free(c);
  options->solverData = NULL;
}

void gfc3dgpu_options_delete(SolverOptions *options) {
  gfc3dgpu_release(options);
  fc3dgpu_options_delete(options);
}

int gfc3dgpu_compute_error(GlobalFrictionContactProblem *problem, double *reaction, double *velocity,
                           double *globalVelocity, double tolerance, double norm_q, double norm_b, double *error) {
  (void)norm_b;
  int rc = check_problem(problem, 1);
  if (rc) return rc;
  if (!reaction || !velocity || !globalVelocity || !error) return NUMERICS_ERR_NULL_POINTER;
  if (problem->numberOfContacts == 0) {
    fc3dgpu_set_error("gfc3dgpu_compute_error: no contact");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  gfc3dgpu_ctx *ctx = gfc3dgpu_ctx_create(0);
  if (!ctx) return NUMERICS_ERR_NOT_IMPLEMENTED;
  rc = upload(ctx, problem);
  if (!rc) rc = gfc3dgpu_ctx_set_start(ctx, reaction, globalVelocity);
  if (!rc) rc = gfc3dgpu_ctx_compute_error(ctx, norm_q >= 0.0 ? norm_q : 0.0, error);
  if (!rc) rc = gfc3dgpu_ctx_get(ctx, NULL, velocity, NULL);
  gfc3dgpu_ctx_destroy(ctx);
  if (rc) return rc;
  return *error > tolerance ? 1 : 0;
}
