/* Host side of the GPU NSGS solver for 2D friction contact, in C: the
 * registry-facing solve, init, free and set_default functions, option
 * handling and the outputs the reference solver writes.  The device work
 * goes through the fc2dgpu_ctx_* C-ABI (fc2dgpu.cu).
 *
 * Reference behaviour mirrored here:
 *   fc2d_driver validation (no trivial case)   fc2d_driver.c:40-145
 *   fc2d_nsgs_set_default                      fc2d_nsgs.c:787-792
 *   registry defaults (1000 iterations, 1e-4)  fc2d_nsgs.c:820-826
 *   outputs iparam[1] / dparam[1], info        fc2d_nsgs.c:496-512 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fc2dgpu.h"
#include "fc3dgpu_bcsr.h"

#define FC2DGPU_CACHE_MAGIC 0x46433244u

/* Device copy of W, kept in options->solverData between calls on the same
 * matrix (same M and storage pointers, same version number). */
typedef struct {
  unsigned magic;
  fc2dgpu_ctx *ctx;
  const void *M, *sbm;
  unsigned long long version;
  int nc;
  int colouring;
} fc2dgpu_cache;

static int check_problem(const FrictionContactProblem *P, const double *r, const double *u) {
  if (!P || !r || !u || !P->M || !P->q || !P->mu) {
    fc3dgpu_set_error("null problem, reaction, velocity, M, q or mu");
    return NUMERICS_ERR_NULL_POINTER;
  }
  if (P->M->size0 <= 0 || P->M->size1 <= 0) {
    fc3dgpu_set_error("Matrix has invalid dimensions");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (P->numberOfContacts <= 0) {
    fc3dgpu_set_error("Number of contacts must be positive");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (P->dimension != 2) {
    fc3dgpu_set_error("Invalid dimension: expected 2, got %d", P->dimension);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (P->M->size0 != 2 * P->numberOfContacts || P->M->size1 != 2 * P->numberOfContacts) {
    fc3dgpu_set_error("M is %d x %d, expected %d", P->M->size0, P->M->size1, 2 * P->numberOfContacts);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  return 0;
}

static int check_options(const SolverOptions *o) {
  if (!o || !o->iparam || !o->dparam || o->iSize < OPTIONS_PARAM_SIZE || o->dSize < OPTIONS_PARAM_SIZE) {
    fc3dgpu_set_error("options are not set");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  if (o->iparam[SICONOS_FRICTION_3D_NSGS_FREEZING_CONTACT] > 0) {
    fc3dgpu_set_error("GPU fc2d NSGS sweeps in colour order: contact freezing is not supported");
    return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  return 0;
}

void fc2dgpu_nsgs_set_default(SolverOptions *options) {
  if (!options || !options->iparam) return;
  options->iparam[SICONOS_IPARAM_NSGS_SHUFFLE] = 0;
  options->iparam[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION] =
      SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL;
}

SolverOptions *fc2dgpu_options_create(void) {
  SolverOptions *o = fc3dgpu_options_alloc(SICONOS_FRICTION_2D_NSGS_GPU, 1000, 1e-4);
  if (!o) return NULL;
  fc2dgpu_nsgs_set_default(o);
  return o;
}

static int cached_ctx(FrictionContactProblem *P, SolverOptions *o, fc2dgpu_ctx **out) {
  fc2dgpu_cache *c = (fc2dgpu_cache *)o->solverData;
  if (c && c->magic != FC2DGPU_CACHE_MAGIC) {
    fc3dgpu_set_error("options->solverData holds foreign data");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  const NumericsMatrix *M = P->M;
  const void *sbm = M->storageType == NM_SPARSE_BLOCK ? (const void *)M->matrix1 : (const void *)M->matrix0;
  const unsigned long long ver =
      M->storageType == NM_SPARSE_BLOCK && M->matrix1 ? M->matrix1->version.number : M->version.number;
  const int kind = o->iparam[FC3DGPU_IPARAM_COLOURING] ? o->iparam[FC3DGPU_IPARAM_COLOURING]
                                                        : FC3DGPU_COLOURING_DEFAULT;
  /* the device W is reused for a W whose version number is unchanged (a
   * value change bumps it); q and mu are sent again on every call */
  if (c && c->ctx && c->M == (const void *)M && c->sbm == sbm && c->version == ver && ver != 0 &&
      c->nc == P->numberOfContacts && c->colouring == kind) {
    *out = c->ctx;
    return 1;
  }
  if (!c) {
    c = (fc2dgpu_cache *)calloc(1, sizeof(fc2dgpu_cache));
    if (!c) {
      fc3dgpu_set_error("host allocation failed");
      return NUMERICS_ERR_MEMORY;
    }
    c->magic = FC2DGPU_CACHE_MAGIC;
    o->solverData = c;
  }
  if (!c->ctx) {
    c->ctx = fc2dgpu_ctx_create(0);
    if (!c->ctx) return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  Bcsr b;
  int rc = fc3dgpu_bcsr_from_problem(P, 2, &b);
  if (rc) return rc;
  rc = fc2dgpu_ctx_set_problem(c->ctx, b.nc, b.rowptr, b.colidx, b.blocks, P->q, P->mu, kind);
  fc3dgpu_bcsr_free(&b);
  if (rc) {
    c->M = NULL;
    return rc;
  }
  c->M = M;
  c->sbm = sbm;
  c->version = ver;
  c->nc = P->numberOfContacts;
  c->colouring = kind;
  *out = c->ctx;
  return 0;
}

static void release(SolverOptions *o) {
  if (!o || !o->solverData) return;
  fc2dgpu_cache *c = (fc2dgpu_cache *)o->solverData;
  if (c->magic != FC2DGPU_CACHE_MAGIC) return;
  fc2dgpu_ctx_destroy(c->ctx);
  free(c);
  o->solverData = NULL;
}

int fc2dgpu_nsgs(FrictionContactProblem *problem, double *reaction, double *velocity, SolverOptions *options) {
  int rc = check_problem(problem, reaction, velocity);
  if (rc) return rc;
  rc = check_options(options);
  if (rc) return rc;
  fc2dgpu_ctx *ctx = NULL;
  rc = cached_ctx(problem, options, &ctx);
  if (rc < 0) return rc;
  /* W unchanged: only q and mu go up again, into the same layout */
  if (rc == 1) rc = fc2dgpu_ctx_set_q_mu(ctx, problem->q, problem->mu);
  if (!rc) rc = fc2dgpu_ctx_set_r(ctx, reaction);
  if (rc) return rc;
  const int prec = options->iparam[FC3DGPU_IPARAM_PRECISION];
  if (prec != 0 && prec != 1) {
    fc3dgpu_set_error("iparam[FC3DGPU_IPARAM_PRECISION] must be 0 (FP32 + FP64 polish) or 1 (FP64)");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  const double sw = options->dparam[FC3DGPU_DPARAM_SWITCH_TOL];
  const double stall = options->dparam[FC3DGPU_DPARAM_STALL];
  rc = fc2dgpu_ctx_set_precision(ctx, prec, sw > 0 ? sw : 0.0, stall > 0 ? (int)stall : 0);
  if (rc) return rc;
  const int eval = options->iparam[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION];
  int iters = 0, info = 1;
  double error = INFINITY, ms = 0.0;
  rc = fc2dgpu_ctx_solve(ctx, options->dparam[SICONOS_DPARAM_TOL], options->iparam[SICONOS_IPARAM_MAX_ITER], eval,
                         &iters, &error, &info, &ms);
  if (rc) return rc;
  /* the velocity is written by fc2d_compute_error only (full-final mode) */
  const int full = eval == SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL && isfinite(error);
  rc = fc2dgpu_ctx_get_r_u(ctx, reaction, full ? velocity : NULL);
  if (rc) return rc;
  options->iparam[SICONOS_IPARAM_ITER_DONE] = iters;
  options->dparam[SICONOS_DPARAM_RESIDU] = error;
  options->iparam[FC3DGPU_IPARAM_COLOURS] = fc2dgpu_ctx_colours(ctx, NULL);
  fc2dgpu_ctx_last_sweeps(ctx, &options->iparam[FC3DGPU_IPARAM_SWEEPS_FP32],
                          &options->iparam[FC3DGPU_IPARAM_SWEEPS_FP64]);
  options->dparam[FC3DGPU_DPARAM_MS_SOLVE] = ms;
  if (options->callback && options->callback->collectStatsIteration && iters > 0) {
    /* the sweeps run on the device: the per-iteration callback is replayed
     * after the solve with each sweep's light error and the final iterate */
    double *tr = (double *)malloc(sizeof(double) * (size_t)iters);
    if (tr) {
      const int m = fc2dgpu_ctx_trace(ctx, tr, iters);
      for (int k = 0; k < m; k++)
        options->callback->collectStatsIteration(options->callback->env, (size_t)(2 * problem->numberOfContacts),
                                                 reaction, velocity, tr[k], NULL);
      free(tr);
    }
  }
  return info;
}

int fc2dgpu_driver(FrictionContactProblem *problem, double *reaction, double *velocity, SolverOptions *options) {
  int rc = check_problem(problem, reaction, velocity);
  if (rc) return rc;
  if (!options || !options->iparam || !options->dparam) {
    fc3dgpu_set_error("options are not set");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  options->iparam[SICONOS_IPARAM_ITER_DONE] = 0;
  options->dparam[SICONOS_DPARAM_RESIDU] = 0.0;
  if (options->solverId != SICONOS_FRICTION_2D_NSGS_GPU) {
    fc3dgpu_set_error("fc2d_driver: solver ID %d not found in registry", options->solverId);
    return NUMERICS_ERR_INVALID_SOLVER;
  }
  /* the registry's init then solve then free (fc2d_driver.c:113-135) */
  rc = fc2dgpu_nsgs_init_wrap(problem, options);
  if (rc) return rc;
  rc = fc2dgpu_nsgs_solve_wrap(problem, reaction, velocity, options);
  fc2dgpu_nsgs_free_wrap(problem, options);
  return rc;
}

int fc2dgpu_nsgs_solve_wrap(void *problem, double *reaction, double *velocity, SolverOptions *options) {
  return fc2dgpu_nsgs((FrictionContactProblem *)problem, reaction, velocity, options);
}

/* as fc2d_nsgs_init_wrap (fc2d_nsgs.c:802-805): the defaults are applied on
 * every driver call */
int fc2dgpu_nsgs_init_wrap(void *problem, SolverOptions *options) {
  (void)problem;
  fc2dgpu_nsgs_set_default(options);
  return NUMERICS_OK;
}

/* the device copy lives until the options are freed (fc2dgpu_release), so
 * repeated driver calls on one problem reuse it */
void fc2dgpu_nsgs_free_wrap(void *problem, SolverOptions *options) {
  (void)problem;
  (void)options;
}

void fc2dgpu_release(SolverOptions *options) { release(options); }

void fc2dgpu_options_delete(SolverOptions *options) {
  release(options);
  fc3dgpu_options_delete(options);
}

int fc2dgpu_compute_error(FrictionContactProblem *problem, double *reaction, double *velocity, double tolerance,
                          double norm_q, double *error) {
  int rc = check_problem(problem, reaction, velocity);
  if (rc) return rc;
  if (!error) return NUMERICS_ERR_NULL_POINTER;
  fc2dgpu_ctx *ctx = fc2dgpu_ctx_create(0);
  if (!ctx) return NUMERICS_ERR_NOT_IMPLEMENTED;
  Bcsr b;
  rc = fc3dgpu_bcsr_from_problem(problem, 2, &b);
  if (!rc) {
    rc = fc2dgpu_ctx_set_problem(ctx, b.nc, b.rowptr, b.colidx, b.blocks, problem->q, problem->mu, 0);
    fc3dgpu_bcsr_free(&b);
  }
  if (!rc) rc = fc2dgpu_ctx_set_r(ctx, reaction);
  if (!rc) rc = fc2dgpu_ctx_compute_error(ctx, norm_q, error);
  if (!rc) rc = fc2dgpu_ctx_get_r_u(ctx, NULL, velocity);
  fc2dgpu_ctx_destroy(ctx);
  if (rc) return rc;
  return *error > tolerance ? 1 : 0;
}
