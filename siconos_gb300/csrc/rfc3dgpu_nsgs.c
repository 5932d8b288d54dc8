/* Host side of the GPU NSGS solver for 3D rolling friction, in C: the
 * registry-facing solve, init, free and set_default functions, option
 * handling and the outputs the reference solver writes.  The device work
 * goes through the rfc3dgpu_ctx_* C-ABI (rfc3dgpu.cu).
 *
 * Reference behaviour mirrored here:
 *   rolling_friction_3d_driver checks and trivial case   rolling_friction_3d_driver.c:44-135
 *   rolling_friction_3d_nsgs_set_default                  rolling_friction_3d_nsgs.c:617-668
 *   one-contact NSN defaults (10 iterations, 1e-12,
 *   spectral-norm rho, natural map)                       rolling_friction_3d_onecone_nonsmooth_Newton_solvers.c:543-582
 *   outputs iparam[1] / dparam[1], info                  rolling_friction_3d_nsgs.c:592-600 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fc3dgpu_bcsr.h"
#include "rfc3dgpu.h"

#define RFC3DGPU_CACHE_MAGIC 0x52464333u

/* the device context kept in options->solverData between calls */
typedef struct {
  unsigned magic;
  rfc3dgpu_ctx *ctx;
} rfc3dgpu_cache;

static int check_problem(const RollingFrictionContactProblem *P, const double *r, const double *u) {
  if (!P || !r || !u || !P->M || !P->q || !P->mu || !P->mu_r) {
    fc3dgpu_set_error("null problem, reaction, velocity, M, q, mu or mu_r");
    return NUMERICS_ERR_NULL_POINTER;
  }
  if (P->numberOfContacts <= 0) {
    fc3dgpu_set_error("Number of contacts must be positive");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (P->dimension != 5) {
    fc3dgpu_set_error("Invalid dimension: expected 5, got %d", P->dimension);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (P->M->size0 != 5 * P->numberOfContacts || P->M->size1 != 5 * P->numberOfContacts) {
    fc3dgpu_set_error("M is %d x %d, expected %d", P->M->size0, P->M->size1, 5 * P->numberOfContacts);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  return 0;
}

static int check_options(const SolverOptions *o) {
  if (!o || !o->iparam || !o->dparam || o->iSize < OPTIONS_PARAM_SIZE || o->dSize < OPTIONS_PARAM_SIZE) {
    fc3dgpu_set_error("options are not set");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  const int *ip = o->iparam;
  if (ip[SICONOS_FRICTION_3D_NSGS_SHUFFLE] != 0 || ip[SICONOS_FRICTION_3D_NSGS_FREEZING_CONTACT] > 0 ||
      ip[SICONOS_FRICTION_3D_NSGS_RELAXATION] != 0 || ip[SICONOS_FRICTION_3D_NSGS_FILTER_LOCAL_SOLUTION] != 0) {
    fc3dgpu_set_error("GPU rolling NSGS sweeps in colour order: shuffle, freezing, relaxation and filter are not "
                      "supported");
    return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  if (ip[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION] != SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL ||
      ip[SICONOS_FRICTION_3D_IPARAM_INTERNAL_ERROR_STRATEGY] != SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_GIVEN_VALUE) {
    fc3dgpu_set_error("GPU rolling NSGS supports LIGHT_WITH_FULL_FINAL and GIVEN_VALUE only");
    return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  if (o->numberOfInternalSolvers < 1 || !o->internalSolvers || !o->internalSolvers[0] ||
      !o->internalSolvers[0]->iparam || !o->internalSolvers[0]->dparam) {
    fc3dgpu_set_error("The NSGS method needs options for the internal solvers");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  const SolverOptions *lo = o->internalSolvers[0];
  if (lo->solverId != SICONOS_ROLLING_FRICTION_3D_ONECONTACT_NSN ||
      lo->iparam[SICONOS_FRICTION_3D_NSN_FORMULATION] != SICONOS_FRICTION_3D_NSN_FORMULATION_NATURALMAP ||
      lo->iparam[SICONOS_FRICTION_3D_NSN_RHO_STRATEGY] != SICONOS_FRICTION_3D_NSN_FORMULATION_RHO_STRATEGY_SPECTRAL_NORM) {
    fc3dgpu_set_error("GPU rolling NSGS runs the ONECONTACT_NSN local solver (natural map, spectral-norm rho) only");
    return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  return 0;
}

static void options_free(SolverOptions *o) {
  if (!o) return;
  for (size_t i = 0; i < o->numberOfInternalSolvers; i++)
    if (o->internalSolvers) options_free(o->internalSolvers[i]);
  free(o->internalSolvers);
  free(o->iparam);
  free(o->dparam);
  free(o->dWork);
  free(o->iWork);
  free(o);
}

/* solver_options_create(SICONOS_ROLLING_FRICTION_3D_ONECONTACT_NSN):
 * registry defaults 10 / 1e-12 and its set_default */
static SolverOptions *local_options_create(void) {
  SolverOptions *o = fc3dgpu_options_alloc(SICONOS_ROLLING_FRICTION_3D_ONECONTACT_NSN, 10, 1e-12);
  if (!o) return NULL;
  o->dparam[SICONOS_FRICTION_3D_NSN_RHO] = 1.0;
  o->iparam[SICONOS_FRICTION_3D_NSN_RHO_STRATEGY] = SICONOS_FRICTION_3D_NSN_FORMULATION_RHO_STRATEGY_SPECTRAL_NORM;
  o->iparam[SICONOS_FRICTION_3D_NSN_FORMULATION] = SICONOS_FRICTION_3D_NSN_FORMULATION_NATURALMAP;
  return o;
}

void rfc3dgpu_nsgs_set_default(SolverOptions *options) {
  if (!options || !options->iparam || !options->dparam) return;
  int *ip = options->iparam;
  double *dp = options->dparam;
  ip[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION] = SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL;
  ip[SICONOS_FRICTION_3D_IPARAM_INTERNAL_ERROR_STRATEGY] = SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_GIVEN_VALUE;
  ip[SICONOS_FRICTION_3D_NSGS_SHUFFLE] = 0;
  ip[SICONOS_FRICTION_3D_NSGS_SHUFFLE_SEED] = 0;
  ip[SICONOS_FRICTION_3D_NSGS_FREEZING_CONTACT] = 0;
  ip[SICONOS_FRICTION_3D_NSGS_FILTER_LOCAL_SOLUTION] = 0;
  ip[SICONOS_FRICTION_3D_NSGS_RELAXATION] = 0;
  ip[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION_FREQUENCY] = 0;
  dp[SICONOS_DPARAM_TOL] = 1e-4;
  dp[SICONOS_FRICTION_3D_DPARAM_INTERNAL_ERROR_RATIO] = 10.0;
  ip[FC3DGPU_IPARAM_PRECISION] = 0;  /* FP32 sweeps, then the reference's FP64 loop */
  dp[FC3DGPU_DPARAM_SWITCH_TOL] = 0.0;
  dp[FC3DGPU_DPARAM_STALL] = 0.0;
  if (options->numberOfInternalSolvers == 0 || !options->internalSolvers) {
    options->numberOfInternalSolvers = 1;
    options->internalSolvers = (SolverOptions **)calloc(1, sizeof(SolverOptions *));
  } else {
    options_free(options->internalSolvers[0]);
  }
  if (options->internalSolvers) options->internalSolvers[0] = local_options_create();
}

SolverOptions *rfc3dgpu_options_create(void) {
  SolverOptions *o = fc3dgpu_options_alloc(SICONOS_ROLLING_FRICTION_3D_NSGS_GPU, 1000, 1e-4);
  if (!o) return NULL;
  rfc3dgpu_nsgs_set_default(o);
  return o;
}

void rfc3dgpu_release(SolverOptions *options) {
  if (!options || !options->solverData) return;
  rfc3dgpu_cache *c = (rfc3dgpu_cache *)options->solverData;
  if (c->magic != RFC3DGPU_CACHE_MAGIC) return;
  rfc3dgpu_ctx_destroy(c->ctx);
  free(c);
  options->solverData = NULL;
}

void rfc3dgpu_options_delete(SolverOptions *options) {
  if (!options) return;
  rfc3dgpu_release(options);
  options_free(options);
}

/* W as block-CSR of 5x5 blocks, through the 3D solver's converter */
static int bcsr_of(const RollingFrictionContactProblem *P, Bcsr *b) {
  FrictionContactProblem view;
  memset(&view, 0, sizeof(view));
  view.dimension = 5;
  view.numberOfContacts = P->numberOfContacts;
  view.M = P->M;
  view.q = P->q;
  view.mu = P->mu;
  return fc3dgpu_bcsr_from_problem(&view, 5, b);
}

/* The device context is kept between calls; the problem (layout,
 * colouring, rho) is sent on every call. */
static int cached_ctx(RollingFrictionContactProblem *P, SolverOptions *o, rfc3dgpu_ctx **out) {
  rfc3dgpu_cache *c = (rfc3dgpu_cache *)o->solverData;
  if (c && c->magic != RFC3DGPU_CACHE_MAGIC) {
    fc3dgpu_set_error("options->solverData holds foreign data");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  if (!c) {
    c = (rfc3dgpu_cache *)calloc(1, sizeof(rfc3dgpu_cache));
    if (!c) {
      fc3dgpu_set_error("host allocation failed");
      return NUMERICS_ERR_MEMORY;
    }
    c->magic = RFC3DGPU_CACHE_MAGIC;
    o->solverData = c;
  }
  if (!c->ctx) {
    c->ctx = rfc3dgpu_ctx_create(0);
    if (!c->ctx) return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  Bcsr b;
  int rc = bcsr_of(P, &b);
  if (rc) return rc;
  rc = rfc3dgpu_ctx_set_problem(c->ctx, b.nc, b.rowptr, b.colidx, b.blocks, P->q, P->mu, P->mu_r,
                                o->iparam[FC3DGPU_IPARAM_COLOURING]);
  fc3dgpu_bcsr_free(&b);
  if (rc) return rc;
  *out = c->ctx;
  return 0;
}

int rfc3dgpu_nsgs(RollingFrictionContactProblem *problem, double *reaction, double *velocity,
                  SolverOptions *options) {
  int rc = check_problem(problem, reaction, velocity);
  if (rc) return rc;
  rc = check_options(options);
  if (rc) return rc;
  rfc3dgpu_ctx *ctx = NULL;
  rc = cached_ctx(problem, options, &ctx);
  if (!rc) rc = rfc3dgpu_ctx_set_r(ctx, reaction);
  if (rc) return rc;
  const int prec = options->iparam[FC3DGPU_IPARAM_PRECISION];
  if (prec != 0 && prec != 1) {
    fc3dgpu_set_error("iparam[FC3DGPU_IPARAM_PRECISION] must be 0 (FP32 + FP64 loop) or 1 (FP64)");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  const double sw = options->dparam[FC3DGPU_DPARAM_SWITCH_TOL];
  const double stall = options->dparam[FC3DGPU_DPARAM_STALL];
  rc = rfc3dgpu_ctx_set_precision(ctx, prec, sw > 0 ? sw : 0.0, stall > 0 ? (int)stall : 0);
  if (rc) return rc;
  const SolverOptions *lo = options->internalSolvers[0];
  int iters = 0, info = 1;
  double error = INFINITY, ms = 0.0;
  rc = rfc3dgpu_ctx_solve(ctx, options->dparam[SICONOS_DPARAM_TOL], options->iparam[SICONOS_IPARAM_MAX_ITER],
                          lo->dparam[SICONOS_DPARAM_TOL], lo->iparam[SICONOS_IPARAM_MAX_ITER], &iters, &error,
                          &info, &ms);
  if (!rc) rc = rfc3dgpu_ctx_get_r_u(ctx, reaction, velocity);
  if (rc) return rc;
  options->iparam[SICONOS_IPARAM_ITER_DONE] = iters;
  options->dparam[SICONOS_DPARAM_RESIDU] = error;
  options->iparam[FC3DGPU_IPARAM_COLOURS] = rfc3dgpu_ctx_colours(ctx, NULL);
  options->dparam[FC3DGPU_DPARAM_MS_SOLVE] = ms;
  rfc3dgpu_ctx_last_sweeps(ctx, &options->iparam[FC3DGPU_IPARAM_SWEEPS_FP32],
                           &options->iparam[FC3DGPU_IPARAM_SWEEPS_FP64]);
  if (options->callback && options->callback->collectStatsIteration && iters > 0) {
    double *tr = (double *)malloc(sizeof(double) * (size_t)iters);
    if (tr) {
      const int m = rfc3dgpu_ctx_trace(ctx, tr, iters);
      for (int k = 0; k < m; k++)
        options->callback->collectStatsIteration(options->callback->env, (size_t)(5 * problem->numberOfContacts),
                                                 reaction, velocity, tr[k], NULL);
      free(tr);
    }
  }
  return info;
}

int rfc3dgpu_driver(RollingFrictionContactProblem *problem, double *reaction, double *velocity,
                    SolverOptions *options) {
  int rc = check_problem(problem, reaction, velocity);
  if (rc) return rc;
  if (!options || !options->iparam || !options->dparam) {
    fc3dgpu_set_error("options are not set");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  options->iparam[SICONOS_IPARAM_ITER_DONE] = 0;
  options->dparam[SICONOS_DPARAM_RESIDU] = 0.0;
  const int nc = problem->numberOfContacts;
  int trivial = 1;
  for (int i = 0; i < nc; i++)
    if (problem->q[5 * i] < -DBL_EPSILON) {
      trivial = 0;
      break;
    }
  if (trivial) {
    for (int i = 0; i < 5 * nc; i++) {
      velocity[i] = problem->q[i];
      reaction[i] = 0.0;
    }
    return NUMERICS_OK;
  }
  if (options->solverId != SICONOS_ROLLING_FRICTION_3D_NSGS_GPU) {
    fc3dgpu_set_error("rolling_friction_3d_driver: solver ID %d not found in registry", options->solverId);
    return NUMERICS_ERR_INVALID_SOLVER;
  }
  return rfc3dgpu_nsgs(problem, reaction, velocity, options);
}

int rfc3dgpu_nsgs_solve_wrap(void *problem, double *reaction, double *velocity, SolverOptions *options) {
  return rfc3dgpu_nsgs((RollingFrictionContactProblem *)problem, reaction, velocity, options);
}

int rfc3dgpu_nsgs_init_wrap(void *problem, SolverOptions *options) {
  (void)problem;
  (void)options;
  return NUMERICS_OK;
}

/* the device copy stays in options->solverData until rfc3dgpu_release */
void rfc3dgpu_nsgs_free_wrap(void *problem, SolverOptions *options) {
  (void)problem;
  (void)options;
}

int rfc3dgpu_compute_error(RollingFrictionContactProblem *problem, double *reaction, double *velocity,
                           double tolerance, double norm_q, double *error) {
  int rc = check_problem(problem, reaction, velocity);
  if (rc) return rc;
  if (!error) return NUMERICS_ERR_NULL_POINTER;
  rfc3dgpu_ctx *ctx = rfc3dgpu_ctx_create(0);
  if (!ctx) return NUMERICS_ERR_NOT_IMPLEMENTED;
  Bcsr b;
  rc = bcsr_of(problem, &b);
  if (!rc) {
    rc = rfc3dgpu_ctx_set_problem(ctx, b.nc, b.rowptr, b.colidx, b.blocks, problem->q, problem->mu, problem->mu_r, 0);
    fc3dgpu_bcsr_free(&b);
  }
  if (!rc) rc = rfc3dgpu_ctx_set_r(ctx, reaction);
  if (!rc) rc = rfc3dgpu_ctx_compute_error(ctx, norm_q, error);
  if (!rc) rc = rfc3dgpu_ctx_get_r_u(ctx, NULL, velocity);
  rfc3dgpu_ctx_destroy(ctx);
  if (rc) return rc;
  return *error > tolerance ? 1 : 0;
}
