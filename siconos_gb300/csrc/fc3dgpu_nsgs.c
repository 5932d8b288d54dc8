/* Host side of the GPU NSGS solver, in C: the registry-facing solve and
 * set_default functions, option handling, the SBM -> block-CSR repack and
 * the outputs the reference solver writes.  All device work goes through the
 * device-resident C-ABI (fc3dgpu_ctx_*), implemented in CUDA.
 *
 * Reference behaviour mirrored here:
 *   fc3d_driver validation and trivial case  fc3d_driver.c:51-145
 *   fc3d_nsgs_set_default                     fc3d_nsgs.c:919-950
 *   one-contact local solver defaults         onecontact.c:1037-1056, REGISTER :1139-1143
 *   solver_options_initialize                 SolverOptions.c:44-96
 *   outputs iparam[1] / dparam[1], info       fc3d_nsgs.c:894-900
 *   per-iteration callback                    fc3d_nsgs.c:103-110 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "fc3dgpu.h"
#include "fc3dgpu_bcsr.h"

void fc3dgpu_set_error(const char *fmt, ...);

#define FC3DGPU_CACHE_MAGIC 0x46433344u

typedef struct {
  unsigned magic;
  fc3dgpu_ctx *ctx;
  const void *M;
  const void *sbm;
  unsigned long long version;
  int nc;
  long long nnzb;
  int colouring;
} fc3dgpu_cache;

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* calloc'd options as solver_options_initialize does */
SolverOptions *fc3dgpu_options_alloc(int id, int max_iter, double tol) {
  SolverOptions *o = (SolverOptions *)calloc(1, sizeof(SolverOptions));
  if (!o) return NULL;
  o->solverId = id;
  o->iSize = OPTIONS_PARAM_SIZE;
  o->dSize = OPTIONS_PARAM_SIZE;
  o->iparam = (int *)calloc(OPTIONS_PARAM_SIZE, sizeof(int));
  o->dparam = (double *)calloc(OPTIONS_PARAM_SIZE, sizeof(double));
  if (!o->iparam || !o->dparam) {
    free(o->iparam);
    free(o->dparam);
    free(o);
    return NULL;
  }
  o->iparam[SICONOS_IPARAM_MAX_ITER] = max_iter;
  o->dparam[SICONOS_DPARAM_TOL] = tol;
  o->dparam[SICONOS_DPARAM_RESIDU] = INFINITY;
  o->filterOn = true;
  o->isSet = true;
  return o;
}

/* fc3d_onecontact_nsn_gp_set_default on registry defaults (100, 1e-14) */
static SolverOptions *local_options_create(void) {
  SolverOptions *o = fc3dgpu_options_alloc(SICONOS_FRICTION_3D_ONECONTACT_NSN_GP_HYBRID, 100, 1e-14);
  if (!o) return NULL;
  o->iparam[SICONOS_FRICTION_3D_NSN_RHO_STRATEGY] = SICONOS_FRICTION_3D_NSN_FORMULATION_RHO_STRATEGY_SPLIT_SPECTRAL_NORM;
  o->dparam[SICONOS_FRICTION_3D_NSN_RHO] = 1.0;
  o->iparam[SICONOS_FRICTION_3D_NSN_FORMULATION] = SICONOS_FRICTION_3D_NSN_FORMULATION_ALARTCURNIER_STD;
  o->iparam[SICONOS_FRICTION_3D_NSN_LINESEARCH] = SICONOS_FRICTION_3D_NSN_LINESEARCH_GOLDSTEINPRICE;
  o->iparam[SICONOS_FRICTION_3D_NSN_LINESEARCH_MAX_ITER] = 10;
  o->iparam[SICONOS_FRICTION_3D_NSN_HYBRID_STRATEGY] = SICONOS_FRICTION_3D_NSN_HYBRID_STRATEGY_NSN_AND_PLI_NSN_LOOP;
  o->iparam[SICONOS_FRICTION_3D_NSN_HYBRID_MAX_LOOP] = 1;
  o->iparam[SICONOS_FRICTION_3D_NSN_HYBRID_MAX_ITER] = 100;
  return o;
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
  free(o->solverData);
  free(o);
}

void fc3dgpu_nsgs_set_default(SolverOptions *options) {
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
  ip[SICONOS_FRICTION_3D_NSGS_PRINTING_LIKE_IPM] = 1;
  ip[FC3DGPU_IPARAM_PRECISION] = 0;
  ip[FC3DGPU_IPARAM_LANES] = 0;
  ip[FC3DGPU_IPARAM_WARMSTART] = 0;
  ip[FC3DGPU_IPARAM_COLOURING] = FC3DGPU_COLOURING_DEFAULT;
  dp[FC3DGPU_DPARAM_SWITCH_TOL] = 1e-6;
  dp[FC3DGPU_DPARAM_LOCAL_TOL32] = 1e-5;
  dp[FC3DGPU_DPARAM_STALL] = 64;
  if (options->numberOfInternalSolvers == 0 || !options->internalSolvers) {
    options->numberOfInternalSolvers = 1;
    options->internalSolvers = (SolverOptions **)calloc(1, sizeof(SolverOptions *));
  } else {
    options_free(options->internalSolvers[0]);
  }
  if (options->internalSolvers) options->internalSolvers[0] = local_options_create();
}

SolverOptions *fc3dgpu_options_create(void) {
  SolverOptions *o = fc3dgpu_options_alloc(SICONOS_FRICTION_3D_NSGS_GPU, 1000, 1e-4);
  if (!o) return NULL;
  fc3dgpu_nsgs_set_default(o);
  return o;
}

void fc3dgpu_options_delete(SolverOptions *options) {
  if (!options) return;
  fc3dgpu_release(options);
  options_free(options);
}

void fc3dgpu_release(SolverOptions *options) {
  if (!options || !options->solverData) return;
  fc3dgpu_cache *c = (fc3dgpu_cache *)options->solverData;
  if (c->magic != FC3DGPU_CACHE_MAGIC) return;
  fc3dgpu_ctx_destroy(c->ctx);
  free(c);
  options->solverData = NULL;
}

/* Block-CSR view of W (fc3dgpu_bcsr.h): SBM storage is repacked (its blocks
 * are scattered pointers, BlockCSRMatrix.cpp:249); dense storage keeps every
 * d x d block holding a nonzero, plus the diagonal. */
void fc3dgpu_bcsr_free(Bcsr *b) {
  if (!b->borrowed) {
    free(b->rowptr);
    free(b->colidx);
    free(b->blocks);
  }
  memset(b, 0, sizeof(*b));
}

static int bcsr_impl(const FrictionContactProblem *P, int d, Bcsr *out, int block_ptrs) {
  memset(out, 0, sizeof(*out));
  const int nc = P->numberOfContacts;
  const NumericsMatrix *M = P->M;
  const size_t dd = (size_t)d * (size_t)d;
  out->nc = nc;
  if (M->storageType == NM_SPARSE_BLOCK) {
    const SparseBlockStructuredMatrix *S = M->matrix1;
    if (!S || !S->index1_data || !S->index2_data || !S->block) {
      fc3dgpu_set_error("SBM storage without data");
      return NUMERICS_ERR_NULL_POINTER;
    }
    if ((int)S->blocknumber0 != nc || (int)S->blocknumber1 != nc) {
      fc3dgpu_set_error("SBM has %zu x %zu block rows/columns, expected %d", S->blocknumber0, S->blocknumber1, nc);
      return NUMERICS_ERR_INVALID_ARGUMENT;
    }
    for (int i = 0; i < nc; i++) {
      size_t lo = i ? S->blocksize0[i - 1] : 0, lo1 = i ? S->blocksize1[i - 1] : 0;
      if (S->blocksize0[i] - lo != (size_t)d || S->blocksize1[i] - lo1 != (size_t)d) {
        fc3dgpu_set_error("SBM block %d is not %dx%d", i, d, d);
        return NUMERICS_ERR_INVALID_ARGUMENT;
      }
    }
    const size_t nrows_filled = S->filled1 ? S->filled1 - 1 : 0;
    const long long nnzb = (long long)(nrows_filled ? S->index1_data[nrows_filled] : 0);
    out->nnzb = nnzb;
    /* Zero-copy view when every block row is filled and the blocks sit
     * back to back in one allocation (size_t and int64_t share a layout on
     * the LP64 targets this library builds for). */
    if (sizeof(size_t) == sizeof(int64_t) && nrows_filled == (size_t)nc && nnzb > 0 && block_ptrs) {
      out->rowptr = (int64_t *)S->index1_data;
      out->colidx = (int64_t *)S->index2_data;
      out->block = (const double *const *)S->block;
      out->borrowed = 1;
      return 0;
    }
    if (sizeof(size_t) == sizeof(int64_t) && nrows_filled == (size_t)nc && nnzb > 0) {
      int contiguous = 1;
      for (long long k = 1; k < nnzb && contiguous; k++) contiguous = (S->block[k] == S->block[0] + dd * k);
      if (contiguous) {
        out->rowptr = (int64_t *)S->index1_data;
        out->colidx = (int64_t *)S->index2_data;
        out->blocks = S->block[0];
        out->borrowed = 1;
        return 0;
      }
    }
    out->rowptr = (int64_t *)malloc(sizeof(int64_t) * ((size_t)nc + 1));
    out->colidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nnzb ? nnzb : 1));
    out->blocks = (double *)malloc(sizeof(double) * dd * (size_t)(nnzb ? nnzb : 1));
    if (!out->rowptr || !out->colidx || !out->blocks) {
      fc3dgpu_bcsr_free(out);
      fc3dgpu_set_error("host allocation failed");
      return NUMERICS_ERR_MEMORY;
    }
    for (int i = 0; i <= nc; i++)
      out->rowptr[i] = (int64_t)((size_t)i <= nrows_filled ? S->index1_data[i] : S->index1_data[nrows_filled]);
    for (long long k = 0; k < nnzb; k++) {
      out->colidx[k] = (int64_t)S->index2_data[k];
      memcpy(&out->blocks[dd * k], S->block[k], dd * sizeof(double));
    }
    return 0;
  }
  if (M->storageType == NM_DENSE) {
    const double *A = M->matrix0;
    if (!A) {
      fc3dgpu_set_error("dense storage without data");
      return NUMERICS_ERR_NULL_POINTER;
    }
    const size_t n = (size_t)d * (size_t)nc;
    long long cnt = 0;
    for (int bi = 0; bi < nc; bi++)
      for (int bj = 0; bj < nc; bj++) {
        int nz = (bi == bj);
        for (int a = 0; a < d && !nz; a++)
          for (int b = 0; b < d && !nz; b++) nz = A[(size_t)(d * bj + b) * n + (size_t)(d * bi + a)] != 0.0;
        cnt += nz;
      }
    out->nnzb = cnt;
    out->rowptr = (int64_t *)malloc(sizeof(int64_t) * ((size_t)nc + 1));
    out->colidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)cnt);
    out->blocks = (double *)malloc(sizeof(double) * dd * (size_t)cnt);
    if (!out->rowptr || !out->colidx || !out->blocks) {
      fc3dgpu_bcsr_free(out);
      fc3dgpu_set_error("host allocation failed");
      return NUMERICS_ERR_MEMORY;
    }
    long long k = 0;
    for (int bi = 0; bi < nc; bi++) {
      out->rowptr[bi] = k;
      for (int bj = 0; bj < nc; bj++) {
        int nz = (bi == bj);
        for (int a = 0; a < d && !nz; a++)
          for (int b = 0; b < d && !nz; b++) nz = A[(size_t)(d * bj + b) * n + (size_t)(d * bi + a)] != 0.0;
        if (!nz) continue;
        out->colidx[k] = bj;
        for (int b = 0; b < d; b++)
          for (int a = 0; a < d; a++)
            out->blocks[dd * k + (size_t)(d * b + a)] = A[(size_t)(d * bj + b) * n + (size_t)(d * bi + a)];
        k++;
      }
    }
    out->rowptr[nc] = k;
    return 0;
  }
  fc3dgpu_set_error("storage type %d is not supported (SBM or dense only)", (int)M->storageType);
  return NUMERICS_ERR_NOT_IMPLEMENTED;
}

int fc3dgpu_bcsr_from_problem(const FrictionContactProblem *P, int d, Bcsr *out) { return bcsr_impl(P, d, out, 0); }

int fc3dgpu_bcsr_view(const FrictionContactProblem *P, int d, Bcsr *out) { return bcsr_impl(P, d, out, 1); }

/* W of the problem onto the device: new values keep the layout when the
 * structure is unchanged (fc3dgpu_ctx_update_W[_ptrs]). */
static int upload_W(fc3dgpu_ctx *ctx, const FrictionContactProblem *P, int kind, long long *nnzb) {
  Bcsr b;
  int rc = fc3dgpu_bcsr_view(P, 3, &b);
  if (rc) return rc;
  rc = b.block ? fc3dgpu_ctx_update_W_ptrs(ctx, b.nc, b.rowptr, b.colidx, b.block, kind)
               : fc3dgpu_ctx_update_W(ctx, b.nc, b.rowptr, b.colidx, b.blocks, kind);
  if (nnzb) *nnzb = b.nnzb;
  fc3dgpu_bcsr_free(&b);
  return rc;
}

static int check_problem(const FrictionContactProblem *P, const double *r, const double *u) {
  if (!P || !r || !u || !P->M || !P->q || !P->mu) {
    fc3dgpu_set_error("null problem, reaction, velocity, M, q or mu");
    return NUMERICS_ERR_NULL_POINTER;
  }
  if (P->numberOfContacts <= 0) {
    fc3dgpu_set_error("Number of contacts must be positive");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (P->dimension != 3) {
    fc3dgpu_set_error("dimension must be 3");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (P->M->size0 != 3 * P->numberOfContacts || P->M->size1 != 3 * P->numberOfContacts) {
    fc3dgpu_set_error("M is %d x %d, expected %d", P->M->size0, P->M->size1, 3 * P->numberOfContacts);
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  for (int i = 0; i < P->numberOfContacts; i++)
    if (!(P->mu[i] >= 0.0) || isinf(P->mu[i])) {
      fc3dgpu_set_error("mu[%d] = %g is not a friction coefficient", i, P->mu[i]);
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
  /* value checks as fc3d_nsgs.c:630-665 makes them */
  const int shuffle = ip[SICONOS_FRICTION_3D_NSGS_SHUFFLE], em = ip[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION];
  if (shuffle < 0 || shuffle > 2) {
    fc3dgpu_set_error("iparam[SICONOS_FRICTION_3D_NSGS_SHUFFLE] must be 0, 1 or 2");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (em < SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_FULL || em > SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_ADAPTIVE) {
    fc3dgpu_set_error("iparam[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION] must be 0, 1, 2 or 3");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  if (shuffle != 0 || ip[SICONOS_FRICTION_3D_NSGS_FREEZING_CONTACT] > 0) {
    fc3dgpu_set_error("GPU NSGS sweeps in colour order: shuffle and freezing are not supported");
    return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  if (o->numberOfInternalSolvers < 1 || !o->internalSolvers || !o->internalSolvers[0]) {
    fc3dgpu_set_error("The NSGS method needs options for the internal solvers");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  if (o->internalSolvers[0]->solverId != SICONOS_FRICTION_3D_ONECONTACT_NSN_GP_HYBRID) {
    fc3dgpu_set_error("GPU NSGS runs the OC_NSN_GP_HYBRID local solver only");
    return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  return 0;
}

static void params_from_options(const SolverOptions *o, fc3dgpu_params *p) {
  fc3dgpu_params_default(p);
  const int *ip = o->iparam;
  const double *dp = o->dparam;
  const SolverOptions *lo = o->internalSolvers[0];
  p->tol = dp[SICONOS_DPARAM_TOL];
  p->max_iter = ip[SICONOS_IPARAM_MAX_ITER];
  p->precision = ip[FC3DGPU_IPARAM_PRECISION];
  p->lanes = ip[FC3DGPU_IPARAM_LANES];
  if (dp[FC3DGPU_DPARAM_SWITCH_TOL] > 0) p->switch_tol = dp[FC3DGPU_DPARAM_SWITCH_TOL];
  if (dp[FC3DGPU_DPARAM_LOCAL_TOL32] > 0) p->local_tol32 = dp[FC3DGPU_DPARAM_LOCAL_TOL32];
  if (dp[FC3DGPU_DPARAM_STALL] > 0) p->stall_window = (int)dp[FC3DGPU_DPARAM_STALL];
  p->local_tol = lo->dparam[SICONOS_DPARAM_TOL];
  /* relaxation and the filter of local solutions (fc3d_nsgs.c:760-830) are
   * steps of the FP64 sweeps: with either, FP64 sweeps only */
  p->relax = ip[SICONOS_FRICTION_3D_NSGS_RELAXATION] == 1;
  p->omega = dp[SICONOS_FRICTION_3D_NSGS_RELAXATION_VALUE];
  p->filter = ip[SICONOS_FRICTION_3D_NSGS_FILTER_LOCAL_SOLUTION] == 1;
  if (p->relax || p->filter) p->precision = (p->precision == 2 || p->precision == 3) ? 3 : 1;
  p->newton_max = lo->iparam[SICONOS_IPARAM_MAX_ITER];
  if (lo->iparam[SICONOS_FRICTION_3D_NSN_HYBRID_MAX_ITER] > 0) p->pli_max = lo->iparam[SICONOS_FRICTION_3D_NSN_HYBRID_MAX_ITER];
  if (lo->iparam[SICONOS_FRICTION_3D_NSN_LINESEARCH_MAX_ITER] > 0) p->ls_max = lo->iparam[SICONOS_FRICTION_3D_NSN_LINESEARCH_MAX_ITER];
}

/* Get (or build) the cached device copy of W for this problem. */
static int cached_ctx(FrictionContactProblem *P, SolverOptions *o, fc3dgpu_ctx **out) {
  fc3dgpu_cache *c = (fc3dgpu_cache *)o->solverData;
  if (c && c->magic != FC3DGPU_CACHE_MAGIC) {
    fc3dgpu_set_error("options->solverData holds foreign data");
    return NUMERICS_ERR_INVALID_OPTION;
  }
  const NumericsMatrix *M = P->M;
  const void *sbm = M->storageType == NM_SPARSE_BLOCK ? (const void *)M->matrix1 : (const void *)M->matrix0;
  unsigned long long ver =
      M->storageType == NM_SPARSE_BLOCK && M->matrix1 ? M->matrix1->version.number : M->version.number;
  const int kind = o->iparam[FC3DGPU_IPARAM_COLOURING];
  if (c && c->ctx && c->M == (const void *)M && c->sbm == sbm && c->version == ver && c->nc == P->numberOfContacts &&
      c->colouring == kind && ver != 0) {
    *out = c->ctx;
    return 0;
  }
  if (!c) {
    c = (fc3dgpu_cache *)calloc(1, sizeof(fc3dgpu_cache));
    if (!c) {
      fc3dgpu_set_error("host allocation failed");
      return NUMERICS_ERR_MEMORY;
    }
    c->magic = FC3DGPU_CACHE_MAGIC;
    o->solverData = c;
  }
  if (!c->ctx) {
    c->ctx = fc3dgpu_ctx_create(0);
    if (!c->ctx) return NUMERICS_ERR_NOT_IMPLEMENTED;
  }
  /* a W that changed since the cached one is most often new values on the
   * same structure (time stepping with fixed contacts): keep the layout then */
  int rc = upload_W(c->ctx, P, kind, &c->nnzb);
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

/* |q| computed on a host thread while W uploads */
typedef struct {
  const double *q;
  long long n;
  double norm;
} NormJob;

static void *norm_job(void *p) {
  NormJob *j = (NormJob *)p;
  j->norm = fc3dgpu_norm_q_host(j->q, j->n);
  return NULL;
}

/* The options whose loop runs on the host (fc3d_nsgs.c:711-900, the
 * general branch): an error evaluation other than LIGHT_WITH_FULL_FINAL, or
 * a local tolerance set from the error at each iteration
 * (fc3d_set_internalsolver_tolerance.c:31-63). */
static int host_loop_options(const SolverOptions *o) {
  const int em = o->iparam[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION];
  const int st = o->iparam[SICONOS_FRICTION_3D_IPARAM_INTERNAL_ERROR_STRATEGY];
  return em != SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL ||
         st == SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_ADAPTIVE ||
         st == SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_ADAPTIVE_N_CONTACT;
}

/* That loop: one FP64 sweep in colour order a device call
 * (fc3dgpu_ctx_solve with a budget of one sweep and a zero tolerance, which
 * reports the sweep's light error and the full error of its iterate, u on
 * the device), the decisions on the host as the reference takes them:
 *   local tolerance at the start of each iteration: ADAPTIVE
 *     max(error / ratio, tol / nc), ADAPTIVE_N_CONTACT error / (ratio nc),
 *     from the previous iteration's error (infinite before the first);
 *   FULL: the full error every iteration, or every `freq` iterations
 *     (1e24 between evaluations, fc3d_nsgs.c:392-412), against the tolerance;
 *   LIGHT: the light error against the tolerance, no full error, u as given;
 *   LIGHT_WITH_FULL_FINAL: the tolerance manager (tolerance_manager.h) and
 *     the final full error, as the device loop of the default options;
 *   ADAPTIVE: the reference's loop has no branch for it: the budget runs
 *     out, info -20, residual infinite, u as given.
 * The per-iteration error is kept for the callback, replayed after the loop
 * as for the device loop.  Returns info; the outputs as the reference's. */
static int nsgs_host_loop(fc3dgpu_ctx *ctx, FrictionContactProblem *P, double *reaction, double *velocity,
                          SolverOptions *o, const fc3dgpu_params *p0, double *trace, int trace_cap, int *tlen,
                          int *iters, double *residual, double *incr_out, double *ms) {
  const int nc = P->numberOfContacts;
  const int *ip = o->iparam;
  const int em = ip[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION];
  const int freq = ip[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION_FREQUENCY];
  const int strategy = ip[SICONOS_FRICTION_3D_IPARAM_INTERNAL_ERROR_STRATEGY];
  const double ratio = o->dparam[SICONOS_FRICTION_3D_DPARAM_INTERNAL_ERROR_RATIO];
  const double user_tol = p0->tol, min_tol = DBL_EPSILON * 1e-6;
  fc3dgpu_params p = *p0;
  p.max_iter = 1;
  p.tol = 0.0;
  p.precision = (p0->precision == 2 || p0->precision == 3) ? 3 : 1;
  double tolerance = user_tol, local_tol = p0->local_tol;
  double incr = INFINITY, full = INFINITY, last_full = INFINITY;
  int not_conv = 1, iter = 0, nt_trace = 0;
  double *scratch = (double *)malloc(sizeof(double) * 3 * (size_t)nc);
  if (!scratch) {
    fc3dgpu_set_error("host allocation failed");
    return NUMERICS_ERR_MEMORY;
  }
  *ms = 0.0;
  while (iter < p0->max_iter && not_conv > 0) {
    ++iter;
    if (strategy == SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_ADAPTIVE)
      local_tol = fmax(incr / ratio, user_tol / nc);
    else if (strategy == SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_ADAPTIVE_N_CONTACT)
      local_tol = incr / (ratio * nc);
    p.local_tol = local_tol;
    fc3dgpu_stats st;
    int rc = fc3dgpu_ctx_solve(ctx, &p, &st);
    if (rc) {
      free(scratch);
      return rc;
    }
    *ms += st.ms_total;
    last_full = st.error;
    if (em == SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT) {
      incr = st.incr_error;
      not_conv = incr < tolerance ? 0 : 1;
    } else if (em == SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL) {
      incr = st.incr_error;
      if (incr < tolerance) {
        full = st.error;
        if (full <= user_tol) {
          not_conv = 0;
        } else if (incr < 1e-15 || incr < DBL_EPSILON * 100.0) {
          local_tol = fmax(local_tol / 100.0, min_tol);
        } else if (full > 0.0 && incr > 0.0) {
          double nt = incr / full * user_tol;
          const double umin = user_tol * 1e-6, mint = umin > min_tol ? umin : min_tol;
          if (nt < mint) nt = mint;
          if (nt > 0.0 && nt < tolerance) tolerance = nt;
        }
        if (!(tolerance > 0.0)) break; /* before the iteration's callback, as fc3d_nsgs.c:841-846 */
      }
    } else if (em == SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_FULL) {
      full = 1e24;
      if (freq <= 0 || iter % freq == 0) {
        full = st.error;
        /* u of this iterate, as the reference's fc3d_compute_error leaves it */
        rc = fc3dgpu_ctx_get_r_u(ctx, scratch, velocity);
        if (rc) {
          free(scratch);
          return rc;
        }
      }
      incr = full;
      not_conv = full < tolerance ? 0 : 1;
    }
    if (trace && nt_trace < trace_cap) trace[nt_trace] = incr;
    nt_trace++;
  }
  int rc = 0;
  if (em == SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL) {
    /* the final full error: the last call's (that of the final iterate,
     * u left on the device), or one evaluation when no sweep ran */
    full = last_full;
    if (iter == 0) rc = fc3dgpu_ctx_compute_error(ctx, &full);
    if (!rc) rc = fc3dgpu_ctx_get_r_u(ctx, reaction, velocity);
    not_conv = full < user_tol ? 0 : 1;
  } else {
    rc = fc3dgpu_ctx_get_r_u(ctx, reaction, scratch);
  }
  free(scratch);
  if (rc) return rc;
  *iters = iter;
  *tlen = nt_trace;
  *residual = full;
  *incr_out = incr;
  int info = not_conv;
  if (iter == p0->max_iter && not_conv > 0) info = NUMERICS_ERR_MAX_ITER;
  return info;
}

int fc3dgpu_nsgs(FrictionContactProblem *problem, double *reaction, double *velocity, SolverOptions *options) {
  int rc = check_problem(problem, reaction, velocity);
  if (rc) return rc;
  rc = check_options(options);
  if (rc) return rc;
  const double t0 = now_s();
  fc3dgpu_ctx *ctx = NULL;
  NormJob nj = {problem->q, 3LL * problem->numberOfContacts, 0.0};
  pthread_t th;
  const int threaded = pthread_create(&th, NULL, norm_job, &nj) == 0;
  if (!threaded) norm_job(&nj);
  rc = cached_ctx(problem, options, &ctx);
  if (threaded) pthread_join(th, NULL);
  if (rc) return rc;
  rc = fc3dgpu_ctx_set_q_mu_norm(ctx, problem->q, problem->mu, nj.norm);
  if (!rc) rc = fc3dgpu_ctx_set_r(ctx, reaction);
  if (rc) return rc;
  fc3dgpu_params p;
  params_from_options(options, &p);
  if (host_loop_options(options)) {
    const double t1 = now_s();
    const int cap = p.max_iter > 0 ? p.max_iter : 1;
    double *tr = (double *)malloc(sizeof(double) * (size_t)cap);
    int iters = 0, tlen = 0;
    double residual = INFINITY, incr = INFINITY, ms = 0.0;
    const int info = nsgs_host_loop(ctx, problem, reaction, velocity, options, &p, tr, cap, &tlen, &iters,
                                    &residual, &incr, &ms);
    const double t2 = now_s();
    if (info < 0 && info != NUMERICS_ERR_MAX_ITER) {
      free(tr);
      return info;
    }
    int *ip = options->iparam;
    double *dp = options->dparam;
    ip[SICONOS_IPARAM_ITER_DONE] = iters;
    dp[SICONOS_DPARAM_RESIDU] = residual;
    ip[FC3DGPU_IPARAM_SWEEPS_FP32] = 0;
    ip[FC3DGPU_IPARAM_SWEEPS_FP64] = iters;
    dp[SICONOS_DPARAM_TIME_BEFORE_LOOP] = t1 - t0;
    dp[SICONOS_DPARAM_TIME_IN_LOOP] = t2 - t1;
    dp[SICONOS_DPARAM_TIME_AFTER_LOOP] = 0.0;
    dp[FC3DGPU_DPARAM_MS_SWEEP32] = 0.0;
    dp[FC3DGPU_DPARAM_MS_SWEEP64] = iters ? ms / iters : 0.0;
    dp[FC3DGPU_DPARAM_MS_SOLVE] = ms;
    dp[FC3DGPU_DPARAM_INCR_ERROR] = incr;
    if (tr && options->callback && options->callback->collectStatsIteration)
      for (int k = 0; k < tlen && k < cap; k++)
        options->callback->collectStatsIteration(options->callback->env, (size_t)(3 * problem->numberOfContacts),
                                                 reaction, velocity, tr[k], NULL);
    free(tr);
    return info;
  }
  fc3dgpu_stats st;
  const double t1 = now_s();
  rc = fc3dgpu_ctx_solve(ctx, &p, &st);
  const double t2 = now_s();
  if (rc) return rc;
  rc = fc3dgpu_ctx_get_r_u(ctx, reaction, velocity);
  if (rc) return rc;
  const double t3 = now_s();
  int *ip = options->iparam;
  double *dp = options->dparam;
  ip[SICONOS_IPARAM_ITER_DONE] = st.sweeps32 + st.sweeps64;
  dp[SICONOS_DPARAM_RESIDU] = st.error;
  ip[FC3DGPU_IPARAM_SWEEPS_FP32] = st.sweeps32;
  ip[FC3DGPU_IPARAM_SWEEPS_FP64] = st.sweeps64;
  ip[FC3DGPU_IPARAM_COLOURS] = st.colours;
  dp[SICONOS_DPARAM_TIME_BEFORE_LOOP] = t1 - t0;
  dp[SICONOS_DPARAM_TIME_IN_LOOP] = t2 - t1;
  dp[SICONOS_DPARAM_TIME_AFTER_LOOP] = t3 - t2;
  dp[FC3DGPU_DPARAM_MS_SWEEP32] = st.sweeps32 ? st.ms_fp32 / st.sweeps32 : 0.0;
  dp[FC3DGPU_DPARAM_MS_SWEEP64] = st.sweeps64 ? st.ms_fp64 / st.sweeps64 : 0.0;
  dp[FC3DGPU_DPARAM_MS_SOLVE] = st.ms_total;
  dp[FC3DGPU_DPARAM_INCR_ERROR] = st.incr_error;
  if (options->callback && options->callback->collectStatsIteration) {
    /* The sweeps run on the device without host round trips, so the
     * per-iteration callback is replayed after the solve: one call per
     * sweep with that sweep's incremental error and the final iterate. */
    int n = st.sweeps32 + st.sweeps64;
    double *tr = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (tr) {
      int m = fc3dgpu_ctx_trace(ctx, tr, n);
      for (int k = 0; k < m; k++)
        options->callback->collectStatsIteration(options->callback->env, (size_t)(3 * problem->numberOfContacts),
                                                 reaction, velocity, tr[k], NULL);
      free(tr);
    }
  }
  return st.info;
}

/* fc3d_driver (fc3d_driver.c:77-145) for this solver id: validation,
 * outputs reset, trivial take-off case (all q_n >= -DBL_EPSILON gives r = 0,
 * u = q, fc3d_driver.c:51-71), dispatch, [WARN] on a non-zero status. */
int fc3dgpu_driver(FrictionContactProblem *problem, double *reaction, double *velocity, SolverOptions *options) {
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
    if (problem->q[3 * i] < -DBL_EPSILON) {
      trivial = 0;
      break;
    }
  if (trivial) {
    for (int i = 0; i < 3 * nc; i++) {
      velocity[i] = problem->q[i];
      reaction[i] = 0.0;
    }
    return NUMERICS_OK;
  }
  if (options->solverId != SICONOS_FRICTION_3D_NSGS_GPU) {
    fc3dgpu_set_error("Solver ID not found in registry");
    return NUMERICS_ERR_INVALID_SOLVER;
  }
  rc = fc3dgpu_nsgs(problem, reaction, velocity, options);
  if (rc != NUMERICS_OK) fprintf(stderr, "[WARN] fc3dgpu_driver: solver returned status %d\n", rc);
  return rc;
}

int fc3dgpu_nsgs_solve_wrap(void *problem, double *reaction, double *velocity, SolverOptions *options) {
  return fc3dgpu_nsgs((FrictionContactProblem *)problem, reaction, velocity, options);
}

int fc3dgpu_nsgs_init_wrap(void *problem, SolverOptions *options) {
  (void)problem;
  (void)options;
  return NUMERICS_OK;
}

void fc3dgpu_nsgs_free_wrap(void *problem, SolverOptions *options) {
  /* the device copy of W stays cached in options->solverData across
   * fc3d_driver calls; fc3dgpu_release frees it */
  (void)problem;
  (void)options;
}

int fc3dgpu_compute_error(FrictionContactProblem *problem, double *reaction, double *velocity, double tolerance,
                          double norm_q, double *error) {
  int rc = check_problem(problem, reaction, velocity);
  if (rc) return rc;
  if (!error) return NUMERICS_ERR_NULL_POINTER;
  fc3dgpu_ctx *ctx = fc3dgpu_ctx_create(0);
  if (!ctx) return NUMERICS_ERR_NOT_IMPLEMENTED;
  rc = upload_W(ctx, problem, 0, NULL);
  if (!rc) rc = fc3dgpu_ctx_set_q_mu(ctx, problem->q, problem->mu);
  if (!rc) rc = fc3dgpu_ctx_set_r(ctx, reaction);
  if (!rc) rc = fc3dgpu_ctx_set_norm_q(ctx, norm_q);
  if (!rc) rc = fc3dgpu_ctx_compute_error(ctx, error);
  if (!rc) rc = fc3dgpu_ctx_get_r_u(ctx, NULL, velocity);
  fc3dgpu_ctx_destroy(ctx);
  if (rc) return rc;
  return *error > tolerance ? 1 : 0;
}

int fc3dgpu_nsgs_batch(int nproblems, FrictionContactProblem **problems, double **reactions, double **velocities,
                       SolverOptions *options, int *info) {
  if (nproblems < 0 || (nproblems > 0 && (!problems || !reactions || !velocities || !info))) {
    fc3dgpu_set_error("fc3dgpu_nsgs_batch: invalid argument");
    return NUMERICS_ERR_INVALID_ARGUMENT;
  }
  int worst = 0;
  for (int k = 0; k < nproblems; k++) {
    fc3dgpu_release(options);
    info[k] = fc3dgpu_nsgs(problems[k], reactions[k], velocities[k], options);
    if (info[k] < worst) worst = info[k];
  }
  fc3dgpu_release(options);
  return worst < 0 ? worst : 0;
}
