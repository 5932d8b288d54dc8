/* rfc3dgpu: GB300 coloured NSGS for the 3D rolling-friction contact problem
 * (5 components per contact: normal, two tangential, two rolling), a
 * drop-in solver beside the reference's SICONOS_ROLLING_FRICTION_3D_NSGS
 * (RollingFrictionContact/rolling_friction_3d_nsgs.c:285-615).
 *
 * Same algorithm as the reference with its default options: per contact
 * q_loc = q_i + sum_{j != i} W_ij r_j (the dense matrix's row sums in
 * column order, as the reference forms them), the take-off test, the
 * one-contact direct nonsmooth Newton on the rolling natural map (at most 10
 * iterations, tolerance 1e-12, rho = 1 / largest eigenvalue of W_ii), the
 * light error and LIGHT_WITH_FULL_FINAL with the reference's tolerance
 * manager (including the local-tolerance tightening), and
 * rolling_friction_3d_compute_error.  Contacts are visited in colour order:
 * the FP64 iterates are those of the reference's sequential sweep in that
 * order, bit for bit.  All sweeps of a solve run in one cooperative launch
 * with a grid barrier between colours and the convergence logic on the
 * device.  Mixed precision (the solver-level default, iparam[23] = 0): FP32
 * sweeps of the same loop first (one-contact tolerance 1e-6), until the
 * light error drops below dparam[23] (0: max(tol, 1e-6)) or stalls for
 * dparam[25] sweeps (0: 64), then the reference's FP64 loop from their
 * iterate; iparam[23] = 1 runs the FP64 loop only.  iparam[27] / [28] report
 * the FP32 and FP64 sweeps. 
 *
 * Buffers of the solver-level calls are HOST memory owned by the caller. */
#ifndef RFC3DGPU_H
#define RFC3DGPU_H

#ifdef FC3DGPU_USE_SICONOS_HEADERS
#include "RollingFrictionContactProblem.h"
#endif
#include "fc3dgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* New solver id in the free range of the 3D rolling-friction solvers
 * (RollingFrictionContact_options.h:61-80 uses 3000-3005 and 3010). */
#define SICONOS_ROLLING_FRICTION_3D_NSGS_GPU 3020

/* Registry-facing functions, shapes as rolling_friction_3d_nsgs's wrappers
 * (rolling_friction_3d_nsgs.c:670-697).  Options the GPU solver does not
 * implement (shuffle, freezing, relaxation, filter, error evaluations other
 * than LIGHT_WITH_FULL_FINAL, internal-error strategies other than
 * GIVEN_VALUE, local solvers other than ONECONTACT_NSN with the natural map
 * and the spectral-norm rho) give NUMERICS_ERR_NOT_IMPLEMENTED. */
int rfc3dgpu_nsgs(RollingFrictionContactProblem *problem, double *reaction, double *velocity,
                  SolverOptions *options);
int rfc3dgpu_nsgs_solve_wrap(void *problem, double *reaction, double *velocity, SolverOptions *options);
int rfc3dgpu_nsgs_init_wrap(void *problem, SolverOptions *options);
void rfc3dgpu_nsgs_free_wrap(void *problem, SolverOptions *options);
/* rolling_friction_3d_nsgs_set_default (rolling_friction_3d_nsgs.c:617-668)
 * with the one-contact NSN defaults (10 iterations, tolerance 1e-12, natural
 * map, spectral-norm rho). */
void rfc3dgpu_nsgs_set_default(SolverOptions *options);
SolverOptions *rfc3dgpu_options_create(void);
void rfc3dgpu_release(SolverOptions *options);
void rfc3dgpu_options_delete(SolverOptions *options);
/* rolling_friction_3d_driver (rolling_friction_3d_driver.c:56-135) for this
 * solver id: checks, the trivial take-off case, dispatch. */
int rfc3dgpu_driver(RollingFrictionContactProblem *problem, double *reaction, double *velocity,
                    SolverOptions *options);
/* rolling_friction_3d_compute_error on the GPU; returns 1 when the error
 * exceeds tolerance, else 0 (<0 on failure). */
int rfc3dgpu_compute_error(RollingFrictionContactProblem *problem, double *reaction, double *velocity,
                           double tolerance, double norm_q, double *error);

/* Device-resident context. */
typedef struct rfc3dgpu_ctx rfc3dgpu_ctx;
rfc3dgpu_ctx *rfc3dgpu_ctx_create(int device);
void rfc3dgpu_ctx_destroy(rfc3dgpu_ctx *ctx);
/* W as block-CSR of 5x5 column-major blocks (any order within a row; the
 * sums follow ascending column order), q[5 nc], mu[nc], mu_r[nc];
 * colour_kind as for fc3dgpu_colour (0 = default). */
int rfc3dgpu_ctx_set_problem(rfc3dgpu_ctx *ctx, int nc, const int64_t *rowptr, const int64_t *colidx,
                             const double *blocks, const double *q, const double *mu, const double *mu_r,
                             int colour_kind);
int rfc3dgpu_ctx_set_r(rfc3dgpu_ctx *ctx, const double *r);
/* Solve from the context's reaction with the reference's defaults;
 * local_tol / local_max_iter are the one-contact Newton's (1e-12, 10 by
 * default).  *iters sweeps, *error the final error, *info 0 / 1, *ms device
 * time.  Output pointers may be NULL. */
int rfc3dgpu_ctx_solve(rfc3dgpu_ctx *ctx, double tol, int max_iter, double local_tol, int local_max_iter,
                       int *iters, double *error, int *info, double *ms);
int rfc3dgpu_ctx_get_r_u(rfc3dgpu_ctx *ctx, double *r, double *u);
int rfc3dgpu_ctx_compute_error(rfc3dgpu_ctx *ctx, double norm_q, double *error);
int rfc3dgpu_ctx_colours(rfc3dgpu_ctx *ctx, int32_t *colour);
int rfc3dgpu_ctx_trace(rfc3dgpu_ctx *ctx, double *out, int cap);
/* rho of each contact (contact order), as the solve uses it. */
int rfc3dgpu_ctx_rho(rfc3dgpu_ctx *ctx, double *rho);
/* 1: FP64 sweeps only (the context's default); 0: FP32 sweeps until the
 * light error drops below switch_tol (0: max(tol, 1e-6)) or makes no 1 %
 * progress for stall_window sweeps (0: 64), then the FP64 loop. */
int rfc3dgpu_ctx_set_precision(rfc3dgpu_ctx *ctx, int precision, double switch_tol, int stall_window);
/* FP32 and FP64 sweeps of the last solve. */
int rfc3dgpu_ctx_last_sweeps(rfc3dgpu_ctx *ctx, int *sweeps32, int *sweeps64);

#ifdef __cplusplus
}
#endif
#endif
