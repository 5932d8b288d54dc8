/* fc2dgpu: GB300 coloured NSGS for the 2D Coulomb friction-contact problem,
 * as a drop-in solver beside the reference's SICONOS_FRICTION_2D_NSGS and
 * its CUDA variants (SICONOS_FRICTION_2D_NSGS_GRAPH_PERMUT_CUDA,
 * parallel/gpu/fc2d_nsgs_graph_permut_cuda.cu).
 *
 * The sweep is the reference's fc2d_nsgs (fc2d_nsgs.c:299-520): per contact
 * q_loc = q_i + sum_{j != i} W_ij r_j, the closed-form 2x2 local solve, the
 * light error, LIGHT_WITH_FULL_FINAL with fc2d_compute_error, info 0 / 1 as
 * the reference returns it.  Contacts are visited in colour order (contacts
 * of one colour share no W block), so the FP64 iterates are those of the
 * reference's sequential sweep run in that order, bit for bit.  One
 * thread-block cluster (up to 16 SMs; a cooperative grid over every SM when
 * a colour is larger than a cluster) runs all sweeps of a problem in one
 * launch, with a hardware barrier between colours and the convergence logic
 * on the device: no host round trip per sweep.
 *
 * Buffers of the solver-level calls are HOST memory owned by the caller. */
#ifndef FC2DGPU_H
#define FC2DGPU_H

#include "fc3dgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* New solver id in the free FC2D range (FrictionContact_options.h:60-73 uses
 * 400-411). */
#define SICONOS_FRICTION_2D_NSGS_GPU 412

/* Registry-facing functions, shapes as fc2d_nsgs's wrappers (fc2d_nsgs.c:
 * 800-825).  Options the GPU solver does not implement (shuffle, freezing,
 * other error evaluations) give NUMERICS_ERR_NOT_IMPLEMENTED. */
int fc2dgpu_nsgs(FrictionContactProblem *problem, double *reaction, double *velocity, SolverOptions *options);
int fc2dgpu_nsgs_solve_wrap(void *problem, double *reaction, double *velocity, SolverOptions *options);
int fc2dgpu_nsgs_init_wrap(void *problem, SolverOptions *options);
void fc2dgpu_nsgs_free_wrap(void *problem, SolverOptions *options);
/* fc2d_nsgs_set_default (fc2d_nsgs.c:787-792): no shuffle,
 * LIGHT_WITH_FULL_FINAL.  GPU knobs as for the 3D solver:
 * iparam[FC3DGPU_IPARAM_PRECISION] 0 = FP32 sweeps + FP64 polish (default),
 * 1 = FP64 sweeps only; dparam[FC3DGPU_DPARAM_SWITCH_TOL] and
 * dparam[FC3DGPU_DPARAM_STALL] the switch (see fc2dgpu_ctx_set_precision);
 * iparam[FC3DGPU_IPARAM_COLOURING] the colouring (0 = default).  Outputs:
 * iparam[FC3DGPU_IPARAM_SWEEPS_FP32 / _FP64], iparam[FC3DGPU_IPARAM_COLOURS],
 * dparam[FC3DGPU_DPARAM_MS_SOLVE]. */
void fc2dgpu_nsgs_set_default(SolverOptions *options);
/* Options as solver_options_create(SICONOS_FRICTION_2D_NSGS_GPU) gives them
 * once registered: max_iter 1000, tol 1e-4. */
SolverOptions *fc2dgpu_options_create(void);
/* Free the device copy of W the options hold between calls (as
 * fc3dgpu_release), and the options themselves. */
void fc2dgpu_release(SolverOptions *options);
void fc2dgpu_options_delete(SolverOptions *options);
/* fc2d_compute_error (fc2d_compute_error.c:40-140) on the GPU: velocity =
 * q + W reaction, *error the relative natural-map error; returns 1 when it
 * exceeds tolerance, else 0 (<0 on failure). */
int fc2dgpu_compute_error(FrictionContactProblem *problem, double *reaction, double *velocity, double tolerance,
                          double norm_q, double *error);
/* fc2d_driver (fc2d_driver.c:40-145) restricted to this solver id. */
int fc2dgpu_driver(FrictionContactProblem *problem, double *reaction, double *velocity, SolverOptions *options);

/* Device-resident context (W, q, mu uploaded once, solved many times). */
typedef struct fc2dgpu_ctx fc2dgpu_ctx;
fc2dgpu_ctx *fc2dgpu_ctx_create(int device);
void fc2dgpu_ctx_destroy(fc2dgpu_ctx *ctx);
/* W as block-CSR of 2x2 column-major blocks (every contact needs its
 * diagonal block), q[2 nc], mu[nc]; colour_kind as for fc3dgpu_colour.
 * Returns NUMERICS_ERR_INVALID_ARGUMENT on a bad structure. */
int fc2dgpu_ctx_set_problem(fc2dgpu_ctx *ctx, int nc, const int64_t *rowptr, const int64_t *colidx,
                            const double *blocks, const double *q, const double *mu, int colour_kind);
/* New q and mu for the structure and W values already in the context. */
int fc2dgpu_ctx_set_q_mu(fc2dgpu_ctx *ctx, const double *q, const double *mu);
int fc2dgpu_ctx_set_r(fc2dgpu_ctx *ctx, const double *r);
/* Solve from the context's reaction.  error_evaluation is the reference's
 * SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION value, with fc2d_nsgs's
 * meaning (fc2d_nsgs.c:438-448, :496-500): LIGHT_WITH_FULL_FINAL stops on
 * the light error confirmed by fc2d_compute_error and reports the latter;
 * LIGHT stops on and reports the light error; any other value evaluates no
 * error (max_iter sweeps, error INFINITY, info 1).  *iters sweeps, *info
 * 0 / 1 (1 at once, with error INFINITY, when a diagonal block's
 * determinant is below DBL_EPSILON, fc2d_nsgs.c:318-333), *ms the device
 * time.  Any output pointer may be NULL. */
int fc2dgpu_ctx_solve(fc2dgpu_ctx *ctx, double tol, int max_iter, int error_evaluation, int *iters, double *error,
                      int *info, double *ms);
/* Precision of the sweeps.  1 (a new context's default): FP64 sweeps only,
 * the reference's iterates bit for bit.  0: FP32 sweeps until the FP32
 * light error is below switch_tol (0 = max(tol, 1e-6)) or has not
 * reached a new low for stall_window sweeps (0 = 64), then the reference's
 * FP64 loop from that iterate on the remaining budget; FP64 is slow on this
 * GPU (about 64-cycle latency per operation, 550 for a division), FP32 an
 * order of magnitude faster.  Both phases run back to back on the device. */
int fc2dgpu_ctx_set_precision(fc2dgpu_ctx *ctx, int precision, double switch_tol, int stall_window);
/* FP32 and FP64 sweeps of the last solve. */
int fc2dgpu_ctx_last_sweeps(fc2dgpu_ctx *ctx, int *sweeps32, int *sweeps64);
/* Reaction and velocity in contact order; the velocity is the one the last
 * fc2d_compute_error produced (LIGHT_WITH_FULL_FINAL only).  Either may be
 * NULL. */
int fc2dgpu_ctx_get_r_u(fc2dgpu_ctx *ctx, double *r, double *u);
/* fc2d_compute_error of the context's reaction (the velocity it makes is
 * kept for fc2dgpu_ctx_get_r_u), relative to max(|r|, |u|, norm_q). */
int fc2dgpu_ctx_compute_error(fc2dgpu_ctx *ctx, double norm_q, double *error);
/* Colour of each contact and the number of colours (return value). */
int fc2dgpu_ctx_colours(fc2dgpu_ctx *ctx, int32_t *colour);
/* Launch shape of the sweep kernel: a thread-block cluster of
 * cluster_blocks blocks (1..16; -1: a cooperative grid over every SM) of
 * `threads` threads (32..512, a multiple of 32), the reactions kept in HBM
 * (reactions = 1) or replicated in every cluster block's shared memory (2,
 * up to 13,312 contacts); 0 picks each from the problem (the default).
 * fc2dgpu_ctx_launch_shape reports a grid as minus its block count.  The
 * iterates do not depend on the shape; the reduction order of the errors
 * does. */
int fc2dgpu_ctx_set_launch(fc2dgpu_ctx *ctx, int cluster_blocks, int threads, int reactions);
int fc2dgpu_ctx_launch_shape(fc2dgpu_ctx *ctx, int *cluster_blocks, int *threads, int *reactions);
/* Per-sweep light error of the last solve (cap entries); returns how many. */
int fc2dgpu_ctx_trace(fc2dgpu_ctx *ctx, double *out, int cap);

#ifdef __cplusplus
}
#endif
#endif
