/* gfc3dgpu: GB300 solver for the global 3D friction-contact problem
 * (GlobalFrictionContactProblem: M v = q + H r, u = H^T v + b, r in the
 * Coulomb cones of coefficients mu), as a drop-in beside the reference's
 * SICONOS_GLOBAL_FRICTION_3D_NSGS (gfc3d_nsgs.c:62-198, dispatched by
 * gfc3d_driver.c:171).
 *
 * The reference's iteration updates every contact from the same velocity
 * (a projected Jacobi step, despite its name): v = M^-1 (q + H r),
 * u = b + H^T v, r_c <- proj_K(r_c - (u_N + mu |u_T|, u_T)), then
 * gfc3d_compute_error (gfc3d_compute_error.c:38-160) after every iteration
 * (or every ERROR_EVALUATION_FREQUENCY iterations).  The GPU runs all
 * iterations of a solve in one cooperative launch: row products of H and
 * H^T from slot-major slabs, M^-1 by LU factors of the connected components
 * of M's pattern (a division by the diagonal when every component is one
 * degree of freedom), the error's norms reduced in a fixed order, and the
 * stop decision on the device.  FP64 without FMA contraction, in the
 * reference's operation order: r, u and v equal the reference's bit for bit
 * (its dense LU is an unblocked partial-pivoting LU, which the per-component
 * factors reproduce); the error's sums run in another order, so the error
 * agrees to rounding.
 *
 * Buffers of the solver-level calls are HOST memory owned by the caller. */
#ifndef GFC3DGPU_H
#define GFC3DGPU_H

#include "fc3dgpu.h"
#ifdef FC3DGPU_USE_SICONOS_HEADERS
#include "GlobalFrictionContactProblem.h"
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* New solver id in the free part of the GFC3D range
 * (FrictionContact_options.h:182-204 uses 600-618 and 620). */
#define SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU 619

/* gfc3d_nsgs (gfc3d_nsgs.c:62-198) on the GPU.  M and H may be stored dense
 * (NM_DENSE) or sparse-block (NM_SPARSE_BLOCK); NM_SPARSE gives
 * NUMERICS_ERR_NOT_IMPLEMENTED.  reaction (3 nc) and globalVelocity (n) are
 * the start on entry; on exit reaction, velocity = b + H^T v and
 * globalVelocity hold the last iterate, dparam[SICONOS_DPARAM_RESIDU] the
 * error, and the return value is the reference's info: 0 converged, 1 not,
 * -1 when no iteration ran (max_iter 0).  Like the reference, the iteration
 * count is not written to the options; options are the reference's:
 * iparam[SICONOS_IPARAM_MAX_ITER], dparam[SICONOS_DPARAM_TOL],
 * iparam[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION_FREQUENCY].  A singular
 * M gives NUMERICS_ERR_INVALID_ARGUMENT.  Negative returns other than -1 are
 * NUMERICS_ERR_* codes with a message in fc3dgpu_last_error(). */
int gfc3dgpu_nsgs(GlobalFrictionContactProblem *problem, double *reaction, double *velocity, double *globalVelocity,
                  SolverOptions *options);
/* Registry shapes (gfc3d_nsgs.c:210-230). */
int gfc3dgpu_nsgs_solve_wrap(void *problem, double *reaction, double *velocity, double *globalVelocity,
                             SolverOptions *options);
int gfc3dgpu_nsgs_init_wrap(void *problem, SolverOptions *options);
void gfc3dgpu_nsgs_free_wrap(void *problem, SolverOptions *options);
/* gfc3d_nsgs_set_default (gfc3d_nsgs.c:200-208): fc3d_nsgs_set_default's
 * values (tol 1e-4, error every iteration). */
void gfc3dgpu_nsgs_set_default(SolverOptions *options);
/* Options as solver_options_create(SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU)
 * gives them once registered: max_iter 1000, tol 1e-4. */
SolverOptions *gfc3dgpu_options_create(void);
/* Free the device context the options hold between calls, and the options. */
void gfc3dgpu_release(SolverOptions *options);
void gfc3dgpu_options_delete(SolverOptions *options);
/* gfc3d_driver (gfc3d_driver.c:77-120, :171-174) restricted to this solver
 * id: with no contact, globalVelocity = M^-1 q and 0. */
int gfc3dgpu_driver(GlobalFrictionContactProblem *problem, double *reaction, double *velocity,
                    double *globalVelocity, SolverOptions *options);
/* gfc3d_compute_error of (reaction, globalVelocity) on the GPU: writes
 * velocity = b + H^T v and *error; returns 1 when it exceeds tolerance,
 * else 0 (<0 on failure).  norm_q scales the equation residual as in the
 * reference; norm_b is unused, as there. */
int gfc3dgpu_compute_error(GlobalFrictionContactProblem *problem, double *reaction, double *velocity,
                           double *globalVelocity, double tolerance, double norm_q, double norm_b, double *error);

/* Device-resident context: M, H, q, b, mu uploaded once, solved many
 * times. */
typedef struct gfc3dgpu_ctx gfc3dgpu_ctx;
gfc3dgpu_ctx *gfc3dgpu_ctx_create(int device);
void gfc3dgpu_ctx_destroy(gfc3dgpu_ctx *ctx);
/* M (n x n) and H (n x 3 nc) as CSR: row pointers (n + 1), column indices
 * ascending within a row, values; q[n], b[3 nc], mu[nc].  M is factorised
 * on the device by the connected components of its pattern (at most
 * GFC3DGPU_MAX_COMPONENT degrees of freedom each).  Returns
 * NUMERICS_ERR_INVALID_ARGUMENT on a bad structure, a component too large
 * or a singular M. */
#define GFC3DGPU_MAX_COMPONENT 256
int gfc3dgpu_ctx_set_problem(gfc3dgpu_ctx *ctx, int64_t n, int nc, const int64_t *Mp, const int64_t *Mi,
                             const double *Mx, const int64_t *Hp, const int64_t *Hi, const double *Hx,
                             const double *q, const double *b, const double *mu);
/* Start of the next solve: reaction (3 nc) and global velocity (n); the
 * velocity only matters for a solve with max_iter 0.  Either may be NULL
 * (zeros). */
int gfc3dgpu_ctx_set_start(gfc3dgpu_ctx *ctx, const double *r, const double *v);
/* Solve from the context's start (then from the last iterate: a second
 * solve continues).  freq is ERROR_EVALUATION_FREQUENCY (0: every
 * iteration).  *iters iterations run, *error the reported error, *info the
 * reference's info, *ms the device time.  Any output may be NULL. */
int gfc3dgpu_ctx_solve(gfc3dgpu_ctx *ctx, double tol, int max_iter, int freq, int *iters, double *error, int *info,
                       double *ms);
/* The last iterate: reaction, local velocity u = b + H^T v, global velocity.
 * Any may be NULL. */
int gfc3dgpu_ctx_get(gfc3dgpu_ctx *ctx, double *r, double *u, double *v);
/* gfc3d_compute_error of the context's current (r, v) with the given |q|
 * (negative: |q| of the context's q); u is kept for gfc3dgpu_ctx_get. */
int gfc3dgpu_ctx_compute_error(gfc3dgpu_ctx *ctx, double norm_q, double *error);
/* Per-iteration error of the last solve (as the reference's loop sees it,
 * cap entries); returns how many. */
int gfc3dgpu_ctx_trace(gfc3dgpu_ctx *ctx, double *out, int cap);
/* Structure of the device problem: components of M, the largest one, 1 when
 * M^-1 is a division by the diagonal, the bytes one iteration moves at the
 * least (the unpadded arrays it streams, each once) and the grid size. */
int gfc3dgpu_ctx_info(gfc3dgpu_ctx *ctx, int *ncomp, int *max_component, int *diagonal, double *bytes_per_iteration,
                      int *grid);
/* Arithmetic of the row products: 0 (a new context's default) the
 * reference's, a multiply and an add each rounded, so r, u and v equal the
 * reference's bit for bit; 1 (opt-in) fused multiply-adds, which halve the
 * FP64 operations of the products (the kernel is bound by the FP64 pipe) and
 * give iterates equal to the reference's to rounding, not bit for bit.
 * Through the solver options: iparam[FC3DGPU_IPARAM_PRECISION] = 2 selects
 * the fused products, any other value the reference's. */
int gfc3dgpu_ctx_set_arithmetic(gfc3dgpu_ctx *ctx, int fused);
/* Poll limit of every grid-barrier wait (0: the default of 2^22 polls). */
int gfc3dgpu_ctx_spin_limit(gfc3dgpu_ctx *ctx, unsigned long long polls);

#ifdef __cplusplus
}
#endif
#endif
