/* Internal helpers shared by the host-side solver entry points (not part of
 * the C-ABI in include/). */
#ifndef FC3DGPU_BCSR_H
#define FC3DGPU_BCSR_H

#include <stdint.h>

#include "fc3dgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* W of a friction-contact problem as block-CSR of d x d column-major blocks */
typedef struct {
  int nc;
  long long nnzb;
  int64_t *rowptr;
  int64_t *colidx;
  double *blocks;
  const double *const *block; /* or one pointer per block (then blocks is NULL) */
  int borrowed;               /* arrays point into the caller's SBM, not owned */
} Bcsr;

/* Flat blocks: SBM storage whose blocks already sit back to back is viewed,
 * other SBM storage and dense storage are repacked. */
int fc3dgpu_bcsr_from_problem(const FrictionContactProblem *P, int d, Bcsr *out);
/* As fc3dgpu_bcsr_from_problem, but SBM storage with every block row filled
 * is viewed as is, blocks through its block pointer array (no pass over the
 * blocks; for fc3dgpu_ctx_update_W_ptrs). */
int fc3dgpu_bcsr_view(const FrictionContactProblem *P, int d, Bcsr *out);
void fc3dgpu_bcsr_free(Bcsr *b);
/* SolverOptions with iparam/dparam of the reference's size, max_iter and tol
 * set, as solver_options_create does. */
SolverOptions *fc3dgpu_options_alloc(int id, int max_iter, double tol);
void fc3dgpu_set_error(const char *fmt, ...);
/* |q| as fc3dgpu_ctx_set_q_mu computes it, and fc3dgpu_ctx_set_q_mu with
 * that value given (so the host can compute it while W uploads). */
double fc3dgpu_norm_q_host(const double *q, long long n);
int fc3dgpu_ctx_set_q_mu_norm(fc3dgpu_ctx *ctx, const double *q, const double *mu, double norm_q);

#ifdef __cplusplus
}
#endif
#endif
