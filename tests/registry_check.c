/* A Siconos user's program, unchanged but for the solver id: it reads a
 * friction-contact problem with the reference's reader, creates the options
 * with the reference's solver_options_create and solves through the
 * reference's fc3d_driver, which finds the GPU solver in the reference's
 * registry (the constructor of fc3d_nsgs_gpu_register.c, linked in).
 *
 * Prints one `key value` pair per line for tests/test_registry.py:
 *   name, solve_is_gpu, iparam/dparam defaults, info, iterations, residual,
 *   the reference's own fc3d_compute_error of the returned reaction (when
 *   the solve returned one) and the GPU library's last message.
 *
 * With a fifth argument (a GFC3D .dat file) it does the same for the global
 * solver: the registry entry of SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU, the
 * options the reference's solver_options_create gives it, and a solve
 * through the entry's solve3 (what gfc3d_driver's case for the id calls),
 * checked with the reference's own gfc3d_compute_error (keys prefixed g_).
 */
#define FC3DGPU_USE_SICONOS_HEADERS
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "FrictionContactProblem.h"
#include "FrictionContact_options.h"
#include "NonSmoothDrivers.h"
#include "SolverOptions.h"
#include "fc3d_compute_error.h"
#include "fc3dgpu.h"
#include "gfc3dgpu.h"
#include "GlobalFrictionContactProblem.h"
#include "gfc3d_compute_error.h"
#include "solver_registry.h"

int main(int argc, char **argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s problem.dat [tol max_iter]\n", argv[0]);
    return 2;
  }
  const double tol = argc > 2 ? atof(argv[2]) : 1e-8;
  const int max_iter = argc > 3 ? atoi(argv[3]) : 10000;
  FrictionContactProblem *problem = frictionContact_new_from_filename(argv[1]);
  if (!problem) {
    fprintf(stderr, "cannot read %s\n", argv[1]);
    return 2;
  }
  const SolverEntry *e = solver_registry_lookup(SICONOS_FRICTION_3D_NSGS_GPU);
  printf("registered %d\n", e != NULL);
  if (!e) return 3;
  printf("name %s\n", e->name);
  printf("solve_is_gpu %d\n", e->solve == fc3dgpu_nsgs_solve_wrap);
  SolverOptions *options = solver_options_create(SICONOS_FRICTION_3D_NSGS_GPU);
  if (!options) return 4;
  printf("solverId %d\n", options->solverId);
  printf("default_max_iter %d\n", options->iparam[SICONOS_IPARAM_MAX_ITER]);
  printf("default_tol %.17g\n", options->dparam[SICONOS_DPARAM_TOL]);
  printf("iparam_error_evaluation %d\n", options->iparam[SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION]);
  printf("internal_solver %d\n", options->numberOfInternalSolvers > 0 ? options->internalSolvers[0]->solverId : -1);
  options->dparam[SICONOS_DPARAM_TOL] = tol;
  options->iparam[SICONOS_IPARAM_MAX_ITER] = max_iter;
  const int n = problem->dimension * problem->numberOfContacts;
  double *r = calloc((size_t)n, sizeof(double));
  double *u = calloc((size_t)n, sizeof(double));
  const int info = fc3d_driver(problem, r, u, options);
  printf("info %d\n", info);
  printf("iterations %d\n", options->iparam[SICONOS_IPARAM_ITER_DONE]);
  printf("residual %.17g\n", options->dparam[SICONOS_DPARAM_RESIDU]);
  if (info >= 0) {
    double err = 0.0;
    double norm_q = 0.0;
    for (int i = 0; i < n; i++) norm_q += problem->q[i] * problem->q[i];
    fc3d_compute_error(problem, r, u, tol, options, sqrt(norm_q), &err);
    printf("reference_error %.17g\n", err);
  }
  printf("message %s\n", fc3dgpu_last_error());
  fc3dgpu_release(options);
  solver_options_delete(options);
  frictionContactProblem_free(problem);
  free(r);
  free(u);
  if (argc > 4) {
    GlobalFrictionContactProblem *gp = globalFrictionContact_new_from_filename(argv[4]);
    if (!gp) {
      fprintf(stderr, "cannot read %s\n", argv[4]);
      return 2;
    }
    const SolverEntry *g = solver_registry_lookup(SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU);
    printf("g_registered %d\n", g != NULL);
    if (!g) return 3;
    printf("g_name %s\n", g->name);
    printf("g_solve3_is_gpu %d\n", g->has_3var && g->solve3 == gfc3dgpu_nsgs_solve_wrap);
    SolverOptions *go = solver_options_create(SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU);
    printf("g_default_max_iter %d\n", go->iparam[SICONOS_IPARAM_MAX_ITER]);
    printf("g_default_tol %.17g\n", go->dparam[SICONOS_DPARAM_TOL]);
    go->dparam[SICONOS_DPARAM_TOL] = tol;
    go->iparam[SICONOS_IPARAM_MAX_ITER] = max_iter;
    const int m = 3 * gp->numberOfContacts, nd = gp->M->size0;
    double *gr = calloc((size_t)m, sizeof(double)), *gu = calloc((size_t)m, sizeof(double));
    double *gv = calloc((size_t)nd, sizeof(double));
    const int ginfo = g->solve3(gp, gr, gu, gv, go);
    printf("g_info %d\n", ginfo);
    printf("g_residual %.17g\n", go->dparam[SICONOS_DPARAM_RESIDU]);
    if (ginfo >= 0) {
      double err = 0.0, nq = 0.0, nb = 0.0;
      for (int i = 0; i < nd; i++) nq += gp->q[i] * gp->q[i];
      for (int i = 0; i < m; i++) nb += gp->b[i] * gp->b[i];
      gfc3d_compute_error(gp, gr, gu, gv, tol, go, sqrt(nq), sqrt(nb), &err);
      printf("g_reference_error %.17g\n", err);
    }
    printf("g_message %s\n", fc3dgpu_last_error());
    gfc3dgpu_release(go);
    solver_options_delete(go);
    globalFrictionContact_free(gp);
    free(gr);
    free(gu);
    free(gv);
  }
  return 0;
}
