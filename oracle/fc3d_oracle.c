/* CPU restatement of the reference's FC3D NSGS path -- TEST INFRASTRUCTURE.
 *
 * This file is the oracle: only tests, the smoke check and the bench's CPU
 * baseline load it.  The product never links it.  It restates, in this
 * project's own code, the algorithm of the reference's default
 * SICONOS_FRICTION_3D_NSGS solve on a 3x3 block-sparse W:
 *
 *   fc3d_driver trivial case        fc3d_driver.c:51-71
 *   NSGS outer loop, general branch fc3d_nsgs.c:711-900 (error evaluation
 *                                   FULL with its frequency, LIGHT,
 *                                   LIGHT_WITH_FULL_FINAL or ADAPTIVE; local
 *                                   tolerance GIVEN_VALUE, ADAPTIVE or
 *                                   ADAPTIVE_N_CONTACT,
 *                                   fc3d_set_internalsolver_tolerance.c:31-63;
 *                                   relaxation, filter and freezing; no
 *                                   shuffle)
 *   light error                     fc3d_nsgs.c:80-96
 *   tolerance manager               tolerance_manager.h:63-241
 *   local q                         fc3d_local_problem_tools.c:48-63,
 *                                   SparseBlockMatrix.c:1431-1490
 *   AC rho (split spectral norm)    fc3d_AlartCurnier_functions.c:784-812
 *   hybrid local solver             fc3d_onecontact_nonsmooth_Newton_solvers.c:920-1015
 *   damped AC Newton + GP search    same file :562-854
 *   keep/discard, local error       same file :856-918
 *   AC function (STD)               fc3d_AlartCurnier_functions.c:506-646
 *   PLI projection solver           fc3d_projection.c:350-514
 *   cone projection                 projectionOnCone.c:32-49
 *   3x3 solve with partial pivoting op3x3.h:868-980
 *   fc3d_compute_error              fc3d_compute_error.c:42-122, SparseBlockMatrix.c:360-419
 *
 * Arithmetic follows the reference's operation order, and the file is built
 * with -ffp-contract=off, so on the same inputs it reproduces the reference
 * (built in oracle/_ref with the same flag) bit for bit; tests pin that.
 * Vector norms are plain sums of squares, as in the project's BLAS shim.
 *
 * One extension: `order` lets a caller visit contacts in a given order (for
 * instance grouped by colour), which is the sweep order of the coloured
 * GPU solver. */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ---------------- BLAS-1 as in the project's shim ---------------- */
static double nrm2(int n, const double *x) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s += x[i] * x[i];
  return sqrt(s);
}

/* ---------------- 3x3 helpers (op3x3.h semantics) ---------------- */
/* r += a v, a column-major; column by column as op3x3.h:342 */
static void mvp3x3(const double *a, const double *v, double *r) {
  r[0] += a[0] * v[0];
  r[1] += a[1] * v[0];
  r[2] += a[2] * v[0];
  r[0] += a[3] * v[1];
  r[1] += a[4] * v[1];
  r[2] += a[5] * v[1];
  r[0] += a[6] * v[2];
  r[1] += a[7] * v[2];
  r[2] += a[8] * v[2];
}

/* c = a b (column-major), op3x3.h:449 */
static void mm3x3(const double *a, const double *b, double *c) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c[i + 3 * j] = a[i] * b[3 * j] + a[i + 3] * b[1 + 3 * j] + a[i + 6] * b[2 + 3 * j];
}

int oracle_solve_3x3_gepp(const double *a, double *b) {
  double lp0, lp1, lp2, lm1, lm2, ln1, ln2, bl, bm, bn, f1, f2, s0, s1, s2, alp0;
  double a0 = a[0], a1 = a[1], a2 = a[2];
  double aa0 = fabs(a0), aa1 = fabs(a1), aa2 = fabs(a2);
  int p1 = aa0 >= aa1 ? (aa0 >= aa2 ? 0 : 2) : (aa1 >= aa2 ? 1 : 2);
  if (p1 == 0) {
    f1 = a1 / a0; f2 = a2 / a0; lp0 = a0; alp0 = fabs(a0); lp1 = a[3]; lp2 = a[6];
    lm1 = a[4] - f1 * lp1; lm2 = a[7] - f1 * lp2; ln1 = a[5] - f2 * lp1; ln2 = a[8] - f2 * lp2;
    bl = b[0]; bm = b[1] - f1 * bl; bn = b[2] - f2 * bl;
  } else if (p1 == 1) {
    f1 = a0 / a1; f2 = a2 / a1; lp0 = a1; alp0 = fabs(a1); lp1 = a[4]; lp2 = a[7];
    lm1 = a[3] - f1 * lp1; lm2 = a[6] - f1 * lp2; ln1 = a[5] - f2 * lp1; ln2 = a[8] - f2 * lp2;
    bl = b[1]; bm = b[0] - f1 * bl; bn = b[2] - f2 * bl;
  } else {
    f1 = a0 / a2; f2 = a1 / a2; lp0 = a2; alp0 = fabs(a2); lp1 = a[5]; lp2 = a[8];
    lm1 = a[3] - f1 * lp1; lm2 = a[6] - f1 * lp2; ln1 = a[4] - f2 * lp1; ln2 = a[7] - f2 * lp2;
    bl = b[2]; bm = b[0] - f1 * bl; bn = b[1] - f2 * bl;
  }
  if (alp0 <= DBL_EPSILON) return 1;
  double alm1 = fabs(lm1), aln1 = fabs(ln1);
  if (alm1 >= aln1) {
    if (alm1 < DBL_EPSILON) return 1;
    f1 = ln1 / lm1;
    s2 = (bn - f1 * bm) / (ln2 - f1 * lm2);
    s1 = (bm - lm2 * s2) / lm1;
  } else {
    if (aln1 < DBL_EPSILON) return 1;
    f1 = lm1 / ln1;
    s2 = (bm - f1 * bn) / (lm2 - f1 * ln2);
    s1 = (bn - ln2 * s2) / ln1;
  }
  s0 = (bl - s1 * lp1 - s2 * lp2) / lp0;
  b[0] = s0;
  b[1] = s1;
  b[2] = s2;
  return 0;
}

/* ---------------- cone projection and errors ---------------- */
unsigned oracle_projection_on_cone(double *r, double mu) {
  double normT = sqrt(r[1] * r[1] + r[2] * r[2]);
  if (mu * normT <= -r[0]) {
    r[0] = 0.0;
    r[1] = 0.0;
    r[2] = 0.0;
    return 0;
  } else if (normT <= mu * r[0]) {
    return 1;
  } else {
    double mu2 = mu * mu;
    r[0] = (mu * normT + r[0]) / (mu2 + 1.0);
    r[1] = mu * r[0] * r[1] / normT;
    r[2] = mu * r[0] * r[2] / normT;
    return 2;
  }
}

static void unitary_error(const double r[3], const double u[3], double mu, double *error) {
  double w[3];
  w[0] = r[0] - u[0] - mu * sqrt(u[1] * u[1] + u[2] * u[2]);
  w[1] = r[1] - u[1];
  w[2] = r[2] - u[2];
  oracle_projection_on_cone(w, mu);
  w[0] = r[0] - w[0];
  w[1] = r[1] - w[1];
  w[2] = r[2] - w[2];
  *error += w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
}

/* fc3d_compute_error: u = q + W r, relative natural-map error. */
double oracle_fc3d_compute_error(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                                 const double *q, const double *mu, const double *r, double *u, double norm_q) {
  int n = 3 * nc;
  memcpy(u, q, sizeof(double) * (size_t)n);
  for (int i = 0; i < nc; i++)
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) mvp3x3(&blocks[9 * k], &r[3 * colidx[k]], &u[3 * i]);
  double e = 0.0;
  for (int i = 0; i < nc; i++) unitary_error(&r[3 * i], &u[3 * i], mu[i], &e);
  e = sqrt(e);
  double nr = nrm2(n, r), nu = nrm2(n, u);
  double scal = fmax(norm_q, fmax(nr, nu));
  if (fabs(scal) > DBL_EPSILON) e /= scal;
  return e;
}

/* ---------------- Alart-Curnier STD function ---------------- */
void oracle_ac_std(const double R[3], const double v[3], double mu, const double rho[3], double F[3], double *A,
                   double *B) {
  double RhoN = rho[0], RhoT = rho[1];
  double RVN = R[0] - RhoN * v[0];
  double RVT = R[1] - RhoT * v[1];
  double RVS = R[2] - RhoT * v[2];
  double RV = sqrt(RVT * RVT + RVS * RVS);
  double Radius;
  if (A) {
    A[3] = 0.; A[6] = 0.; A[1] = 0.; A[2] = 0.;
  }
  if (B) {
    B[3] = 0.; B[6] = 0.; B[1] = 0.; B[2] = 0.;
  }
  if (RVN > 0.0) {
    Radius = mu * RVN;
    F[0] = RhoN * v[0];
    if (A && B) {
      A[0] = RhoN;
      B[0] = 0.0;
    }
  } else {
    Radius = 0.0;
    F[0] = R[0];
    if (A && B) {
      A[0] = 0.0;
      B[0] = 1.0;
    }
  }
  if (RV <= Radius) {
    F[1] = RhoT * v[1];
    F[2] = RhoT * v[2];
    if (A && B) {
      A[4] = RhoT; A[7] = 0.0; A[5] = 0.0; A[8] = RhoT;
      B[1] = 0.0; B[4] = 0.0; B[7] = 0.0; B[2] = 0.0; B[5] = 0.0; B[8] = 0.0;
    }
  } else if (RV > Radius) {
    if (Radius > 0) {
      double RV1 = 1.0 / RV;
      F[1] = R[1] - Radius * RVT * RV1;
      F[2] = R[2] - Radius * RVS * RV1;
      if (A && B) {
        double RV3 = RV1 * RV1 * RV1;
        double GTT = RV1 - RVT * RVT * RV3;
        double GTS = -RVT * RVS * RV3;
        double GST = GTS;
        double GSS = RV1 - RVS * RVS * RV3;
        A[1] = mu * RhoN * RVT * RV1;
        A[2] = mu * RhoN * RVS * RV1;
        A[4] = GTT * RhoT * Radius;
        A[7] = GTS * RhoT * Radius;
        A[5] = GST * RhoT * Radius;
        A[8] = GSS * RhoT * Radius;
        B[1] = -mu * RVT * RV1;
        B[4] = 1.0 - GTT * Radius;
        B[7] = -GTS * Radius;
        B[2] = -mu * RVS * RV1;
        B[5] = -GST * Radius;
        B[8] = 1.0 - GSS * Radius;
      }
    } else {
      F[1] = R[1];
      F[2] = R[2];
      if (A && B) {
        A[4] = 0.0; A[7] = 0.0; A[5] = 0.0; A[8] = 0.0;
        B[1] = 0.0; B[4] = 1.0; B[7] = 0.0; B[2] = 0.0; B[5] = 0.0; B[8] = 1.0;
      }
    }
  }
}

/* ---------------- local solver ---------------- */
typedef struct {
  const double *M; /* diagonal block, column-major */
  double q[3];     /* local q */
  double mu;
  const double *rho; /* AC rho[3] */
  double *rho_pli;   /* PLI rho, persists across sweeps */
  double tol;        /* local tolerance */
  int newton_max;    /* 100 */
  int pli_max;       /* 100 */
  int ls_max;        /* 10 */
  double residual;   /* SOLVER_RESIDUAL of the local options */
} Local;

static double local_error(const Local *L, const double *r) {
  double nq = nrm2(3, L->q);
  double v[3] = {L->q[0], L->q[1], L->q[2]};
  mvp3x3(L->M, r, v);
  double e = 0.0;
  unitary_error(r, v, L->mu, &e);
  e = sqrt(e);
  if (fabs(nq) > DBL_EPSILON) e /= nq;
  return e;
}

static void line_search_gp(const Local *L, double *t_opt, const double r[3], const double dR[3], double *F,
                           const double *A, const double *B, double *v) {
  double alpha = *t_opt, inf = 1e20, amin = 0.0, amax = inf, m1 = 0.1, m2 = 0.9;
  const double *M = L->M;
  double q0 = 0.5 * (((0.0 + F[0] * F[0]) + F[1] * F[1]) + F[2] * F[2]);
  double tmp[3], AWB[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      AWB[i + 3 * j] = 0.0;
      for (int k = 0; k < 3; k++) AWB[i + 3 * j] += A[i + 3 * k] * M[k + j * 3];
      AWB[i + 3 * j] += B[i + 3 * j];
    }
  for (int i = 0; i < 3; i++) {
    tmp[i] = 0.0;
    for (int j = 0; j < 3; j++) tmp[i] += AWB[i + 3 * j] * dR[j];
  }
  double dqdt0 = 0.0;
  for (int i = 0; i < 3; i++) dqdt0 += F[i] * tmp[i];
  for (int it = 0; it < L->ls_max; it++) {
    for (int i = 0; i < 3; i++) tmp[i] = r[i] + alpha * dR[i];
    for (int i = 0; i < 3; i++) v[i] = M[i] * tmp[0] + L->q[i] + M[i + 3] * tmp[1] + M[i + 6] * tmp[2];
    oracle_ac_std(tmp, v, L->mu, L->rho, F, NULL, NULL);
    double qv = 0.5 * (((0.0 + F[0] * F[0]) + F[1] * F[1]) + F[2] * F[2]);
    double slope = (qv - q0) / alpha;
    int C1 = (slope >= m2 * dqdt0), C2 = (slope <= m1 * dqdt0);
    if (C1 && C2) {
      *t_opt = alpha;
      return;
    } else if (!C1) {
      amin = alpha;
    } else {
      amax = alpha;
    }
    if (alpha < inf)
      alpha = 0.5 * (amin + amax);
    else
      alpha = 10 * alpha;
  }
  *t_opt = alpha;
}

/* returns info (0 converged) */
static int newton_damped(Local *L, double *r) {
  double nq = sqrt(L->q[0] * L->q[0] + L->q[1] * L->q[1] + L->q[2] * L->q[2]);
  double nrel = 1.0;
  if (nq > DBL_EPSILON) nrel /= nq;
  const double *M = L->M;
  double dR[3] = {0., 0., 0.}, F[3] = {0., 0., 0.};
  double A[9] = {0}, B[9] = {0}, AWB[9] = {0};
  double v[3] = {L->q[0], L->q[1], L->q[2]};
  mvp3x3(M, r, v);
  int itermax = L->newton_max, inew = 0;
  double t = 1., t_opt = 1., t_init = 1.;
  oracle_ac_std(r, v, L->mu, L->rho, F, NULL, NULL);
  L->residual = sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]) * nrel;
  if (L->residual < L->tol) return 0;
  for (inew = 1; inew < itermax; ++inew) {
    oracle_ac_std(r, v, L->mu, L->rho, F, A, B);
    mm3x3(A, M, AWB);
    for (int e = 0; e < 9; e++) AWB[e] += B[e];
    for (int e = 0; e < 9; e++) AWB[e] *= -1.;
    dR[0] = F[0];
    dR[1] = F[1];
    dR[2] = F[2];
    int info3 = oracle_solve_3x3_gepp(AWB, dR);
    if (info3) {
      dR[0] = 0;
      dR[1] = 0;
      dR[2] = 0;
    }
    if (!info3) {
      t_opt = t_init;
      line_search_gp(L, &t_opt, r, dR, F, A, B, v);
      t = t_opt;
    }
    r[0] = r[0] + t * dR[0];
    r[1] = r[1] + t * dR[1];
    r[2] = r[2] + t * dR[2];
    v[0] = L->q[0];
    v[1] = L->q[1];
    v[2] = L->q[2];
    mvp3x3(M, r, v);
    oracle_ac_std(r, v, L->mu, L->rho, F, NULL, NULL);
    L->residual = sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]) * nrel;
    if (info3) break;
    if (L->residual < L->tol) return 0;
    if (sqrt(dR[0] * dR[0] + dR[1] * dR[1] + dR[2] * dR[2]) < 10 * DBL_EPSILON) return 1;
  }
  return 1;
}

static int pli_solve(Local *L, double *r) {
  const double *M = L->M;
  double mu = L->mu, rho = *L->rho_pli, rho_k;
  double vel[3], vel_k[3], r_k[3];
  double localerror = 1.0, localerror_k, a1 = 0, a2 = 0;
  int localiter = 0, ls_itermax = 10;
  double tau = 2.0 / 3.0, tauinv = 3.0 / 2.0, Lc = 0.9, Lmin = 0.3;
  while ((localerror > L->tol) && (localiter < L->pli_max)) {
    localiter++;
    localerror_k = localerror;
    r_k[0] = r[0];
    r_k[1] = r[1];
    r_k[2] = r[2];
    for (int i = 0; i < 3; i++) vel_k[i] = M[i] * r[0] + L->q[i] + M[i + 3] * r[1] + M[i + 6] * r[2];
    int ls = 0, success = 0;
    rho_k = rho / tau;
    double normUT = sqrt(vel_k[1] * vel_k[1] + vel_k[2] * vel_k[2]);
    while (!success && (ls < ls_itermax)) {
      rho_k = rho_k * tau;
      r[0] = r_k[0] - rho_k * (vel_k[0] + mu * normUT);
      r[1] = r_k[1] - rho_k * vel_k[1];
      r[2] = r_k[2] - rho_k * vel_k[2];
      oracle_projection_on_cone(r, mu);
      for (int i = 0; i < 3; i++) vel[i] = M[i] * r[0] + L->q[i] + M[i + 3] * r[1] + M[i + 6] * r[2];
      a1 = sqrt((vel_k[0] - vel[0]) * (vel_k[0] - vel[0]) + (vel_k[1] - vel[1]) * (vel_k[1] - vel[1]) +
                (vel_k[2] - vel[2]) * (vel_k[2] - vel[2]));
      a2 = sqrt((r_k[0] - r[0]) * (r_k[0] - r[0]) + (r_k[1] - r[1]) * (r_k[1] - r[1]) +
                (r_k[2] - r[2]) * (r_k[2] - r[2]));
      success = (rho_k * a1 <= Lc * a2) ? 1 : 0;
      ls++;
    }
    localerror = 0.0;
    unitary_error(r, vel, mu, &localerror);
    if ((rho_k * a1 < Lmin * a2) && (localerror < localerror_k))
      rho = rho_k * tauinv;
    else
      rho = rho_k;
  }
  *L->rho_pli = rho;
  L->residual = localerror;
  return localerror > L->tol ? 1 : 0;
}

static void keep_or_discard(Local *L, double *r, double *rb, double *cur) {
  double e = local_error(L, r);
  int bad = isnan(L->residual) || isinf(L->residual);
  if (bad) {
    r[0] = rb[0]; r[1] = rb[1]; r[2] = rb[2];
  } else if (e <= L->tol || e <= *cur) {
    *cur = e;
    rb[0] = r[0]; rb[1] = r[1]; rb[2] = r[2];
  } else {
    r[0] = rb[0]; r[1] = rb[1]; r[2] = rb[2];
  }
}

/* fc3d_onecontact_nonsmooth_Newton_solvers_solve with OC_NSN_GP_HYBRID and
 * NSN_AND_PLI_NSN_LOOP, max_loop 1 */
static void local_solve(Local *L, double *r) {
  if (L->q[0] > -DBL_EPSILON) {
    r[0] = 0.0;
    r[1] = 0.0;
    r[2] = 0.0;
    L->residual = 0.0;
    return;
  }
  double rb[3] = {r[0], r[1], r[2]};
  double cur = local_error(L, r);
  newton_damped(L, r);
  keep_or_discard(L, r, rb, &cur);
  if (cur <= L->tol) {
    L->residual = cur;
    return;
  }
  int loop = 0, max_loop = 1;
  while (loop < max_loop && cur >= L->tol) {
    loop++;
    pli_solve(L, r);
    keep_or_discard(L, r, rb, &cur);
    if (cur < L->tol) break;
    newton_damped(L, r);
    keep_or_discard(L, r, rb, &cur);
  }
  L->residual = cur;
}

static void ac_rho_split_spectral(const double *M, double rho[3]) {
  double sw = M[1 + 1 * 3] + M[2 + 2 * 3];
  double dw = sw * sw - 4.0 * (sw - M[2 + 1 * 3] + M[1 + 2 * 3]);
  if (dw > 0.0)
    dw = sqrt(dw);
  else
    dw = 0.0;
  rho[0] = 1.0 / M[0];
  rho[1] = 2.0 / (sw + dw);
  rho[2] = rho[1];
}

/* ---------------- NSGS driver ---------------- */
typedef struct {
  double user_tol, working_tol, min_tol, local_tol;
} TolMgr;

/* The NSGS options beyond the defaults that the loop below follows
 * (fc3d_nsgs.c:711-900, the general branch): the error evaluation
 * (SICONOS_NSGS_ERROR_EVALUATION_FULL 0, LIGHT 1, LIGHT_WITH_FULL_FINAL 2,
 * ADAPTIVE 3, NonSmoothGaussSeidel_options.h:125-143), the full-error
 * frequency of FULL (calculateFullErrorAdaptiveInterval, fc3d_nsgs.c:392-412),
 * and the local tolerance strategy applied at the start of each iteration
 * (fc3d_set_internalsolver_tolerance.c:31-63: ADAPTIVE 0, GIVEN_VALUE 1,
 * ADAPTIVE_N_CONTACT 2) with its ratio (dparam INTERNAL_ERROR_RATIO); and
 * per contact the relaxation of the new reaction (performRelaxation_3,
 * fc3d_nsgs.c:73-78, before its light-error term) and the filter that keeps
 * the old reaction when the local solver's residual is not finite or above
 * 1 (acceptLocalReactionFiltered, fc3d_nsgs.c:338-389); and contact freezing
 * (fc3d_nsgs.c:719-810): from the 10th iteration a contact whose light-error
 * term is small against its reaction, or whose reaction is small against the
 * last light error's |r|, is skipped for `freeze` sweeps, its stored term
 * still summed; all counters reset when nc - 1 contacts are frozen. */
typedef struct {
  int err_mode, freq, strategy;
  double ratio;
  int relax, filter; /* RELAXATION == TRUE, FILTER_LOCAL_SOLUTION == TRUE */
  double omega;      /* RELAXATION_VALUE */
  int freeze;        /* FREEZING_CONTACT: sweeps a converged contact is skipped */
} NsgsOpts;

/* Returns info: 0 converged, 1 not converged, -20 max iterations (and the
 * driver's trivial-case 0).  r is the warm start on entry.  *u_written
 * (optional) tells whether u was written: the reference computes u only
 * with the full error, so the LIGHT and ADAPTIVE evaluations leave it as
 * given, FULL with a frequency leaves the u of the last evaluated iterate. */
static int nsgs_impl(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks, const double *q,
                     const double *mu, double *r, double *u, double tol, int maxiter, const int32_t *order,
                     const NsgsOpts *op, int *iters, double *err, double *trace, int trace_cap, int *trace_len,
                     int *u_written) {
  int n = 3 * nc;
  if (iters) *iters = 0;
  if (err) *err = 0.0;
  if (trace_len) *trace_len = 0;
  if (u_written) *u_written = 0;
  /* driver trivial case */
  int trivial = 1;
  for (int i = 0; i < nc; i++)
    if (q[3 * i] < -DBL_EPSILON) {
      trivial = 0;
      break;
    }
  if (trivial) {
    memcpy(u, q, sizeof(double) * (size_t)n);
    memset(r, 0, sizeof(double) * (size_t)n);
    if (u_written) *u_written = 1;
    return 0;
  }
  double norm_q = nrm2(n, q);
  /* per-contact state */
  int64_t *diag = (int64_t *)malloc(sizeof(int64_t) * (size_t)nc);
  double *rho = (double *)malloc(sizeof(double) * 3 * (size_t)nc);
  double *rho_pli = (double *)malloc(sizeof(double) * (size_t)nc);
  for (int i = 0; i < nc; i++) {
    diag[i] = -1;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++)
      if (colidx[k] == i) {
        diag[i] = k;
        break;
      }
    if (diag[i] >= 0) ac_rho_split_spectral(&blocks[9 * diag[i]], &rho[3 * i]);
    rho_pli[i] = 1.0;
  }
  const double local_tol0 = 1e-14;
  TolMgr tm = {tol, tol, DBL_EPSILON * 1e-6, local_tol0};
  double tolerance = tm.working_tol;
  double incr_error = INFINITY, full_error = INFINITY;
  int hasNotConverged = 1, iter = 0;
  int tlen = 0;
  Local L;
  L.newton_max = 100;
  L.pli_max = 100;
  L.ls_max = 10;
  /* freezing state: counters, each contact's last light-error term, and |r|
   * of the last light error (1e24 before any) */
  unsigned *frozen = NULL;
  double *le2 = NULL, norm_r = 1e24;
  if (op->freeze > 0) {
    frozen = (unsigned *)calloc((size_t)nc, sizeof(unsigned));
    le2 = (double *)calloc((size_t)nc, sizeof(double));
  }
  while (iter < maxiter && hasNotConverged > 0) {
    ++iter;
    double light = 0.0;
    const double tmp = (double)nc * (double)nc / 1000.;
    const double crit1 = tolerance * tolerance / tmp, crit2 = norm_r * norm_r / tmp;
    if (frozen) {
      unsigned nfrozen = 0;
      for (int i = 0; i < nc; i++)
        if (frozen[i] > 0) nfrozen++;
      if ((size_t)nfrozen >= (size_t)nc - 1)
        for (int i = 0; i < nc; i++) frozen[i] = 0;
    }
    /* fc3d_set_internalsolver_tolerance: the local solver's tolerance from
     * the previous iteration's error */
    if (op->strategy == 0)
      tm.local_tol = fmax(incr_error / op->ratio, tol / nc);
    else if (op->strategy == 2)
      tm.local_tol = incr_error / (op->ratio * nc);
    for (int ii = 0; ii < nc; ii++) {
      int c = order ? order[ii] : ii;
      if (frozen && frozen[c] > 0) {
        frozen[c] -= 1;
        light += le2[c];
        continue;
      }
      L.M = &blocks[9 * diag[c]];
      L.q[0] = q[3 * c];
      L.q[1] = q[3 * c + 1];
      L.q[2] = q[3 * c + 2];
      for (int64_t k = rowptr[c]; k < rowptr[c + 1]; k++)
        if (colidx[k] != c) mvp3x3(&blocks[9 * k], &r[3 * colidx[k]], L.q);
      L.mu = mu[c];
      L.rho = &rho[3 * c];
      L.rho_pli = &rho_pli[c];
      L.tol = tm.local_tol;
      double lr[3] = {r[3 * c], r[3 * c + 1], r[3 * c + 2]};
      local_solve(&L, lr);
      if (op->relax) {
        lr[0] = op->omega * lr[0] + (1.0 - op->omega) * r[3 * c];
        lr[1] = op->omega * lr[1] + (1.0 - op->omega) * r[3 * c + 1];
        lr[2] = op->omega * lr[2] + (1.0 - op->omega) * r[3 * c + 2];
      }
      double d0 = r[3 * c] - lr[0], d1 = r[3 * c + 1] - lr[1], d2 = r[3 * c + 2] - lr[2];
      const double e2 = d0 * d0 + d1 * d1 + d2 * d2;
      light += e2;
      if (frozen) {
        le2[c] = e2;
        const double sq = lr[0] * lr[0] + lr[1] * lr[1] + lr[2] * lr[2];
        if ((e2 <= crit1 * sq || sq <= crit2) && iter >= 10) frozen[c] = (unsigned)op->freeze;
      }
      if (op->filter && (isnan(L.residual) || isinf(L.residual) || L.residual > 1.0)) continue;
      r[3 * c] = lr[0];
      r[3 * c + 1] = lr[1];
      r[3 * c + 2] = lr[2];
    }
    if (op->err_mode == 1) {
      /* LIGHT: the light error against the working tolerance */
      incr_error = sqrt(light);
      double nr = nrm2(n, r);
      norm_r = nr;
      if (fabs(nr) > DBL_EPSILON) incr_error /= nr;
      hasNotConverged = incr_error < tolerance ? 0 : 1;
    } else if (op->err_mode == 2) {
      /* LIGHT_WITH_FULL_FINAL: light error, then check_convergence_with_adaptation */
      incr_error = sqrt(light);
      double nr = nrm2(n, r);
      norm_r = nr;
      if (fabs(nr) > DBL_EPSILON) incr_error /= nr;
      if (incr_error >= tolerance) {
        hasNotConverged = 1;
      } else {
        full_error = oracle_fc3d_compute_error(nc, rowptr, colidx, blocks, q, mu, r, u, norm_q);
        if (u_written) *u_written = 1;
        if (full_error <= tm.user_tol) {
          hasNotConverged = 0;
        } else if (incr_error < 1e-15 || incr_error < DBL_EPSILON * 100.0) {
          double nt = fmax(tm.local_tol / 100.0, tm.min_tol);
          tm.local_tol = nt;
          hasNotConverged = 1;
        } else {
          if (full_error > 0.0 && incr_error > 0.0) {
            double ratio = incr_error / full_error;
            double nt = ratio * tm.user_tol;
            double user_min = tm.user_tol * 1e-6;
            double mint = user_min > tm.min_tol ? user_min : tm.min_tol;
            if (nt < mint) nt = mint;
            if (nt > 0.0 && nt < tolerance) tolerance = nt;
          }
          hasNotConverged = 1;
        }
        if (!(tolerance > 0.0)) break;
      }
    } else if (op->err_mode == 0) {
      /* FULL: the full error every iteration, or every freq iterations
       * (1e24 between evaluations) */
      full_error = 1e24;
      if (op->freq <= 0 || iter % op->freq == 0) {
        full_error = oracle_fc3d_compute_error(nc, rowptr, colidx, blocks, q, mu, r, u, norm_q);
        if (u_written) *u_written = 1;
      }
      incr_error = full_error;
      hasNotConverged = full_error < tolerance ? 0 : 1;
    }
    /* ADAPTIVE (3): the loop has no branch for it; it runs to the budget */
    if (trace && tlen < trace_cap) trace[tlen] = incr_error;
    tlen++;
  }
  if (op->err_mode == 2) {
    full_error = oracle_fc3d_compute_error(nc, rowptr, colidx, blocks, q, mu, r, u, norm_q);
    if (u_written) *u_written = 1;
    hasNotConverged = full_error < tol ? 0 : 1;
  }
  int info = hasNotConverged;
  if (iter == maxiter && hasNotConverged > 0) info = -20;
  if (iters) *iters = iter;
  if (err) *err = full_error;
  if (trace_len) *trace_len = tlen;
  free(diag);
  free(rho);
  free(rho_pli);
  free(frozen);
  free(le2);
  return info;
}

/* The reference's default options: LIGHT_WITH_FULL_FINAL, GIVEN_VALUE. */
int oracle_fc3d_nsgs(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks, const double *q,
                     const double *mu, double *r, double *u, double tol, int maxiter, const int32_t *order,
                     int *iters, double *err, double *trace, int trace_cap, int *trace_len) {
  const NsgsOpts op = {2, 0, 1, 10.0, 0, 0, 1.0, 0};
  return nsgs_impl(nc, rowptr, colidx, blocks, q, mu, r, u, tol, maxiter, order, &op, iters, err, trace, trace_cap,
                   trace_len, NULL);
}

/* Any error evaluation (0-3), frequency, local tolerance strategy (0-2),
 * relaxation, filter and freezing: opts6 = {err_mode, freq, strategy, relax,
 * filter, freeze}, dopts2 = {INTERNAL_ERROR_RATIO, RELAXATION_VALUE}. */
int oracle_fc3d_nsgs_opts(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                          const double *q, const double *mu, double *r, double *u, double tol, int maxiter,
                          const int32_t *order, const int32_t *opts6, const double *dopts2, int *iters, double *err,
                          double *trace, int trace_cap, int *trace_len, int *u_written) {
  const NsgsOpts op = {opts6[0], opts6[1], opts6[2], dopts2[0], opts6[3] == 1, opts6[4] == 1, dopts2[1], opts6[5]};
  return nsgs_impl(nc, rowptr, colidx, blocks, q, mu, r, u, tol, maxiter, order, &op, iters, err, trace, trace_cap,
                   trace_len, u_written);
}

/* One contact's local solve from the reference's default local options, for
 * unit tests of the local solver.  r in/out; returns the local residual. */
double oracle_local_solve(const double *M, const double *qloc, double mu, double *r, double *rho_pli, double tol) {
  double rho[3];
  ac_rho_split_spectral(M, rho);
  Local L;
  L.M = M;
  L.q[0] = qloc[0];
  L.q[1] = qloc[1];
  L.q[2] = qloc[2];
  L.mu = mu;
  L.rho = rho;
  L.rho_pli = rho_pli;
  L.tol = tol;
  L.newton_max = 100;
  L.pli_max = 100;
  L.ls_max = 10;
  local_solve(&L, r);
  return L.residual;
}
