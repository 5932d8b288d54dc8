/* CPU restatement of the reference's 3D rolling-friction NSGS -- TEST
 * INFRASTRUCTURE (the checker of the GPU rolling-friction solver; never the
 * product).
 *
 * Follows rolling_friction_3d_nsgs (RollingFrictionContact/
 * rolling_friction_3d_nsgs.c:285-615) with its default options
 * (rolling_friction_3d_nsgs_set_default :617-668: LIGHT_WITH_FULL_FINAL,
 * GIVEN_VALUE internal tolerance, no shuffle, freezing, filter or
 * relaxation; local solver SICONOS_ROLLING_FRICTION_3D_ONECONTACT_NSN with
 * its registry defaults, 10 iterations and tolerance 1e-12,
 * rolling_friction_3d_onecone_nonsmooth_Newton_solvers.c:543-582), on a
 * block-CSR W of 5x5 column-major blocks:
 *   - rho per contact = 1 / (largest eigenvalue of W_ii), the cyclic Jacobi
 *     iteration of eigvals_sym5x5_for_loop (linalg/op5x5.h:775-870);
 *   - W as the reference's rolling NSGS takes it, a dense matrix (its
 *     sparse-block diagonal extraction asserts, NumericsMatrix.c:1870): per
 *     sweep and contact q_loc = q_i + (sum over the row of W with the
 *     contact's own columns zeroed, in column order) as NM_row_prod_no_diag's
 *     dense branch (NumericsMatrix.c:385-412, one ddot per row); over the
 *     stored blocks of a row in ascending column order that is one running
 *     sum per component, added to q_i at the end; the take-off test q_loc,n > -DBL_EPSILON (:228-245); else
 *     the direct nonsmooth Newton on the rolling natural map (:344-505,
 *     rolling_naturalmap_functions.c:31-165, projectionOnRollingCone.c,
 *     5x5 GEPP of op5x5.h:642-700), with the reference's residual formulas
 *     as written (including the cubed third component after a Newton step);
 *   - the light error, determine_convergence_with_full_final with the
 *     local-tolerance tightening when the light error is below DBL_EPSILON
 *     (rolling_friction_3d_nsgs.c:243-285), and the final
 *     rolling_friction_3d_compute_error (rolling_friction_3d_compute_error.c:
 *     58-110: u = 1.0 q + 1.0 (W r), the dense dgemv's row sums over all
 *     columns, natural-map error relative to max(|q|, |r|, |u|)).
 * Blocks of a row must be stored in ascending column order (the dense
 * matrix's column order).
 * Norms are plain sums of squares in index order (the CBLAS shim the
 * reference is built with here); pow(x, 2) is the C library's, as in the
 * reference.  `order` (optional) is the contact visiting order of a sweep. */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { RC_DUAL = 0, RC_INSIDE, RC_FRICTION, RC_ROLLING, RC_FRICTION_ROLLING };

#define E(M, i, j) (M)[(i) + 5 * (j)]

static double nrm2(int64_t n, const double *x) {
  double s = 0.0;
  for (int64_t i = 0; i < n; i++) s += x[i] * x[i];
  return sqrt(s);
}

/* r += a v, column by column (mvp5x5, op5x5.h:229-275) */
static void mvp5(const double *a, const double *v, double *r) {
  for (int j = 0; j < 5; j++)
    for (int i = 0; i < 5; i++) r[i] += a[i + 5 * j] * v[j];
}

/* s += a v, columns in order: a block's share of the dense row sums */
static void acc5(const double *a, const double *v, double *s) {
  for (int k = 0; k < 5; k++)
    for (int i = 0; i < 5; i++) s[i] += a[i + 5 * k] * v[k];
}

/* c = a b, each entry one left-to-right sum (mm5x5) */
static void mm5(const double *a, const double *b, double *c) {
  for (int j = 0; j < 5; j++)
    for (int i = 0; i < 5; i++)
      E(c, i, j) = E(a, i, 0) * E(b, 0, j) + E(a, i, 1) * E(b, 1, j) + E(a, i, 2) * E(b, 2, j) +
                   E(a, i, 3) * E(b, 3, j) + E(a, i, 4) * E(b, 4, j);
}

/* Gaussian elimination with partial pivoting; b unchanged when a pivot is
 * below 1e-16 (solve_5x5_gepp_for_loop) */
static int gepp5(const double *a, double *b) {
  double A[25], x[5];
  memcpy(A, a, sizeof(A));
  memcpy(x, b, sizeof(x));
  for (int i = 0; i < 5; i++) {
    int p = i;
    double best = fabs(E(A, i, i));
    for (int k = i + 1; k < 5; k++)
      if (fabs(E(A, k, i)) > best) {
        best = fabs(E(A, k, i));
        p = k;
      }
    if (best < 1e-16) return i + 1;
    if (p != i) {
      for (int j = 0; j < 5; j++) {
        const double t = E(A, i, j);
        E(A, i, j) = E(A, p, j);
        E(A, p, j) = t;
      }
      const double t = x[i];
      x[i] = x[p];
      x[p] = t;
    }
    for (int k = i + 1; k < 5; k++) {
      const double f = E(A, k, i) / E(A, i, i);
      for (int j = i; j < 5; j++) E(A, k, j) -= f * E(A, i, j);
      x[k] -= f * x[i];
    }
  }
  for (int i = 4; i >= 0; i--) {
    double s = 0;
    for (int j = i + 1; j < 5; j++) s += E(A, i, j) * x[j];
    x[i] = (x[i] - s) / E(A, i, i);
  }
  memcpy(b, x, sizeof(x));
  return 0;
}

/* largest eigenvalue of the symmetric part given by the lower triangle:
 * cyclic Jacobi rotations (angle from atan2), at most 50 sweeps, stop when
 * the sum of the squared off-diagonal entries visited is below 1e-24 */
double oracle_rfc3d_max_eig(const double *a) {
  double A[25];
  for (int j = 0; j < 5; j++)
    for (int i = 0; i < 5; i++) E(A, i, j) = i >= j ? E(a, i, j) : 0.0;
  for (int j = 0; j < 5; j++)
    for (int i = j + 1; i < 5; i++) E(A, j, i) = E(A, i, j);
  for (int sweep = 0; sweep < 50; sweep++) {
    double off = 0.0;
    for (int p = 0; p < 5; p++)
      for (int q = p + 1; q < 5; q++) {
        const double apq = E(A, q, p);
        if (fabs(apq) < 1e-12) continue;
        off += apq * apq;
        const double app = E(A, p, p), aqq = E(A, q, q);
        const double phi = 0.5 * atan2(2.0 * apq, aqq - app);
        const double c = cos(phi), s = sin(phi);
        for (int i = 0; i < 5; i++) {
          const double aip = E(A, i, p), aiq = E(A, i, q);
          E(A, i, p) = c * aip - s * aiq;
          E(A, i, q) = s * aip + c * aiq;
        }
        for (int j = 0; j < 5; j++) {
          const double apj = E(A, p, j), aqj = E(A, q, j);
          E(A, p, j) = c * apj - s * aqj;
          E(A, q, j) = s * apj + c * aqj;
        }
        E(A, p, p) = c * c * app - 2.0 * c * s * apq + s * s * aqq;
        E(A, q, q) = s * s * app + 2.0 * c * s * apq + c * c * aqq;
        E(A, q, p) = 0.0;
        E(A, p, q) = 0.0;
      }
    if (off < 1e-12 * 1e-12) break;
  }
  double ev[5] = {E(A, 0, 0), E(A, 1, 1), E(A, 2, 2), E(A, 3, 3), E(A, 4, 4)};
  for (int i = 0; i < 4; i++)
    for (int j = i + 1; j < 5; j++)
      if (ev[j] < ev[i]) {
        const double t = ev[i];
        ev[i] = ev[j];
        ev[j] = t;
      }
  return ev[4];
}

/* projection on the rolling cone, in place; the region it was in */
static int proj_rcone(double *r, double mu, double mur) {
  const double nT = sqrt(r[1] * r[1] + r[2] * r[2]);
  const double nM = sqrt(r[3] * r[3] + r[4] * r[4]);
  if (mu * nT + mur * nM <= -r[0]) {
    for (int i = 0; i < 5; i++) r[i] = 0.0;
    return RC_DUAL;
  }
  if ((nT <= mu * r[0]) && (nM <= mur * r[0])) return RC_INSIDE;
  const double mu2 = mu * mu, mur2 = mur * mur;
  double t = (mu * nT + mur * nM + r[0]) / (mur2 + mu2 + 1.0);
  if ((nT > mu * t) && (nM > mur * t)) {
    r[0] = t;
    r[1] = mu * r[0] * r[1] / nT;
    r[2] = mu * r[0] * r[2] / nT;
    r[3] = mur * r[0] * r[3] / nM;
    r[4] = mur * r[0] * r[4] / nM;
    return RC_FRICTION_ROLLING;
  }
  t = (mu * nT + r[0]) / (mu2 + 1.0);
  if ((nT > mu * t) && (nM <= mur * t)) {
    r[0] = t;
    r[1] = mu * r[0] * r[1] / nT;
    r[2] = mu * r[0] * r[2] / nT;
    return RC_FRICTION;
  }
  t = (mur * nM + r[0]) / (mur2 + 1.0);
  if ((nT <= mu * t) && (nM > mur * t)) {
    r[0] = t;
    r[3] = mur * r[0] * r[3] / nM;
    r[4] = mur * r[0] * r[4] / nM;
    return RC_ROLLING;
  }
  return 20;
}

/* an element of the subdifferential of the projection at r (H zeroed
 * first: the reference leaves it unset in the unreachable last case) */
static void subdiff_rcone(double *H, const double *r, double mu, double mur) {
  memset(H, 0, 25 * sizeof(double));
  const double nT = sqrt(r[1] * r[1] + r[2] * r[2]);
  const double nM = sqrt(r[3] * r[3] + r[4] * r[4]);
  if (mu * nT + mur * nM <= -r[0]) return;
  if ((nT <= mu * r[0]) && (nM <= mur * r[0])) {
    for (int i = 0; i < 5; i++) E(H, i, i) = 1.;
    return;
  }
  const double mu2 = mu * mu, mur2 = mur * mur;
  const double a1 = mu * nT + mur * nM + r[0];
  double k = 1. / (1. + mu2 + mur2);
  double t = a1 * k;
  if ((nT > mu * t) && (nM > mur * t)) {
    E(H, 0, 0) = 1. * k;
    const double s1 = r[1] / nT, s2 = r[2] / nT;
    const double mk = mu * k;
    E(H, 0, 1) = mk * s1;
    E(H, 0, 2) = mk * s2;
    const double s3 = r[3] / nM, s4 = r[4] / nM;
    const double rk = mur * k;
    E(H, 0, 3) = rk * s3;
    E(H, 0, 4) = rk * s4;
    E(H, 1, 0) = E(H, 0, 1);
    E(H, 2, 0) = E(H, 0, 2);
    E(H, 3, 0) = E(H, 0, 3);
    E(H, 4, 0) = E(H, 0, 4);
    const double mkT = mk / nT, a2 = r[0] + mur * nM;
    E(H, 1, 1) = mkT * (-a2 * s1 * s1 + a1);
    E(H, 1, 2) = mkT * (-a2 * s1 * s2);
    E(H, 1, 3) = mk * s1 * mur * s3;
    E(H, 1, 4) = mk * s1 * mur * s4;
    E(H, 2, 1) = mkT * (-a2 * s1 * s2);
    E(H, 2, 2) = mkT * (-a2 * s2 * s2 + a1);
    E(H, 2, 3) = mk * s2 * mur * s3;
    E(H, 2, 4) = mk * s2 * mur * s4;
    const double rkM = rk / nM, a3 = r[0] + mu * nT;
    E(H, 3, 3) = rkM * (-a3 * s3 * s3 + a1);
    E(H, 3, 4) = rkM * (-a3 * s3 * s4);
    E(H, 3, 1) = E(H, 1, 3);
    E(H, 3, 2) = E(H, 2, 3);
    E(H, 4, 3) = rkM * (-a3 * s3 * s4);
    E(H, 4, 4) = rkM * (-a3 * s4 * s4 + a1);
    E(H, 4, 1) = E(H, 1, 4);
    E(H, 4, 2) = E(H, 2, 4);
    return;
  }
  const double b1 = r[0] + mu * nT;
  k = 1. / (1. + mu2);
  t = b1 * k;
  if ((nT > mu * t) && (nM <= mur * t)) {
    E(H, 0, 0) = 1. * k;
    const double s1 = r[1] / nT, s2 = r[2] / nT;
    const double mk = mu * k;
    E(H, 1, 0) = mk * s1;
    E(H, 2, 0) = mk * s2;
    E(H, 0, 1) = E(H, 1, 0);
    E(H, 0, 2) = E(H, 2, 0);
    const double mkT = mk / nT;
    E(H, 1, 1) = mkT * (-r[0] * s1 * s1 + b1);
    E(H, 1, 2) = mkT * (-r[0] * s1 * s2);
    E(H, 2, 1) = mkT * (-r[0] * s1 * s2);
    E(H, 2, 2) = mkT * (-r[0] * s2 * s2 + b1);
    E(H, 3, 3) = 1.;
    E(H, 4, 4) = 1.;
    return;
  }
  const double c1 = mur * nM + r[0];
  const double kr = 1. / (1. + mur2);
  t = c1 * kr;
  if ((nT <= mu * t) && (nM > mur * t)) {
    E(H, 0, 0) = 1. * kr;
    const double s3 = r[3] / nM, s4 = r[4] / nM;
    const double rk = mur * kr;
    E(H, 3, 0) = rk * s3;
    E(H, 4, 0) = rk * s4;
    E(H, 0, 3) = E(H, 3, 0);
    E(H, 0, 4) = E(H, 4, 0);
    const double rkM = rk / nM;
    E(H, 3, 3) = rkM * (-r[0] * s3 * s3 + c1);
    E(H, 3, 4) = rkM * (-r[0] * s3 * s4);
    E(H, 4, 3) = rkM * (-r[0] * s3 * s4);
    E(H, 4, 4) = rkM * (-r[0] * s4 * s4 + c1);
    E(H, 1, 1) = 1.;
    E(H, 2, 2) = 1.;
  }
}

/* rolling natural map F(R) = R - P(R - rho (v + mu |v_T| e_n + mur |w_T| e_n))
 * and, when A is given, the generalised Jacobians A (d/dv) and B (d/dR) */
static void natural_map(const double *R, const double *v, double mu, double mur, double rho, double *F, double *A,
                        double *B) {
  const double nVT = sqrt(v[1] * v[1] + v[2] * v[2]);
  const double nOT = sqrt(v[3] * v[3] + v[4] * v[4]);
  double RV[5];
  RV[0] = R[0] - rho * (v[0] + mu * nVT + mur * nOT);
  RV[1] = R[1] - rho * v[1];
  RV[2] = R[2] - rho * v[2];
  RV[3] = R[3] - rho * v[3];
  RV[4] = R[4] - rho * v[4];
  memcpy(F, RV, sizeof(RV));
  const int where = proj_rcone(F, mu, mur);
  for (int i = 0; i < 5; i++) F[i] = R[i] - F[i];
  if (!A) return;
  double s1, s2, s3, s4;
  if (where == RC_DUAL) {
    memset(A, 0, 25 * sizeof(double));
    memset(B, 0, 25 * sizeof(double));
    for (int i = 0; i < 5; i++) E(B, i, i) = 1.;
    return;
  }
  if (nVT <= 0.0) {
    s1 = 1.;
    s2 = 0.;
  } else {
    s1 = v[1] / nVT;
    s2 = v[2] / nVT;
  }
  if (nOT <= 0.0) {
    s3 = 1.;
    s4 = 0.;
  } else {
    s3 = v[3] / nOT;
    s4 = v[4] / nOT;
  }
  double D[25];
  memset(D, 0, sizeof(D));
  E(D, 0, 0) = rho;
  E(D, 0, 1) = rho * mu * s1;
  E(D, 0, 2) = rho * mu * s2;
  E(D, 0, 3) = rho * mur * s3;
  E(D, 0, 4) = rho * mur * s4;
  E(D, 1, 1) = rho;
  E(D, 2, 2) = rho;
  E(D, 3, 3) = rho;
  E(D, 4, 4) = rho;
  if (where == RC_INSIDE) {
    memcpy(A, D, sizeof(D));
    memset(B, 0, 25 * sizeof(double));
    return;
  }
  double H[25];
  subdiff_rcone(H, RV, mu, mur);
  mm5(H, D, A);
  for (int i = 0; i < 25; i++) B[i] = 0.;
  for (int i = 0; i < 5; i++) E(B, i, i) = 1.;
  for (int i = 0; i < 25; i++) B[i] -= H[i];
}

/* the one-contact direct nonsmooth Newton (after the take-off test) */
static void local_nsn(const double *M, const double *q, double mu, double mur, double rho, double *r, double tol,
                      int itermax) {
  const double nq = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3] + q[4] * q[4]);
  double rel = 1.0;
  if (nq > DBL_EPSILON) rel /= nq;
  double v[5], F[5], A[25], B[25], AWB[25], dR[5];
  memcpy(v, q, sizeof(v));
  mvp5(M, r, v);
  natural_map(r, v, mu, mur, rho, F, NULL, NULL);
  double res = sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3] + F[4] * F[4]) * rel;
  if (res < tol) return;
  for (int it = 1; it < itermax; it++) {
    natural_map(r, v, mu, mur, rho, F, A, B);
    mm5(A, M, AWB);
    for (int i = 0; i < 25; i++) AWB[i] += B[i];
    for (int i = 0; i < 25; i++) AWB[i] *= -1.;
    memcpy(dR, F, sizeof(dR));
    gepp5(AWB, dR);
    for (int i = 0; i < 5; i++) r[i] += dR[i];
    memcpy(v, q, sizeof(v));
    mvp5(M, r, v);
    natural_map(r, v, mu, mur, rho, F, NULL, NULL);
    const double e2 = (F[0] * F[0] + F[1] * F[1] + F[2] * F[2] * F[2] + F[3] * F[3] + F[4] * F[4]) * rel;
    const double old = res;
    res = sqrt(fmax(0.0, e2));
    if (res < tol) return;
    if (fabs(res - old) < DBL_EPSILON) return;
  }
}

double oracle_rfc3d_compute_error(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                                  const double *q, const double *mu, const double *mur, const double *r, double *u,
                                  double norm_q) {
  const int64_t n = 5LL * nc;
  for (int i = 0; i < nc; i++) {
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) acc5(&blocks[25 * k], &r[5 * colidx[k]], s);
    for (int a = 0; a < 5; a++) u[5 * i + a] = 1.0 * q[5 * i + a] + 1.0 * s[a];
  }
  double err = 0.0;
  for (int i = 0; i < nc; i++) {
    const double *ri = &r[5 * i], *ui = &u[5 * i];
    double w[5];
    w[0] = ri[0] - ui[0] - mu[i] * sqrt(ui[1] * ui[1] + ui[2] * ui[2]) - mur[i] * sqrt(ui[3] * ui[3] + ui[4] * ui[4]);
    for (int a = 1; a < 5; a++) w[a] = ri[a] - ui[a];
    proj_rcone(w, mu[i], mur[i]);
    for (int a = 0; a < 5; a++) w[a] = ri[a] - w[a];
    err += w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + w[3] * w[3] + w[4] * w[4];
  }
  err = sqrt(err);
  double norm = fmax(norm_q, nrm2(n, r));
  norm = fmax(norm, nrm2(n, u));
  if (fabs(norm) > DBL_EPSILON) err /= norm;
  return err;
}

/* Returns info (0 converged, 1 not; -1 when a contact has no diagonal block). */
int oracle_rfc3d_nsgs(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks, const double *q,
                      const double *mu, const double *mur, double *r, double *u, double tol, int maxiter,
                      const int32_t *order, int *iters, double *error, double *trace, int trace_cap, int *trace_len) {
  const int64_t n = 5LL * nc;
  const double norm_q = nrm2(n, q);
  int64_t *diag = (int64_t *)malloc(sizeof(int64_t) * (size_t)nc);
  double *rho = (double *)malloc(sizeof(double) * (size_t)nc);
  for (int i = 0; i < nc; i++) {
    diag[i] = -1;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++)
      if (colidx[k] == i && diag[i] < 0) diag[i] = k;
    if (diag[i] < 0) {
      free(diag);
      free(rho);
      return -1;
    }
    rho[i] = 1.0 / oracle_rfc3d_max_eig(&blocks[25 * diag[i]]);
  }
  double local_tol = 1e-12;
  const int local_max = 10;
  double tolerance = tol, err = 1.;
  int iter = 0, not_conv = 1, tl = 0;
  while (iter < maxiter && not_conv) {
    ++iter;
    double lsum = 0.0;
    for (int t = 0; t < nc; t++) {
      const int c = order ? order[t] : t;
      double ql[5], rl[5], s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
      for (int64_t k = rowptr[c]; k < rowptr[c + 1]; k++)
        if (colidx[k] != c) acc5(&blocks[25 * k], &r[5 * colidx[k]], s);
      for (int a = 0; a < 5; a++) ql[a] = q[5 * c + a] + s[a];
      memcpy(rl, &r[5 * c], sizeof(rl));
      if (ql[0] > -DBL_EPSILON) {
        for (int a = 0; a < 5; a++) rl[a] = 0.0;
      } else {
        local_nsn(&blocks[25 * diag[c]], ql, mu[c], mur[c], rho[c], rl, local_tol, local_max);
      }
      const double *o = &r[5 * c];
      lsum += (pow(o[0] - rl[0], 2) + pow(o[1] - rl[1], 2) + pow(o[2] - rl[2], 2) + pow(o[3] - rl[3], 2) +
               pow(o[4] - rl[4], 2));
      memcpy(&r[5 * c], rl, sizeof(rl));
    }
    err = sqrt(lsum);
    const double nr = nrm2(n, r);
    if (fabs(nr) > DBL_EPSILON) err /= nr;
    if (trace && tl < trace_cap) trace[tl++] = err;
    not_conv = 1;
    if (err < tolerance) {
      not_conv = 0;
      const double full = oracle_rfc3d_compute_error(nc, rowptr, colidx, blocks, q, mu, mur, r, u, norm_q);
      if (full > tol) {
        if (err < DBL_EPSILON)
          local_tol = fmax(local_tol / 100., DBL_EPSILON * 1e-6);
        else
          tolerance = err / full * tol;
        not_conv = 1;
      }
    }
  }
  err = oracle_rfc3d_compute_error(nc, rowptr, colidx, blocks, q, mu, mur, r, u, norm_q);
  not_conv = err < tol ? 0 : 1;
  *iters = iter;
  *error = err;
  if (trace_len) *trace_len = tl;
  free(diag);
  free(rho);
  return not_conv;
}
