/* CPU restatement of the reference's 2D friction-contact NSGS -- TEST
 * INFRASTRUCTURE (the checker of the GPU fc2d solver; never the product).
 *
 * Follows fc2d_nsgs (FrictionContact/fc2d_nsgs.c:299-520) with its default
 * options (fc2d_nsgs_set_default :787: no shuffle, no freezing,
 * LIGHT_WITH_FULL_FINAL), on a block-CSR W of 2x2 column-major blocks:
 *   - the diagonal blocks' determinants (:194-210), a failure when one is
 *     below DBL_EPSILON (:318-333);
 *   - per sweep and contact: q_loc = q_i + sum_{j != i} W_ij r_j in the
 *     row's block order (SBM_row_prod_no_diag_2x2, SparseBlockMatrix.c:1492,
 *     with mvp2x2's update order, op3x3.h), the closed-form local solve
 *     (fc2d_nsgs_local_solve :212-252), the light error (:90-96, :126-146);
 *   - determine_convergence_with_full_final (:187-228): when the light
 *     error is below the working tolerance, fc2d_compute_error decides, and
 *     the working tolerance becomes error / full * tol when it is not met;
 *   - the final fc2d_compute_error and info = (error < tol ? 0 : 1).
 * fc2d_compute_error (fc2d_compute_error.c:40-140): w = q + W z block by
 * block (SBM_gemv with a 2x2 dgemv per block: w_i += (a_i0 z0 + a_i1 z1)),
 * the natural-map error summed contact by contact, divided by
 * max(|z|, |w|, |q|) when that exceeds DBL_EPSILON.  Norms are plain sums of
 * squares in index order (the CBLAS shim the reference is built with here).
 * `order` (optional) is the contact visiting order of a sweep. */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SGN(x) ((x) < 0 ? -1 : (x) > 0 ? 1 : 0)

static double nrm2(int64_t n, const double *x) {
  double s = 0.0;
  for (int64_t i = 0; i < n; i++) s += x[i] * x[i];
  return sqrt(s);
}

static void mvp2x2(const double *a, const double *v, double *r) {
  r[0] += a[0] * v[0];
  r[1] += a[1] * v[0];
  r[0] += a[2] * v[1];
  r[1] += a[3] * v[1];
}

double oracle_fc2d_compute_error(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                                 const double *q, const double *mu, const double *z, double *w, double norm_q) {
  const int64_t n = 2LL * nc;
  memcpy(w, q, sizeof(double) * (size_t)n);
  for (int i = 0; i < nc; i++)
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
      const double *a = &blocks[4 * k];
      const double *x = &z[2 * colidx[k]];
      for (int r = 0; r < 2; r++) {
        double s = 0.0;
        s += a[r] * x[0];
        s += a[2 + r] * x[1];
        w[2 * i + r] = 1.0 * w[2 * i + r] + 1.0 * s;
      }
    }
  double err = 0.0;
  for (int i = 0; i < nc; i++) {
    const double *r = &z[2 * i], *u = &w[2 * i];
    double t0 = r[0] - u[0] - mu[i] * fabs(u[1]);
    double t1 = r[1] - u[1];
    double normT = fabs(t1);
    if (mu[i] * normT <= -t0) {
      t0 = 0.;
      t1 = 0.;
    } else if (normT > mu[i] * t0) {
      t0 = (mu[i] * normT + t0) / (mu[i] * mu[i] + 1.0);
      t1 = mu[i] * t0 * SGN(t1);
    }
    t0 = r[0] - t0;
    t1 = r[1] - t1;
    err += t0 * t0 + t1 * t1;
  }
  err = sqrt(err);
  double nr = nrm2(n, z), nw = nrm2(n, w);
  double scal = fmax(nr, fmax(nw, norm_q));
  if (fabs(scal) > DBL_EPSILON) err /= scal;
  return err;
}

static void local_solve(const double *W, double D, const double *q, double mu, double *P) {
  const double Wnn = W[0], Wtn = W[1], Wnt = W[2], Wtt = W[3];
  if (q[0] > 0) {
    P[0] = 0;
    P[1] = 0;
  } else {
    P[0] = -(Wtt * q[0] - Wnt * q[1]) / D;
    P[1] = -(-Wtn * q[0] + Wnn * q[1]) / D;
    double muPn = mu * P[0];
    if (fabs(P[1]) > muPn) {
      if (P[1] + muPn < 0) {
        P[0] = -q[0] / (Wnn - mu * Wnt);
        P[1] = -mu * P[0];
      } else {
        P[0] = -q[0] / (Wnn + mu * Wnt);
        P[1] = mu * P[0];
      }
    }
  }
}

/* Returns info (0 converged, 1 not; -1 on a singular diagonal block). */
int oracle_fc2d_nsgs(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks, const double *q,
                     const double *mu, double *r, double *u, double tol, int maxiter, const int32_t *order,
                     int *iters, double *error, double *trace, int trace_cap, int *trace_len) {
  const int64_t n = 2LL * nc;
  const double norm_q = nrm2(n, q);
  int64_t *diag = (int64_t *)malloc(sizeof(int64_t) * (size_t)nc);
  double *det = (double *)malloc(sizeof(double) * (size_t)nc);
  for (int i = 0; i < nc; i++) {
    diag[i] = -1;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++)
      if (colidx[k] == i && diag[i] < 0) diag[i] = k;
    if (diag[i] < 0) {
      free(diag);
      free(det);
      return -1;
    }
    const double *b = &blocks[4 * diag[i]];
    det[i] = b[0] * b[3] - b[1] * b[2];
    if (det[i] < DBL_EPSILON) {
      *iters = 0;
      *error = INFINITY;
      if (trace_len) *trace_len = 0;
      free(diag);
      free(det);
      return 1;
    }
  }
  double tolerance = tol;
  int iter = 0, not_conv = 1, tl = 0;
  double err = INFINITY;
  while (iter < maxiter && not_conv) {
    ++iter;
    double lsum = 0.0;
    for (int t = 0; t < nc; t++) {
      const int c = order ? order[t] : t;
      double loc[2] = {r[2 * c], r[2 * c + 1]};
      double ql[2] = {q[2 * c], q[2 * c + 1]};
      for (int64_t k = rowptr[c]; k < rowptr[c + 1]; k++)
        if (colidx[k] != c) mvp2x2(&blocks[4 * k], &r[2 * colidx[k]], ql);
      local_solve(&blocks[4 * diag[c]], det[c], ql, mu[c], loc);
      const double x0 = r[2 * c] - loc[0], x1 = r[2 * c + 1] - loc[1];
      lsum += x0 * x0 + x1 * x1;
      r[2 * c] = loc[0];
      r[2 * c + 1] = loc[1];
    }
    err = sqrt(lsum);
    const double nr = nrm2(n, r);
    if (fabs(nr) > DBL_EPSILON) err /= nr;
    if (trace && tl < trace_cap) trace[tl++] = err;
    if (err < tolerance) {
      not_conv = 0;
      const double full = oracle_fc2d_compute_error(nc, rowptr, colidx, blocks, q, mu, r, u, norm_q);
      if (full > tol) {
        tolerance = err / full * tol;
        not_conv = 1;
      }
    }
  }
  err = oracle_fc2d_compute_error(nc, rowptr, colidx, blocks, q, mu, r, u, norm_q);
  not_conv = err < tol ? 0 : 1;
  *iters = iter;
  *error = err;
  if (trace_len) *trace_len = tl;
  free(diag);
  free(det);
  return not_conv;
}

/* The FP32 phase of the GPU solver's mixed-precision mode, for checking it:
 * `nsweeps` sweeps of the same algorithm in single precision, visiting
 * contacts in `order`.  W, q, mu and the reaction are rounded to float, the
 * diagonal determinants computed in float from the rounded blocks, every
 * operation in float in the same order as the FP64 sweep (no contraction),
 * and the reaction returned widened to double. */
static void mvp2x2_f(const float *a, const float *v, float *r) {
  r[0] += a[0] * v[0];
  r[1] += a[1] * v[0];
  r[0] += a[2] * v[1];
  r[1] += a[3] * v[1];
}

static void local_solve_f(const float *W, float D, const float *q, float mu, float *P) {
  const float Wnn = W[0], Wtn = W[1], Wnt = W[2], Wtt = W[3];
  if (q[0] > 0) {
    P[0] = 0;
    P[1] = 0;
  } else {
    P[0] = -(Wtt * q[0] - Wnt * q[1]) / D;
    P[1] = -(-Wtn * q[0] + Wnn * q[1]) / D;
    float muPn = mu * P[0];
    if (fabsf(P[1]) > muPn) {
      if (P[1] + muPn < 0) {
        P[0] = -q[0] / (Wnn - mu * Wnt);
        P[1] = -mu * P[0];
      } else {
        P[0] = -q[0] / (Wnn + mu * Wnt);
        P[1] = mu * P[0];
      }
    }
  }
}

int oracle_fc2d_sweeps_f32(int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                           const double *q, const double *mu, double *r, int nsweeps, const int32_t *order) {
  const int64_t nnzb = rowptr[nc];
  float *W = (float *)malloc(sizeof(float) * 4 * (size_t)(nnzb ? nnzb : 1));
  float *qf = (float *)malloc(sizeof(float) * 2 * (size_t)nc);
  float *mf = (float *)malloc(sizeof(float) * (size_t)nc);
  float *rf = (float *)malloc(sizeof(float) * 2 * (size_t)nc);
  float *det = (float *)malloc(sizeof(float) * (size_t)nc);
  int64_t *diag = (int64_t *)malloc(sizeof(int64_t) * (size_t)nc);
  int rc = 0;
  for (int64_t k = 0; k < 4 * nnzb; k++) W[k] = (float)blocks[k];
  for (int64_t k = 0; k < 2LL * nc; k++) {
    qf[k] = (float)q[k];
    rf[k] = (float)r[k];
  }
  for (int i = 0; i < nc; i++) {
    mf[i] = (float)mu[i];
    diag[i] = -1;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++)
      if (colidx[k] == i && diag[i] < 0) diag[i] = k;
    if (diag[i] < 0) {
      rc = -1;
      goto done;
    }
    const float *b = &W[4 * diag[i]];
    det[i] = b[0] * b[3] - b[1] * b[2];
  }
  for (int s = 0; s < nsweeps; s++)
    for (int t = 0; t < nc; t++) {
      const int c = order ? order[t] : t;
      float loc[2] = {rf[2 * c], rf[2 * c + 1]};
      float ql[2] = {qf[2 * c], qf[2 * c + 1]};
      for (int64_t k = rowptr[c]; k < rowptr[c + 1]; k++)
        if (colidx[k] != c) mvp2x2_f(&W[4 * k], &rf[2 * colidx[k]], ql);
      local_solve_f(&W[4 * diag[c]], det[c], ql, mf[c], loc);
      rf[2 * c] = loc[0];
      rf[2 * c + 1] = loc[1];
    }
  for (int64_t k = 0; k < 2LL * nc; k++) r[k] = (double)rf[k];
done:
  free(W);
  free(qf);
  free(mf);
  free(rf);
  free(det);
  free(diag);
  return rc;
}
