/* CPU restatement of the reference's global FC3D NSGS -- TEST INFRASTRUCTURE.
 *
 * Only tests, the smoke check and the bench's CPU baseline load this file;
 * the product never links it.  It restates, in this project's own code, the
 * reference's SICONOS_GLOBAL_FRICTION_3D_NSGS solve of a
 * GlobalFrictionContactProblem (M v = q + H r, u = H^T v + b, r in the
 * Coulomb cones):
 *
 *   gfc3d_driver, no-contact case        gfc3d_driver.c:107-114,
 *                                        GlobalFrictionContactProblem.c:270-300
 *   gfc3d_nsgs loop (projection local    gfc3d_nsgs.c:62-198
 *     solver, error every iteration or
 *     every ERROR_EVALUATION_FREQUENCY)
 *   gfc3d_compute_error                  gfc3d_compute_error.c:38-160
 *   dense LU of M (NM_LU_solve, dense)   NumericsMatrix.c:3543-3590, :3699-3735
 *   cone projection                      projectionOnCone.c:32-49
 *
 * M and H come as CSR (rows in ascending column order).  A matrix-vector
 * product row is summed from +0.0 in ascending column order and then added
 * to the scaled output, as the project's BLAS shim computes the reference's
 * dense dgemv; entries that are zero change no such sum, so dense storage
 * and CSR give the same values bit for bit.  M is factorised by connected
 * components of its pattern: an unblocked LU with partial pivoting (first
 * largest pivot, the multipliers by division) per component, which on a
 * dense M equals the shim's dgetrf of the whole matrix value for value (no
 * fill crosses components and every pivot row lies in the pivot's
 * component).  Vector norms are plain sums of squares, as in the shim.
 * Built with -ffp-contract=off like the reference in oracle/_ref. */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

unsigned oracle_projection_on_cone(double *r, double mu);

static double nrm2(int64_t n, const double *x) {
  double s = 0.0;
  for (int64_t i = 0; i < n; i++) s += x[i] * x[i];
  return sqrt(s);
}

/* y[i] = beta*y[i] + alpha*(sum_k A[i,k] x[k]) with beta in {0, 1}, the
 * shim's dgemv order (a zero beta stores 0.0 + alpha*s). */
static void csr_gemv(int64_t rows, const int64_t *p, const int64_t *ix, const double *v, double alpha,
                     const double *x, double beta, double *y) {
  for (int64_t i = 0; i < rows; i++) {
    double s = 0.0;
    for (int64_t k = p[i]; k < p[i + 1]; k++) s += v[k] * x[ix[k]];
    y[i] = (beta == 0.0 ? 0.0 : beta * y[i]) + alpha * s;
  }
}

/* fc3d_unitary_compute_and_add_error (fc3d_compute_error.c:42-56) */
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

/* ---------------- M's components and their LU factors ---------------- */

typedef struct {
  int ncomp;
  int64_t *cptr;  /* component c holds DOFs dof[cptr[c] .. cptr[c+1]) */
  int64_t *dof;   /* ascending within a component */
  int64_t *luoff; /* column-major s x s factors of component c at lu[luoff[c]] */
  double *lu;
  int *piv; /* local pivot rows, cptr-indexed */
} Factors;

static int64_t uf_find(int64_t *par, int64_t i) {
  while (par[i] != i) {
    par[i] = par[par[i]];
    i = par[i];
  }
  return i;
}

/* Components of the pattern of M (an entry (i, j) joins i and j), listed
 * by their smallest DOF; returns 0, or 1 when a pivot is exactly zero. */
int oracle_gfc3d_components(int64_t n, const int64_t *Mp, const int64_t *Mi, int64_t *comp_of) {
  int64_t *par = malloc(sizeof(int64_t) * (n > 0 ? n : 1));
  for (int64_t i = 0; i < n; i++) par[i] = i;
  for (int64_t i = 0; i < n; i++)
    for (int64_t k = Mp[i]; k < Mp[i + 1]; k++) {
      int64_t a = uf_find(par, i), b = uf_find(par, Mi[k]);
      if (a != b) {
        if (a < b)
          par[b] = a;
        else
          par[a] = b;
      }
    }
  int64_t nc = 0;
  int64_t *id = malloc(sizeof(int64_t) * (n > 0 ? n : 1));
  for (int64_t i = 0; i < n; i++) id[i] = -1;
  for (int64_t i = 0; i < n; i++) {
    int64_t r = uf_find(par, i);
    if (id[r] < 0) id[r] = nc++;
    comp_of[i] = id[r];
  }
  free(id);
  free(par);
  return (int)nc;
}

static int factorise(int64_t n, const int64_t *Mp, const int64_t *Mi, const double *Mx, Factors *F) {
  int64_t *comp_of = malloc(sizeof(int64_t) * (n > 0 ? n : 1));
  F->ncomp = oracle_gfc3d_components(n, Mp, Mi, comp_of);
  const int nc = F->ncomp;
  F->cptr = calloc(nc + 1, sizeof(int64_t));
  for (int64_t i = 0; i < n; i++) F->cptr[comp_of[i] + 1]++;
  for (int c = 0; c < nc; c++) F->cptr[c + 1] += F->cptr[c];
  F->dof = malloc(sizeof(int64_t) * (n > 0 ? n : 1));
  int64_t *fill = malloc(sizeof(int64_t) * (nc > 0 ? nc : 1));
  for (int c = 0; c < nc; c++) fill[c] = F->cptr[c];
  int64_t *local = malloc(sizeof(int64_t) * (n > 0 ? n : 1)); /* position of a DOF in its component */
  for (int64_t i = 0; i < n; i++) {
    local[i] = fill[comp_of[i]] - F->cptr[comp_of[i]];
    F->dof[fill[comp_of[i]]++] = i;
  }
  free(fill);
  F->luoff = malloc(sizeof(int64_t) * (nc + 1));
  F->luoff[0] = 0;
  for (int c = 0; c < nc; c++) {
    int64_t s = F->cptr[c + 1] - F->cptr[c];
    F->luoff[c + 1] = F->luoff[c] + s * s;
  }
  F->lu = calloc(F->luoff[nc] > 0 ? F->luoff[nc] : 1, sizeof(double));
  F->piv = malloc(sizeof(int) * (n > 0 ? n : 1));
  for (int64_t i = 0; i < n; i++) {
    const int c = (int)comp_of[i];
    const int64_t s = F->cptr[c + 1] - F->cptr[c];
    double *A = F->lu + F->luoff[c];
    for (int64_t k = Mp[i]; k < Mp[i + 1]; k++) A[local[Mi[k]] * s + local[i]] = Mx[k];
  }
  free(local);
  free(comp_of);
  int singular = 0;
  for (int c = 0; c < nc; c++) {
    const int64_t s = F->cptr[c + 1] - F->cptr[c];
    double *A = F->lu + F->luoff[c];
    int *piv = F->piv + F->cptr[c];
    for (int64_t j = 0; j < s; j++) {
      int64_t p = j;
      double best = -1.0;
      for (int64_t i = j; i < s; i++)
        if (fabs(A[j * s + i]) > best) {
          best = fabs(A[j * s + i]);
          p = i;
        }
      piv[j] = (int)p;
      if (A[j * s + p] == 0.0) {
        singular = 1;
        continue;
      }
      if (p != j)
        for (int64_t k = 0; k < s; k++) {
          double t = A[k * s + j];
          A[k * s + j] = A[k * s + p];
          A[k * s + p] = t;
        }
      for (int64_t i = j + 1; i < s; i++) A[j * s + i] = A[j * s + i] / A[j * s + j];
      for (int64_t k = j + 1; k < s; k++)
        for (int64_t i = j + 1; i < s; i++) A[k * s + i] = A[k * s + i] - A[j * s + i] * A[k * s + j];
    }
  }
  return singular;
}

static void factors_free(Factors *F) {
  free(F->cptr);
  free(F->dof);
  free(F->luoff);
  free(F->lu);
  free(F->piv);
}

/* x <- M^-1 x with the factors: row swaps in order, unit-lower forward
 * substitution (subtractions in ascending column order), upper back
 * substitution (descending), then the division by the pivot. */
static void lu_solve(const Factors *F, double *x, double *work) {
  for (int c = 0; c < F->ncomp; c++) {
    const int64_t o = F->cptr[c], s = F->cptr[c + 1] - o;
    const double *A = F->lu + F->luoff[c];
    const int *piv = F->piv + o;
    double *y = work;
    for (int64_t i = 0; i < s; i++) y[i] = x[F->dof[o + i]];
    for (int64_t i = 0; i < s; i++)
      if (piv[i] != i) {
        double t = y[i];
        y[i] = y[piv[i]];
        y[piv[i]] = t;
      }
    for (int64_t i = 0; i < s; i++) {
      double v = y[i];
      for (int64_t k = 0; k < i; k++) v = v - A[k * s + i] * y[k];
      y[i] = v;
    }
    for (int64_t i = s - 1; i >= 0; i--) {
      double v = y[i];
      for (int64_t k = s - 1; k > i; k--) v = v - A[k * s + i] * y[k];
      y[i] = v / A[i * s + i];
    }
    for (int64_t i = 0; i < s; i++) x[F->dof[o + i]] = y[i];
  }
}

/* ---------------- the solve ---------------- */

typedef struct {
  int64_t n, m;
  const int64_t *Mp, *Mi, *Hp, *Hi;
  const double *Mx, *Hx;
  int64_t *Tp, *Ti; /* H^T as CSR (rows = contact DOFs, ascending DOF) */
  double *Tx;
  const double *q, *b, *mu;
} Global;

static void transpose(Global *G) {
  const int64_t n = G->n, m = G->m, nnz = G->Hp[n];
  G->Tp = calloc(m + 1, sizeof(int64_t));
  G->Ti = malloc(sizeof(int64_t) * (nnz > 0 ? nnz : 1));
  G->Tx = malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
  for (int64_t k = 0; k < nnz; k++) G->Tp[G->Hi[k] + 1]++;
  for (int64_t j = 0; j < m; j++) G->Tp[j + 1] += G->Tp[j];
  int64_t *fill = malloc(sizeof(int64_t) * (m > 0 ? m : 1));
  memcpy(fill, G->Tp, sizeof(int64_t) * (m > 0 ? m : 1));
  for (int64_t i = 0; i < n; i++)
    for (int64_t k = G->Hp[i]; k < G->Hp[i + 1]; k++) {
      int64_t d = fill[G->Hi[k]]++;
      G->Ti[d] = i;
      G->Tx[d] = G->Hx[k];
    }
  free(fill);
}

/* gfc3d_compute_error (gfc3d_compute_error.c:38-160): writes u = b + H^T v
 * and returns the error. */
static double compute_error(const Global *G, const double *r, double *u, const double *v, double norm_q,
                            double *tmp, double *tmp1) {
  const int64_t n = G->n, m = G->m;
  const int nc = (int)(m / 3);
  const double norm_r = nrm2(m, r);
  memcpy(tmp1, G->q, sizeof(double) * n);
  if (nc > 0) csr_gemv(n, G->Hp, G->Hi, G->Hx, 1.0, r, 0.0, tmp);
  /* with no contact, tmp keeps what it held (the reference's work array) */
  const double norm_Hr = nrm2(n, tmp);
  for (int64_t i = 0; i < n; i++) tmp1[i] += 1.0 * tmp[i];
  csr_gemv(n, G->Mp, G->Mi, G->Mx, -1.0, v, 0.0, tmp);
  const double norm_Mv = nrm2(n, tmp);
  for (int64_t i = 0; i < n; i++) tmp1[i] += 1.0 * tmp[i];
  const double rel = fmax(norm_q, fmax(norm_Mv, norm_Hr));
  double error = nrm2(n, tmp1);
  const double min_rel = sqrt(DBL_EPSILON);
  if (fabs(rel) > min_rel) error = error / rel;
  memcpy(u, G->b, sizeof(double) * m);
  csr_gemv(m, G->Tp, G->Ti, G->Tx, 1.0, v, 1.0, u);
  const double norm_u = nrm2(m, u);
  double ec = 0.0;
  for (int c = 0; c < nc; c++) unitary_error(&r[3 * c], &u[3 * c], G->mu[c], &ec);
  ec = sqrt(ec);
  const double rel2 = fmax(norm_u, norm_r);
  if (fabs(rel2) > min_rel) ec = ec / rel2;
  return error + ec;
}

/* Returns info as gfc3d_nsgs leaves it: -1 when no iteration ran, else 0
 * (converged) or 1; -2 when M is singular; -3 when a work array could not
 * be allocated.  freq is SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION_FREQUENCY
 * (0: the error after every iteration).  r, v are the start on entry. */
int oracle_gfc3d_nsgs(int64_t n, int nc, const int64_t *Mp, const int64_t *Mi, const double *Mx, const int64_t *Hp,
                      const int64_t *Hi, const double *Hx, const double *q, const double *b, const double *mu,
                      double *r, double *u, double *v, double tol, int maxiter, int freq, int *iters,
                      double *error_out, double *trace, int trace_cap) {
  Global G = {n, 3 * (int64_t)nc, Mp, Mi, Hp, Hi, Mx, Hx, NULL, NULL, NULL, q, b, mu};
  Factors F;
  if (factorise(n, Mp, Mi, Mx, &F)) {
    factors_free(&F);
    return -2;
  }
  if (nc == 0) {
    /* gfc3d_driver's no-contact case: v = M^-1 q */
    double *work = malloc(sizeof(double) * (n > 0 ? n : 1));
    memcpy(v, q, sizeof(double) * n);
    lu_solve(&F, v, work);
    free(work);
    factors_free(&F);
    if (iters) *iters = 0;
    if (error_out) *error_out = 0.0;
    return 0;
  }
  transpose(&G);
  const int64_t m = G.m;
  double *tmp = calloc(n > 0 ? n : 1, sizeof(double)), *tmp1 = calloc(n > 0 ? n : 1, sizeof(double));
  double *work = malloc(sizeof(double) * (n > 0 ? n : 1));
  const double norm_q = nrm2(n, q);
  int info = -1, iter = 0, not_conv = 1;
  double error = 1.0;
  while (iter < maxiter && not_conv > 0) {
    ++iter;
    memcpy(v, q, sizeof(double) * n);
    csr_gemv(n, Hp, Hi, Hx, 1.0, r, 1.0, v);
    lu_solve(&F, v, work);
    memcpy(u, b, sizeof(double) * m);
    csr_gemv(m, G.Tp, G.Ti, G.Tx, 1.0, v, 1.0, u);
    for (int c = 0; c < nc; c++) {
      double *rc = &r[3 * c];
      const double *uc = &u[3 * c];
      const double normUT = sqrt(uc[1] * uc[1] + uc[2] * uc[2]);
      const double an = 1.0;
      rc[0] -= an * (uc[0] + mu[c] * normUT);
      rc[1] -= an * uc[1];
      rc[2] -= an * uc[2];
      oracle_projection_on_cone(rc, mu[c]);
    }
    if (freq > 0) {
      if (!(iter % freq)) error = compute_error(&G, r, u, v, norm_q, tmp, tmp1);
    } else {
      error = compute_error(&G, r, u, v, norm_q, tmp, tmp1);
    }
    if (trace && iter - 1 < trace_cap) trace[iter - 1] = error;
    if (error < tol) not_conv = 0;
    info = not_conv;
  }
  if (iter == maxiter) error = compute_error(&G, r, u, v, norm_q, tmp, tmp1);
  if (iters) *iters = iter;
  if (error_out) *error_out = error;
  free(tmp);
  free(tmp1);
  free(work);
  free(G.Tp);
  free(G.Ti);
  free(G.Tx);
  factors_free(&F);
  return info;
}

/* gfc3d_compute_error of (r, v) alone: u = b + H^T v is written. */
double oracle_gfc3d_compute_error(int64_t n, int nc, const int64_t *Mp, const int64_t *Mi, const double *Mx,
                                  const int64_t *Hp, const int64_t *Hi, const double *Hx, const double *q,
                                  const double *b, const double *mu, const double *r, const double *v, double *u) {
  Global G = {n, 3 * (int64_t)nc, Mp, Mi, Hp, Hi, Mx, Hx, NULL, NULL, NULL, q, b, mu};
  transpose(&G);
  double *tmp = calloc(n > 0 ? n : 1, sizeof(double)), *tmp1 = calloc(n > 0 ? n : 1, sizeof(double));
  const double e = compute_error(&G, r, u, v, nrm2(n, q), tmp, tmp1);
  free(tmp);
  free(tmp1);
  free(G.Tp);
  free(G.Ti);
  free(G.Tx);
  return e;
}
