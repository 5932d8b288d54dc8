/* Seeded sphere-lattice scene generator: geometry, W = H M^-1 H^T in
 * block-CSR and q = H v_free.  See include/fc3dgpu_scene.h. */
#include "fc3dgpu_scene.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define RADIUS 0.5
#define MASS 1.0
#define INERTIA 0.1

struct fc3dgpu_lattice {
  int nx, ny, nz, nb, nc;
  double *pos;   /* 3*nb */
  double *vel;   /* 6*nb: linear then angular */
  int32_t *cA;   /* nc, -1 = ground */
  int32_t *cB;   /* nc */
  double *frame; /* 9*nc: rows n, t1, t2 */
  double *cpt;   /* 3*nc contact point */
  double *gap;   /* nc */
  /* per-body incident contact lists (CSR) */
  int32_t *bptr; /* nb+1 */
  int32_t *blist;
};

/* ---- random numbers: splitmix64, uniform (0,1), polar-method normals ---- */
static uint64_t splitmix64(uint64_t *s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static double uniform01(uint64_t *s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

/* Natural logarithm for x in (0, 1]: x = m 2^e with m in [0.5, 1) (frexp is
 * exact), ln m = 2 atanh(z) = 2 (z + z^3/3 + z^5/5 + ...) with
 * z = (m - 1)/(m + 1) in (-1/3, 0]; 40 terms reach double precision.  Only
 * IEEE basic operations, so the result is the same on every platform. */
static double series_log(double x) {
  int e;
  double m = frexp(x, &e);
  double z = (m - 1.0) / (m + 1.0), z2 = z * z, term = z, s = 0.0;
  for (int k = 0; k < 40; k++) {
    s += term / (double)(2 * k + 1);
    term *= z2;
  }
  return 2.0 * s + (double)e * 0.693147180559945309417232121458176568;
}

typedef struct {
  uint64_t s;
  int have;
  double spare;
} NormalStream;

static double normal(NormalStream *ns) {
  if (ns->have) {
    ns->have = 0;
    return ns->spare;
  }
  for (;;) {
    double u = 2.0 * uniform01(&ns->s) - 1.0, v = 2.0 * uniform01(&ns->s) - 1.0;
    double w = u * u + v * v;
    if (w <= 0.0 || w >= 1.0) continue;
    double f = sqrt(-2.0 * series_log(w) / w);
    ns->spare = v * f;
    ns->have = 1;
    return u * f;
  }
}

void fc3dgpu_normal_fill(uint64_t seed, double *out, int64_t n) {
  NormalStream ns = {seed, 0, 0.0};
  for (int64_t i = 0; i < n; i++) out[i] = normal(&ns);
}

/* ---- small 3-vector helpers ---- */
static void cross(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

/* Frame rows n, t1, t2: t1 by Gram-Schmidt of e_x against n (e_y when n is
 * within ~25 degrees of e_x), t2 = n x t1. */
static void make_frame(const double n[3], double F[9]) {
  double e[3] = {1.0, 0.0, 0.0};
  if (fabs(n[0]) > 0.9) {
    e[0] = 0.0;
    e[1] = 1.0;
  }
  double d = e[0] * n[0] + e[1] * n[1] + e[2] * n[2];
  double t[3] = {e[0] - d * n[0], e[1] - d * n[1], e[2] - d * n[2]};
  double tn = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
  t[0] /= tn;
  t[1] /= tn;
  t[2] /= tn;
  double s[3];
  cross(n, t, s);
  for (int i = 0; i < 3; i++) {
    F[i] = n[i];
    F[3 + i] = t[i];
    F[6 + i] = s[i];
  }
}

fc3dgpu_lattice *fc3dgpu_lattice_create(int nx, int ny, int nz, uint64_t seed, double jitter_std, double v0_std) {
  if (nx < 1 || ny < 1 || nz < 1) return NULL;
  fc3dgpu_lattice *L = (fc3dgpu_lattice *)calloc(1, sizeof(*L));
  if (!L) return NULL;
  L->nx = nx;
  L->ny = ny;
  L->nz = nz;
  L->nb = nx * ny * nz;
  int nc = (nx - 1) * ny * nz + nx * (ny - 1) * nz + nx * ny * (nz - 1) + nx * ny;
  L->nc = nc;
  L->pos = (double *)malloc(sizeof(double) * 3 * (size_t)L->nb);
  L->vel = (double *)malloc(sizeof(double) * 6 * (size_t)L->nb);
  L->cA = (int32_t *)malloc(sizeof(int32_t) * (size_t)nc);
  L->cB = (int32_t *)malloc(sizeof(int32_t) * (size_t)nc);
  L->frame = (double *)malloc(sizeof(double) * 9 * (size_t)nc);
  L->cpt = (double *)malloc(sizeof(double) * 3 * (size_t)nc);
  L->gap = (double *)malloc(sizeof(double) * (size_t)nc);
  L->bptr = (int32_t *)calloc((size_t)L->nb + 1, sizeof(int32_t));
  L->blist = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)nc);
  if (!L->pos || !L->vel || !L->cA || !L->cB || !L->frame || !L->cpt || !L->gap || !L->bptr || !L->blist) {
    fc3dgpu_lattice_free(L);
    return NULL;
  }
  /* positions: one stream, then velocities: a second stream */
  NormalStream ps = {seed * 2 + 1, 0, 0.0}, vs = {seed * 2 + 2, 0, 0.0};
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        int b = i + nx * (j + ny * k);
        L->pos[3 * b + 0] = (double)i + jitter_std * normal(&ps);
        L->pos[3 * b + 1] = (double)j + jitter_std * normal(&ps);
        L->pos[3 * b + 2] = (double)k + 0.5 + jitter_std * normal(&ps);
      }
  for (int b = 0; b < L->nb; b++)
    for (int d = 0; d < 6; d++) L->vel[6 * b + d] = v0_std * normal(&vs);
  /* contacts in body order: ground (bottom layer), +x, +y, +z neighbours */
  int c = 0;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        int b = i + nx * (j + ny * k);
        int nbr[4] = {-2, i + 1 < nx ? b + 1 : -2, j + 1 < ny ? b + nx : -2, k + 1 < nz ? b + nx * ny : -2};
        if (k == 0) nbr[0] = -1;
        for (int t = 0; t < 4; t++) {
          if (nbr[t] == -2) continue;
          double n[3];
          const double *pb = &L->pos[3 * (t == 0 ? b : nbr[t])];
          if (t == 0) {
            /* ground plane z = 0 below body b: A = ground, B = b */
            L->cA[c] = -1;
            L->cB[c] = b;
            n[0] = 0.0;
            n[1] = 0.0;
            n[2] = 1.0;
            L->gap[c] = pb[2] - RADIUS;
            L->cpt[3 * c + 0] = pb[0];
            L->cpt[3 * c + 1] = pb[1];
            L->cpt[3 * c + 2] = pb[2] - RADIUS;
          } else {
            const double *pa = &L->pos[3 * b];
            L->cA[c] = b;
            L->cB[c] = nbr[t];
            double d[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
            double dn = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            for (int a = 0; a < 3; a++) n[a] = d[a] / dn;
            L->gap[c] = dn - 2.0 * RADIUS;
            for (int a = 0; a < 3; a++) L->cpt[3 * c + a] = pa[a] + 0.5 * d[a];
          }
          make_frame(n, &L->frame[9 * c]);
          c++;
        }
      }
  /* body -> incident contacts, in contact order */
  for (c = 0; c < nc; c++) {
    if (L->cA[c] >= 0) L->bptr[L->cA[c] + 1]++;
    L->bptr[L->cB[c] + 1]++;
  }
  for (int b = 0; b < L->nb; b++) L->bptr[b + 1] += L->bptr[b];
  int32_t *fill = (int32_t *)malloc(sizeof(int32_t) * (size_t)L->nb);
  if (!fill) {
    fc3dgpu_lattice_free(L);
    return NULL;
  }
  memcpy(fill, L->bptr, sizeof(int32_t) * (size_t)L->nb);
  for (c = 0; c < nc; c++) {
    if (L->cA[c] >= 0) L->blist[fill[L->cA[c]]++] = c;
    L->blist[fill[L->cB[c]]++] = c;
  }
  free(fill);
  return L;
}

void fc3dgpu_lattice_free(fc3dgpu_lattice *L) {
  if (!L) return;
  free(L->pos);
  free(L->vel);
  free(L->cA);
  free(L->cB);
  free(L->frame);
  free(L->cpt);
  free(L->gap);
  free(L->bptr);
  free(L->blist);
  free(L);
}

int fc3dgpu_lattice_sizes(const fc3dgpu_lattice *L, int *nbodies, int *ncontacts, int64_t *nnzb) {
  if (!L) return -1;
  if (nbodies) *nbodies = L->nb;
  if (ncontacts) *ncontacts = L->nc;
  if (nnzb) {
    /* diagonal + one block per other contact sharing a body (two contacts
     * share at most one body on a lattice) */
    int64_t s = L->nc;
    for (int b = 0; b < L->nb; b++) {
      int64_t d = L->bptr[b + 1] - L->bptr[b];
      s += d * (d - 1);
    }
    *nnzb = s;
  }
  return 0;
}

/* Jacobian of contact c w.r.t. body b, as the two 3x3 parts of the
 * 3x6 block H_cb = s R [I | -[d]x], d = contact point - body centre,
 * s = +1 for body B, -1 for body A.  Returns rows of R and d. */
static void contact_arm(const fc3dgpu_lattice *L, int c, int b, double *sign, double d[3]) {
  *sign = (L->cB[c] == b) ? 1.0 : -1.0;
  for (int a = 0; a < 3; a++) d[a] = L->cpt[3 * c + a] - L->pos[3 * b + a];
}

/* Block W_ij contribution of a shared body b, added to Wblk (column-major):
 * s_i s_j R_i (I/m - [d_i]x [d_j]x / I) R_j^T. */
static void add_body_block(const fc3dgpu_lattice *L, int ci, int cj, int b, double *Wblk) {
  double si, sj, di[3], dj[3];
  contact_arm(L, ci, b, &si, di);
  contact_arm(L, cj, b, &sj, dj);
  /* K = I/m - [di]x [dj]x / I ; [a]x[b]x = b a^T - (a.b) I */
  double ab = di[0] * dj[0] + di[1] * dj[1] + di[2] * dj[2];
  double K[3][3];
  for (int r = 0; r < 3; r++)
    for (int s = 0; s < 3; s++) {
      double cxx = dj[r] * di[s] - (r == s ? ab : 0.0);
      K[r][s] = (r == s ? 1.0 / MASS : 0.0) - cxx / INERTIA;
    }
  const double *Ri = &L->frame[9 * ci], *Rj = &L->frame[9 * cj];
  double KR[3][3]; /* K Rj^T */
  for (int r = 0; r < 3; r++)
    for (int s = 0; s < 3; s++) KR[r][s] = K[r][0] * Rj[3 * s + 0] + K[r][1] * Rj[3 * s + 1] + K[r][2] * Rj[3 * s + 2];
  double sg = si * sj;
  for (int r = 0; r < 3; r++)
    for (int s = 0; s < 3; s++) {
      double v = Ri[3 * r + 0] * KR[0][s] + Ri[3 * r + 1] * KR[1][s] + Ri[3 * r + 2] * KR[2][s];
      Wblk[r + 3 * s] += sg * v;
    }
}

static int cmp_i32(const void *a, const void *b) {
  int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

int fc3dgpu_lattice_fill_W(const fc3dgpu_lattice *L, int64_t *rowptr, int64_t *colidx, double *blocks) {
  if (!L) return -1;
  int64_t k = 0;
  int32_t nbr[32];
  for (int c = 0; c < L->nc; c++) {
    rowptr[c] = k;
    int cnt = 0;
    int bodies[2] = {L->cA[c], L->cB[c]};
    for (int t = 0; t < 2; t++) {
      int b = bodies[t];
      if (b < 0) continue;
      for (int32_t p = L->bptr[b]; p < L->bptr[b + 1]; p++)
        if (cnt < 32) nbr[cnt++] = L->blist[p];
    }
    qsort(nbr, (size_t)cnt, sizeof(int32_t), cmp_i32);
    int u = 0;
    for (int t = 0; t < cnt; t++)
      if (t == 0 || nbr[t] != nbr[t - 1]) nbr[u++] = nbr[t];
    for (int t = 0; t < u; t++) {
      int j = nbr[t];
      double *W = &blocks[9 * k];
      for (int e = 0; e < 9; e++) W[e] = 0.0;
      for (int s = 0; s < 2; s++) {
        int b = bodies[s];
        if (b < 0) continue;
        if (L->cA[j] == b || L->cB[j] == b) add_body_block(L, c, j, b, W);
      }
      colidx[k] = j;
      k++;
    }
  }
  rowptr[L->nc] = k;
  return 0;
}

int fc3dgpu_lattice_fill_q(const fc3dgpu_lattice *L, double h, double *q) {
  if (!L) return -1;
  for (int c = 0; c < L->nc; c++) {
    double u[3] = {0.0, 0.0, 0.0};
    int bodies[2] = {L->cA[c], L->cB[c]};
    for (int t = 0; t < 2; t++) {
      int b = bodies[t];
      if (b < 0) continue;
      double s, d[3];
      contact_arm(L, c, b, &s, d);
      const double *v = &L->vel[6 * b];
      double vf[3] = {v[0], v[1], v[2] - 9.81 * h};
      double w[3] = {v[3], v[4], v[5]}, wxd[3];
      cross(w, d, wxd);
      for (int a = 0; a < 3; a++) u[a] += s * (vf[a] + wxd[a]);
    }
    const double *R = &L->frame[9 * c];
    for (int r = 0; r < 3; r++) q[3 * c + r] = R[3 * r + 0] * u[0] + R[3 * r + 1] * u[1] + R[3 * r + 2] * u[2];
  }
  return 0;
}

int fc3dgpu_lattice_global_sizes(const fc3dgpu_lattice *L, int64_t *n, int64_t *nnzH) {
  if (!L) return -1;
  if (n) *n = 6 * (int64_t)L->nb;
  if (nnzH) *nnzH = 18 * (int64_t)L->bptr[L->nb];
  return 0;
}

int fc3dgpu_lattice_fill_global(const fc3dgpu_lattice *L, double h, double mass_scale, int64_t *Mp, int64_t *Mi, double *Mx,
                                int64_t *Hp, int64_t *Hi, double *Hx, double *q, double *b) {
  if (!L) return -1;
  int64_t k = 0;
  for (int bd = 0; bd < L->nb; bd++) {
    const double *v = &L->vel[6 * bd];
    for (int a = 0; a < 6; a++) {
      const int64_t i = 6 * (int64_t)bd + a;
      const double mass = mass_scale * (a < 3 ? MASS : INERTIA);
      Mp[i] = i;
      Mi[i] = i;
      Mx[i] = mass;
      q[i] = mass * (a == 2 ? v[2] - 9.81 * h : v[a]);
      Hp[i] = k;
      /* incident contacts in ascending order (blist is in contact order) */
      for (int32_t p = L->bptr[bd]; p < L->bptr[bd + 1]; p++) {
        const int c = L->blist[p];
        double s, d[3];
        contact_arm(L, c, bd, &s, d);
        const double *R = &L->frame[9 * c];
        for (int r = 0; r < 3; r++) {
          double x;
          if (a < 3) {
            x = R[3 * r + a];
          } else {
            double dxr[3];
            cross(d, &R[3 * r], dxr);
            x = dxr[a - 3];
          }
          Hi[k] = 3 * (int64_t)c + r;
          Hx[k] = s * x;
          k++;
        }
      }
    }
  }
  Mp[6 * (int64_t)L->nb] = 6 * (int64_t)L->nb;
  Hp[6 * (int64_t)L->nb] = k;
  for (int64_t j = 0; j < 3 * (int64_t)L->nc; j++) b[j] = 0.0;
  return 0;
}

int fc3dgpu_lattice_fill_geometry(const fc3dgpu_lattice *L, double *gap, int32_t *bodyA, int32_t *bodyB) {
  if (!L) return -1;
  if (gap) memcpy(gap, L->gap, sizeof(double) * (size_t)L->nc);
  if (bodyA) memcpy(bodyA, L->cA, sizeof(int32_t) * (size_t)L->nc);
  if (bodyB) memcpy(bodyB, L->cB, sizeof(int32_t) * (size_t)L->nc);
  return 0;
}

int fc3dgpu_lattice_fill_contacts(const fc3dgpu_lattice *L, double *frame, double *point, double *body_pos,
                                  double *body_mass, double *body_inertia, double *vel) {
  if (!L) return -1;
  if (frame) memcpy(frame, L->frame, sizeof(double) * 9 * (size_t)L->nc);
  if (point) memcpy(point, L->cpt, sizeof(double) * 3 * (size_t)L->nc);
  if (body_pos) memcpy(body_pos, L->pos, sizeof(double) * 3 * (size_t)L->nb);
  if (vel) memcpy(vel, L->vel, sizeof(double) * 6 * (size_t)L->nb);
  for (int b = 0; b < L->nb; b++) {
    if (body_mass) body_mass[b] = MASS;
    if (body_inertia) body_inertia[b] = INERTIA;
  }
  return 0;
}

int fc3dgpu_lattice_perturb_velocities(fc3dgpu_lattice *L, uint64_t seed, double std) {
  if (!L) return -1;
  NormalStream ns = {seed * 2 + 0x5151ULL, 0, 0.0};
  for (int b = 0; b < L->nb; b++)
    for (int d = 0; d < 6; d++) L->vel[6 * b + d] += std * normal(&ns);
  return 0;
}
