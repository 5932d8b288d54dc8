/* Text (.dat) files of 3D friction-contact problems, in the format the
 * reference reads and writes (frictionContact_newFromFile /
 * frictionContact_printInFile, FrictionContactProblem.c:67-132):
 *
 *   dimension (3)            number of contacts nc
 *   matrix: storage type, rows, columns, then
 *     0 (dense):             rows, columns again, rows*columns values in
 *                            column order (NM_new_from_file, NumericsMatrix.c)
 *     1 (sparse block):      number of blocks, block rows, block columns, the
 *                            cumulative block sizes of rows and of columns,
 *                            filled1, filled2, the row pointer (filled1
 *                            entries), the column indices (filled2 entries),
 *                            then per block its number and its values in
 *                            column order (SBM_new_from_file /
 *                            SBM_write_in_file, SparseBlockMatrix.c:1619-1850)
 *   q (3 nc values)          mu (nc values)
 *
 * Values are written as "%32.24e" (25 significant digits: a double reads
 * back exactly); the reference reads block values with a 32-character field
 * and q, mu with a plain field, and so does this reader.  A dense matrix
 * becomes block-CSR with every 3x3 block holding a nonzero entry, and every
 * diagonal block.  Other storage types (CSparse) are not read. */
#include "fc3dgpu_dat.h"

#include <ctype.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct fc3dgpu_dat {
  int dim, nc;
  int64_t nnzb;
  int64_t *rowptr, *colidx;
  double *blocks, *q, *mu;
};

static char g_dat_err[256];
const char *fc3dgpu_dat_last_error(void) { return g_dat_err; }

typedef struct {
  const char *p, *end;
} Cursor;

static int next_token(Cursor *c, char *buf, size_t cap, size_t maxlen) {
  while (c->p < c->end && isspace((unsigned char)*c->p)) c->p++;
  if (c->p >= c->end) return 0;
  size_t n = 0;
  while (c->p < c->end && !isspace((unsigned char)*c->p) && n < maxlen && n + 1 < cap) buf[n++] = *c->p++;
  buf[n] = 0;
  return n > 0;
}

static int read_i64(Cursor *c, int64_t *v) {
  char b[64], *e;
  if (!next_token(c, b, sizeof b, 63)) return 0;
  errno = 0;
  long long x = strtoll(b, &e, 10);
  if (*e || errno) return 0;
  *v = x;
  return 1;
}

/* maxlen: the reference's field width (32 for block values, unlimited
 * otherwise) */
static int read_f64(Cursor *c, double *v, size_t maxlen) {
  char b[512], *e;
  if (!next_token(c, b, sizeof b, maxlen)) return 0;
  *v = strtod(b, &e);
  return *e == 0;
}

void fc3dgpu_dat_close(fc3dgpu_dat *d) {
  if (!d) return;
  free(d->rowptr);
  free(d->colidx);
  free(d->blocks);
  free(d->q);
  free(d->mu);
  free(d);
}

#define FAIL(...)                                                  \
  do {                                                             \
    snprintf(g_dat_err, sizeof g_dat_err, __VA_ARGS__);            \
    goto fail;                                                     \
  } while (0)

static fc3dgpu_dat *parse(const char *text, size_t len) {
  Cursor c = {text, text + len};
  fc3dgpu_dat *d = (fc3dgpu_dat *)calloc(1, sizeof(*d));
  int64_t *bs0 = NULL, *bs1 = NULL, *i1 = NULL, *i2 = NULL;
  double *dense = NULL;
  if (!d) FAIL("out of memory");
  int64_t dim, nc, st, s0, s1;
  if (!read_i64(&c, &dim) || !read_i64(&c, &nc)) FAIL("missing dimension or number of contacts");
  if (dim != 3) FAIL("dimension %lld: only 3D friction-contact problems", (long long)dim);
  if (nc <= 0 || nc > 100000000) FAIL("bad number of contacts %lld", (long long)nc);
  d->dim = 3;
  d->nc = (int)nc;
  const int64_t n = 3 * nc;
  if (!read_i64(&c, &st) || !read_i64(&c, &s0) || !read_i64(&c, &s1)) FAIL("missing matrix header");
  if (s0 != n || s1 != n) FAIL("matrix is %lld x %lld, expected %lld x %lld", (long long)s0, (long long)s1,
                               (long long)n, (long long)n);
  d->rowptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nc + 1));
  if (!d->rowptr) FAIL("out of memory");
  if (st == 0) {
    int64_t r0, r1;
    if (!read_i64(&c, &r0) || !read_i64(&c, &r1) || r0 != n || r1 != n) FAIL("bad dense matrix sizes");
    dense = (double *)malloc(sizeof(double) * (size_t)(n * n));
    if (!dense) FAIL("out of memory");
    for (int64_t i = 0; i < n * n; i++)
      if (!read_f64(&c, &dense[i], 511)) FAIL("dense value %lld unreadable", (long long)i);
    int64_t k = 0;
    for (int pass = 0; pass < 2; pass++) {
      k = 0;
      for (int64_t bi = 0; bi < nc; bi++) {
        if (pass) d->rowptr[bi] = k;
        for (int64_t bj = 0; bj < nc; bj++) {
          int nz = bi == bj;
          for (int a = 0; a < 3 && !nz; a++)
            for (int b = 0; b < 3 && !nz; b++) nz = dense[(3 * bj + b) * n + 3 * bi + a] != 0.0;
          if (!nz) continue;
          if (pass) {
            d->colidx[k] = bj;
            for (int b = 0; b < 3; b++)
              for (int a = 0; a < 3; a++) d->blocks[9 * k + 3 * b + a] = dense[(3 * bj + b) * n + 3 * bi + a];
          }
          k++;
        }
      }
      if (!pass) {
        d->colidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)(k ? k : 1));
        d->blocks = (double *)malloc(sizeof(double) * 9 * (size_t)(k ? k : 1));
        if (!d->colidx || !d->blocks) FAIL("out of memory");
      }
    }
    d->rowptr[nc] = k;
    d->nnzb = k;
  } else if (st == 1) {
    int64_t nb, bn0, bn1, f1, f2;
    if (!read_i64(&c, &nb) || nb <= 0) FAIL("sparse block matrix without blocks");
    if (!read_i64(&c, &bn0) || !read_i64(&c, &bn1) || bn0 != nc || bn1 != nc)
      FAIL("block counts must equal the number of contacts");
    bs0 = (int64_t *)malloc(sizeof(int64_t) * (size_t)nc);
    bs1 = (int64_t *)malloc(sizeof(int64_t) * (size_t)nc);
    if (!bs0 || !bs1) FAIL("out of memory");
    for (int64_t i = 0; i < nc; i++)
      if (!read_i64(&c, &bs0[i]) || bs0[i] != 3 * (i + 1)) FAIL("row block %lld is not 3x3", (long long)i);
    for (int64_t i = 0; i < nc; i++)
      if (!read_i64(&c, &bs1[i]) || bs1[i] != 3 * (i + 1)) FAIL("column block %lld is not 3x3", (long long)i);
    if (!read_i64(&c, &f1) || !read_i64(&c, &f2) || f1 < 1 || f1 > nc + 1 || f2 != nb)
      FAIL("bad filled1 / filled2");
    i1 = (int64_t *)malloc(sizeof(int64_t) * (size_t)f1);
    i2 = (int64_t *)malloc(sizeof(int64_t) * (size_t)f2);
    d->colidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)nb);
    d->blocks = (double *)malloc(sizeof(double) * 9 * (size_t)nb);
    if (!i1 || !i2 || !d->colidx || !d->blocks) FAIL("out of memory");
    for (int64_t i = 0; i < f1; i++)
      if (!read_i64(&c, &i1[i]) || i1[i] < 0 || i1[i] > nb || (i && i1[i] < i1[i - 1]))
        FAIL("bad row pointer entry %lld", (long long)i);
    if (i1[0] != 0 || i1[f1 - 1] != nb) FAIL("row pointer does not span the blocks");
    for (int64_t i = 0; i < f2; i++)
      if (!read_i64(&c, &i2[i]) || i2[i] < 0 || i2[i] >= nc) FAIL("bad column index %lld", (long long)i);
    for (int64_t r = 0; r + 1 < f1; r++)
      for (int64_t b = i1[r]; b < i1[r + 1]; b++) {
        int64_t num;
        if (!read_i64(&c, &num) || num != b) FAIL("block %lld out of sequence", (long long)b);
        for (int e = 0; e < 9; e++)
          if (!read_f64(&c, &d->blocks[9 * b + e], 32)) FAIL("block %lld value unreadable", (long long)b);
        d->colidx[b] = i2[b];
      }
    /* trailing rows without blocks keep the last pointer */
    for (int64_t i = 0; i <= nc; i++) d->rowptr[i] = i < f1 ? i1[i] : i1[f1 - 1];
    d->nnzb = nb;
  } else {
    FAIL("matrix storage type %lld is not read (0 dense, 1 sparse block)", (long long)st);
  }
  d->q = (double *)malloc(sizeof(double) * (size_t)n);
  d->mu = (double *)malloc(sizeof(double) * (size_t)nc);
  if (!d->q || !d->mu) FAIL("out of memory");
  for (int64_t i = 0; i < n; i++)
    if (!read_f64(&c, &d->q[i], 511)) FAIL("q[%lld] unreadable", (long long)i);
  for (int64_t i = 0; i < nc; i++)
    if (!read_f64(&c, &d->mu[i], 511)) FAIL("mu[%lld] unreadable", (long long)i);
  free(bs0);
  free(bs1);
  free(i1);
  free(i2);
  free(dense);
  g_dat_err[0] = 0;
  return d;
fail:
  free(bs0);
  free(bs1);
  free(i1);
  free(i2);
  free(dense);
  fc3dgpu_dat_close(d);
  return NULL;
}

fc3dgpu_dat *fc3dgpu_dat_open(const char *path) {
  if (!path) {
    snprintf(g_dat_err, sizeof g_dat_err, "null path");
    return NULL;
  }
  FILE *f = fopen(path, "rb");
  if (!f) {
    snprintf(g_dat_err, sizeof g_dat_err, "cannot open %s", path);
    return NULL;
  }
  fseek(f, 0, SEEK_END);
  long len = ftell(f);
  fseek(f, 0, SEEK_SET);
  char *text = (char *)malloc((size_t)(len > 0 ? len : 1));
  if (!text || (len > 0 && fread(text, 1, (size_t)len, f) != (size_t)len)) {
    fclose(f);
    free(text);
    snprintf(g_dat_err, sizeof g_dat_err, "cannot read %s", path);
    return NULL;
  }
  fclose(f);
  fc3dgpu_dat *d = parse(text, (size_t)(len > 0 ? len : 0));
  free(text);
  return d;
}

int fc3dgpu_dat_sizes(const fc3dgpu_dat *d, int *nc, int64_t *nnzb) {
  if (!d) return -1;
  if (nc) *nc = d->nc;
  if (nnzb) *nnzb = d->nnzb;
  return 0;
}

int fc3dgpu_dat_get(const fc3dgpu_dat *d, int64_t *rowptr, int64_t *colidx, double *blocks, double *q, double *mu) {
  if (!d) return -1;
  if (rowptr) memcpy(rowptr, d->rowptr, sizeof(int64_t) * (size_t)(d->nc + 1));
  if (colidx) memcpy(colidx, d->colidx, sizeof(int64_t) * (size_t)d->nnzb);
  if (blocks) memcpy(blocks, d->blocks, sizeof(double) * 9 * (size_t)d->nnzb);
  if (q) memcpy(q, d->q, sizeof(double) * 3 * (size_t)d->nc);
  if (mu) memcpy(mu, d->mu, sizeof(double) * (size_t)d->nc);
  return 0;
}

int fc3dgpu_dat_write(const char *path, int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                      const double *q, const double *mu) {
  if (!path || nc <= 0 || !rowptr || !colidx || !blocks || !q || !mu) {
    snprintf(g_dat_err, sizeof g_dat_err, "invalid argument");
    return -1;
  }
  const int64_t nb = rowptr[nc];
  if (rowptr[0] != 0 || nb <= 0) {
    snprintf(g_dat_err, sizeof g_dat_err, "row pointer must start at 0 and hold blocks");
    return -1;
  }
  FILE *f = fopen(path, "w");
  if (!f) {
    snprintf(g_dat_err, sizeof g_dat_err, "cannot open %s for writing", path);
    return -1;
  }
  fprintf(f, "%d\n%d\n", 3, nc);
  fprintf(f, "%d\n%d\n%d\n", 1, 3 * nc, 3 * nc);
  fprintf(f, "%lld\n%d\n%d\n", (long long)nb, nc, nc);
  for (int i = 0; i < nc; i++) fprintf(f, "%d\t", 3 * (i + 1));
  fprintf(f, "\n");
  for (int i = 0; i < nc; i++) fprintf(f, "%d\t", 3 * (i + 1));
  fprintf(f, "\n%d\n%lld\n", nc + 1, (long long)nb);
  for (int i = 0; i <= nc; i++) fprintf(f, "%lld\t", (long long)rowptr[i]);
  fprintf(f, "\n");
  for (int64_t k = 0; k < nb; k++) fprintf(f, "%lld\t", (long long)colidx[k]);
  fprintf(f, "\n");
  for (int64_t k = 0; k < nb; k++) {
    fprintf(f, "%lld\n", (long long)k);
    for (int e = 0; e < 9; e++) fprintf(f, "%32.24e\n", blocks[9 * k + e]);
  }
  for (int64_t i = 0; i < 3LL * nc; i++) fprintf(f, "%32.24e ", q[i]);
  fprintf(f, "\n");
  for (int i = 0; i < nc; i++) fprintf(f, "%32.24e ", mu[i]);
  fprintf(f, "\n");
  int bad = ferror(f);
  if (fclose(f) != 0 || bad) {
    snprintf(g_dat_err, sizeof g_dat_err, "write to %s failed", path);
    return -1;
  }
  return 0;
}
