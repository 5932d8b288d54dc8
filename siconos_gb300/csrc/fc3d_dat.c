/* Text (.dat) files of friction-contact problems (2D and 3D), in the format
 * the reference reads and writes (frictionContact_newFromFile /
 * frictionContact_printInFile, FrictionContactProblem.c:67-132):
 *
 *   dimension d (2 or 3)     number of contacts nc
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
 *     2 (sparse):            the storage's origin, then the CSparse text
 *                            print of the matrix: a version line, a header
 *                            "m-by-n, nzmax: .. nnz: .." ("csr:" or
 *                            "triplet:" before it for those forms), then per
 *                            column (row) "col j : locations a to b" and one
 *                            "i : value" line per entry, or for triplets one
 *                            "i j : value" line per entry
 *                            (NSM_new_from_file NumericsSparseMatrix.c:555,
 *                            CSparseMatrix_new_from_file CSparseMatrix.c:651,
 *                            CSparseMatrix_print_in_file CSparseMatrix.c:883)
 *   q (d nc values)          mu (nc values)
 *
 * Values are written as "%32.24e" (25 significant digits: a double reads
 * back exactly); the reference reads sparse-block values with a 32-character
 * field and q, mu with a plain field, and so does this reader.  Whatever the
 * storage, the matrix comes out as block-CSR of d x d column-major blocks,
 * columns increasing in each block row: from a dense or a sparse matrix
 * every block holding an entry (dense: a nonzero entry), and every diagonal
 * block.  (Sparse files print values with 6 significant digits: those
 * matrices are only that accurate.) */
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

static _Thread_local char g_dat_err[256];
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

/* the rest of the current line, without its end of line */
static int next_line(Cursor *c, char *buf, size_t cap) {
  if (c->p >= c->end) return 0;
  size_t n = 0;
  while (c->p < c->end && *c->p != '\n') {
    if (n + 1 < cap) buf[n++] = *c->p;
    c->p++;
  }
  if (c->p < c->end) c->p++;
  buf[n] = 0;
  return 1;
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

/* maxlen: the reference's field width (32 for sparse-block values,
 * unlimited otherwise) */
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

#define FAIL(...)                                       \
  do {                                                  \
    snprintf(g_dat_err, sizeof g_dat_err, __VA_ARGS__); \
    goto fail;                                          \
  } while (0)

typedef struct {
  int64_t r, c;
  double v;
} Entry;

static int64_t g_bs;
static int cmp_entry(const void *a, const void *b) {
  const Entry *x = (const Entry *)a, *y = (const Entry *)b;
  int64_t kx = x->r / g_bs, ky = y->r / g_bs;
  if (kx != ky) return kx < ky ? -1 : 1;
  kx = x->c / g_bs;
  ky = y->c / g_bs;
  if (kx != ky) return kx < ky ? -1 : 1;
  return 0;
}

/* Block-CSR of bs x bs blocks from entries (any order; duplicates summed),
 * with every diagonal block present. */
static int entries_to_blocks(fc3dgpu_dat *d, Entry *e, int64_t ne, int64_t bs) {
  const int64_t nc = d->nc;
  /* add a zero entry on every diagonal block so that it exists */
  Entry *all = (Entry *)malloc(sizeof(Entry) * (size_t)(ne + nc));
  if (!all) return -1;
  memcpy(all, e, sizeof(Entry) * (size_t)ne);
  for (int64_t i = 0; i < nc; i++) all[ne + i] = (Entry){bs * i, bs * i, 0.0};
  ne += nc;
  g_bs = bs;
  qsort(all, (size_t)ne, sizeof(Entry), cmp_entry);
  int64_t nb = 0;
  for (int64_t k = 0; k < ne; k++)
    if (k == 0 || cmp_entry(&all[k], &all[k - 1]) != 0) nb++;
  d->colidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)nb);
  d->blocks = (double *)calloc((size_t)(bs * bs * nb), sizeof(double));
  if (!d->colidx || !d->blocks) {
    free(all);
    return -1;
  }
  int64_t b = -1;
  for (int64_t i = 0; i <= nc; i++) d->rowptr[i] = 0;
  for (int64_t k = 0; k < ne; k++) {
    if (k == 0 || cmp_entry(&all[k], &all[k - 1]) != 0) {
      b++;
      d->colidx[b] = all[k].c / bs;
      d->rowptr[all[k].r / bs + 1]++;
    }
    d->blocks[bs * bs * b + bs * (all[k].c % bs) + all[k].r % bs] += all[k].v;
  }
  for (int64_t i = 0; i < nc; i++) d->rowptr[i + 1] += d->rowptr[i];
  d->nnzb = nb;
  free(all);
  return 0;
}

/* The CSparse text print of an n x n matrix (origin already read). */
static int parse_csparse(fc3dgpu_dat *d, Cursor *c, int64_t n, int64_t bs) {
  char line[2048];
  int64_t m = -1, ncol = -1, nnz = -1;
  int is_csr = 0, is_triplet = 0;
  /* the header line is the first one holding "-by-" */
  for (int tries = 0; tries < 8 && m < 0; tries++) {
    if (!next_line(c, line, sizeof line)) break;
    const char *by = strstr(line, "-by-");
    if (!by) continue;
    is_csr = strstr(line, "csr:") != NULL;
    is_triplet = strstr(line, "triplet:") != NULL;
    const char *s = by;
    while (s > line && isdigit((unsigned char)s[-1])) s--;
    m = strtoll(s, NULL, 10);
    ncol = strtoll(by + 4, NULL, 10);
    const char *z = strstr(line, "nnz:");
    if (z) nnz = strtoll(z + 4, NULL, 10);
  }
  if (m != n || ncol != n) {
    snprintf(g_dat_err, sizeof g_dat_err, "sparse matrix header missing or not %lld x %lld", (long long)n,
             (long long)n);
    return -1;
  }
  if (nnz < 0) {
    snprintf(g_dat_err, sizeof g_dat_err, "sparse matrix without its number of entries");
    return -1;
  }
  Entry *e = (Entry *)malloc(sizeof(Entry) * (size_t)(nnz ? nnz : 1));
  if (!e) {
    snprintf(g_dat_err, sizeof g_dat_err, "out of memory");
    return -1;
  }
  int64_t k = 0;
  if (is_triplet) {
    for (; k < nnz; k++) {
      int64_t i, j;
      char colon[8];
      if (!read_i64(c, &i) || !read_i64(c, &j) || !next_token(c, colon, sizeof colon, 7) || strcmp(colon, ":") ||
          !read_f64(c, &e[k].v, 511) || i < 0 || i >= n || j < 0 || j >= n)
        goto bad;
      e[k].r = i;
      e[k].c = j;
    }
  } else {
    for (int64_t j = 0; j < n; j++) {
      char w[64];
      int64_t jj, a, b;
      /* "col j : locations a to b" (or "row j : ...") */
      if (!next_token(c, w, sizeof w, 63) || (strcmp(w, "col") && strcmp(w, "row")) || !read_i64(c, &jj) ||
          jj != j || !next_token(c, w, sizeof w, 63) || strcmp(w, ":") || !next_token(c, w, sizeof w, 63) ||
          strcmp(w, "locations") || !read_i64(c, &a) || !next_token(c, w, sizeof w, 63) || strcmp(w, "to") ||
          !read_i64(c, &b) || a != k || b + 1 < a || b + 1 > nnz)
        goto bad;
      for (; k <= b; k++) {
        int64_t i;
        if (!read_i64(c, &i) || !next_token(c, w, sizeof w, 63) || strcmp(w, ":") || !read_f64(c, &e[k].v, 511) ||
            i < 0 || i >= n)
          goto bad;
        e[k].r = is_csr ? j : i;
        e[k].c = is_csr ? i : j;
      }
    }
    if (k != nnz) goto bad;
  }
  {
    int rc = entries_to_blocks(d, e, nnz, bs);
    free(e);
    if (rc) snprintf(g_dat_err, sizeof g_dat_err, "out of memory");
    return rc;
  }
bad:
  snprintf(g_dat_err, sizeof g_dat_err, "sparse matrix entry %lld unreadable", (long long)k);
  free(e);
  return -1;
}

static fc3dgpu_dat *parse(const char *text, size_t len) {
  Cursor c = {text, text + len};
  fc3dgpu_dat *d = (fc3dgpu_dat *)calloc(1, sizeof(*d));
  int64_t *bs0 = NULL, *bs1 = NULL, *i1 = NULL, *i2 = NULL;
  double *dense = NULL;
  if (!d) FAIL("out of memory");
  int64_t dim, nc, st, s0, s1;
  if (!read_i64(&c, &dim) || !read_i64(&c, &nc)) FAIL("missing dimension or number of contacts");
  if (dim != 2 && dim != 3) FAIL("dimension %lld: 2D or 3D friction-contact problems only", (long long)dim);
  if (nc <= 0 || nc > 100000000) FAIL("bad number of contacts %lld", (long long)nc);
  const int64_t bs = dim;
  d->dim = (int)dim;
  d->nc = (int)nc;
  const int64_t n = bs * nc;
  if (!read_i64(&c, &st) || !read_i64(&c, &s0) || !read_i64(&c, &s1)) FAIL("missing matrix header");
  if (s0 != n || s1 != n)
    FAIL("matrix is %lld x %lld, expected %lld x %lld", (long long)s0, (long long)s1, (long long)n, (long long)n);
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
          for (int64_t a = 0; a < bs && !nz; a++)
            for (int64_t b = 0; b < bs && !nz; b++) nz = dense[(bs * bj + b) * n + bs * bi + a] != 0.0;
          if (!nz) continue;
          if (pass) {
            d->colidx[k] = bj;
            for (int64_t b = 0; b < bs; b++)
              for (int64_t a = 0; a < bs; a++)
                d->blocks[bs * bs * k + bs * b + a] = dense[(bs * bj + b) * n + bs * bi + a];
          }
          k++;
        }
      }
      if (!pass) {
        d->colidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)(k ? k : 1));
        d->blocks = (double *)malloc(sizeof(double) * (size_t)(bs * bs * (k ? k : 1)));
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
      if (!read_i64(&c, &bs0[i]) || bs0[i] != bs * (i + 1))
        FAIL("row block %lld is not %lldx%lld", (long long)i, (long long)bs, (long long)bs);
    for (int64_t i = 0; i < nc; i++)
      if (!read_i64(&c, &bs1[i]) || bs1[i] != bs * (i + 1))
        FAIL("column block %lld is not %lldx%lld", (long long)i, (long long)bs, (long long)bs);
    if (!read_i64(&c, &f1) || !read_i64(&c, &f2) || f1 < 1 || f1 > nc + 1 || f2 != nb)
      FAIL("bad filled1 / filled2");
    i1 = (int64_t *)malloc(sizeof(int64_t) * (size_t)f1);
    i2 = (int64_t *)malloc(sizeof(int64_t) * (size_t)f2);
    d->colidx = (int64_t *)malloc(sizeof(int64_t) * (size_t)nb);
    d->blocks = (double *)malloc(sizeof(double) * (size_t)(bs * bs * nb));
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
        for (int64_t e = 0; e < bs * bs; e++)
          if (!read_f64(&c, &d->blocks[bs * bs * b + e], 32)) FAIL("block %lld value unreadable", (long long)b);
        d->colidx[b] = i2[b];
      }
    /* trailing rows without blocks keep the last pointer */
    for (int64_t i = 0; i <= nc; i++) d->rowptr[i] = i < f1 ? i1[i] : i1[f1 - 1];
    d->nnzb = nb;
  } else if (st == 2) {
    int64_t origin;
    if (!read_i64(&c, &origin)) FAIL("sparse matrix without its origin");
    if (parse_csparse(d, &c, n, bs)) goto fail;
  } else {
    FAIL("matrix storage type %lld is not read (0 dense, 1 sparse block, 2 sparse)", (long long)st);
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

int fc3dgpu_dat_sizes(const fc3dgpu_dat *d, int *dim, int *nc, int64_t *nnzb) {
  if (!d) return -1;
  if (dim) *dim = d->dim;
  if (nc) *nc = d->nc;
  if (nnzb) *nnzb = d->nnzb;
  return 0;
}

int fc3dgpu_dat_get(const fc3dgpu_dat *d, int64_t *rowptr, int64_t *colidx, double *blocks, double *q, double *mu) {
  if (!d) return -1;
  const size_t bs = (size_t)d->dim;
  if (rowptr) memcpy(rowptr, d->rowptr, sizeof(int64_t) * (size_t)(d->nc + 1));
  if (colidx) memcpy(colidx, d->colidx, sizeof(int64_t) * (size_t)d->nnzb);
  if (blocks) memcpy(blocks, d->blocks, sizeof(double) * bs * bs * (size_t)d->nnzb);
  if (q) memcpy(q, d->q, sizeof(double) * bs * (size_t)d->nc);
  if (mu) memcpy(mu, d->mu, sizeof(double) * (size_t)d->nc);
  return 0;
}

int fc3dgpu_dat_write(const char *path, int dim, int nc, const int64_t *rowptr, const int64_t *colidx,
                      const double *blocks, const double *q, const double *mu) {
  if (!path || (dim != 2 && dim != 3) || nc <= 0 || !rowptr || !colidx || !blocks || !q || !mu) {
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
  const int bs = dim;
  fprintf(f, "%d\n%d\n", dim, nc);
  fprintf(f, "%d\n%d\n%d\n", 1, bs * nc, bs * nc);
  fprintf(f, "%lld\n%d\n%d\n", (long long)nb, nc, nc);
  for (int i = 0; i < nc; i++) fprintf(f, "%d\t", bs * (i + 1));
  fprintf(f, "\n");
  for (int i = 0; i < nc; i++) fprintf(f, "%d\t", bs * (i + 1));
  fprintf(f, "\n%d\n%lld\n", nc + 1, (long long)nb);
  for (int i = 0; i <= nc; i++) fprintf(f, "%lld\t", (long long)rowptr[i]);
  fprintf(f, "\n");
  for (int64_t k = 0; k < nb; k++) fprintf(f, "%lld\t", (long long)colidx[k]);
  fprintf(f, "\n");
  for (int64_t k = 0; k < nb; k++) {
    fprintf(f, "%lld\n", (long long)k);
    for (int e = 0; e < bs * bs; e++) fprintf(f, "%32.24e\n", blocks[(int64_t)bs * bs * k + e]);
  }
  for (int64_t i = 0; i < (int64_t)bs * nc; i++) fprintf(f, "%32.24e ", q[i]);
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
