/* Reading and writing 2D and 3D friction-contact problems in the reference's
 * .dat text format (frictionContact_newFromFile / frictionContact_printInFile,
 * FrictionContactProblem.c:67-132), so that problems saved by Siconos can be
 * loaded without it, and the other way round.  The matrix is returned and
 * written as block-CSR of d x d column-major blocks (d = the dimension; the
 * sparse-block storage); a dense or a CSparse matrix in a file becomes every
 * block holding an entry (dense: a nonzero entry), plus the diagonal
 * blocks. */
#ifndef FC3DGPU_DAT_H
#define FC3DGPU_DAT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fc3dgpu_dat fc3dgpu_dat;

/* Parse a file; NULL on failure (fc3dgpu_dat_last_error() says why). */
fc3dgpu_dat *fc3dgpu_dat_open(const char *path);
void fc3dgpu_dat_close(fc3dgpu_dat *d);
/* Dimension (2 or 3), contacts and blocks of the parsed problem. */
int fc3dgpu_dat_sizes(const fc3dgpu_dat *d, int *dim, int *nc, int64_t *nnzb);
/* Copy out W (rowptr[nc+1], colidx[nnzb], blocks[d*d nnzb]), q[d nc], mu[nc];
 * any pointer may be NULL. */
int fc3dgpu_dat_get(const fc3dgpu_dat *d, int64_t *rowptr, int64_t *colidx, double *blocks, double *q, double *mu);
/* Write a problem of dimension dim with W in sparse-block storage, values as
 * "%32.24e". */
int fc3dgpu_dat_write(const char *path, int dim, int nc, const int64_t *rowptr, const int64_t *colidx,
                      const double *blocks, const double *q, const double *mu);
const char *fc3dgpu_dat_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
