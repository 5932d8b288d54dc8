/* Reading and writing 3D friction-contact problems in the reference's .dat
 * text format (frictionContact_newFromFile / frictionContact_printInFile,
 * FrictionContactProblem.c:67-132), so that problems saved by Siconos can be
 * loaded without it, and the other way round.  The matrix is returned and
 * written as block-CSR of 3x3 column-major blocks (the sparse-block storage);
 * a dense matrix in a file becomes every 3x3 block holding a nonzero entry,
 * plus the diagonal blocks. */
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
/* Contacts and 3x3 blocks of the parsed problem. */
int fc3dgpu_dat_sizes(const fc3dgpu_dat *d, int *nc, int64_t *nnzb);
/* Copy out W (rowptr[nc+1], colidx[nnzb], blocks[9 nnzb]), q[3 nc], mu[nc];
 * any pointer may be NULL. */
int fc3dgpu_dat_get(const fc3dgpu_dat *d, int64_t *rowptr, int64_t *colidx, double *blocks, double *q, double *mu);
/* Write a problem with W in sparse-block storage, values as "%32.24e". */
int fc3dgpu_dat_write(const char *path, int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                      const double *q, const double *mu);
const char *fc3dgpu_dat_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
