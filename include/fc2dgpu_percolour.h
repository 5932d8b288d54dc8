/* fc2dgpu_percolour: the reference's own GPU design for 2D friction contact,
 * re-implemented on this library's colouring so that it can be measured on
 * the same GPU as the cluster-resident solver of fc2dgpu.h.
 *
 * The reference solver SICONOS_FRICTION_2D_NSGS_GRAPH_PERMUT_CUDA
 * (FrictionContact/parallel/gpu/fc2d_nsgs_graph_permut_cuda.cu:303-710)
 * colours the contacts with PETSc (graph_tools.c:942), which is not available
 * here, so the file itself does not build.  Its structure is kept:
 *   - rows and columns permuted by colour; per colour a scalar CSR of the
 *     off-diagonal blocks' rows (64-bit indices, FP64);
 *   - per sweep, one CUDA graph replay of: a memset, then per colour a
 *     cuSPARSE SpMV y_c = A_c z and a local-solve kernel (one thread per
 *     contact, 256 threads per block) that adds q, solves the 2x2 problem and
 *     accumulates |z|^2 and |dz|^2 with a block tree and atomicAdd;
 *   - after each replay, two blocking 8-byte device-to-host copies and the
 *     convergence test on the host; the full error (when the light error is
 *     below the working tolerance, and at the end) on the host after a
 *     device-to-host copy of z.
 * This is a comparator, not a solver of the drop-in API: the sums of the
 * SpMV differ in order from the reference CPU sweep, so its iterates agree
 * with the oracle's to rounding, not bit for bit. */
#ifndef FC2DGPU_PERCOLOUR_H
#define FC2DGPU_PERCOLOUR_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fc2dgpu_percolour fc2dgpu_percolour;

/* W as block-CSR of 2x2 column-major blocks, q[2 nc], mu[nc]; colour_kind as
 * for fc3dgpu_colour.  NULL on failure (message in fc3dgpu_last_error). */
fc2dgpu_percolour *fc2dgpu_percolour_create(int device, int nc, const int64_t *rowptr, const int64_t *colidx,
                                            const double *blocks, const double *q, const double *mu,
                                            int colour_kind);
void fc2dgpu_percolour_destroy(fc2dgpu_percolour *h);
/* Solve from r0 (contact order; NULL = zero) with LIGHT_WITH_FULL_FINAL as
 * the reference's CUDA solver runs it; *ms is the host wall time of the
 * iteration loop (graph replays and the per-sweep copies included). */
int fc2dgpu_percolour_solve(fc2dgpu_percolour *h, const double *r0, double tol, int max_iter, int *iters,
                            double *error, int *info, double *ms);
/* Run the reference's own local-solve kernel in the sweep instead of this
 * library's: `path` names a CUDA library image (cubin or fatbin for this
 * device) holding fc2d_nsgs_local_solve_kernel_range_reduce compiled from
 * fc2d_nsgs_graph_permut_cuda.cu:213-300, or ..._range_reduce_2 from
 * fc2d_nsgs_graph_permut_cuda_blocklegacy.cu:215-300 (C++ linkage; arguments as that
 * file launches it at :583-586: colour range [k1, k2) in the permuted
 * numbering, SpMV output indexed by the global row).  The sweep graph is
 * recaptured; 0 on success, NUMERICS_ERR_INVALID_ARGUMENT when the image
 * does not load or lacks the kernel (message in fc3dgpu_last_error). */
int fc2dgpu_percolour_use_kernel_file(fc2dgpu_percolour *h, const char *path);
/* on = 1: sweep as the reference's BLOCKLEGACY variant
 * (SICONOS_FRICTION_2D_NSGS_GRAPH_PERMUT_CUDA_BLOCKLEGACY,
 * fc2d_nsgs_graph_permut_cuda_blocklegacy.cu:380-567): per colour
 * cusparseDbsrmv of its block rows (2x2 blocks, column-major, int32 indices,
 * diagonal blocks kept with zero values) and the local-solve kernel, issued
 * every sweep without a graph; 0: back to the graph of scalar-CSR SpMVs.
 * The kernel is this library's or the image's (..._range_reduce_2 in an
 * image of the BLOCKLEGACY file). */
int fc2dgpu_percolour_use_bsr(fc2dgpu_percolour *h, int on);
/* Reaction and velocity of the last solve in contact order. */
int fc2dgpu_percolour_get_r_u(fc2dgpu_percolour *h, double *r, double *u);

#ifdef __cplusplus
}
#endif
#endif
