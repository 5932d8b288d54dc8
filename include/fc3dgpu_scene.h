/* Seeded sphere-lattice friction-contact scenes.
 *
 * The reference ships no generator for its benchmark scenes; this one builds
 * the workload the benchmarks are quoted on: X*Y*Z rigid spheres (radius
 * 0.5, mass 1, inertia 0.1*I3) on a cubic lattice of spacing 1.0, centres at
 * (i, j, k + 0.5) jittered by N(0, jitter_std^2) per coordinate, contacts
 * between face-neighbour spheres plus a ground plane under the bottom layer.
 * Each contact's frame has the normal along the centre-to-centre line (ground:
 * +z) and Gram-Schmidt tangents.  W = H M^-1 H^T is assembled in FP64 as 3x3
 * column-major blocks in block-CSR order (the SparseBlockStructuredMatrix
 * layout of the reference, SparseBlockMatrix.h:82-121), and
 * q = H (v0 + h g) with v0 ~ N(0, v0_std^2) per degree of freedom.
 *
 * Random numbers come from splitmix64 and the Marsaglia polar method with a
 * logarithm written from its series definition, built with
 * -ffp-contract=off, so a seed gives the same scene bit for bit on x86-64
 * and aarch64.
 */
#ifndef FC3DGPU_SCENE_H
#define FC3DGPU_SCENE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fc3dgpu_lattice fc3dgpu_lattice;

/* Create the scene geometry and the initial velocities.  Returns NULL on a
 * bad size (any dimension < 1) or allocation failure. */
fc3dgpu_lattice *fc3dgpu_lattice_create(int nx, int ny, int nz, uint64_t seed, double jitter_std, double v0_std);
void fc3dgpu_lattice_free(fc3dgpu_lattice *L);

/* Number of bodies, contacts and 3x3 blocks (diagonal included) of W. */
int fc3dgpu_lattice_sizes(const fc3dgpu_lattice *L, int *nbodies, int *ncontacts, int64_t *nnzb);

/* Fill W in block-CSR: rowptr[nc+1], colidx[nnzb] (sorted per row),
 * blocks[9*nnzb] column-major.  Returns 0. */
int fc3dgpu_lattice_fill_W(const fc3dgpu_lattice *L, int64_t *rowptr, int64_t *colidx, double *blocks);

/* q = H (v + h g) for the current body velocities; g = -9.81 e_z. */
int fc3dgpu_lattice_fill_q(const fc3dgpu_lattice *L, double h, double *q);

/* Per-contact normal gap (centre distance minus radii; ground: height minus
 * radius) and contact bodies (A = -1 for the ground; B > A). */
int fc3dgpu_lattice_fill_geometry(const fc3dgpu_lattice *L, double *gap, int32_t *bodyA, int32_t *bodyB);

/* Contact geometry for an assembly of W and q elsewhere: frames (rows n, t1,
 * t2; 9 per contact), contact points (3 per contact), body centres (3 per
 * body), masses, isotropic inertias and velocities (6 per body).  Any
 * pointer may be NULL. */
int fc3dgpu_lattice_fill_contacts(const fc3dgpu_lattice *L, double *frame, double *point, double *body_pos,
                                  double *body_mass, double *body_inertia, double *vel);

/* The same scene in the global form of the reference's
 * GlobalFrictionContactProblem (M v = q + H r, u = H^T v + b): 6 degrees of
 * freedom per body (linear then angular velocity), M = diag(m I3, I I3),
 * H (6 nb x 3 nc) with, for contact c on body b (sign s = +1 for body B, -1
 * for body A, arm d = contact point - centre, frame rows R_0..R_2),
 * H[6b + a, 3c + k] = s R_k[a] and H[6b + 3 + a, 3c + k] = s (d x R_k)[a],
 * so that H^T M^-1 H is the W of fc3dgpu_lattice_fill_W divided by
 * mass_scale, the factor applied to every mass and inertia (the reference's
 * global NSGS takes unit steps, r <- proj(r - u), and diverges once W has
 * an eigenvalue above 2: about 19 at unit mass, so 10 is the scale of the
 * global benchmark); q = M (v + h g), b = 0.  Sizes: n = 6 nb,
 * nnz(M) = n, nnz(H) = 18 x (body-contact incidences). */
int fc3dgpu_lattice_global_sizes(const fc3dgpu_lattice *L, int64_t *n, int64_t *nnzH);
/* M and H as CSR (row pointers n + 1, ascending columns, values), q[n],
 * b[3 nc]. */
int fc3dgpu_lattice_fill_global(const fc3dgpu_lattice *L, double h, double mass_scale, int64_t *Mp, int64_t *Mi, double *Mx,
                                int64_t *Hp, int64_t *Hi, double *Hx, double *q, double *b);

/* Random walk of the body velocities: v += N(0, std^2) per degree of
 * freedom, from its own stream seeded by seed. */
int fc3dgpu_lattice_perturb_velocities(fc3dgpu_lattice *L, uint64_t seed, double std);

/* Standard normal samples from the generator's own stream (exposed for
 * tests of the sampler). */
void fc3dgpu_normal_fill(uint64_t seed, double *out, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
