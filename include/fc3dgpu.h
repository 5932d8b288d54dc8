/* fc3dgpu: GB300 (sm_103a) coloured NSGS for the 3D Coulomb friction-contact
 * problem, as a drop-in solver beside the reference's
 * SICONOS_FRICTION_3D_NSGS.
 *
 * The entry points below are what the reference's solver registry binds
 * (solver_registry.h:75-95): a solve function with the registry's
 * SolverSolveFunc signature and a set_default function.  Host code is C;
 * the CUDA work sits behind the device-resident API at the end of this
 * header.  All buffers in the solver-level calls are HOST memory owned by the
 * caller, exactly as for the reference solver.
 *
 * Error behaviour follows the reference: the solve returns 0 on
 * convergence, 1 when not converged, NUMERICS_ERR_MAX_ITER (-20) when the
 * iteration budget ran out, and a negative NUMERICS_ERR_* code for invalid
 * input.  There is no CPU fallback: without a usable CUDA device the solve
 * returns NUMERICS_ERR_NOT_IMPLEMENTED and fc3dgpu_last_error() says why.
 */
#ifndef FC3DGPU_H
#define FC3DGPU_H

#ifdef FC3DGPU_USE_SICONOS_HEADERS
#include "FrictionContactProblem.h"
#include "SolverOptions.h"
#include "numerics_errors.h"
#else
#include "siconos_numerics_abi.h"
#endif
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* New solver id in the free FC3D range (FrictionContact_options.h:83-131
 * uses 500-530; the driver accepts 500-599, fc3d_driver.c:212).  A Siconos
 * build that lists it in that enum defines FC3DGPU_ID_IN_SICONOS_ENUM. */
#ifndef FC3DGPU_ID_IN_SICONOS_ENUM
#define SICONOS_FRICTION_3D_NSGS_GPU 531
#endif

/* GPU knobs live in option slots the NSGS solver does not use.  dparam
 * 20-22 keep the reference's timing meaning (SolverOptions.h:118-120). */
#define FC3DGPU_IPARAM_PRECISION 23   /* in: 0 FP32 sweeps + FP64 polish (default), 1 FP64 sweeps only */
#define FC3DGPU_IPARAM_LANES 24       /* in: lanes per contact 1, 2, 4, 8; 0 = autotune (default) */
#define FC3DGPU_IPARAM_WARMSTART 25   /* in: 0 = reaction on entry (default), 1 = learned proposal */
#define FC3DGPU_IPARAM_COLOURING 26   /* in: colouring kind, see FC3DGPU_COLOURING_DEFAULT */
#define FC3DGPU_IPARAM_SWEEPS_FP32 27 /* out: FP32 sweeps done */
/* Colouring kind: low byte 0 = hash priority, 1 = largest degree first;
 * FC3DGPU_COLOUR_PASSES(n) adds n iterated-greedy recolouring passes (the
 * classes revisited in reverse order), which shrink the small last colours:
 * on the 60x60x30 lattice 10 colours become 8; FC3DGPU_COLOUR_KEMPE then
 * empties classes by Kempe-chain exchanges (fc3dgpu_colour_reduce, each
 * problem of a batch on its own): 8 become 6, for about 70 ms of host work
 * per new structure at 320,400 contacts (worth it when a structure is solved
 * more than a few times; leave it out when the contact set changes at every
 * call). */
#define FC3DGPU_COLOUR_PASSES(n) ((n) << 8)
#define FC3DGPU_COLOUR_KEMPE (1 << 16)
#define FC3DGPU_COLOURING_DEFAULT (FC3DGPU_COLOUR_PASSES(4) | FC3DGPU_COLOUR_KEMPE)
#define FC3DGPU_IPARAM_SWEEPS_FP64 28 /* out: FP64 sweeps done */
#define FC3DGPU_IPARAM_COLOURS 29     /* out: number of colours */
#define FC3DGPU_DPARAM_SWITCH_TOL 23  /* in: FP32 -> FP64 switch on the incremental error (default 1e-6) */
#define FC3DGPU_DPARAM_LOCAL_TOL32 24 /* in: FP32 local Newton tolerance (default 1e-5) */
#define FC3DGPU_DPARAM_STALL 25       /* in: FP32 stall window in sweeps (default 64) */
#define FC3DGPU_DPARAM_MS_SWEEP32 26  /* out: mean device time of one FP32 sweep (ms) */
#define FC3DGPU_DPARAM_MS_SWEEP64 27  /* out: mean device time of one FP64 sweep (ms) */
#define FC3DGPU_DPARAM_MS_SOLVE 28    /* out: device time of the whole solve (ms) */
#define FC3DGPU_DPARAM_INCR_ERROR 29  /* out: last incremental error */

/* Registry-facing solver functions.  fc3dgpu_nsgs has the signature of
 * fc3d_nsgs's wrapper (fc3d_nsgs.c:968): problem, reaction (in: warm start,
 * out: solution), velocity (out: W r + q), options. */
int fc3dgpu_nsgs(FrictionContactProblem *problem, double *reaction, double *velocity, SolverOptions *options);
int fc3dgpu_nsgs_solve_wrap(void *problem, double *reaction, double *velocity, SolverOptions *options);
int fc3dgpu_nsgs_init_wrap(void *problem, SolverOptions *options);
void fc3dgpu_nsgs_free_wrap(void *problem, SolverOptions *options);

/* fc3d_driver (fc3d_driver.c:77-145) restricted to this solver id:
 * validation, trivial take-off case (r = 0, u = q when every q_n >=
 * -DBL_EPSILON), then fc3dgpu_nsgs.  Inside Siconos the reference's own
 * fc3d_driver plays this part once the solver is registered. */
int fc3dgpu_driver(FrictionContactProblem *problem, double *reaction, double *velocity, SolverOptions *options);

/* Defaults of fc3d_nsgs_set_default (fc3d_nsgs.c:919-950) -- LIGHT_WITH_FULL_FINAL,
 * GIVEN_VALUE local tolerance, no shuffle/freezing/filter/relaxation, tol
 * 1e-4, one internal OC_NSN_GP_HYBRID solver with the one-contact defaults
 * (onecontact.c:1037-1056: 100 Newton iterations, tol 1e-14, GP line search
 * of 10, NSN_AND_PLI_NSN_LOOP, one loop, 100 PLI iterations) -- plus the GPU
 * knobs above.  Internal solver options are allocated with calloc, like
 * solver_options_create, when options has none.  fc3dgpu_nsgs also honours
 * the other error evaluations (FULL with its frequency, LIGHT, ADAPTIVE) and
 * the ADAPTIVE / ADAPTIVE_N_CONTACT local tolerances as fc3d_nsgs.c:711-900
 * does, with FP64 sweeps, one device call a sweep; relaxation and the filter
 * of local solutions in the FP64 sweeps; shuffle and freezing give
 * NUMERICS_ERR_NOT_IMPLEMENTED. */
void fc3dgpu_nsgs_set_default(SolverOptions *options);

/* Stand-alone options (what solver_options_create(SICONOS_FRICTION_3D_NSGS_GPU)
 * returns once the solver is registered): max_iter 1000, tol 1e-4. */
SolverOptions *fc3dgpu_options_create(void);
void fc3dgpu_options_delete(SolverOptions *options);

/* Release the device copy of W cached in options->solverData. */
void fc3dgpu_release(SolverOptions *options);

/* fc3d_compute_error (fc3d_compute_error.c:70-122) on the GPU in FP64:
 * velocity <- W reaction + q, *error = relative natural-map error.
 * Returns 0 when error <= tolerance, 1 otherwise, <0 on failure. */
int fc3dgpu_compute_error(FrictionContactProblem *problem, double *reaction, double *velocity, double tolerance,
                          double norm_q, double *error);

/* Many independent problems in one persistent launch (uneven sizes).  Each
 * problem uses the options' tolerance and budget; info[k] per problem. */
int fc3dgpu_nsgs_batch(int nproblems, FrictionContactProblem **problems, double **reactions, double **velocities,
                       SolverOptions *options, int *info);

/* Device colouring of the contact conflict graph of a block-CSR structure
 * (two contacts conflict when W has a block between them).  Greedy in
 * decreasing priority, computed in Jones-Plassmann rounds on the GPU.
 * Returns the number of colours, <0 on failure. */
int fc3dgpu_colour(int nc, const int64_t *rowptr, const int64_t *colidx, int kind, int32_t *colour);
/* Host Kempe-chain reduction of a proper colouring: empties the highest
 * colour classes while each of their contacts can take a lower colour,
 * directly or after exchanging two colours on Kempe components (on a cubic
 * sphere lattice: the greedy 8 colours become 6).  gptr/adj: the conflict
 * graph as symmetric CSR; work_cap bounds one Kempe search (<= 0: nc).
 * Returns the new number of colours (<0: out of memory, colour still
 * proper).  Colouring kinds with FC3DGPU_COLOUR_KEMPE apply it after the
 * device colouring. */
int fc3dgpu_colour_reduce(int nc, const int *gptr, const int *adj, int *colour, int ncol, int work_cap);
/* The same for a batch: each group (rows group_off[g] .. group_off[g+1]-1,
 * conflicting only within the group; gptr/adj over all rows) reduced on its
 * own, exactly as fc3dgpu_colour_reduce reduces it alone, by up to nthreads
 * host threads.  Returns the largest number of colours over the groups (<0:
 * out of memory, colour still proper). */
int fc3dgpu_colour_reduce_groups(int ngroups, const int *group_off, const int *gptr, const int *adj, int *colour,
                                 int nthreads);

/* Device facts: SM count, L2 bytes, whether kernels can read pageable host
 * memory (and through the host page tables), cooperative launch support,
 * compute capability (major*10+minor).  Returns 0 or a negative code. */
int fc3dgpu_device_info(int device, long long *out6);

/* Last error message of this thread ("" when none). */
const char *fc3dgpu_last_error(void);

/* ------------------------------------------------------------------
 * Device-resident API: a problem uploaded once and solved many times with
 * inputs already in HBM (time stepping, benchmarks).
 * ------------------------------------------------------------------ */
typedef struct fc3dgpu_ctx fc3dgpu_ctx;

typedef struct {
  double tol;          /* user tolerance on fc3d_compute_error */
  int max_iter;        /* total sweep budget */
  int precision;       /* 0 mixed (FP32 sweeps + FP64 polish), 1 FP64 only,
                          2 mixed with the fast FP64 polish, 3 fast FP64 only
                          (fast: the one-contact solver's FP64 divisions and
                          square roots refined from FP32 seeds, about 1e-14
                          relative; the error that decides convergence stays
                          exact FP64) */
  int lanes;           /* lanes per contact (1,2,4,8); 0 = autotune */
  double switch_tol;   /* FP32 phase ends when incr error < switch_tol ... */
  int stall_window;    /* ... or has not improved for this many sweeps */
  double local_tol;    /* FP64 local solver tolerance (1e-14) */
  double local_tol32;  /* FP32 local solver tolerance */
  int newton_max;      /* 100 */
  int pli_max;         /* 100 */
  int ls_max;          /* 10 */
  int fp32_only;       /* 1: run FP32 sweeps only, for throughput runs */
  int local_mode32;    /* FP32 one-contact solver: 0 the reference's hybrid
                          (default), 1 damped Newton alone */
  int relax;           /* FP64 sweeps: each new reaction relaxed,
                          omega r_new + (1 - omega) r_old (0 = off) */
  double omega;
  int filter;          /* FP64 sweeps: keep the old reaction when the local
                          residual is not finite or above 1 (0 = off); the
                          FP32 sweeps do neither, so a solve with either
                          runs FP64 sweeps only */
} fc3dgpu_params;

typedef struct {
  int info;            /* as the solver's return value */
  int status;          /* device status word; 0 = ok, else a FC3DGPU_STATUS_* bit */
  int sweeps32, sweeps64;
  int colours, lanes, grid;
  double incr_error;   /* last incremental error */
  double error;        /* final fc3d_compute_error (FP64) */
  double ms_total;     /* device time of the solve (CUDA events) */
  double ms_fp32, ms_fp64;
  double bytes_sweep32, bytes_sweep64; /* algorithmic bytes per sweep */
} fc3dgpu_stats;

#define FC3DGPU_STATUS_BARRIER_TIMEOUT 1
#define FC3DGPU_STATUS_NONFINITE 2

void fc3dgpu_params_default(fc3dgpu_params *p);
fc3dgpu_ctx *fc3dgpu_ctx_create(int device);
void fc3dgpu_ctx_destroy(fc3dgpu_ctx *ctx);
/* Upload W as block-CSR (blocks: 9 doubles per block, column-major) and
 * build the coloured device layout. */
int fc3dgpu_ctx_set_W(fc3dgpu_ctx *ctx, int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                      int colour_kind);
/* Many independent problems as one block-diagonal W: the union block-CSR
 * (problem k owns the contacts after those of problems 0..k-1; no block may
 * join two problems), the number of problems and each one's contact count.
 * Each problem is coloured as it would be alone.  q, mu and r are then
 * passed as the concatenation of the problems' vectors. */
/* fc3dgpu_ctx_set_W for new values of W: when the block structure (rowptr,
 * colidx) and the colouring kind equal the current ones (compared on the
 * device), only the blocks are uploaded and refilled into the current
 * layout; otherwise it is fc3dgpu_ctx_set_W.  Time stepping with fixed
 * contacts and the driver's cache use it. */
int fc3dgpu_ctx_update_W(fc3dgpu_ctx *ctx, int nc, const int64_t *rowptr, const int64_t *colidx, const double *blocks,
                         int colour_kind);
/* fc3dgpu_ctx_update_W with the values given as one pointer per block
 * (block[k] -> the 9 doubles of block k, column-major): the block array of
 * a SparseBlockStructuredMatrix (SparseBlockMatrix.h), so SBM storage needs
 * no repacking.  The pointers are checked first (by up to four host
 * threads); runs of blocks adjacent in memory are then copied straight from
 * there, scattered blocks gathered through pinned staging buffers. */
int fc3dgpu_ctx_update_W_ptrs(fc3dgpu_ctx *ctx, int nc, const int64_t *rowptr, const int64_t *colidx,
                              const double *const *block, int colour_kind);
int fc3dgpu_ctx_set_W_batch(fc3dgpu_ctx *ctx, int nproblems, const int *problem_nc, const int64_t *rowptr,
                            const int64_t *colidx, const double *blocks, int colour_kind);
/* Solve every problem of the batch (persistent kernels with a work queue,
 * recorded once into a CUDA graph and replayed).  Per problem: FP32 and FP64
 * sweeps, final fc3d_compute_error and info (as fc3dgpu_nsgs returns it);
 * *ms = device time.  Arrays may be NULL. */
int fc3dgpu_ctx_solve_batch(fc3dgpu_ctx *ctx, const fc3dgpu_params *p, int *sweeps32, int *sweeps64, double *error,
                            int *info, double *ms);
int fc3dgpu_ctx_set_q_mu(fc3dgpu_ctx *ctx, const double *q, const double *mu);
int fc3dgpu_ctx_set_r(fc3dgpu_ctx *ctx, const double *r);
int fc3dgpu_ctx_solve(fc3dgpu_ctx *ctx, const fc3dgpu_params *p, fc3dgpu_stats *st);
int fc3dgpu_ctx_get_r_u(fc3dgpu_ctx *ctx, double *r, double *u);
int fc3dgpu_ctx_compute_error(fc3dgpu_ctx *ctx, double *error);
/* Per-sweep incremental error trace of the last solve (FP32 then FP64). */
int fc3dgpu_ctx_trace(fc3dgpu_ctx *ctx, double *out, int cap);
int fc3dgpu_ctx_colours(fc3dgpu_ctx *ctx, int32_t *colour);
/* Sweep work counters since the last call: Newton iterations, PLI
 * iterations, line-search evaluations, local solves, largest Newton count of
 * one solve, summed and largest SM cycles of one warp work unit, number of
 * units.  enable != 0 keeps counting in later solves.  out8 may be NULL. */
int fc3dgpu_ctx_counters(fc3dgpu_ctx *ctx, int enable, unsigned long long *out8);
/* Phase timeline: in the next solves, record for sweep `sweep` (1-based),
 * per colour and block, out[(colour*grid + block)*8 + {0..5}] = globaltimer
 * (ns) at the phase start, at the end of the block's work, after its
 * row-product pass, its number of local solves, and (staged sweeps) after the
 * staging wait and after the first slab round (entries 6, 7 spare); copies
 * the last record into out (cap entries) and returns how many were copied.
 * sweep 0 stops.  With the dataflow sweep (fc3dgpu_ctx_flow) the record is
 * per slab: out[slab*8 + {0..7}] = globaltimer before the wait for its
 * column slabs, after it, after its data landed in shared memory, after the
 * row products, after the light-error sums that follow the local solves, its
 * number of local solves, after the next slab's bulk copies were issued (just
 * before the local solves), and after the local solves with their stores. */
int fc3dgpu_ctx_timeline(fc3dgpu_ctx *ctx, int sweep, unsigned long long *out, int cap);
/* Bulk-copy (TMA) staging of each block's slab range into shared memory
 * in the FP32 sweeps: 1 on (default), 0 off.  Returns the previous value. */
int fc3dgpu_ctx_staging(fc3dgpu_ctx *ctx, int on);
/* Synchronisation between the colours of a sweep (one lane per contact):
 * 1 (default) each block waits only for the blocks whose rows share a W block
 * with its own, 0 a grid-wide barrier after every colour.  Both give the same
 * iterates.  Returns the previous setting. */
int fc3dgpu_ctx_sync(fc3dgpu_ctx *ctx, int neighbourhood);
/* FP32 sweeps as a slab dataflow (1, default): each warp updates whole
 * 32-row slabs once the slabs holding their columns reached the state the
 * sequential sweep in colour order reads (per-slab completion counters, no
 * barrier between colours); 0 the coloured kernel above.  The same sweep
 * either way.  Applies with one lane per contact when no slab has more
 * than 16 off-diagonal slots.  Returns the previous setting. */
int fc3dgpu_ctx_flow(fc3dgpu_ctx *ctx, int on);
/* Warps per block of the dataflow sweep: 8, 10 or 12 (0: the default, 10,
 * or the autotuner's choice); fewer when the per-warp buffers of the current
 * layout do not fit.  Returns the previous request. */
int fc3dgpu_ctx_flow_warps(fc3dgpu_ctx *ctx, int nw);
/* Measuring autotuner of the sweep variant, run at the first solve of a new
 * structure with automatic lanes (fc3dgpu_params.lanes = 0): it times a few
 * sweeps of each candidate from the current reaction (restored afterwards)
 * and keeps the fastest for the structure.  mode 1 (default): only variants
 * with the same iterates bit for bit (the dataflow sweep with 8, 10 or 12
 * warps a block, the coloured kernel with one lane per contact; FP64 sweeps
 * keep one lane per contact, the oracle's iterates); mode 2: also 2, 4 and
 * 8 lanes per contact in both precisions (other summation orders); mode 0:
 * off.  Returns the previous mode. */
int fc3dgpu_ctx_autotune(fc3dgpu_ctx *ctx, int mode);
/* The autotuner's choice for the current structure: choice4 = {dataflow
 * sweep (0/1), its warps a block, FP32 lanes, FP64 lanes}; ms11 = device time
 * of one sweep of each candidate (FP32: dataflow 8, 10, 12 warps, coloured
 * 1, 2, 4, 8 lanes; FP64: 1, 2, 4, 8 lanes; infinity when not run).  Returns
 * 1 when the structure is not tuned yet, 0 otherwise. */
int fc3dgpu_ctx_tuning(fc3dgpu_ctx *ctx, int *choice4, float *ms11);
/* Polls before a barrier, slab-counter or bulk-copy wait of the sweep
 * kernels gives up (0: the default 2^22, seconds); the kernel then records
 * FC3DGPU_STATUS_BARRIER_TIMEOUT, every block leaves (each after its own
 * bulk copies in flight have landed) and the solve returns an error; the
 * context stays usable.  Returns the previous setting. */
unsigned long long fc3dgpu_ctx_spin_limit(fc3dgpu_ctx *ctx, unsigned long long polls);
/* r = 0 on the device (PLI steps reset), without a host copy. */
int fc3dgpu_ctx_zero_r(fc3dgpu_ctx *ctx);
/* The CUDA stream (cudaStream_t) every kernel of this context runs on, for
 * callers that time or order work around a solve. */
void *fc3dgpu_ctx_stream(fc3dgpu_ctx *ctx);
/* Number of kernels this context has launched so far. */
unsigned long long fc3dgpu_ctx_launches(fc3dgpu_ctx *ctx);
/* Norm of q used by the relative error (default: computed from q). */
int fc3dgpu_ctx_set_norm_q(fc3dgpu_ctx *ctx, double norm_q);
/* Problem sizes of the context: contacts, 3x3 blocks of W, colours. */
int fc3dgpu_ctx_sizes(fc3dgpu_ctx *ctx, int *nc, long long *nnzb, int *ncolours);
/* W as the context holds it, block-CSR in contact order (sizes from
 * fc3dgpu_ctx_sizes; any pointer may be NULL). */
int fc3dgpu_ctx_get_W(fc3dgpu_ctx *ctx, int64_t *rowptr, int64_t *colidx, double *blocks);

/* ---- Assembly of W and q on the device ---------------------------------
 * What the reference's mechanics layer does on the host before calling
 * fc3d_driver (the Delassus matrix W = H M^-1 H^T of the one-step problem and
 * q = H v_free; OSNSMatrix / BlockCSRMatrix fill in Siconos' kernel), here for
 * rigid bodies with a scalar mass and an isotropic inertia.  Contact k joins
 * body bodyA[k] (-1: a fixed obstacle) and body bodyB[k]; frame[9k..9k+8]
 * holds its rows n, t1, t2 and point[3k..3k+2] its point; H of contact k and
 * body b is s R [I | -[d]x] with d = point - body position, s = +1 for body B
 * and -1 for body A.  W's block structure (contacts sharing a body, columns
 * increasing) and its FP64 blocks are built on the device, then coloured and
 * laid out as fc3dgpu_ctx_set_W does.  Host arrays in, nothing returned to the
 * host. */
int fc3dgpu_ctx_set_contacts(fc3dgpu_ctx *ctx, int nbodies, int ncontacts, const int32_t *bodyA, const int32_t *bodyB,
                             const double *frame, const double *point, const double *body_pos,
                             const double *body_mass, const double *body_inertia, int colour_kind);
/* Friction coefficients of the contacts (host array). */
int fc3dgpu_ctx_set_mu(fc3dgpu_ctx *ctx, const double *mu);
/* Body velocities (host, 6 per body: linear then angular) and the time step:
 * q = H (v + h g), g = -9.81 e_z, formed on the device. */
int fc3dgpu_ctx_set_velocities(fc3dgpu_ctx *ctx, const double *vel, double h);
/* One random-walk step of the body velocities on the device, v += std N(0, 1)
 * per degree of freedom (normals from a counter-based hash of seed and index),
 * then q re-formed: a time step without any host-device traffic but q's norm. */
int fc3dgpu_ctx_random_walk(fc3dgpu_ctx *ctx, uint64_t seed, double std);
/* The context's q (contact order, host array of 3 nc) and body velocities. */
int fc3dgpu_ctx_get_q(fc3dgpu_ctx *ctx, double *q);
int fc3dgpu_ctx_get_velocities(fc3dgpu_ctx *ctx, double *vel);

/* ---- Error evaluation without allocation --------------------------------
 * No counterpart in the reference (whose fc3d_compute_error,
 * fc3d_compute_error.c:70-122, is host code).  For callers that cannot let a
 * library allocate device memory: an application whose memory pool owns the
 * device, where a cudaMalloc or cudaFree would synchronise the device
 * mid-step or find no memory left.
 *
 * Computes velocity = W reaction + q and the relative natural-map error of
 * fc3d_compute_error on the current device, on `stream` (a cudaStream_t; NULL
 * is the default stream), asynchronously: *error is written when the stream
 * reaches the kernel.  Every pointer is memory the device can access: W as
 * block-CSR (rowptr[nc+1], colidx[nnz], blocks[9 nnz], 3x3 blocks
 * column-major), q, mu, reaction as in FrictionContactProblem.  velocity may
 * be NULL.  A row pointer or column index out of range makes *error NaN.
 *
 * Scratch is a fixed device array of FC3DGPU_NOALLOC_SCRATCH_BYTES inside the
 * library; no call allocates or frees memory.  The first call on a device
 * looks the array up (once per device and CUDA context, normally the
 * device's primary context; a new context, e.g. after cudaDeviceReset, is
 * looked up again at its first call): make that call before any stream
 * capture starts.  Calls share the array, so two calls in flight at once on
 * the same device (other streams or host threads) race: order them on one
 * stream.  Every pointer must be memory the current device can use as given
 * (its own device memory, managed memory, or mapped pinned host memory);
 * others, including another device's memory, are refused with
 * NUMERICS_ERR_INVALID_ARGUMENT before any device work.
 * More than FC3DGPU_NOALLOC_MAX_CONTACTS contacts is rejected with
 * NUMERICS_ERR_INVALID_ARGUMENT before any device work. */
#define FC3DGPU_NOALLOC_MAX_CONTACTS 4194304
#define FC3DGPU_NOALLOC_SCRATCH_BYTES (8 * (3 * (FC3DGPU_NOALLOC_MAX_CONTACTS / 256) + 32))
int fc3dgpu_compute_error_device(int nc, int64_t nnz, const int64_t *rowptr, const int64_t *colidx,
                                 const double *blocks, const double *q, const double *mu, const double *reaction,
                                 double norm_q, double *velocity, double *error, void *stream);

#ifdef __cplusplus
}
#endif
#endif
