/* Layout-compatible declarations of the reference's numerics types and
 * constants that the GPU solver's C-ABI exchanges.
 *
 * Inside a Siconos build, include the reference's own headers instead
 * (define FC3DGPU_USE_SICONOS_HEADERS before including fc3dgpu.h); this file
 * exists so the library and its tests build stand-alone.  Every struct below
 * has the member order and types of the reference definition it mirrors, so
 * pointers pass unchanged across the boundary:
 *
 *   NumericsDataVersion          core/NumericsDataVersion.h:28-31
 *   SparseBlockStructuredMatrix  linalg/SparseBlockMatrix.h:82-121
 *   NumericsMatrix               linalg/NumericsMatrix.h:73-89 (only the
 *                                members up to `version` are read)
 *   FrictionContactProblem       FrictionContact/FrictionContactProblem.h:33-46
 *   RollingFrictionContactProblem RollingFrictionContact/RollingFrictionContactProblem.h:33-53
 *   GlobalFrictionContactProblem FrictionContact/GlobalFrictionContactProblem.h:34-66
 *   Callback, SolverOptions      core/SolverOptions.h:36-91
 */
#ifndef SICONOS_NUMERICS_ABI_H
#define SICONOS_NUMERICS_ABI_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint64_t version_t;
typedef struct {
  version_t number;
} NumericsDataVersion;

typedef enum { NM_DENSE = 0, NM_SPARSE_BLOCK = 1, NM_SPARSE = 2, NM_UNKNOWN = 99 } NM_types;

typedef struct SparseBlockStructuredMatrix {
  size_t nbblocks;
  double **block;
  size_t blocknumber0;
  size_t blocknumber1;
  size_t *blocksize0;
  size_t *blocksize1;
  size_t filled1;
  size_t filled2;
  size_t *index1_data;
  size_t *index2_data;
  size_t *diagonal_blocks;
  NumericsDataVersion version;
} SparseBlockStructuredMatrix;

struct NumericsSparseMatrix;
struct NumericsMatrixInternalData;

typedef struct NumericsMatrix {
  NM_types storageType;
  int size0;
  int size1;
  double *matrix0;
  SparseBlockStructuredMatrix *matrix1;
  struct NumericsSparseMatrix *matrix2;
  struct NumericsMatrixInternalData *internalData;
  NumericsDataVersion version;
  struct NumericsMatrix *destructible;
} NumericsMatrix;

typedef struct FrictionContactProblem {
  int dimension;
  int numberOfContacts;
  NumericsMatrix *M;
  double *q;
  double *mu;
} FrictionContactProblem;

/* RollingFrictionContact/RollingFrictionContactProblem.h:33-53 */
typedef struct RollingFrictionContactProblem {
  int dimension;
  int numberOfContacts;
  NumericsMatrix *M;
  double *q;
  double *mu;
  double *mu_r;
} RollingFrictionContactProblem;

/* FrictionContact/GlobalFrictionContactProblem.h:34-66 */
typedef struct GlobalFrictionContactProblem {
  int dimension;
  int numberOfContacts;
  NumericsMatrix *M;
  NumericsMatrix *H;
  double *q;
  double norm_q;
  double *b;
  double norm_b;
  double *mu;
  NumericsMatrix *M_inverse;
  char *name;
  void *env;
} GlobalFrictionContactProblem;

typedef struct {
  void *env;
  void (*collectStatsIteration)(void *env, size_t size, double *reaction, double *velocity, double error,
                                void *extra_data);
} Callback;

#define OPTIONS_PARAM_SIZE 30

typedef struct SolverOptions {
  int solverId;
  bool isSet;
  size_t iSize;
  int *iparam;
  size_t dSize;
  double *dparam;
  bool filterOn;
  size_t dWorkSize;
  double *dWork;
  size_t iWorkSize;
  int *iWork;
  size_t numberOfInternalSolvers;
  struct SolverOptions **internalSolvers;
  Callback *callback;
  void *solverParameters;
  void *solverData;
} SolverOptions;

/* solver ids (FrictionContact_options.h:83, :152) */
#define SICONOS_FRICTION_2D_NSGS 400
#define SICONOS_FRICTION_3D_NSGS 500
#define SICONOS_ROLLING_FRICTION_3D_NSGS 3000
#define SICONOS_ROLLING_FRICTION_3D_ONECONTACT_NSN 3003
#define SICONOS_FRICTION_3D_ONECONTACT_NSN_GP_HYBRID 565
#define SICONOS_GLOBAL_FRICTION_3D_NSGS 605

/* generic indices (SolverOptions.h:94-121) */
#define SICONOS_IPARAM_MAX_ITER 0
#define SICONOS_IPARAM_ITER_DONE 1
#define SICONOS_IPARAM_NSGS_SHUFFLE 5
#define SICONOS_DPARAM_TOL 0
#define SICONOS_DPARAM_RESIDU 1
#define SICONOS_DPARAM_TIME_BEFORE_LOOP 20
#define SICONOS_DPARAM_TIME_IN_LOOP 21
#define SICONOS_DPARAM_TIME_AFTER_LOOP 22

/* fc3d / NSGS indices (FrictionContact_options.h:220-236,
 * NonSmoothGaussSeidel_options.h:50-100).  The error-evaluation indices are
 * the ones the reference's compiled solvers use: NonSmoothGaussSeidel_options.h:275-276
 * and :284 re-map SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION(_FREQUENCY) and
 * SICONOS_FRICTION_3D_DPARAM_INTERNAL_ERROR_RATIO onto the generic NSGS
 * slots 13, 14 and 11 after FrictionContact_options.h declares them as 7, 8
 * and 2, so fc3d_nsgs.c, fc2d_nsgs.c and rolling_friction_3d_nsgs.c read
 * slots 13, 14 (iparam) and 11 (dparam). */
#define SICONOS_FRICTION_3D_IPARAM_INTERNAL_ERROR_STRATEGY 2
#define SICONOS_FRICTION_3D_CURRENT_CONTACT_NUMBER 5
#define SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION 13
#define SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION_FREQUENCY 14
#define SICONOS_FRICTION_3D_NSGS_RELAXATION 10
#define SICONOS_FRICTION_3D_NSGS_SHUFFLE 11
#define SICONOS_FRICTION_3D_NSGS_SHUFFLE_SEED 12
#define SICONOS_FRICTION_3D_NSGS_FREEZING_CONTACT 15
#define SICONOS_FRICTION_3D_NSGS_FILTER_LOCAL_SOLUTION 16
#define SICONOS_FRICTION_3D_NSGS_PRINTING_LIKE_IPM 17
#define SICONOS_FRICTION_3D_NSGS_RELAXATION_VALUE 10
#define SICONOS_FRICTION_3D_DPARAM_INTERNAL_ERROR_RATIO 11
#define SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_FULL 0
#define SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT 1
#define SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL 2
#define SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_ADAPTIVE 3
/* local tolerance strategies (NonSmoothGaussSeidel_options.h:222-228) */
#define SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_ADAPTIVE 0
#define SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_GIVEN_VALUE 1
#define SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_ADAPTIVE_N_CONTACT 2

/* one-contact local solver indices (FrictionContact_options.h:294-365) */
#define SICONOS_FRICTION_3D_NSN_RHO_STRATEGY 9
#define SICONOS_FRICTION_3D_NSN_FORMULATION 10
#define SICONOS_FRICTION_3D_NSN_LINESEARCH 11
#define SICONOS_FRICTION_3D_NSN_LINESEARCH_MAX_ITER 12
#define SICONOS_FRICTION_3D_NSN_HYBRID_STRATEGY 14
#define SICONOS_FRICTION_3D_NSN_HYBRID_MAX_LOOP 15
#define SICONOS_FRICTION_3D_NSN_HYBRID_MAX_ITER 16
#define SICONOS_FRICTION_3D_NSN_RHO 3
#define SICONOS_FRICTION_3D_NSN_FORMULATION_RHO_STRATEGY_SPECTRAL_NORM 1
#define SICONOS_FRICTION_3D_NSN_FORMULATION_RHO_STRATEGY_SPLIT_SPECTRAL_NORM 3
#define SICONOS_FRICTION_3D_NSN_FORMULATION_NATURALMAP 4
#define SICONOS_FRICTION_3D_NSN_FORMULATION_ALARTCURNIER_STD 0
#define SICONOS_FRICTION_3D_NSN_LINESEARCH_GOLDSTEINPRICE 0
#define SICONOS_FRICTION_3D_NSN_HYBRID_STRATEGY_NSN_AND_PLI_NSN_LOOP 2

/* error codes (numerics_errors.h:41-67) */
#define NUMERICS_OK 0
#define NUMERICS_ERR_NULL_POINTER -1
#define NUMERICS_ERR_INVALID_ARGUMENT -2
#define NUMERICS_ERR_INVALID_OPTION -3
#define NUMERICS_ERR_INVALID_SOLVER -4
#define NUMERICS_ERR_NOT_IMPLEMENTED -5
#define NUMERICS_ERR_MEMORY -6
#define NUMERICS_ERR_MAX_ITER -20
#define NUMERICS_ERR_DIVERGENCE -21
#define NUMERICS_ERR_LOCAL_SOLVER -24
#define NUMERICS_ERR_INFEASIBLE -40
#define NUMERICS_ERR_UNKNOWN -99

#ifdef __cplusplus
}
#endif
#endif
