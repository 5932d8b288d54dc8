/* Registration of the GPU solver in a Siconos numerics build.
 *
 * This translation unit is compiled INTO the reference's libsiconos_numerics
 * (it needs the reference's own headers, FC3DGPU_USE_SICONOS_HEADERS), not
 * into libfc3dgpu.so.  Its constructor adds SICONOS_FRICTION_3D_NSGS_GPU (531)
 * to the solver registry exactly as fc3d_nsgs.c:981-987 adds
 * SICONOS_FRICTION_3D_NSGS through REGISTER_SOLVER (utils/solver_registry.h:75-95):
 * afterwards solver_options_create(531) (utils/SolverOptions.c:310-334) sets
 * the GPU solver's defaults and fc3d_driver (FrictionContact/fc3d_driver.c:77-145)
 * dispatches to fc3dgpu_nsgs_solve_wrap through solver_registry_lookup
 * (utils/solver_registry.c:48).  The default budget and tolerance are the
 * stock NSGS solver's (1000 iterations, 1e-4).
 *
 * The global solver SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU (619) registers the
 * same way as gfc3d_nsgs.c:232-237 registers GFC3D_NSGS
 * (REGISTER_SOLVER_3VAR, solve3 = gfc3dgpu_nsgs_solve_wrap); the reference's
 * gfc3d_driver dispatches by a switch on the id (gfc3d_driver.c:120-293),
 * so a build that adds it also adds one case there that looks the id up in
 * the registry and calls the entry's solve3.
 *
 * fc3dgpu.h defines the ids as macros; a build that adds them to the
 * enum of FrictionContact_options.h instead compiles this file with
 * -DFC3DGPU_ID_IN_SICONOS_ENUM.
 */
#define FC3DGPU_USE_SICONOS_HEADERS
#include "fc3dgpu.h"
#include "gfc3dgpu.h"
#include "solver_registry.h"

REGISTER_SOLVER(SICONOS_FRICTION_3D_NSGS_GPU, "FC3D_NSGS_GPU",
                "Coloured non-smooth Gauss-Seidel for 3D friction contact on GB300", fc3dgpu_nsgs_init_wrap,
                fc3dgpu_nsgs_solve_wrap, fc3dgpu_nsgs_free_wrap, NULL, fc3dgpu_nsgs_set_default, 1000, 1e-4, 0)

REGISTER_SOLVER_3VAR(SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU, "GFC3D_NSGS_GPU",
                     "Global 3D friction contact NSGS (projected iteration) on GB300", gfc3dgpu_nsgs_init_wrap,
                     gfc3dgpu_nsgs_solve_wrap, gfc3dgpu_nsgs_free_wrap, NULL, gfc3dgpu_nsgs_set_default, 1000,
                     1e-4, 0)
