"""The C-ABI library: loads, exports every function include/*.h declares,
mirrors the reference's option defaults and error behaviour.  No GPU
compute is called here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions(comparator=False):
    """Functions include/*.h declares: the solver library's, or (comparator)
    those of the measurement-only per-colour library."""
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        if (h.name == "fc2dgpu_percolour.h") != comparator:
            continue
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b((?:g?fc[23]|rfc3)dgpu_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_functions()
    for must in ["fc3dgpu_nsgs", "fc3dgpu_nsgs_set_default", "fc3dgpu_nsgs_batch", "fc3dgpu_compute_error",
                 "fc3dgpu_driver", "fc3dgpu_colour", "fc3dgpu_ctx_solve", "fc3dgpu_lattice_create",
                 "fc2dgpu_nsgs", "fc2dgpu_driver", "fc2dgpu_ctx_solve",
                 "rfc3dgpu_nsgs", "rfc3dgpu_driver", "rfc3dgpu_ctx_solve",
                 "gfc3dgpu_nsgs", "gfc3dgpu_driver", "gfc3dgpu_ctx_solve"]:
        assert must in names
    assert "fc2dgpu_percolour_solve" in declared_functions(comparator=True)


@pytest.mark.parametrize("name", declared_functions())
def test_library_exports(built_lib, name):
    assert hasattr(built_lib, name), name


@pytest.mark.parametrize("name", declared_functions(comparator=True))
def test_comparator_library_exports(built_lib, name):
    import siconos_gb300.numerics as sn
    assert hasattr(sn.comparator_lib(), name), name


def test_solver_library_links_no_cusparse(built_lib):
    """The solver library has no library GEMM/SpMV backend: cuSPARSE is
    linked only into the measurement-only comparator."""
    import subprocess
    from siconos_gb300 import build as B
    dyn = subprocess.run(["readelf", "-d", str(B.LIB)], capture_output=True, text=True).stdout
    assert "cusparse" not in dyn
    assert "cusparse" in subprocess.run(["readelf", "-d", str(B.COMPARATOR)], capture_output=True, text=True).stdout


def test_options_mirror_reference_defaults(built_lib):
    import siconos_gb300.numerics as sn
    o = sn.SolverOptions(sn.SICONOS_FRICTION_3D_NSGS_GPU)
    ip, dp = o.iparam, o.dparam
    # fc3d_nsgs_set_default (fc3d_nsgs.c:919-950) with registry defaults
    assert ip[0] == 1000 and dp[0] == 1e-4
    # error evaluation in slot 13 and the internal error ratio in dparam 11:
    # the slots the reference's compiled fc3d_nsgs reads (NonSmoothGaussSeidel_options.h:275-284)
    assert ip[13] == 2 and ip[2] == 1 and ip[11] == 0 and ip[15] == 0 and ip[16] == 0 and ip[10] == 0
    assert dp[11] == 10.0 and ip[17] == 1 and ip[14] == 0
    loc = o.internalSolvers[0]
    # fc3d_onecontact_nsn_gp_set_default (onecontact.c:1037-1056), registry 100 / 1e-14
    assert loc.solverId == 565
    assert loc.iparam[0] == 100 and loc.dparam[0] == 1e-14
    assert loc.iparam[9] == 3 and loc.iparam[10] == 0 and loc.iparam[11] == 0 and loc.iparam[12] == 10
    assert loc.iparam[14] == 2 and loc.iparam[15] == 1 and loc.iparam[16] == 100


def _tiny_problem(q):
    import siconos_gb300.numerics as sn
    W = sn.SparseBlockMatrix(1, [0, 1], [0], np.eye(3).reshape(1, 9, order="F").reshape(-1))
    return sn.FrictionContactProblem(3, 1, W, np.array(q, float), np.array([0.5]))


def test_driver_trivial_case_on_host(built_lib):
    import siconos_gb300.numerics as sn
    P = _tiny_problem([1.0, 0.2, -0.3])
    r = np.ones(3)
    u = np.zeros(3)
    o = sn.SolverOptions()
    assert sn.fc3d_driver(P, r, u, o) == 0
    assert not r.any() and np.array_equal(u, P.q())
    assert np.may_share_memory(P.q(), P.q())


def test_invalid_inputs_rejected(built_lib):
    import siconos_gb300.numerics as sn
    L = sn.lib()
    o = sn.SolverOptions()
    P = _tiny_problem([-1.0, 0.0, 0.0])
    r, u = np.zeros(3), np.zeros(3)
    assert L.fc3dgpu_driver(None, r.ctypes.data_as(sn._DP), u.ctypes.data_as(sn._DP), o.ptr) == sn.NUMERICS_ERR_NULL_POINTER
    P.c.dimension = 2
    assert sn.fc3d_driver(P, r, u, o) == sn.NUMERICS_ERR_INVALID_ARGUMENT
    P.c.dimension = 3
    P.mu()[0] = -0.1
    assert sn.fc3d_driver(P, r, u, o) == sn.NUMERICS_ERR_INVALID_ARGUMENT
    P.mu()[0] = 0.5
    o.iparam[11] = 1  # shuffle
    assert sn.fc3d_driver(P, r, u, o) == sn.NUMERICS_ERR_NOT_IMPLEMENTED
    assert "shuffle" in sn.last_error()
    # values the reference refuses (fc3d_nsgs.c:630-665): invalid argument
    o.iparam[11] = 5
    assert sn.fc3d_driver(P, r, u, o) == sn.NUMERICS_ERR_INVALID_ARGUMENT
    o.iparam[11] = 0
    o.iparam[sn.SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION] = 7
    assert sn.fc3d_driver(P, r, u, o) == sn.NUMERICS_ERR_INVALID_ARGUMENT
    assert "ERROR_EVALUATION" in sn.last_error()


@pytest.mark.parametrize("em,strategy,relax,filt", [(0, 1, 0, 0), (1, 1, 0, 0), (3, 1, 0, 0), (2, 0, 0, 0),
                                                   (2, 2, 0, 0), (2, 1, 1, 0), (2, 1, 0, 1), (0, 0, 1, 1)])
def test_other_nsgs_options_pass_the_checks(built_lib, em, strategy, relax, filt):
    """The reference's other error evaluations, local tolerance strategies,
    relaxation and filter are accepted; on a machine without a GPU the solve
    then stops at the device, not at the option checks."""
    import siconos_gb300.numerics as sn
    ctx = sn.lib().fc3dgpu_ctx_create(0)
    if ctx:
        sn.lib().fc3dgpu_ctx_destroy(ctx)
        pytest.skip("a GPU is present")
    o = sn.SolverOptions()
    o.iparam[sn.SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION] = em
    o.iparam[sn.SICONOS_FRICTION_3D_IPARAM_INTERNAL_ERROR_STRATEGY] = strategy
    o.iparam[10] = relax  # SICONOS_FRICTION_3D_NSGS_RELAXATION
    o.iparam[16] = filt  # SICONOS_FRICTION_3D_NSGS_FILTER_LOCAL_SOLUTION
    P = _tiny_problem([-1.0, 0.0, 0.0])
    r, u = np.zeros(3), np.zeros(3)
    assert sn.fc3d_driver(P, r, u, o) == sn.NUMERICS_ERR_NOT_IMPLEMENTED
    assert "only" not in sn.last_error() and "not supported" not in sn.last_error()


def test_solve_fails_loudly_without_gpu(built_lib):
    import siconos_gb300.numerics as sn
    n = C.c_int()
    cudart_ok = sn.lib().fc3dgpu_ctx_create(0)
    if cudart_ok:
        sn.lib().fc3dgpu_ctx_destroy(cudart_ok)
        pytest.skip("a GPU is present")
    P = _tiny_problem([-1.0, 0.0, 0.0])
    r, u = np.zeros(3), np.zeros(3)
    rc = sn.fc3d_driver(P, r, u, sn.SolverOptions())
    assert rc == sn.NUMERICS_ERR_NOT_IMPLEMENTED
    assert "CUDA" in sn.last_error() or "device" in sn.last_error()
