"""The drop-in through the reference's own solver registry.

`siconos_gb300/csrc/fc3d_nsgs_gpu_register.c` (the registration unit a
Siconos build compiles in) and `tests/registry_check.c` (a user program that
only changes the solver id) are compiled against the reference's headers and
linked with the reference's numerics (`oracle/_ref`) and `libfc3dgpu.so`.
The reference's `solver_options_create(531)` must then apply the GPU
solver's defaults (fc3d_nsgs_set_default, fc3d_nsgs.c:919-950, with the
registry's 1000 iterations / 1e-4), and the reference's `fc3d_driver`
(fc3d_driver.c:77-145) must dispatch to `fc3dgpu_nsgs_solve_wrap` through
`solver_registry_lookup` (solver_registry.c:48).

Without a GPU the solve returns NUMERICS_ERR_NOT_IMPLEMENTED with the
solver's message (no CPU fallback); with one it converges on KaplasTower and
the reference's own fc3d_compute_error of the result is below 1e-8.  Needs
the reference checkout ($SICONOS_REFERENCE or the one oracle/_ref was built
from): skipped where it is absent.
"""
import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import ROOT, load_case

NUMERICS_ERR_NOT_IMPLEMENTED = -5


def _reference():
    from oracle import build_ref
    src = build_ref.source_dir()
    if src is None or not build_ref.LIB.exists():
        pytest.skip("reference checkout or oracle/_ref not available")
    return build_ref, src


@pytest.fixture(scope="module")
def registry_program(tmp_path_factory, built_lib):
    build_ref, src = _reference()
    out = tmp_path_factory.mktemp("registry") / "registry_check"
    lib_ref = build_ref.LIB.parent
    lib_gpu = ROOT / "siconos_gb300" / "_lib"
    cmd = ["gcc", "-std=gnu11", "-O1", "-DCS_LONG", "-DNCOMPLEX", "-w", *build_ref.include_flags(src),
           f"-I{ROOT / 'include'}", str(ROOT / "tests" / "registry_check.c"),
           str(ROOT / "siconos_gb300" / "csrc" / "fc3d_nsgs_gpu_register.c"), "-o", str(out),
           f"-L{lib_ref}", "-lsiconos_numerics_ref", f"-L{lib_gpu}", "-lfc3dgpu", f"-Wl,-rpath,{lib_ref}",
           f"-Wl,-rpath,{lib_gpu}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def _run(prog, dat, tol=1e-8, max_iter=10000, gdat=None):
    args = [str(prog), str(dat), repr(tol), str(max_iter)] + ([str(gdat)] if gdat else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {}
    for line in r.stdout.splitlines():
        k, _, v = line.partition(" ")
        out[k] = v
    return out, r.stderr


def _gpu_present() -> bool:
    import ctypes as C
    import siconos_gb300.numerics as sn
    info = (C.c_longlong * 6)()
    return sn.lib().fc3dgpu_device_info(0, info) == 0


def test_reference_driver_dispatches_to_gpu_solver(registry_program, tmp_path):
    P, g = load_case("fixture_KaplasTower_i1061_4")
    dat = tmp_path / "kaplas.dat"
    O.write_dat_ref(P, dat)
    out, err = _run(registry_program, dat)
    # registered by the unit's constructor, found by the reference's lookup
    assert out["registered"] == "1" and out["name"] == "FC3D_NSGS_GPU" and out["solve_is_gpu"] == "1"
    # the reference's solver_options_create applied the registry defaults and
    # fc3dgpu_nsgs_set_default (LIGHT_WITH_FULL_FINAL error evaluation = 2,
    # internal solver ONECONTACT_NSN_GP_HYBRID = 565)
    assert out["solverId"] == "531"
    assert out["default_max_iter"] == "1000" and float(out["default_tol"]) == 1e-4
    assert out["iparam_error_evaluation"] == "2" and out["internal_solver"] == "565"
    info = int(out["info"])
    if _gpu_present():
        assert info == 0, out
        assert float(out["reference_error"]) <= 1e-8
        assert abs(float(out["residual"]) - float(out["reference_error"])) <= 1e-9 * float(out["reference_error"])
    else:
        # no CPU fallback: the GPU solver's own refusal, passed through the
        # reference's driver (which prints its [WARN] line)
        assert info == NUMERICS_ERR_NOT_IMPLEMENTED, out
        assert "CUDA" in out["message"] or "device" in out["message"], out["message"]
        assert "fc3d_driver: solver returned status -5" in err


def test_reference_driver_trivial_case_never_reaches_solver(registry_program, tmp_path):
    """q_n >= 0 everywhere: the reference's fc3d_checkTrivialCase answers
    before the registry lookup, as for the stock NSGS."""
    P, _ = load_case("fixture_FC3D_Example1_SBM")
    q = np.abs(P.q)
    T = O.Problem(P.nc, P.rowptr, P.colidx, P.blocks, q, P.mu)
    dat = tmp_path / "trivial.dat"
    O.write_dat_ref(T, dat)
    out, _ = _run(registry_program, dat)
    assert int(out["info"]) == 0 and int(out["iterations"]) == 0


def test_global_solver_registered_and_solves_through_solve3(registry_program, tmp_path):
    """SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU in the reference's registry: the
    reference's solver_options_create(619) gives the registry defaults, and
    the entry's solve3 (what the id's case in gfc3d_driver calls) solves the
    reference's GFC3D_TwoRods1 problem as read by the reference's reader."""
    build_ref, src = _reference()
    P, g = load_case("fixture_FC3D_Example1_SBM")
    dat = tmp_path / "fc3d.dat"
    O.write_dat_ref(P, dat)
    gdat = src / "numerics" / "src" / "FrictionContact" / "test" / "data" / "GFC3D_TwoRods1.dat"
    out, err = _run(registry_program, dat, 1e-8, 1000, gdat)
    assert out["g_registered"] == "1" and out["g_name"] == "GFC3D_NSGS_GPU" and out["g_solve3_is_gpu"] == "1"
    assert out["g_default_max_iter"] == "1000" and float(out["g_default_tol"]) == 1e-4
    info = int(out["g_info"])
    if _gpu_present():
        gold = np.load(ROOT / "tests" / "golden" / "gfc3d_GFC3D_TwoRods1.npz")
        assert info == 0, out
        assert float(out["g_reference_error"]) <= 1e-8
        assert abs(float(out["g_residual"]) - float(gold["error"])) <= 1e-12 * float(gold["error"])
    else:
        assert info == NUMERICS_ERR_NOT_IMPLEMENTED, out
        assert "CUDA" in out["g_message"] or "device" in out["g_message"], out["g_message"]


@pytest.mark.parametrize("ref_id, ours", [(500, 531), (400, 412), (3000, 3020), (605, 619)])
def test_option_slots_equal_reference_defaults(built_lib, ref_id, ours):
    """Every option slot the GPU solvers share with the reference's stock NSGS
    (fc3d, fc2d, rolling) holds the reference's default after the reference's
    own solver_options_create; the GPU knobs live in slots 23-29 only."""
    import ctypes as C
    import siconos_gb300.numerics as sn
    build_ref, _ = _reference()
    ref = C.CDLL(str(build_ref.LIB))
    ref.solver_options_create.restype = C.POINTER(sn._SO)
    ref.solver_options_create.argtypes = [C.c_int]
    ref.solver_options_delete.argtypes = [C.POINTER(sn._SO)]
    a = ref.solver_options_create(ref_id)
    b = sn.SolverOptions(ours)
    try:
        n = sn.OPTIONS_PARAM_SIZE
        ia = np.ctypeslib.as_array(a.contents.iparam, shape=(n,)).copy()
        da = np.ctypeslib.as_array(a.contents.dparam, shape=(n,)).copy()
        keep = [k for k in range(n) if not 23 <= k <= 29]
        assert np.array_equal(ia[keep], b.iparam[keep]), (ia, b.iparam)
        assert np.array_equal(da[keep], b.dparam[keep]), (da, b.dparam)
        assert a.contents.numberOfInternalSolvers == len(b.internalSolvers)
        for k, loc in enumerate(b.internalSolvers):
            la = a.contents.internalSolvers[k].contents
            assert la.solverId == loc.solverId
            assert np.array_equal(np.ctypeslib.as_array(la.iparam, shape=(n,)), loc.iparam)
            assert np.array_equal(np.ctypeslib.as_array(la.dparam, shape=(n,)), loc.dparam)
    finally:
        ref.solver_options_delete(a)
