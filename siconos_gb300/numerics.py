"""Python mirror of the reference's ``siconos.numerics`` friction-contact API
for the GPU solver (numerics/python/friction_contact_pybind11.cpp:165,525).

Names, argument meaning and return conventions follow the reference:

* ``FrictionContactProblem(dim, nc, M, q, mu)`` -- ``M`` a dense
  Fortran-ordered numpy matrix or a :class:`SparseBlockMatrix` (3x3 block
  CSR); ``q`` and ``mu`` are shared, not copied, as the reference's tests
  check with ``np.may_share_memory``;
* ``SolverOptions(solver_id)`` -- ``iparam`` / ``dparam`` are numpy views on
  the C arrays;
* ``fc3d_driver(problem, reaction, velocity, options)`` returns ``info``
  (0 converged, negative ``NUMERICS_ERR_*`` codes on invalid input);
* ``fc3d_compute_error(problem, reaction, velocity, tol, norm_q)`` returns
  ``(info, error)``.

Everything runs through the C-ABI of ``libfc3dgpu.so`` (``include/fc3dgpu.h``);
there is no Python or CPU implementation of the solve.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libfc3dgpu.so"

SICONOS_FRICTION_2D_NSGS = 400
SICONOS_FRICTION_2D_NSGS_GPU = 412
SICONOS_FRICTION_3D_NSGS = 500
SICONOS_ROLLING_FRICTION_3D_NSGS = 3000
SICONOS_ROLLING_FRICTION_3D_ONECONTACT_NSN = 3003
SICONOS_ROLLING_FRICTION_3D_NSGS_GPU = 3020
SICONOS_FRICTION_3D_NSGS_GPU = 531
SICONOS_FRICTION_3D_ONECONTACT_NSN_GP_HYBRID = 565
SICONOS_GLOBAL_FRICTION_3D_NSGS = 605
SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU = 619
SICONOS_IPARAM_MAX_ITER = 0
SICONOS_IPARAM_ITER_DONE = 1
SICONOS_IPARAM_NSGS_SHUFFLE = 5
SICONOS_DPARAM_TOL = 0
SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION = 13  # the reference's compiled slot (NonSmoothGaussSeidel_options.h:275)
SICONOS_FRICTION_3D_IPARAM_ERROR_EVALUATION_FREQUENCY = 14
SICONOS_FRICTION_3D_NSGS_FREEZING_CONTACT = 15
SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_FULL = 0
SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT = 1
SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL = 2
SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_ADAPTIVE = 3
SICONOS_FRICTION_3D_IPARAM_INTERNAL_ERROR_STRATEGY = 2
SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_ADAPTIVE = 0
SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_GIVEN_VALUE = 1
SICONOS_FRICTION_3D_INTERNAL_ERROR_STRATEGY_ADAPTIVE_N_CONTACT = 2
SICONOS_FRICTION_3D_DPARAM_INTERNAL_ERROR_RATIO = 11
SICONOS_DPARAM_RESIDU = 1
FC3DGPU_IPARAM_PRECISION = 23
FC3DGPU_IPARAM_LANES = 24
FC3DGPU_IPARAM_WARMSTART = 25
FC3DGPU_COLOUR_KEMPE = 1 << 16
FC3DGPU_COLOURING_DEFAULT = (4 << 8) | FC3DGPU_COLOUR_KEMPE  # hash priority, 4 recolouring passes, Kempe reduction
FC3DGPU_IPARAM_COLOURING = 26
FC3DGPU_IPARAM_SWEEPS_FP32 = 27
FC3DGPU_IPARAM_SWEEPS_FP64 = 28
FC3DGPU_IPARAM_COLOURS = 29
FC3DGPU_DPARAM_SWITCH_TOL = 23
FC3DGPU_DPARAM_LOCAL_TOL32 = 24
FC3DGPU_DPARAM_STALL = 25
FC3DGPU_DPARAM_MS_SWEEP32 = 26
FC3DGPU_DPARAM_MS_SWEEP64 = 27
FC3DGPU_DPARAM_MS_SOLVE = 28
FC3DGPU_DPARAM_INCR_ERROR = 29
NUMERICS_OK = 0
NUMERICS_ERR_NULL_POINTER = -1
NUMERICS_ERR_INVALID_ARGUMENT = -2
NUMERICS_ERR_INVALID_OPTION = -3
NUMERICS_ERR_INVALID_SOLVER = -4
NUMERICS_ERR_NOT_IMPLEMENTED = -5
NUMERICS_ERR_MAX_ITER = -20
NM_DENSE, NM_SPARSE_BLOCK = 0, 1
OPTIONS_PARAM_SIZE = 30

_DP = C.POINTER(C.c_double)
_SZP = C.POINTER(C.c_size_t)


class NumericsDataVersion(C.Structure):
    _fields_ = [("number", C.c_uint64)]


class SparseBlockStructuredMatrix(C.Structure):
    _fields_ = [("nbblocks", C.c_size_t), ("block", C.POINTER(_DP)), ("blocknumber0", C.c_size_t),
                ("blocknumber1", C.c_size_t), ("blocksize0", _SZP), ("blocksize1", _SZP), ("filled1", C.c_size_t),
                ("filled2", C.c_size_t), ("index1_data", _SZP), ("index2_data", _SZP),
                ("diagonal_blocks", _SZP), ("version", NumericsDataVersion)]


class NumericsMatrix(C.Structure):
    _fields_ = [("storageType", C.c_int), ("size0", C.c_int), ("size1", C.c_int), ("matrix0", _DP),
                ("matrix1", C.POINTER(SparseBlockStructuredMatrix)), ("matrix2", C.c_void_p),
                ("internalData", C.c_void_p), ("version", NumericsDataVersion), ("destructible", C.c_void_p)]


class _FCP(C.Structure):
    _fields_ = [("dimension", C.c_int), ("numberOfContacts", C.c_int), ("M", C.POINTER(NumericsMatrix)),
                ("q", _DP), ("mu", _DP)]


class _RFCP(C.Structure):
    _fields_ = [("dimension", C.c_int), ("numberOfContacts", C.c_int), ("M", C.POINTER(NumericsMatrix)),
                ("q", _DP), ("mu", _DP), ("mu_r", _DP)]


class _GFCP(C.Structure):
    _fields_ = [("dimension", C.c_int), ("numberOfContacts", C.c_int), ("M", C.POINTER(NumericsMatrix)),
                ("H", C.POINTER(NumericsMatrix)), ("q", _DP), ("norm_q", C.c_double), ("b", _DP),
                ("norm_b", C.c_double), ("mu", _DP), ("M_inverse", C.POINTER(NumericsMatrix)), ("name", C.c_char_p),
                ("env", C.c_void_p)]


CALLBACK_T = C.CFUNCTYPE(None, C.c_void_p, C.c_size_t, _DP, _DP, C.c_double, C.c_void_p)


class Callback(C.Structure):
    _fields_ = [("env", C.c_void_p), ("collectStatsIteration", CALLBACK_T)]


class _SO(C.Structure):
    pass


_SO._fields_ = [("solverId", C.c_int), ("isSet", C.c_bool), ("iSize", C.c_size_t), ("iparam", C.POINTER(C.c_int)),
                ("dSize", C.c_size_t), ("dparam", _DP), ("filterOn", C.c_bool), ("dWorkSize", C.c_size_t),
                ("dWork", _DP), ("iWorkSize", C.c_size_t), ("iWork", C.POINTER(C.c_int)),
                ("numberOfInternalSolvers", C.c_size_t), ("internalSolvers", C.POINTER(C.POINTER(_SO))),
                ("callback", C.POINTER(Callback)), ("solverParameters", C.c_void_p), ("solverData", C.c_void_p)]


class FC3DGPUParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iter", C.c_int), ("precision", C.c_int), ("lanes", C.c_int),
                ("switch_tol", C.c_double), ("stall_window", C.c_int), ("local_tol", C.c_double),
                ("local_tol32", C.c_double), ("newton_max", C.c_int), ("pli_max", C.c_int), ("ls_max", C.c_int),
                ("fp32_only", C.c_int), ("local_mode32", C.c_int), ("relax", C.c_int), ("omega", C.c_double),
                ("filter", C.c_int)]


class FC3DGPUStats(C.Structure):
    _fields_ = [("info", C.c_int), ("status", C.c_int), ("sweeps32", C.c_int), ("sweeps64", C.c_int),
                ("colours", C.c_int), ("lanes", C.c_int), ("grid", C.c_int), ("incr_error", C.c_double),
                ("error", C.c_double), ("ms_total", C.c_double), ("ms_fp32", C.c_double), ("ms_fp64", C.c_double),
                ("bytes_sweep32", C.c_double), ("bytes_sweep64", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None

_I64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_I32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_F64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")

# exported C-ABI symbols: name -> (restype, argtypes)
ABI = {
    "fc3dgpu_nsgs": (C.c_int, [C.POINTER(_FCP), _DP, _DP, C.POINTER(_SO)]),
    "fc3dgpu_nsgs_solve_wrap": (C.c_int, [C.c_void_p, _DP, _DP, C.POINTER(_SO)]),
    "fc3dgpu_nsgs_init_wrap": (C.c_int, [C.c_void_p, C.POINTER(_SO)]),
    "fc3dgpu_nsgs_free_wrap": (None, [C.c_void_p, C.POINTER(_SO)]),
    "fc3dgpu_driver": (C.c_int, [C.POINTER(_FCP), _DP, _DP, C.POINTER(_SO)]),
    "fc3dgpu_nsgs_set_default": (None, [C.POINTER(_SO)]),
    "fc3dgpu_options_create": (C.POINTER(_SO), []),
    "fc3dgpu_options_delete": (None, [C.POINTER(_SO)]),
    "fc3dgpu_release": (None, [C.POINTER(_SO)]),
    "fc3dgpu_compute_error": (C.c_int, [C.POINTER(_FCP), _DP, _DP, C.c_double, C.c_double, _DP]),
    "fc3dgpu_nsgs_batch": (C.c_int, [C.c_int, C.POINTER(C.POINTER(_FCP)), C.POINTER(_DP), C.POINTER(_DP),
                                     C.POINTER(_SO), C.POINTER(C.c_int)]),
    "fc3dgpu_colour": (C.c_int, [C.c_int, _I64, _I64, C.c_int, _I32]),
    "fc3dgpu_colour_reduce": (C.c_int, [C.c_int, _I32, _I32, _I32, C.c_int, C.c_int]),
    "fc3dgpu_colour_reduce_groups": (C.c_int, [C.c_int, _I32, _I32, _I32, _I32, C.c_int]),
    "fc3dgpu_last_error": (C.c_char_p, []),
    "fc3dgpu_device_info": (C.c_int, [C.c_int, C.c_void_p]),
    "fc3dgpu_params_default": (None, [C.POINTER(FC3DGPUParams)]),
    "fc3dgpu_ctx_create": (C.c_void_p, [C.c_int]),
    "fc3dgpu_ctx_destroy": (None, [C.c_void_p]),
    "fc3dgpu_ctx_set_W": (C.c_int, [C.c_void_p, C.c_int, _I64, _I64, _F64, C.c_int]),
    "fc3dgpu_ctx_set_q_mu": (C.c_int, [C.c_void_p, _F64, _F64]),
    "fc3dgpu_ctx_update_W": (C.c_int, [C.c_void_p, C.c_int, _I64, _I64, _F64, C.c_int]),
    "fc3dgpu_ctx_update_W_ptrs": (C.c_int, [C.c_void_p, C.c_int, _I64, _I64, C.c_void_p, C.c_int]),
    "fc3dgpu_ctx_set_W_batch": (C.c_int, [C.c_void_p, C.c_int, _I32, _I64, _I64, _F64, C.c_int]),
    "fc3dgpu_ctx_solve_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p]),
    "fc3dgpu_ctx_set_r": (C.c_int, [C.c_void_p, _F64]),
    "fc3dgpu_ctx_solve": (C.c_int, [C.c_void_p, C.POINTER(FC3DGPUParams), C.POINTER(FC3DGPUStats)]),
    "fc3dgpu_ctx_get_r_u": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_ctx_compute_error": (C.c_int, [C.c_void_p, _DP]),
    "fc3dgpu_ctx_trace": (C.c_int, [C.c_void_p, _F64, C.c_int]),
    "fc3dgpu_ctx_colours": (C.c_int, [C.c_void_p, _I32]),
    "fc3dgpu_ctx_counters": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "fc3dgpu_ctx_set_norm_q": (C.c_int, [C.c_void_p, C.c_double]),
    "fc3dgpu_mlp_nparams": (C.c_int, []),
    "fc3dgpu_mlp_create": (C.c_void_p, [C.c_int]),
    "fc3dgpu_mlp_destroy": (None, [C.c_void_p]),
    "fc3dgpu_mlp_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_mlp_get_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_mlp_set_data": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    "fc3dgpu_mlp_train_step": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_float, C.c_float, C.c_void_p,
                                         C.c_void_p, C.c_int]),
    "fc3dgpu_mlp_train_step_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_float, C.c_float]),
    "fc3dgpu_mlp_infer": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_int]),
    "fc3dgpu_mlp_infer_stream": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_mlp_set_tensor_path": (C.c_int, [C.c_void_p, C.c_int]),
    "fc3dgpu_mlp_set_residual": (C.c_int, [C.c_void_p, C.c_int]),
    "fc3dgpu_mlp_residual": (C.c_int, [C.c_void_p]),
    "fc3dgpu_ctx_warm_start": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_ctx_features": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_ctx_sizes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_ctx_get_W": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_ctx_set_contacts": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "fc3dgpu_ctx_set_mu": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fc3dgpu_ctx_set_velocities": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double]),
    "fc3dgpu_ctx_random_walk": (C.c_int, [C.c_void_p, C.c_uint64, C.c_double]),
    "fc3dgpu_ctx_get_q": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fc3dgpu_ctx_get_velocities": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fc3dgpu_lattice_fill_contacts": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p]),
    "fc3dgpu_dat_open": (C.c_void_p, [C.c_char_p]),
    "fc3dgpu_dat_close": (None, [C.c_void_p]),
    "fc3dgpu_dat_sizes": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_dat_get": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_dat_write": (C.c_int, [C.c_char_p, C.c_int, C.c_int, _I64, _I64, _F64, _F64, _F64]),
    "fc3dgpu_dat_last_error": (C.c_char_p, []),
    "fc3dgpu_compute_error_device": (C.c_int, [C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p,
                                               C.c_void_p]),
    "fc3dgpu_ctx_zero_r": (C.c_int, [C.c_void_p]),
    "fc3dgpu_ctx_staging": (C.c_int, [C.c_void_p, C.c_int]),
    "fc3dgpu_ctx_sync": (C.c_int, [C.c_void_p, C.c_int]),
    "fc3dgpu_ctx_flow": (C.c_int, [C.c_void_p, C.c_int]),
    "fc3dgpu_ctx_flow_warps": (C.c_int, [C.c_void_p, C.c_int]),
    "fc3dgpu_ctx_autotune": (C.c_int, [C.c_void_p, C.c_int]),
    "fc3dgpu_ctx_tuning": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_ctx_spin_limit": (C.c_ulonglong, [C.c_void_p, C.c_ulonglong]),
    "fc3dgpu_ctx_timeline": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    "fc3dgpu_ctx_stream": (C.c_void_p, [C.c_void_p]),
    "fc3dgpu_ctx_launches": (C.c_ulonglong, [C.c_void_p]),
    "fc3dgpu_lattice_create": (C.c_void_p, [C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_double, C.c_double]),
    "fc3dgpu_lattice_free": (None, [C.c_void_p]),
    "fc3dgpu_lattice_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int64)]),
    "fc3dgpu_lattice_fill_W": (C.c_int, [C.c_void_p, _I64, _I64, _F64]),
    "fc3dgpu_lattice_fill_q": (C.c_int, [C.c_void_p, C.c_double, _F64]),
    "fc3dgpu_lattice_fill_geometry": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc3dgpu_lattice_perturb_velocities": (C.c_int, [C.c_void_p, C.c_uint64, C.c_double]),
    "fc3dgpu_normal_fill": (None, [C.c_uint64, _F64, C.c_int64]),
    "fc2dgpu_nsgs": (C.c_int, [C.POINTER(_FCP), _DP, _DP, C.POINTER(_SO)]),
    "fc2dgpu_nsgs_solve_wrap": (C.c_int, [C.c_void_p, _DP, _DP, C.POINTER(_SO)]),
    "fc2dgpu_nsgs_init_wrap": (C.c_int, [C.c_void_p, C.POINTER(_SO)]),
    "fc2dgpu_nsgs_free_wrap": (None, [C.c_void_p, C.POINTER(_SO)]),
    "fc2dgpu_nsgs_set_default": (None, [C.POINTER(_SO)]),
    "fc2dgpu_options_create": (C.POINTER(_SO), []),
    "fc2dgpu_options_delete": (None, [C.POINTER(_SO)]),
    "fc2dgpu_release": (None, [C.POINTER(_SO)]),
    "fc2dgpu_driver": (C.c_int, [C.POINTER(_FCP), _DP, _DP, C.POINTER(_SO)]),
    "fc2dgpu_compute_error": (C.c_int, [C.POINTER(_FCP), _DP, _DP, C.c_double, C.c_double, _DP]),
    "fc2dgpu_ctx_create": (C.c_void_p, [C.c_int]),
    "fc2dgpu_ctx_destroy": (None, [C.c_void_p]),
    "fc2dgpu_ctx_set_problem": (C.c_int, [C.c_void_p, C.c_int, _I64, _I64, _F64, _F64, _F64, C.c_int]),
    "fc2dgpu_ctx_set_q_mu": (C.c_int, [C.c_void_p, _F64, _F64]),
    "fc2dgpu_ctx_set_r": (C.c_int, [C.c_void_p, _F64]),
    "fc2dgpu_ctx_solve": (C.c_int, [C.c_void_p, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int), _DP,
                                    C.POINTER(C.c_int), _DP]),
    "fc2dgpu_ctx_get_r_u": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc2dgpu_ctx_compute_error": (C.c_int, [C.c_void_p, C.c_double, _DP]),
    "fc2dgpu_ctx_colours": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fc2dgpu_ctx_trace": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "fc2dgpu_ctx_set_launch": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "fc2dgpu_ctx_launch_shape": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                           C.POINTER(C.c_int)]),
    "fc2dgpu_ctx_set_precision": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int]),
    "fc2dgpu_ctx_last_sweeps": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "rfc3dgpu_nsgs": (C.c_int, [C.POINTER(_RFCP), _DP, _DP, C.POINTER(_SO)]),
    "rfc3dgpu_nsgs_solve_wrap": (C.c_int, [C.c_void_p, _DP, _DP, C.POINTER(_SO)]),
    "rfc3dgpu_nsgs_init_wrap": (C.c_int, [C.c_void_p, C.POINTER(_SO)]),
    "rfc3dgpu_nsgs_free_wrap": (None, [C.c_void_p, C.POINTER(_SO)]),
    "rfc3dgpu_nsgs_set_default": (None, [C.POINTER(_SO)]),
    "rfc3dgpu_options_create": (C.POINTER(_SO), []),
    "rfc3dgpu_options_delete": (None, [C.POINTER(_SO)]),
    "rfc3dgpu_release": (None, [C.POINTER(_SO)]),
    "rfc3dgpu_driver": (C.c_int, [C.POINTER(_RFCP), _DP, _DP, C.POINTER(_SO)]),
    "rfc3dgpu_compute_error": (C.c_int, [C.POINTER(_RFCP), _DP, _DP, C.c_double, C.c_double, _DP]),
    "rfc3dgpu_ctx_create": (C.c_void_p, [C.c_int]),
    "rfc3dgpu_ctx_destroy": (None, [C.c_void_p]),
    "rfc3dgpu_ctx_set_problem": (C.c_int, [C.c_void_p, C.c_int, _I64, _I64, _F64, _F64, _F64, _F64, C.c_int]),
    "rfc3dgpu_ctx_set_r": (C.c_int, [C.c_void_p, _F64]),
    "rfc3dgpu_ctx_solve": (C.c_int, [C.c_void_p, C.c_double, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_int),
                                     _DP, C.POINTER(C.c_int), _DP]),
    "rfc3dgpu_ctx_get_r_u": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "rfc3dgpu_ctx_compute_error": (C.c_int, [C.c_void_p, C.c_double, _DP]),
    "rfc3dgpu_ctx_colours": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rfc3dgpu_ctx_trace": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "rfc3dgpu_ctx_rho": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rfc3dgpu_ctx_set_precision": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int]),
    "rfc3dgpu_ctx_last_sweeps": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "gfc3dgpu_nsgs": (C.c_int, [C.POINTER(_GFCP), _DP, _DP, _DP, C.POINTER(_SO)]),
    "gfc3dgpu_nsgs_solve_wrap": (C.c_int, [C.c_void_p, _DP, _DP, _DP, C.POINTER(_SO)]),
    "gfc3dgpu_nsgs_init_wrap": (C.c_int, [C.c_void_p, C.POINTER(_SO)]),
    "gfc3dgpu_nsgs_free_wrap": (None, [C.c_void_p, C.POINTER(_SO)]),
    "gfc3dgpu_nsgs_set_default": (None, [C.POINTER(_SO)]),
    "gfc3dgpu_options_create": (C.POINTER(_SO), []),
    "gfc3dgpu_options_delete": (None, [C.POINTER(_SO)]),
    "gfc3dgpu_release": (None, [C.POINTER(_SO)]),
    "gfc3dgpu_driver": (C.c_int, [C.POINTER(_GFCP), _DP, _DP, _DP, C.POINTER(_SO)]),
    "gfc3dgpu_compute_error": (C.c_int, [C.POINTER(_GFCP), _DP, _DP, _DP, C.c_double, C.c_double, C.c_double,
                                         _DP]),
    "gfc3dgpu_ctx_create": (C.c_void_p, [C.c_int]),
    "gfc3dgpu_ctx_destroy": (None, [C.c_void_p]),
    "gfc3dgpu_ctx_set_problem": (C.c_int, [C.c_void_p, C.c_int64, C.c_int, _I64, _I64, _F64, C.c_void_p,
                                           C.c_void_p, C.c_void_p, _F64, C.c_void_p, C.c_void_p]),
    "gfc3dgpu_ctx_set_start": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "gfc3dgpu_ctx_solve": (C.c_int, [C.c_void_p, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int), _DP,
                                     C.POINTER(C.c_int), _DP]),
    "gfc3dgpu_ctx_get": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gfc3dgpu_ctx_compute_error": (C.c_int, [C.c_void_p, C.c_double, _DP]),
    "gfc3dgpu_ctx_trace": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "gfc3dgpu_ctx_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), _DP,
                                    C.POINTER(C.c_int)]),
    "gfc3dgpu_ctx_spin_limit": (C.c_int, [C.c_void_p, C.c_ulonglong]),
    "gfc3dgpu_ctx_set_arithmetic": (C.c_int, [C.c_void_p, C.c_int]),
    "fc3dgpu_lattice_global_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "fc3dgpu_lattice_fill_global": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _I64, _I64, _F64, _I64, _I64, _F64, _F64,
                                              _F64]),
}

# the per-colour comparator (include/fc2dgpu_percolour.h): a separate,
# measurement-only library; the solver library does not link cuSPARSE
COMPARATOR_ABI = {
    "fc2dgpu_percolour_create": (C.c_void_p, [C.c_int, C.c_int, _I64, _I64, _F64, _F64, _F64, C.c_int]),
    "fc2dgpu_percolour_destroy": (None, [C.c_void_p]),
    "fc2dgpu_percolour_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.POINTER(C.c_int), _DP,
                                          C.POINTER(C.c_int), _DP]),
    "fc2dgpu_percolour_get_r_u": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fc2dgpu_percolour_use_kernel_file": (C.c_int, [C.c_void_p, C.c_char_p]),
    "fc2dgpu_percolour_use_bsr": (C.c_int, [C.c_void_p, C.c_int]),
}
_comparator = None


def comparator_lib():
    """The loaded ``libfc2dpercolour.so`` (the reference's per-colour 2D GPU
    design, for measurement beside the solver)."""
    global _comparator
    if _comparator is None:
        lib()  # resolves its dependency on libfc3dgpu.so
        path = LIB_PATH.parent / "libfc2dpercolour.so"
        if not path.exists():
            raise RuntimeError(f"{path} is missing: build it with siconos_gb300.build.build()")
        L = C.CDLL(str(path))
        for name, (res, args) in COMPARATOR_ABI.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _comparator = L
    return _comparator


def lib():
    """The loaded ``libfc3dgpu.so``.  Raises when it has not been built: there
    is no fallback implementation."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with siconos_gb300.build.build()")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in ABI.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def device_info(device: int = 0) -> dict:
    out = np.zeros(6, np.int64)
    if lib().fc3dgpu_device_info(device, out.ctypes.data) != 0:
        raise RuntimeError(last_error())
    return dict(zip(["sms", "l2_bytes", "pageable_access", "pageable_uses_host_page_tables", "cooperative",
                     "cc"], (int(v) for v in out)))


def last_error() -> str:
    v = lib().fc3dgpu_last_error()
    return v.decode() if v else ""


class SparseBlockMatrix:
    """3x3-block CSR matrix exposed to C as a SparseBlockStructuredMatrix
    whose block pointers point into one contiguous numpy array."""

    def __init__(self, nc: int, rowptr, colidx, blocks, block_size: int = 3):
        self.nc = int(nc)
        self.bs = int(block_size)
        if self.bs not in (2, 3, 5):
            raise ValueError("blocks are 2x2, 3x3 or 5x5")
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        self.colidx = np.ascontiguousarray(colidx, dtype=np.int64)
        self.blocks = np.ascontiguousarray(np.asarray(blocks, dtype=np.float64).reshape(-1, self.bs * self.bs))
        nnzb = int(self.rowptr[-1])
        if self.blocks.shape[0] != nnzb or self.colidx.shape[0] != nnzb:
            raise ValueError("block-CSR arrays disagree on the number of blocks")
        # size_t views of the caller's index arrays (non-negative int64 and
        # size_t share a representation on the LP64 targets this builds for):
        # no copy, so buffers the caller allocated (pinned, say) are used as is
        if np.dtype(np.uintp).itemsize == 8 and (self.rowptr.size == 0 or self.rowptr.min() >= 0) and \
                (self.colidx.size == 0 or self.colidx.min() >= 0):
            self._i1 = self.rowptr.view(np.uintp)
            self._i2 = self.colidx.view(np.uintp)
        else:
            self._i1 = self.rowptr.astype(np.uintp)
            self._i2 = self.colidx.astype(np.uintp)
        self._bs = (self.bs * np.arange(1, self.nc + 1)).astype(np.uintp)
        base = self.blocks.ctypes.data
        self._ptrs = self._ptr_array(base, max(nnzb, 1), 8 * self.bs * self.bs)
        s = SparseBlockStructuredMatrix()
        s.nbblocks = nnzb
        s.block = C.cast(self._ptrs, C.POINTER(_DP))
        s.blocknumber0 = s.blocknumber1 = self.nc
        s.blocksize0 = self._bs.ctypes.data_as(_SZP)
        s.blocksize1 = self._bs.ctypes.data_as(_SZP)
        s.filled1 = self.nc + 1
        s.filled2 = nnzb
        s.index1_data = self._i1.ctypes.data_as(_SZP)
        s.index2_data = self._i2.ctypes.data_as(_SZP)
        s.diagonal_blocks = None
        s.version.number = 1
        self.c = s

    @staticmethod
    def _ptr_array(base, n, stride=72):
        arr = (base + stride * np.arange(n, dtype=np.uint64)).astype(np.uintp)
        holder = (_DP * n).from_buffer(arr)
        holder._keep = arr
        return holder

    def bump_version(self):
        """Signal that the block values changed (invalidates the device copy)."""
        self.c.version.number += 1

    def todense(self) -> np.ndarray:
        b = self.bs
        n = b * self.nc
        W = np.zeros((n, n), order="F")
        for i in range(self.nc):
            for k in range(self.rowptr[i], self.rowptr[i + 1]):
                j = self.colidx[k]
                W[b * i:b * i + b, b * j:b * j + b] = self.blocks[k].reshape(b, b, order="F")
        return W


class FrictionContactProblem:
    """``FrictionContactProblem(dim, nc, M, q, mu)`` sharing the numpy buffers."""

    def __init__(self, dim: int, nc: int, M, q, mu):
        if dim not in (2, 3):
            raise ValueError("dimension 2 or 3")
        if isinstance(M, SparseBlockMatrix) and M.bs != dim:
            raise ValueError("block size differs from the dimension")
        self._q = q if (isinstance(q, np.ndarray) and q.dtype == np.float64 and q.flags.c_contiguous) \
            else np.ascontiguousarray(q, dtype=np.float64)
        self._mu = mu if (isinstance(mu, np.ndarray) and mu.dtype == np.float64 and mu.flags.c_contiguous) \
            else np.ascontiguousarray(mu, dtype=np.float64)
        self._M = M
        nm = NumericsMatrix()
        nm.size0 = nm.size1 = dim * nc
        if isinstance(M, SparseBlockMatrix):
            nm.storageType = NM_SPARSE_BLOCK
            nm.matrix1 = C.pointer(M.c)
        else:
            if not (isinstance(M, np.ndarray) and M.dtype == np.float64 and M.flags.f_contiguous):
                raise TypeError("dense M must be a Fortran-ordered float64 numpy array")
            nm.storageType = NM_DENSE
            nm.matrix0 = M.ctypes.data_as(_DP)
        nm.version.number = 1
        self._nm = nm
        p = _FCP()
        p.dimension = dim
        p.numberOfContacts = nc
        p.M = C.pointer(nm)
        p.q = self._q.ctypes.data_as(_DP)
        p.mu = self._mu.ctypes.data_as(_DP)
        self.c = p

    @property
    def numberOfContacts(self) -> int:
        return self.c.numberOfContacts

    @property
    def dimension(self) -> int:
        return self.c.dimension

    def M(self):
        return self._M

    def q(self):
        return self._q

    def mu(self):
        return self._mu


class SolverOptions:
    """``SolverOptions(solver_id)`` for ``SICONOS_FRICTION_3D_NSGS_GPU`` or
    ``SICONOS_FRICTION_2D_NSGS_GPU``."""

    _KINDS = {SICONOS_FRICTION_3D_NSGS_GPU: "fc3dgpu", SICONOS_FRICTION_2D_NSGS_GPU: "fc2dgpu",
              SICONOS_ROLLING_FRICTION_3D_NSGS_GPU: "rfc3dgpu", SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU: "gfc3dgpu"}

    def __init__(self, solver_id: int = SICONOS_FRICTION_3D_NSGS_GPU):
        if solver_id not in self._KINDS:
            raise ValueError(f"solver {solver_id} is not provided by this library")
        self._kind = self._KINDS[solver_id]
        self.ptr = getattr(lib(), self._kind + "_options_create")()
        if not self.ptr:
            raise MemoryError(self._kind + "_options_create failed")
        self._cb = None

    @property
    def solverId(self) -> int:
        return self.ptr.contents.solverId

    @property
    def iparam(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.ptr.contents.iparam, shape=(OPTIONS_PARAM_SIZE,))

    @property
    def dparam(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.ptr.contents.dparam, shape=(OPTIONS_PARAM_SIZE,))

    @property
    def internalSolvers(self):
        o = self.ptr.contents
        return [_InternalOptions(o.internalSolvers[i]) for i in range(o.numberOfInternalSolvers)]

    def set_callback(self, fn):
        """fn(size, reaction, velocity, error) per iteration."""
        def _c(env, size, r, u, err, extra):
            fn(int(size), np.ctypeslib.as_array(r, shape=(size,)), np.ctypeslib.as_array(u, shape=(size,)), err)
        cfun = CALLBACK_T(_c)
        cb = Callback(None, cfun)
        self._cb = (cfun, cb)
        self.ptr.contents.callback = C.pointer(cb)

    def release(self):
        getattr(lib(), self._kind + "_release")(self.ptr)

    def __del__(self):
        try:
            if getattr(self, "ptr", None):
                self.ptr.contents.callback = None
                getattr(lib(), self._kind + "_options_delete")(self.ptr)
                self.ptr = None
        except Exception:
            pass


class _InternalOptions:
    def __init__(self, ptr):
        self.ptr = ptr

    @property
    def solverId(self) -> int:
        return self.ptr.contents.solverId

    @property
    def iparam(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.ptr.contents.iparam, shape=(OPTIONS_PARAM_SIZE,))

    @property
    def dparam(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.ptr.contents.dparam, shape=(OPTIONS_PARAM_SIZE,))


def _vec(x, n):
    if not (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous and x.size == n):
        raise TypeError(f"expected a C-contiguous float64 array of size {n}")
    return x.ctypes.data_as(_DP)


def fc3d_driver(problem: FrictionContactProblem, reaction: np.ndarray, velocity: np.ndarray,
                options: SolverOptions) -> int:
    n = 3 * problem.numberOfContacts
    return lib().fc3dgpu_driver(C.byref(problem.c), _vec(reaction, n), _vec(velocity, n), options.ptr)


def fc3d_nsgs_gpu(problem, reaction, velocity, options) -> int:
    """The solver entry itself (what the registry binds), without the
    driver's trivial-case shortcut."""
    n = 3 * problem.numberOfContacts
    return lib().fc3dgpu_nsgs(C.byref(problem.c), _vec(reaction, n), _vec(velocity, n), options.ptr)


def read_dat(path) -> "FrictionContactProblem":
    """A FrictionContactProblem from a .dat file of the reference's text format
    (frictionContact_new_from_filename for .dat files), W in sparse-block
    storage."""
    L = lib()
    h = L.fc3dgpu_dat_open(str(path).encode())
    if not h:
        raise ValueError(f"{path}: {L.fc3dgpu_dat_last_error().decode()}")
    try:
        dim, nc, nnzb = C.c_int(), C.c_int(), C.c_int64()
        L.fc3dgpu_dat_sizes(h, C.byref(dim), C.byref(nc), C.byref(nnzb))
        d, n, k = dim.value, nc.value, nnzb.value
        rp = np.zeros(n + 1, np.int64)
        ci = np.zeros(k, np.int64)
        bl = np.zeros((k, d * d))
        q = np.zeros(d * n)
        mu = np.zeros(n)
        L.fc3dgpu_dat_get(h, rp.ctypes.data, ci.ctypes.data, bl.ctypes.data, q.ctypes.data, mu.ctypes.data)
    finally:
        L.fc3dgpu_dat_close(h)
    return FrictionContactProblem(d, n, SparseBlockMatrix(n, rp, ci, bl, block_size=d), q, mu)


def write_dat(problem: "FrictionContactProblem", path) -> None:
    """Write a problem with a sparse-block W in the reference's .dat format
    (frictionContact_printInFilename)."""
    M = problem._M
    if not isinstance(M, SparseBlockMatrix):
        raise TypeError("write_dat needs W in sparse-block storage")
    rc = lib().fc3dgpu_dat_write(str(path).encode(), M.bs, M.nc, M.rowptr, M.colidx, M.blocks.reshape(-1),
                                 problem._q, problem._mu)
    if rc != 0:
        raise OSError(lib().fc3dgpu_dat_last_error().decode())


def fc3d_compute_error(problem, reaction, velocity, tolerance: float, norm_q: float):
    n = 3 * problem.numberOfContacts
    err = C.c_double()
    info = lib().fc3dgpu_compute_error(C.byref(problem.c), _vec(reaction, n), _vec(velocity, n), tolerance, norm_q,
                                       C.byref(err))
    return info, err.value


def fc3d_nsgs_batch(problems, reactions, velocities, options):
    k = len(problems)
    P = (C.POINTER(_FCP) * k)(*[C.pointer(p.c) for p in problems])
    R = (_DP * k)(*[_vec(r, 3 * p.numberOfContacts) for r, p in zip(reactions, problems)])
    U = (_DP * k)(*[_vec(u, 3 * p.numberOfContacts) for u, p in zip(velocities, problems)])
    info = (C.c_int * k)()
    rc = lib().fc3dgpu_nsgs_batch(k, P, R, U, options.ptr, info)
    return rc, list(info)


def fc2d_driver(problem: FrictionContactProblem, reaction: np.ndarray, velocity: np.ndarray,
                options: SolverOptions) -> int:
    """fc2d_driver for ``SICONOS_FRICTION_2D_NSGS_GPU``: returns ``info``."""
    n = 2 * problem.numberOfContacts
    return lib().fc2dgpu_driver(C.byref(problem.c), _vec(reaction, n), _vec(velocity, n), options.ptr)


def fc2d_nsgs_gpu(problem, reaction, velocity, options) -> int:
    """The 2D solver entry itself (what the registry binds), options as given."""
    n = 2 * problem.numberOfContacts
    return lib().fc2dgpu_nsgs(C.byref(problem.c), _vec(reaction, n), _vec(velocity, n), options.ptr)


def fc2d_compute_error(problem, reaction, velocity, tolerance: float, norm_q: float):
    n = 2 * problem.numberOfContacts
    err = C.c_double()
    info = lib().fc2dgpu_compute_error(C.byref(problem.c), _vec(reaction, n), _vec(velocity, n), tolerance, norm_q,
                                       C.byref(err))
    return info, err.value


class Fc2dContext:
    """Device-resident 2D problem (``fc2dgpu_ctx_*``): upload once, solve many
    times from any reaction."""

    def __init__(self, nc, rowptr, colidx, blocks, q, mu, colouring: int = 0, device: int = 0):
        L = lib()
        self.ctx = L.fc2dgpu_ctx_create(device)
        if not self.ctx:
            raise RuntimeError(last_error())
        self.nc = int(nc)
        rc = L.fc2dgpu_ctx_set_problem(self.ctx, self.nc, np.ascontiguousarray(rowptr, np.int64),
                                       np.ascontiguousarray(colidx, np.int64),
                                       np.ascontiguousarray(blocks, np.float64).reshape(-1),
                                       np.ascontiguousarray(q, np.float64), np.ascontiguousarray(mu, np.float64),
                                       colouring)
        if rc != 0:
            L.fc2dgpu_ctx_destroy(self.ctx)
            self.ctx = None
            raise ValueError(last_error())

    def set_r(self, r):
        _check(lib().fc2dgpu_ctx_set_r(self.ctx, np.ascontiguousarray(r, np.float64)))

    def set_q_mu(self, q, mu):
        _check(lib().fc2dgpu_ctx_set_q_mu(self.ctx, np.ascontiguousarray(q, np.float64),
                                          np.ascontiguousarray(mu, np.float64)))

    def solve(self, tol: float, max_iter: int,
              error_evaluation: int = SICONOS_FRICTION_3D_NSGS_ERROR_EVALUATION_LIGHT_WITH_FULL_FINAL) -> dict:
        it, info = C.c_int(), C.c_int()
        err, ms = C.c_double(), C.c_double()
        _check(lib().fc2dgpu_ctx_solve(self.ctx, tol, max_iter, error_evaluation, C.byref(it), C.byref(err),
                                       C.byref(info), C.byref(ms)))
        return dict(iterations=it.value, error=err.value, info=info.value, ms=ms.value)

    def get_r_u(self):
        r, u = np.zeros(2 * self.nc), np.zeros(2 * self.nc)
        _check(lib().fc2dgpu_ctx_get_r_u(self.ctx, r.ctypes.data, u.ctypes.data))
        return r, u

    def compute_error(self, norm_q: float) -> float:
        e = C.c_double()
        _check(lib().fc2dgpu_ctx_compute_error(self.ctx, norm_q, C.byref(e)))
        return e.value

    def colours(self):
        out = np.zeros(self.nc, np.int32)
        n = lib().fc2dgpu_ctx_colours(self.ctx, out.ctypes.data)
        if n < 0:
            raise RuntimeError(last_error())
        return n, out

    def set_precision(self, precision: int, switch_tol: float = 0.0, stall_window: int = 0):
        """0: FP32 sweeps, then the FP64 sweeps of the reference's loop from
        their iterate; 1: FP64 sweeps only (the default of a context)."""
        _check(lib().fc2dgpu_ctx_set_precision(self.ctx, precision, switch_tol, stall_window))

    def last_sweeps(self):
        """(FP32 sweeps, FP64 sweeps) of the last solve."""
        a, b = C.c_int(), C.c_int()
        _check(lib().fc2dgpu_ctx_last_sweeps(self.ctx, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_launch(self, cluster_blocks: int = 0, threads: int = 0, reactions: int = 0):
        """Sweep launch shape (0 = automatic; reactions 1 in HBM, 2 replicated
        in shared memory); returns the shape in use."""
        _check(lib().fc2dgpu_ctx_set_launch(self.ctx, cluster_blocks, threads, reactions))
        return self.launch_shape()

    def launch_shape(self):
        cs, nt, rx = C.c_int(), C.c_int(), C.c_int()
        _check(lib().fc2dgpu_ctx_launch_shape(self.ctx, C.byref(cs), C.byref(nt), C.byref(rx)))
        return cs.value, nt.value, rx.value

    def trace(self, cap: int) -> np.ndarray:
        out = np.zeros(max(cap, 1))
        n = lib().fc2dgpu_ctx_trace(self.ctx, out.ctypes.data, cap)
        return out[:max(n, 0)].copy()

    def close(self):
        if getattr(self, "ctx", None):
            lib().fc2dgpu_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RollingFrictionContactProblem:
    """``RollingFrictionContactProblem(5, nc, M, q, mu, mu_r)`` sharing the
    numpy buffers; M dense (Fortran order) or a 5x5 :class:`SparseBlockMatrix`."""

    def __init__(self, dim: int, nc: int, M, q, mu, mu_r):
        if dim != 5:
            raise ValueError("dimension 5")
        if isinstance(M, SparseBlockMatrix) and M.bs != 5:
            raise ValueError("block size differs from the dimension")
        as_f64 = (lambda x: x if (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous)
                  else np.ascontiguousarray(x, dtype=np.float64))
        self._q, self._mu, self._mu_r = as_f64(q), as_f64(mu), as_f64(mu_r)
        self._M = M
        nm = NumericsMatrix()
        nm.size0 = nm.size1 = 5 * nc
        if isinstance(M, SparseBlockMatrix):
            nm.storageType = NM_SPARSE_BLOCK
            nm.matrix1 = C.pointer(M.c)
        else:
            if not (isinstance(M, np.ndarray) and M.dtype == np.float64 and M.flags.f_contiguous):
                raise TypeError("dense M must be a Fortran-ordered float64 numpy array")
            nm.storageType = NM_DENSE
            nm.matrix0 = M.ctypes.data_as(_DP)
        nm.version.number = 1
        self._nm = nm
        p = _RFCP()
        p.dimension = 5
        p.numberOfContacts = nc
        p.M = C.pointer(nm)
        p.q = self._q.ctypes.data_as(_DP)
        p.mu = self._mu.ctypes.data_as(_DP)
        p.mu_r = self._mu_r.ctypes.data_as(_DP)
        self.c = p

    @property
    def numberOfContacts(self) -> int:
        return self.c.numberOfContacts


def rolling_friction_3d_driver(problem: RollingFrictionContactProblem, reaction, velocity, options) -> int:
    """rolling_friction_3d_driver for ``SICONOS_ROLLING_FRICTION_3D_NSGS_GPU``."""
    n = 5 * problem.numberOfContacts
    return lib().rfc3dgpu_driver(C.byref(problem.c), _vec(reaction, n), _vec(velocity, n), options.ptr)


def rolling_friction_3d_compute_error(problem, reaction, velocity, tolerance: float, norm_q: float):
    n = 5 * problem.numberOfContacts
    err = C.c_double()
    info = lib().rfc3dgpu_compute_error(C.byref(problem.c), _vec(reaction, n), _vec(velocity, n), tolerance, norm_q,
                                        C.byref(err))
    return info, err.value


class RollingContext:
    """Device-resident rolling-friction problem (``rfc3dgpu_ctx_*``)."""

    def __init__(self, nc, rowptr, colidx, blocks, q, mu, mu_r, colouring: int = 0, device: int = 0):
        L = lib()
        self.ctx = L.rfc3dgpu_ctx_create(device)
        if not self.ctx:
            raise RuntimeError(last_error())
        self.nc = int(nc)
        rc = L.rfc3dgpu_ctx_set_problem(self.ctx, self.nc, np.ascontiguousarray(rowptr, np.int64),
                                        np.ascontiguousarray(colidx, np.int64),
                                        np.ascontiguousarray(blocks, np.float64).reshape(-1),
                                        np.ascontiguousarray(q, np.float64), np.ascontiguousarray(mu, np.float64),
                                        np.ascontiguousarray(mu_r, np.float64), colouring)
        if rc != 0:
            L.rfc3dgpu_ctx_destroy(self.ctx)
            self.ctx = None
            raise ValueError(last_error())

    def set_r(self, r):
        _check(lib().rfc3dgpu_ctx_set_r(self.ctx, np.ascontiguousarray(r, np.float64)))

    def solve(self, tol: float, max_iter: int, local_tol: float = 1e-12, local_max_iter: int = 10) -> dict:
        it, info = C.c_int(), C.c_int()
        err, ms = C.c_double(), C.c_double()
        _check(lib().rfc3dgpu_ctx_solve(self.ctx, tol, max_iter, local_tol, local_max_iter, C.byref(it),
                                        C.byref(err), C.byref(info), C.byref(ms)))
        return dict(iterations=it.value, error=err.value, info=info.value, ms=ms.value)

    def get_r_u(self):
        r, u = np.zeros(5 * self.nc), np.zeros(5 * self.nc)
        _check(lib().rfc3dgpu_ctx_get_r_u(self.ctx, r.ctypes.data, u.ctypes.data))
        return r, u

    def compute_error(self, norm_q: float) -> float:
        e = C.c_double()
        _check(lib().rfc3dgpu_ctx_compute_error(self.ctx, norm_q, C.byref(e)))
        return e.value

    def colours(self):
        out = np.zeros(self.nc, np.int32)
        n = lib().rfc3dgpu_ctx_colours(self.ctx, out.ctypes.data)
        if n < 0:
            raise RuntimeError(last_error())
        return n, out

    def rho(self) -> np.ndarray:
        out = np.zeros(self.nc)
        _check(lib().rfc3dgpu_ctx_rho(self.ctx, out.ctypes.data))
        return out

    def trace(self, cap: int) -> np.ndarray:
        out = np.zeros(max(cap, 1))
        n = lib().rfc3dgpu_ctx_trace(self.ctx, out.ctypes.data, cap)
        return out[:max(n, 0)].copy()

    def set_precision(self, precision: int, switch_tol: float = 0.0, stall_window: int = 0):
        """0: FP32 sweeps, then the reference's FP64 loop from their iterate;
        1: FP64 sweeps only (the default of a context)."""
        _check(lib().rfc3dgpu_ctx_set_precision(self.ctx, precision, switch_tol, stall_window))

    def last_sweeps(self):
        """(FP32 sweeps, FP64 sweeps) of the last solve."""
        a, b = C.c_int(), C.c_int()
        _check(lib().rfc3dgpu_ctx_last_sweeps(self.ctx, C.byref(a), C.byref(b)))
        return a.value, b.value

    def close(self):
        if getattr(self, "ctx", None):
            lib().rfc3dgpu_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Fc2dPerColour:
    """The reference's per-colour GPU design for fc2d (cuSPARSE SpMV + local
    solve per colour, a CUDA graph per sweep, host convergence test), for
    measurement beside :class:`Fc2dContext` (``include/fc2dgpu_percolour.h``)."""

    def __init__(self, nc, rowptr, colidx, blocks, q, mu, colouring: int = 0, device: int = 0):
        self.nc = int(nc)
        self.h = comparator_lib().fc2dgpu_percolour_create(device, self.nc, np.ascontiguousarray(rowptr, np.int64),
                                                np.ascontiguousarray(colidx, np.int64),
                                                np.ascontiguousarray(blocks, np.float64).reshape(-1),
                                                np.ascontiguousarray(q, np.float64),
                                                np.ascontiguousarray(mu, np.float64), colouring)
        if not self.h:
            raise RuntimeError(last_error())

    def solve(self, tol: float, max_iter: int, r0=None) -> dict:
        it, info = C.c_int(), C.c_int()
        err, ms = C.c_double(), C.c_double()
        r0p = None if r0 is None else np.ascontiguousarray(r0, np.float64)
        _check(comparator_lib().fc2dgpu_percolour_solve(self.h, None if r0p is None else r0p.ctypes.data, tol, max_iter,
                                             C.byref(it), C.byref(err), C.byref(info), C.byref(ms)))
        return dict(iterations=it.value, error=err.value, info=info.value, ms=ms.value)

    def get_r_u(self):
        r, u = np.zeros(2 * self.nc), np.zeros(2 * self.nc)
        _check(comparator_lib().fc2dgpu_percolour_get_r_u(self.h, r.ctypes.data, u.ctypes.data))
        return r, u

    def use_kernel_file(self, path) -> None:
        """Run the local-solve kernel of a CUDA library image (the
        reference's fc2d_nsgs_local_solve_kernel_range_reduce, compiled from
        its own source) in the sweep instead of the comparator's."""
        _check(comparator_lib().fc2dgpu_percolour_use_kernel_file(self.h, str(path).encode()))

    def use_bsr(self, on: bool = True) -> None:
        """Sweep as the reference's BLOCKLEGACY variant: per colour a
        cuSPARSE BSR matvec of 2x2 blocks and the local solve, no graph."""
        _check(comparator_lib().fc2dgpu_percolour_use_bsr(self.h, int(on)))

    def close(self):
        if getattr(self, "h", None):
            comparator_lib().fc2dgpu_percolour_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _check(rc):
    if rc != 0:
        raise RuntimeError(f"status {rc}: {last_error()}")


def colour(rowptr, colidx, kind: int = 0) -> tuple[int, np.ndarray]:
    """Device colouring of a block-CSR structure: (number of colours, colour
    per contact)."""
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    colidx = np.ascontiguousarray(colidx, np.int64)
    nc = rowptr.size - 1
    out = np.zeros(nc, np.int32)
    n = lib().fc3dgpu_colour(nc, rowptr, colidx, kind, out)
    if n < 0:
        raise RuntimeError(last_error())
    return n, out


# ---- global 3D friction contact (M v = q + H r, u = H^T v + b) --------------
class BlockMatrix:
    """A sparse-block matrix with blocks of any sizes (the reference's
    SparseBlockStructuredMatrix in general form): ``row_sizes`` and
    ``col_sizes`` the block sizes, ``blocks`` a dict (block row, block
    column) -> dense block.  Blocks are kept column-major in one array."""

    def __init__(self, row_sizes, col_sizes, blocks: dict):
        self.row_sizes = np.asarray(row_sizes, np.int64)
        self.col_sizes = np.asarray(col_sizes, np.int64)
        keys = sorted(blocks)
        self.shape = (int(self.row_sizes.sum()), int(self.col_sizes.sum()))
        self._cum0 = np.cumsum(self.row_sizes).astype(np.uintp)
        self._cum1 = np.cumsum(self.col_sizes).astype(np.uintp)
        nbr = len(self.row_sizes)
        i1 = np.zeros(nbr + 1, np.uintp)
        for bi, _ in keys:
            i1[bi + 1] += 1
        self._i1 = np.cumsum(i1).astype(np.uintp)
        self._i2 = np.array([bj for _, bj in keys] or [0], np.uintp)
        offs, vals = [], []
        o = 0
        for k in keys:
            a = np.asarray(blocks[k], np.float64)
            if a.shape != (self.row_sizes[k[0]], self.col_sizes[k[1]]):
                raise ValueError(f"block {k} has shape {a.shape}")
            offs.append(o)
            vals.append(a.reshape(-1, order="F"))
            o += a.size
        self.data = np.ascontiguousarray(np.concatenate(vals) if vals else np.zeros(1))
        base = self.data.ctypes.data
        self._ptrs = (_DP * max(len(keys), 1))(*[C.cast(base + 8 * x, _DP) for x in offs])
        s = SparseBlockStructuredMatrix()
        s.nbblocks = len(keys)
        s.block = C.cast(self._ptrs, C.POINTER(_DP))
        s.blocknumber0 = nbr
        s.blocknumber1 = len(self.col_sizes)
        s.blocksize0 = self._cum0.ctypes.data_as(_SZP)
        s.blocksize1 = self._cum1.ctypes.data_as(_SZP)
        s.filled1 = nbr + 1
        s.filled2 = len(keys)
        s.index1_data = self._i1.ctypes.data_as(_SZP)
        s.index2_data = self._i2.ctypes.data_as(_SZP)
        s.diagonal_blocks = None
        s.version.number = 1
        self.c = s

    @staticmethod
    def from_dense(A, row_sizes, col_sizes) -> "BlockMatrix":
        """Every block of A (cut by the sizes) with a nonzero entry."""
        r0 = np.concatenate([[0], np.cumsum(row_sizes)])
        c0 = np.concatenate([[0], np.cumsum(col_sizes)])
        blocks = {}
        for bi in range(len(row_sizes)):
            for bj in range(len(col_sizes)):
                blk = A[r0[bi]:r0[bi + 1], c0[bj]:c0[bj + 1]]
                if np.any(blk != 0):
                    blocks[(bi, bj)] = np.array(blk)
        return BlockMatrix(row_sizes, col_sizes, blocks)


def _nm_of(A, rows, cols):
    nm = NumericsMatrix()
    nm.size0, nm.size1 = rows, cols
    if isinstance(A, BlockMatrix):
        if A.shape != (rows, cols):
            raise ValueError(f"block matrix is {A.shape}, expected {(rows, cols)}")
        nm.storageType = NM_SPARSE_BLOCK
        nm.matrix1 = C.pointer(A.c)
    else:
        if not (isinstance(A, np.ndarray) and A.dtype == np.float64 and A.flags.f_contiguous and
                A.shape == (rows, cols)):
            raise TypeError(f"dense matrices are Fortran-ordered float64 arrays of shape {(rows, cols)}")
        nm.storageType = NM_DENSE
        nm.matrix0 = A.ctypes.data_as(_DP)
    nm.version.number = 1
    return nm


class GlobalFrictionContactProblem:
    """``GlobalFrictionContactProblem(dim, nc, M, H, q, b, mu)``: M (n x n)
    and H (n x 3 nc) dense (Fortran order) or :class:`BlockMatrix`; the numpy
    buffers are shared."""

    def __init__(self, dim: int, nc: int, M, H, q, b, mu):
        if dim != 3:
            raise ValueError("dimension 3")
        as_f64 = (lambda x: x if (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous)
                  else np.ascontiguousarray(x, dtype=np.float64))
        self._q, self._b, self._mu = as_f64(q), as_f64(b), as_f64(mu)
        n = self._q.size
        self._M, self._H = M, H
        self._nm = _nm_of(M, n, n)
        self._nh = _nm_of(H, n, 3 * nc)
        p = _GFCP()
        p.dimension = 3
        p.numberOfContacts = nc
        p.M = C.pointer(self._nm)
        p.H = C.pointer(self._nh)
        p.q = self._q.ctypes.data_as(_DP)
        p.b = self._b.ctypes.data_as(_DP)
        p.mu = self._mu.ctypes.data_as(_DP)
        self.c = p
        self.n = n

    @property
    def numberOfContacts(self) -> int:
        return self.c.numberOfContacts


def gfc3d_driver(problem: GlobalFrictionContactProblem, reaction, velocity, globalVelocity, options) -> int:
    """gfc3d_driver for ``SICONOS_GLOBAL_FRICTION_3D_NSGS_GPU``: returns ``info``."""
    m = 3 * problem.numberOfContacts
    return lib().gfc3dgpu_driver(C.byref(problem.c), _vec(reaction, m) if m else None,
                                 _vec(velocity, m) if m else None, _vec(globalVelocity, problem.n), options.ptr)


def gfc3d_nsgs_gpu(problem, reaction, velocity, globalVelocity, options) -> int:
    """The solver entry itself (what the registry binds), options as given."""
    m = 3 * problem.numberOfContacts
    return lib().gfc3dgpu_nsgs(C.byref(problem.c), _vec(reaction, m), _vec(velocity, m),
                               _vec(globalVelocity, problem.n), options.ptr)


def gfc3d_compute_error(problem, reaction, velocity, globalVelocity, tolerance: float, norm_q: float):
    """(info, error) as the reference's gfc3d_compute_error; writes velocity."""
    m = 3 * problem.numberOfContacts
    err = C.c_double()
    info = lib().gfc3dgpu_compute_error(C.byref(problem.c), _vec(reaction, m), _vec(velocity, m),
                                        _vec(globalVelocity, problem.n), tolerance, norm_q, 0.0, C.byref(err))
    return info, err.value


class Gfc3dContext:
    """Device-resident global problem (``gfc3dgpu_ctx_*``): M and H as CSR
    arrays, uploaded once, solved many times."""

    def __init__(self, n, nc, Mp, Mi, Mx, Hp, Hi, Hx, q, b, mu, device: int = 0):
        L = lib()
        self.ctx = L.gfc3dgpu_ctx_create(device)
        if not self.ctx:
            raise RuntimeError(last_error())
        self.n, self.nc = int(n), int(nc)
        c = np.ascontiguousarray
        self._keep = [c(Hp, np.int64), c(Hi, np.int64), c(Hx, np.float64), c(b, np.float64), c(mu, np.float64)]
        hp, hi, hx, bb, mm = self._keep
        rc = L.gfc3dgpu_ctx_set_problem(self.ctx, self.n, self.nc, c(Mp, np.int64), c(Mi, np.int64),
                                        c(Mx, np.float64), hp.ctypes.data, hi.ctypes.data, hx.ctypes.data,
                                        c(q, np.float64), bb.ctypes.data, mm.ctypes.data)
        if rc != 0:
            L.gfc3dgpu_ctx_destroy(self.ctx)
            self.ctx = None
            raise ValueError(last_error())

    @staticmethod
    def from_problem(P, device: int = 0) -> "Gfc3dContext":
        """From any object with the fields of ``oracle.GlobalProblem``."""
        return Gfc3dContext(P.n, P.nc, P.Mp, P.Mi, P.Mx, P.Hp, P.Hi, P.Hx, P.q, P.b, P.mu, device)

    def set_start(self, r=None, v=None):
        rr = None if r is None else np.ascontiguousarray(r, np.float64)
        vv = None if v is None else np.ascontiguousarray(v, np.float64)
        _check(lib().gfc3dgpu_ctx_set_start(self.ctx, None if rr is None else rr.ctypes.data,
                                            None if vv is None else vv.ctypes.data))

    def solve(self, tol: float, max_iter: int, freq: int = 0) -> dict:
        it, info = C.c_int(), C.c_int()
        err, ms = C.c_double(), C.c_double()
        _check(lib().gfc3dgpu_ctx_solve(self.ctx, tol, max_iter, freq, C.byref(it), C.byref(err), C.byref(info),
                                        C.byref(ms)))
        return dict(iterations=it.value, error=err.value, info=info.value, ms=ms.value)

    def get(self):
        r, u, v = np.zeros(3 * self.nc), np.zeros(3 * self.nc), np.zeros(self.n)
        _check(lib().gfc3dgpu_ctx_get(self.ctx, r.ctypes.data, u.ctypes.data, v.ctypes.data))
        return r, u, v

    def compute_error(self, norm_q: float = -1.0) -> float:
        e = C.c_double()
        _check(lib().gfc3dgpu_ctx_compute_error(self.ctx, norm_q, C.byref(e)))
        return e.value

    def trace(self, cap: int) -> np.ndarray:
        out = np.zeros(max(cap, 1))
        k = lib().gfc3dgpu_ctx_trace(self.ctx, out.ctypes.data, cap)
        return out[:max(k, 0)].copy()

    def info(self) -> dict:
        nc, mx, dg, gr = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        by = C.c_double()
        _check(lib().gfc3dgpu_ctx_info(self.ctx, C.byref(nc), C.byref(mx), C.byref(dg), C.byref(by), C.byref(gr)))
        return dict(components=nc.value, max_component=mx.value, diagonal=bool(dg.value),
                    bytes_per_iteration=by.value, grid=gr.value)

    def spin_limit(self, polls: int):
        _check(lib().gfc3dgpu_ctx_spin_limit(self.ctx, polls))

    def set_arithmetic(self, fused: bool):
        """False: the reference's products (bit-exact iterates, the default);
        True: fused multiply-adds (opt-in, equal to rounding)."""
        _check(lib().gfc3dgpu_ctx_set_arithmetic(self.ctx, int(bool(fused))))

    def close(self):
        if getattr(self, "ctx", None):
            lib().gfc3dgpu_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
