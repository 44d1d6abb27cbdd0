"""ctypes binding of ``libfwi_psv.so`` (the C ABI in ``include/fwi_psv.h``).

There is no CPU fallback: if the library is missing or no GPU is present the
calls that need the device raise :class:`PSVError`.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB, build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

PSV_OK, PSV_ERR_ARG, PSV_ERR_CFL, PSV_ERR_OOM, PSV_ERR_CUDA = 0, 1, 2, 3, 4
PSV_ERR_UNSUPPORTED, PSV_ERR_TIMEOUT, PSV_ERR_STEP_SEARCH, PSV_ERR_IO = 5, 6, 7, 8
PSV_MAX_NZ, PSV_MAX_SHOTS, PSV_MAX_SHOT_ELEMS = 65535, 65535, 2**31 - 1
STENCIL = {"reference": 0, "holberg": 1}
STORAGE = {"auto": 0, "full": 1, "checkpoint": 2, "binomial": 3}


class PSVError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"psv status {status}: {msg}")
        self.status = status


class PsvGrid(C.Structure):
    _fields_ = [
        ("nt", C.c_int), ("nz", C.c_int), ("nx", C.c_int),
        ("dt", C.c_double), ("dx", C.c_double), ("dz", C.c_double),
        ("fdorder", C.c_int), ("stencil", C.c_int), ("surf", C.c_int), ("isurf", C.c_int * 4),
        ("hc", C.c_double * 7),
        ("pml_z", C.c_int), ("pml_x", C.c_int),
        ("a_z", _dp), ("b_z", _dp), ("K_z", _dp), ("a_half_z", _dp), ("b_half_z", _dp),
        ("K_half_z", _dp),
        ("a_x", _dp), ("b_x", _dp), ("K_x", _dp), ("a_half_x", _dp), ("b_half_x", _dp),
        ("K_half_x", _dp),
        ("snap_z1", C.c_int), ("snap_z2", C.c_int), ("snap_x1", C.c_int), ("snap_x2", C.c_int),
        ("snap_dt", C.c_int), ("snap_dz", C.c_int), ("snap_dx", C.c_int),
        ("taper", C.c_int * 8),
        ("imaging_sign", C.c_int),
    ]


class PsvShots(C.Structure):
    _fields_ = [
        ("nshot", C.c_int), ("nsrc", C.c_int), ("nrec", C.c_int), ("stf_type", C.c_int),
        ("rtf_type", C.c_int),
        ("z_src", _ip), ("x_src", _ip), ("src_shot_to_fire", _ip),
        ("stf_z", _dp), ("stf_x", _dp),
        ("z_rec", _ip), ("x_rec", _ip),
    ]


class PsvOptions(C.Structure):
    _fields_ = [
        ("precision", C.c_int), ("storage", C.c_int), ("hbm_budget_gb", C.c_double),
        ("checkpoint_interval", C.c_int), ("max_batch", C.c_int), ("use_graphs", C.c_int),
        ("block_x", C.c_int), ("block_y", C.c_int), ("rows_per_thread", C.c_int),
        ("kernel_family", C.c_int), ("autotune", C.c_int), ("checkpoint_slots", C.c_int),
        ("smooth_hfs", C.c_int), ("pcg", C.c_int), ("chains", C.c_int), ("adjoint", C.c_int),
    ]


# Every symbol include/fwi_psv.h declares, with its C signature.
SIGNATURES = {
    "psv_error_string": (C.c_char_p, [C.c_int]),
    "psv_last_error": (C.c_char_p, []),
    "psv_device_available": (C.c_int, []),
    "psv_holbergcoeff": (C.c_int, [C.c_int, C.c_int, _dp]),
    "psv_cpml_PSV": (C.c_int, [_dp] * 6 + [C.c_double] * 5 + [C.c_int] * 4 + [C.c_double] * 2),
    "psv_wavelet": (C.c_int, [_dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]),
    "psv_checkfd_ssg_elastic": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                          C.c_int, _dp, _dp, _dp, _dp, _dp]),
    "psv_options_default": (None, [C.POINTER(PsvOptions)]),
    "psv_plan_create": (C.c_int, [C.POINTER(PsvGrid), C.POINTER(PsvShots), C.POINTER(PsvOptions),
                                  C.POINTER(C.c_void_p)]),
    "psv_plan_destroy": (C.c_int, [C.c_void_p]),
    "psv_plan_device_bytes": (C.c_longlong, [C.c_void_p]),
    "psv_plan_set_model": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "psv_plan_get_model": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "psv_plan_set_observed": (C.c_int, [C.c_void_p, _dp, _dp]),
    "psv_forward": (C.c_int, [C.c_void_p, _dp, _dp]),
    "psv_gradient": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp]),
    "psv_reset_gradient": (C.c_int, [C.c_void_p]),
    "psv_get_gradient": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "psv_set_gradient": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "psv_get_shot_gradient": (C.c_int, [C.c_void_p, C.c_int] + [_dp] * 8),
    "psv_fwi_iteration": (C.c_int, [C.c_void_p, _dp, _dp, _ip, _dp, C.c_int]),
    "psv_last_timing": (C.c_int, [C.c_void_p, _dp]),
    "psv_save_model": (C.c_int, [C.c_void_p]),
    "psv_taper_gradient": (C.c_int, [C.c_void_p]),
    "psv_trial_misfit": (C.c_int, [C.c_void_p, C.c_double, _dp]),
    "psv_update_model": (C.c_int, [C.c_void_p, C.c_double]),
    "psv_misfit": (C.c_int, [_dp] * 6 + [C.c_int, C.c_int, C.c_int, C.c_double, _dp]),
    "psv_misfit_noalloc": (C.c_int, [C.c_void_p] * 6 + [C.c_int, C.c_int, C.c_int, C.c_double,
                                                          C.c_void_p, C.c_void_p]),
    "psv_plan_stream": (C.c_void_p, [C.c_void_p]),
    "psv_plan_kernel_launches": (C.c_longlong, [C.c_void_p]),
    "psv_profile_kernels": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "psv_plan_autotune": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip, _ip]),
    "psv_plan_shape": (C.c_int, [C.c_void_p, _ip, _ip, _ip]),
    "psv_plan_storage": (C.c_int, [C.c_void_p, _ip, _ip, _ip, C.POINTER(C.c_longlong)]),
    "psv_plan_chains": (C.c_int, [C.c_void_p, _ip]),
    "psv_gauss_filter_kernel": (C.c_int, [C.c_int, _dp]),
    "psv_apply_gauss_filter": (C.c_int, [_dp, C.c_int, C.c_int, C.c_int]),
    "psv_PCG_PSV": (C.c_int, [_dp, _dp, _dp, C.c_int, C.c_int]),
    "psv_pcg_gradient": (C.c_int, [C.c_void_p]),
    "psv_checkpoint_schedule": (C.c_int, [C.c_int, C.c_int, _ip, C.c_int, _ip,
                                          C.POINTER(C.c_longlong)]),
    "psv_multi_forward": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(_dp), C.POINTER(_dp)]),
    "psv_multi_gradient": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, _dp]),
    "psv_joint_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int,
                                   C.POINTER(C.c_void_p)]),
    "psv_joint_forward": (C.c_int, [C.c_void_p, C.POINTER(_dp), C.POINTER(_dp), _dp]),
    "psv_joint_gradient": (C.c_int, [C.c_void_p, _dp, _dp]),
    "psv_joint_launches": (C.c_longlong, [C.c_void_p]),
    "psv_joint_shape": (C.c_int, [C.c_void_p, _ip, _ip]),
    "psv_joint_destroy": (C.c_int, [C.c_void_p]),
    "psv_step_length": (C.c_int, [_dp, C.c_double, C.c_void_p, C.c_void_p, _ip, _dp, C.c_int]),
    "psv_calc_opt_step": (C.c_double, [_dp, _dp]),
    "psv_kernel_PSV": (C.c_int,
                       [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                        C.c_int, _ip, _dp, C.c_int]
                       + [_dp] * 8 + [_dp] * 4 + [_dp] * 5
                       + [C.c_int, _dp, _dp, _dp]
                       + [C.c_int] + [_dp] * 6 + [C.c_int] + [_dp] * 6
                       + [_dp] * 8
                       + [C.c_int, C.c_int, _dp, _dp, _ip, _ip, _ip]
                       + [C.c_int, C.c_int, _dp, _dp, _ip, _ip]
                       + [C.c_int] + [_dp] * 5
                       + [C.c_int] * 7 + [C.c_int, C.c_int]),
    "psv_simulate_PSV": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(PsvOptions)]),
}

TRIAL_FN = C.CFUNCTYPE(C.c_int, C.c_double, _dp, C.c_void_p)

_lib = None


def lib() -> C.CDLL:
    """Load (building first when needed) the engine library."""
    global _lib
    if _lib is None:
        path = LIB
        if not os.path.exists(path):
            path = build()
        _lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib


def check(status: int) -> None:
    if status != PSV_OK:
        raise PSVError(status, lib().psv_last_error().decode())


def device_available() -> bool:
    return bool(lib().psv_device_available())


def dptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


def iptr(a):
    return None if a is None else a.ctypes.data_as(_ip)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)
