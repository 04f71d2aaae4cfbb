"""ctypes binding of libigsolve.so (C-ABI in include/igsolve.h).

The library is the only compute path: there is no CPU fallback.  If the
shared object is missing, or no CUDA device is visible, the solver entry
points raise instead of computing anything.
"""
import ctypes
import os
import threading

import numpy as np

from ion_gym_gb300.build import LIB as LIB_PATH

IG_OK = 0
IG_NOT_CONVERGED = 1
IG_STAGNATED = 2
IG_CYCLE_CAP = 3
IG_INTERRUPTED = 4
IG_BAD_ARG = 5
IG_CUDA_ERROR = 6
IG_NO_DEVICE = 7

_p = ctypes.c_void_p
_d = ctypes.c_double
_l = ctypes.c_long
_i = ctypes.c_int
_ll = ctypes.c_longlong
_pl = ctypes.POINTER(ctypes.c_long)
_pd = ctypes.POINTER(ctypes.c_double)
_pi = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes); must match include/igsolve.h
SIGNATURES = {
    "ig_last_error": (ctypes.c_char_p, []),
    "ig_abi_version": (_i, []),
    "ig_device_count": (_i, []),
    "ig_request_stop": (None, []),
    "ig_clear_stop": (None, []),
    "ig_stop_requested": (_i, []),
    "ig_solve3d": (_i, [_p, _p, _p, _l, _l, _l, _d, _l, _d, _p, _i, _p, _pl,
                        _pd]),
    "ig_solve3d_mg": (_i, [_p, _p, _p, _l, _l, _l, _d, _l, _i, _i, _i, _d,
                           _p, _i, _p, _pl, _pd]),
    "ig_solve3d_vmg": (_i, [_p, _p, _p, _l, _l, _l, _d, _i, _i, _i, _i, _p,
                            _i, _d, _p, _pl, _pd, _pi, _pd]),
    "ig_solve_basis_vmg": (_i, [_p, _p, _d, _p, _l, _l, _l, _d, _i, _i, _i,
                                _i, _d, _p, _pl, _pd, _pi, _pd]),
    "ig_solve_basis_sor": (_i, [_p, _p, _d, _p, _l, _l, _l, _d, _l, _d, _i,
                                _p, _pl, _pd]),
    "ig_cascadic_relres": (_i, [_p, _p, _l, _l, _l, _d, _l, _i, _i, _d, _p,
                                _i, _i, _p, _pl, _pd, _pl, _pi]),
    "ig_sweep_dev": (_i, [_p, _p, _p, _l, _l, _l, _d, _i, _i, _pd, _p]),
    "ig_residual_dev": (_i, [_p, _p, _p, _l, _l, _l, _i, _p, _p]),
    "ig_sweep_rhs_dev": (_i, [_p, _p, _p, _l, _l, _l, _d, _i, _pd, _p]),
    "ig_residual_rhs_dev": (_i, [_p, _p, _p, _l, _l, _l, _p, _p]),
    "ig_restrict_fw_dev": (_i, [_p, _l, _l, _l, _p, _p]),
    "ig_prolong_add_dev": (_i, [_p, _l, _l, _l, _p, _p, _l, _l, _l, _p]),
    "ig_prolongate_dev": (_i, [_p, _l, _l, _l, _p, _l, _l, _l, _p]),
    "ig_coarsen_fixed_any_dev": (_i, [_p, _l, _l, _l, _p, _p]),
    "ig_coarsen_mask_dev": (_i, [_p, _p, _l, _l, _l, _p, _p, _p]),
    "ig_residual_audit_dev": (_i, [_p, _p, _p, _l, _l, _l, _p, _p]),
    "ig_err_sweep_dev": (_i, [_p, _p, _p, _p, _l, _l, _l, _d, _i, _pd, _p]),
    "ig_prof_enable": (None, [_i]),
    "ig_prof_reset": (None, []),
    "ig_prof_read": (None, [_pd, _pl, _pl]),
    "ig_launch_count": (_l, []),
    "ig_mixed_bases": (_i, [_p, _p, _i, _d, _l, _l, _l, _i, _d, _i, _i, _i,
                            _i, _p, _pi, _p]),
    "ig_mixed_bytes": (_l, [_l, _l, _l, _i]),
    "ig_mixed_launch_count": (_l, []),
    "ig_mixed_open": (_i, [_p, _l, _l, _l, _i, _i, _i, _i, _i,
                           ctypes.POINTER(ctypes.c_void_p)]),
    "ig_mixed_open_ex": (_i, [_p, _l, _l, _l, _i, _i, _i, _i, _i, _i, _i,
                              _d, _i, _i, ctypes.POINTER(ctypes.c_void_p)]),
    "ig_mixed_solve_bases": (_i, [_p, _p, _i, _d, _d, _i, _p, _pi, _p]),
    "ig_mixed_solve_unit_bases": (_i, [_p, _p, _i, _d, _d, _i, _p, _pi, _p]),
    "ig_mixed_solve_values": (_i, [_p, _p, _i, _d, _i, _p, _pi, _p]),
    "ig_mixed_close": (None, [_p]),
    "ig_rasterize": (_i, [_p, _i, _p, _i, _l, _l, _l, _p, _p, _p, _p]),
    "ig_theta_scene": (_i, [_p, _i, _p, _l, _l, _l, _i, _i, _p]),
    "ig_shape_xsection": (_i, [_i, _p, _i, _p, _i, _p, _l, _p, _l, _p]),
    "ig_shapes_label": (_i, [_p, _i, _p, _ll, _p, _ll, _p, _i, _l, _l, _l, _p,
                             _p, _p, _p]),
    "ig_device_free_bytes": (_ll, []),
    "ig_unit_bases_dev": (_i, [_p, _ll, _d, _p, _p]),
    "ig_superpose_dev": (_i, [_p, _i, _i, _p, _p, _ll, _p, _ll, _p]),
    "ig_field_aware_dev": (_i, [_p, _i, _ll, _i, _p, _l, _l, _l, _d, _i, _p,
                                _p, _p, _ll, _p]),
    "ig_field_aware_3d": (_i, [_p, _i, _p, _l, _l, _l, _d, _i, _p, _p, _p]),
    "ig_field_check_division": (_i, [_d, ctypes.c_ulonglong, ctypes.c_uint,
                                     _p]),
    "ig_compose_fields": (_i, [_p, _i, _i, _p, _i, _p, _p, _p, _l, _l, _l,
                               _d, _i, _p, _p, _p, _p]),
    "ig_mixed_time_gs": (_i, [_p, _i, _i, _pd, _pd]),
    "ig_mixed_step_bytes": (_i, [_p, _i, _pd]),
    "ig_mixed_rebind": (_i, [_p, _p, _l, _l, _l]),
    "ig_mixed_open_multi": (_i, [_p, _i, _l, _l, _l, _i, _i, _i, _i, _i, _i,
                                 _d, _i, _i, ctypes.POINTER(ctypes.c_void_p)]),
    "ig_mixed_bytes_multi": (_l, [_l, _l, _l, _i]),
    "ig_mixed_solve_values_acc": (_i, [_p, _p, _i, _p, _i, _p, _pi, _p]),
    "ig_mixed_check_fused": (_i, [_p, _i, ctypes.POINTER(ctypes.c_longlong)]),
    "ig_mixed_solve_bytes": (_i, [_p, ctypes.POINTER(ctypes.c_double)]),
    "ig_mixed_set_cycle": (_i, [_p, _i, _i, _i]),
    "ig_mixed_tuning": (_i, [_p, _i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                             ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]),
    "ig_mixed_check_convert": (_i, [_p, ctypes.c_long, ctypes.POINTER(ctypes.c_longlong)]),
    "ig_cascadic_relres_noalloc": (_i, [_p, _p, _l, _l, _l, _d, _l, _i, _i,
                                        _d, _p, _i, _i, _p, _pl, _pd, _pl,
                                        _pi, _p]),
}

_lib = None
_lock = threading.Lock()


class LibraryMissing(RuntimeError):
    """libigsolve.so is not built (or cannot be loaded)."""


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise LibraryMissing(
                    f"{LIB_PATH} is not built; run ion_gym_gb300.build.build() "
                    f"(or __graft_entry__.build()) on a machine with nvcc")
            try:
                L = ctypes.CDLL(LIB_PATH)
            except OSError as e:
                raise LibraryMissing(f"cannot load {LIB_PATH}: {e}") from e
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def last_error():
    m = lib().ig_last_error()
    return m.decode() if m else ""


def require_device():
    if lib().ig_device_count() < 1:
        raise RuntimeError("ion_gym_gb300: no CUDA device is visible; the "
                           "field solve runs only on the GPU")


def ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def as_mask(a):
    return np.ascontiguousarray(a, dtype=bool).view(np.uint8)


def as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def as_f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def check(status, what):
    """Map hard failures to exceptions; solver outcomes (not converged,
    stagnated, interrupted) are returned for the caller to word."""
    if status in (IG_BAD_ARG,):
        raise ValueError(f"{what}: {last_error()}")
    if status == IG_NO_DEVICE:
        raise RuntimeError(f"{what}: no CUDA device is visible")
    if status == IG_CUDA_ERROR:
        raise RuntimeError(f"{what}: CUDA error: {last_error()}")
    return status
