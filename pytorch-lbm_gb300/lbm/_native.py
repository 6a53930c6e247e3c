"""ctypes binding of liblbm_gb300.so (the C ABI in include/lbm_gb300.h).

The library is built in-tree (``lbm/_build.py``) and loaded once.  There is no
fallback: if the shared library is missing or fails to load, every solver
entry point raises.
"""
import ctypes
import os
import threading

import torch  # noqa: F401  (loads the CUDA runtime the library links against)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liblbm_gb300.so")

LBM_F32, LBM_F64, LBM_F16 = 0, 1, 2
LBM_DT_NONE, LBM_DT_F32, LBM_DT_F64 = 0, 1, 2
FIELD_PHI, FIELD_RHO, FIELD_U, FIELD_P, FIELD_PRESS, FIELD_MU = 1, 2, 4, 8, 16, 32
STATUS_NAN, STATUS_MASS_LOW = 1, 2
IFACE_ALLEN_CAHN, IFACE_CAHN_HILLIARD = 0, 1

# every exported entry point declared in include/lbm_gb300.h
EXPORTS = (
    "lbm_create", "lbm_destroy", "lbm_set_geometry", "lbm_set_geometry_device", "lbm_init_fields", "lbm_step", "lbm_step_profiled",
    "lbm_get_fields", "lbm_get_populations", "lbm_get_geometry", "lbm_geometry_host",
    "lbm_get_scalars", "lbm_measure", "lbm_status", "lbm_last_error", "lbm_version",
    "lbm_set_tile", "lbm_get_tile", "lbm_set_layout", "lbm_get_layout", "lbm_autotune", "lbm_measure_static",
    "lbm_footprint",
    "lbm_batch_create", "lbm_batch_step", "lbm_batch_size", "lbm_batch_autotune", "lbm_batch_destroy",
    "lbm_set_launch", "lbm_get_launch", "lbm_batch_get_launch", "lbm_batch_set_cooperative",
    "lbm_cache_limit", "lbm_cache_trim", "lbm_cache_bytes",
    "lbm_inject_droplet", "lbm_set_amplification", "lbm_state_bytes", "lbm_save_state", "lbm_load_state",
    "lbm_write_vtk", "lbm_reduce",
)


class LbmParams(ctypes.Structure):
    _fields_ = [
        ("rho_l", ctypes.c_double), ("rho_g", ctypes.c_double), ("sigma", ctypes.c_double),
        ("xi", ctypes.c_double), ("beta", ctypes.c_double), ("kappa", ctypes.c_double),
        ("phi_c", ctypes.c_double), ("tau_l", ctypes.c_double), ("tau_g", ctypes.c_double),
        ("tau_h", ctypes.c_double), ("theta_eq", ctypes.c_double),
        ("g_force", ctypes.c_double * 3), ("boundary_relax", ctypes.c_double),
        ("sharpen_reduce", ctypes.c_double), ("mu_wall_scale", ctypes.c_double),
        ("geo_amplification", ctypes.c_double), ("ac_scale", ctypes.c_double),
        ("ghost_scale", ctypes.c_double), ("stab_mode", ctypes.c_int32),
        ("geometric_wetting", ctypes.c_int32), ("interface_mode", ctypes.c_int32),
        ("direct_wetting", ctypes.c_int32), ("mu_drive", ctypes.c_double),
    ]


_lib = None
_lock = threading.Lock()
_vp, _i64, _i32, _u32, _dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_uint32, ctypes.c_double


def _declare(L):
    sig = {
        "lbm_create": ([ctypes.POINTER(LbmParams), _i64, _i64, _i64, _i32, ctypes.POINTER(_vp)], _i32),
        "lbm_destroy": ([_vp], _i32),
        "lbm_set_geometry": ([_vp, _vp, _vp, _i32], _i32),
        "lbm_set_geometry_device": ([_vp, _vp, _vp, _i32, _vp], _i32),
        "lbm_init_fields": ([_vp, _vp, _vp, _i32, _i32, _vp], _i32),
        "lbm_step": ([_vp, _i32, _vp], _i32),
        "lbm_step_profiled": ([_vp, _i32, _vp, ctypes.POINTER(ctypes.c_float)], _i32),
        "lbm_get_fields": ([_vp, _u32, _vp, _vp, _vp, _vp, _vp, _vp, _vp], _i32),
        "lbm_get_populations": ([_vp, _vp, _vp, _vp], _i32),
        "lbm_get_geometry": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp], _i32),
        "lbm_geometry_host": ([_i64, _i64, _i64, _vp, _vp, _i32, _dbl, _dbl, _i32,
                               _vp, _vp, _vp, _vp, _vp, _vp], _i32),
        "lbm_get_scalars": ([_vp, ctypes.POINTER(_dbl), ctypes.POINTER(_dbl), ctypes.POINTER(_dbl),
                             ctypes.POINTER(_i64)], _i32),
        "lbm_measure": ([_vp, ctypes.POINTER(_dbl), _vp], _i32),
        "lbm_measure_static": ([_i64, _i64, _i64, _vp, _i32, _vp, _vp, _vp], _i32),
        "lbm_footprint": ([_i64, _i64, _i64, _i32, ctypes.POINTER(_i64)], _i32),
        "lbm_batch_create": ([ctypes.POINTER(_vp), _i32, ctypes.POINTER(_vp)], _i32),
        "lbm_batch_step": ([_vp, _i32, _vp], _i32),
        "lbm_batch_size": ([_vp, ctypes.POINTER(ctypes.c_int)], _i32),
        "lbm_batch_autotune": ([_vp, _i32, _vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)], _i32),
        "lbm_batch_destroy": ([_vp], _i32),
        "lbm_set_launch": ([_vp, _i32, _i32], _i32),
        "lbm_get_launch": ([_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)], _i32),
        "lbm_batch_get_launch": ([_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)], _i32),
        "lbm_batch_set_cooperative": ([_vp, _i32], _i32),
        "lbm_cache_limit": ([ctypes.c_uint64], _i32),
        "lbm_cache_trim": ([_vp], _i32),
        "lbm_cache_bytes": ([_vp], _i32),
        "lbm_inject_droplet": ([_vp, ctypes.POINTER(_dbl), _dbl, _dbl, ctypes.POINTER(_dbl), ctypes.POINTER(_i64),
                                _vp], _i32),
        "lbm_set_amplification": ([_vp, _vp, _i32], _i32),
        "lbm_state_bytes": ([_vp, ctypes.POINTER(_i64)], _i32),
        "lbm_save_state": ([_vp, _vp, _i64, _vp], _i32),
        "lbm_load_state": ([_vp, _vp, _i64, _vp], _i32),
        "lbm_write_vtk": ([ctypes.c_char_p, ctypes.c_char_p, _i64, _vp, _vp, _vp, _vp, _vp], _i32),
        "lbm_reduce": ([_vp, ctypes.POINTER(_dbl), ctypes.POINTER(_dbl), ctypes.POINTER(ctypes.c_int32),
                        ctypes.POINTER(ctypes.c_float), _vp], _i32),
        "lbm_status": ([_vp, ctypes.POINTER(_u32)], _i32),
        "lbm_set_tile": ([_vp, _i32, _i32, _i32], _i32),
        "lbm_set_layout": ([_vp, _i32], _i32),
        "lbm_get_layout": ([_vp, ctypes.POINTER(ctypes.c_int)], _i32),
        "lbm_get_tile": ([_vp, ctypes.POINTER(ctypes.c_int)], _i32),
        "lbm_autotune": ([_vp, _i32, _vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)], _i32),
        "lbm_last_error": ([], ctypes.c_char_p),
        "lbm_version": ([], ctypes.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res


def lib():
    """The loaded library (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise RuntimeError(
                        f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
                        "g.build()\"` (the solver has no CPU fallback)")
                L = ctypes.CDLL(LIB_PATH)
                _declare(L)
                _lib = L
    return _lib


class LbmError(RuntimeError):
    pass


def check(rc, what):
    if rc != 0:
        msg = lib().lbm_last_error().decode(errors="replace")
        raise LbmError(f"{what} failed ({rc}): {msg}")


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def cache_limit(nbytes):
    """Limit of the library's cache of grid state arrays (0 disables it)."""
    check(lib().lbm_cache_limit(int(nbytes)), "lbm_cache_limit")


def cache_trim():
    """Free every cached state array; returns the bytes freed."""
    n = ctypes.c_uint64()
    check(lib().lbm_cache_trim(ctypes.byref(n)), "lbm_cache_trim")
    return int(n.value)


def cache_bytes():
    """Bytes of device memory the cache holds."""
    n = ctypes.c_uint64()
    check(lib().lbm_cache_bytes(ctypes.byref(n)), "lbm_cache_bytes")
    return int(n.value)
