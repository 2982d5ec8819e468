"""ctypes binding of include/aeros_gpu.h (libaeros_gb300.so).

There is no fallback: if the shared library is missing or cannot be loaded,
importing this module raises.  Build it with `python -m aeros_gb300.build`
(or `__graft_entry__.build()`).
"""
import ctypes
import os

from .params import AerosParams

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libaeros_gb300.so")

OK = 0
ERR_ARG = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_SINGULAR = -4
ERR_NONFINITE = -5
ERR_STATE = -6
ERR_UNSUPPORTED = -7

_ERRNAMES = {ERR_ARG: "AEROS_ERR_ARG", ERR_CUDA: "AEROS_ERR_CUDA", ERR_NOMEM: "AEROS_ERR_NOMEM",
             ERR_SINGULAR: "AEROS_ERR_SINGULAR", ERR_NONFINITE: "AEROS_ERR_NONFINITE",
             ERR_STATE: "AEROS_ERR_STATE", ERR_UNSUPPORTED: "AEROS_ERR_UNSUPPORTED"}


class AerosError(RuntimeError):
    def __init__(self, code, where):
        self.code = code
        msg = f"{where} failed: {_ERRNAMES.get(code, code)}"
        try:
            detail = lib().aeros_last_error()
            if detail:
                msg += f" ({detail.decode()})"
        except Exception:
            pass
        super().__init__(msg)


_lib = None


class AerosRelaxation(ctypes.Structure):
    """aeros_relaxation: user data of the ready-made aeros_physics_relaxation hook."""
    _fields_ = [("k_drag", ctypes.c_double), ("k_temp", ctypes.c_double), ("t_ref", ctypes.c_double)]


_vp = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)
_i = ctypes.c_int
_d = ctypes.c_double

# name -> argtypes (all return int unless listed in _RESTYPE)
_PROTOS = {
    "aeros_sht_grid_size": [_i, _ip, _ip],
    "aeros_sht_create": [ctypes.POINTER(_vp), _i, _i, _i, _i],
    "aeros_sht_destroy": [_vp],
    "aeros_sht_info": [_vp, _ip, _ip, _ip, _ip, _vp, _vp, _vp, _vp],
    "aeros_sht_lm": [_vp, _i, _i],
    "aeros_sht_set_precision": [_vp, _i],
    "aeros_sht_set_stream": [_vp, _vp],
    "aeros_sht_synthesis": [_vp, _vp, _vp, _i],
    "aeros_sht_analysis": [_vp, _vp, _vp, _i],
    "aeros_sht_synthesis_vec": [_vp, _vp, _vp, _vp, _vp, _i],
    "aeros_sht_analysis_vec": [_vp, _vp, _vp, _vp, _vp, _i],
    "aeros_sht_gradient": [_vp, _vp, _vp, _vp, _i],
    "aeros_sht_laplacian": [_vp, _vp, _i, _i],
    "aeros_sht_surface_integral": [_vp, _vp, _vp, _i],
    "aeros_uv_from_vordiv": [_vp, _vp, _vp, _vp, _vp, _i],
    "aeros_vordiv_from_uv": [_vp, _vp, _vp, _vp, _vp, _i],
    "aeros_gradient": [_vp, _vp, _vp, _vp, _i],
    "aeros_sht_launch_count": [_vp, ctypes.POINTER(ctypes.c_longlong)],
    "aeros_sht_synthesis_noalloc": [_vp, _vp, _vp, _i],
    "aeros_params_default": [ctypes.POINTER(AerosParams)],
    "aeros_dyn_create": [ctypes.POINTER(_vp), ctypes.POINTER(AerosParams), _vp, _vp],
    "aeros_dyn_destroy": [_vp],
    "aeros_dyn_info": [_vp, _ip, _ip, _ip, _ip, _vp, _vp, _vp, _vp, _vp],
    "aeros_dyn_set_member_forcing": [_vp, _i, _d, _d],
    "aeros_dyn_set_state": [_vp, _vp, _vp, _vp, _vp],
    "aeros_dyn_get_state": [_vp, _vp, _vp, _vp, _vp],
    "aeros_dyn_set_old_state": [_vp, _vp, _vp, _vp, _vp, _i],
    "aeros_dyn_get_old_state": [_vp, _vp, _vp, _vp, _vp],
    "aeros_dyn_set_isothermal": [_vp, _d, _d],
    "aeros_dyn_set_phis": [_vp, _vp],
    "aeros_dyn_hs_perturb": [_vp, _d],
    "aeros_dyn_step": [_vp, _i],
    "aeros_dyn_set_time": [_vp, _d],
    "aeros_dyn_update": [_vp, _d],
    "aeros_dyn_get_time": [_vp, _vp, _vp],
    "aeros_dyn_step_async": [_vp, _i],
    "aeros_dyn_step_packed": [_vp, _vp, _vp, _i, _i, _vp, _vp],
    "aeros_host_register": [_vp, ctypes.c_size_t],
    "aeros_host_unregister": [_vp],
    "aeros_dyn_sync": [_vp],
    "aeros_dyn_profile_step": [_vp, _i, _vp, _vp, _i, _ip],
    "aeros_dyn_tendency": [_vp, _vp, _vp, _vp, _vp],
    "aeros_dyn_tendency_forced": [_vp, _vp, _vp, _vp, _vp],
    "aeros_dyn_set_physics": [_vp, _vp, _vp],
    "aeros_physics_relaxation": [_vp, _vp, _vp],
    "aeros_dyn_diagnose": [_vp, _vp, _vp, _vp, _vp],
    "aeros_dyn_budget": [_vp, _vp, _vp, _vp],
    "aeros_dyn_counters": [_vp, _ip, _dp, _dp, _dp],
    "aeros_dyn_set_mass_target": [_vp, _d],
    "aeros_dyn_member_counters": [_vp, _i, _dp, _dp, _dp],
    "aeros_dyn_set_member_counters": [_vp, _i, _d, _d, _d],
    "aeros_dyn_diag_accumulate": [_vp],
    "aeros_dyn_diag_read": [_vp, _i, _vp, _ip],
    "aeros_dyn_gwspeed": [_vp, _dp],
    "aeros_dyn_set_stream": [_vp, _vp],
    "aeros_dyn_launch_count": [_vp, ctypes.POINTER(ctypes.c_longlong)],
    "aeros_group_create": [ctypes.POINTER(_vp), ctypes.POINTER(_vp), _i],
    "aeros_group_destroy": [_vp],
    "aeros_group_set_stream": [_vp, _vp],
    "aeros_group_step": [_vp, _i],
    "aeros_group_step_async": [_vp, _i],
    "aeros_group_sync": [_vp],
    "aeros_group_launch_count": [_vp, ctypes.POINTER(ctypes.c_longlong)],
    "aeros_group_info": [_vp, ctypes.POINTER(_i), ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)],
    "aeros_sht_synthesis_ad": [_vp, _vp, _vp, _i],
    "aeros_sht_analysis_ad": [_vp, _vp, _vp, _i],
    "aeros_sht_synthesis_vec_ad": [_vp, _vp, _vp, _vp, _vp, _i],
    "aeros_sht_analysis_vec_ad": [_vp, _vp, _vp, _vp, _vp, _i],
    "aeros_dyn_state_size": [_vp, ctypes.POINTER(ctypes.c_longlong)],
    "aeros_dyn_step_ad": [_vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "aeros_dyn_window_forward": [_vp, _i, _i, _vp],
    "aeros_dyn_window_backward": [_vp, _vp, _vp, _vp, _vp],
    "aeros_dyn_autotune": [_vp, _i, _dp, _dp],
    "aeros_dyn_tune_get": [_vp, _vp, _i],
    "aeros_dyn_tune_set": [_vp, _vp, _i],
    "aeros_transport_create": [ctypes.POINTER(_vp), _i, _i, _vp, _vp],
    "aeros_transport_destroy": [_vp],
    "aeros_transport_set_stream": [_vp, _vp],
    "aeros_transport_grid": [_vp, _ip, _ip, _ip],
    "aeros_transport_set_vert_vanleer": [_vp, _i],
    "aeros_transport_step": [_vp, _vp, _vp, _vp, _vp, _d],
    "aeros_transport_last": [_vp, _dp, _ip],
    "aeros_transport_water": [_vp, _vp, _vp, _dp],
    "aeros_last_error": [],
}
_RESTYPE = {"aeros_last_error": ctypes.c_char_p}


def lib():
    """Load the library (raises if it is not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built; run python -m aeros_gb300.build")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _PROTOS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, ctypes.c_int)
        _lib = L
    return _lib


def check(rc, where):
    if rc != OK:
        raise AerosError(rc, where)
    return rc


def exported_symbols():
    return list(_PROTOS)
