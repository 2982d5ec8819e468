"""ctypes mirror of `aeros_params` (include/aeros_gpu.h) and its defaults.

Pure Python, no library load: the CPU test harness uses the same structure.
Defaults are the Held-Suarez benchmark configuration of par/held_suarez.nml
(src/physics/aeros_held_suarez.f90:92-101 for the forcing constants).
"""
import ctypes

PREC_FP64 = 0
PREC_SPLIT = 1


class AerosParams(ctypes.Structure):
    _fields_ = [
        ("trunc", ctypes.c_int),
        ("nlon", ctypes.c_int),
        ("nlat", ctypes.c_int),
        ("nlev", ctypes.c_int),
        ("nmember", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("dt", ctypes.c_double),
        ("eps_filter", ctypes.c_double),
        ("raw_alpha", ctypes.c_double),
        ("si_alpha", ctypes.c_double),
        ("tau_diff", ctypes.c_double),
        ("ndiff", ctypes.c_int),
        ("semi_implicit", ctypes.c_int),
        ("held_suarez", ctypes.c_int),
        ("mass_fixer", ctypes.c_int),
        ("stretch_a", ctypes.c_double),
        ("stretch_r", ctypes.c_double),
        ("sigma_t", ctypes.c_double),
        ("p_top", ctypes.c_double),
        ("ps_ref", ctypes.c_double),
        ("t_ref", ctypes.c_double),
        ("hs_t_equator", ctypes.c_double),
        ("hs_t_min", ctypes.c_double),
        ("hs_dt_y", ctypes.c_double),
        ("hs_dtheta_z", ctypes.c_double),
        ("hs_sigma_b", ctypes.c_double),
        ("hs_p0", ctypes.c_double),
        ("hs_k_a", ctypes.c_double),
        ("hs_k_s", ctypes.c_double),
        ("hs_k_f", ctypes.c_double),
    ]


def held_suarez_params(trunc=31, nlev=20, **overrides) -> AerosParams:
    """The Held-Suarez configuration (par/held_suarez.nml), with overrides."""
    p = AerosParams()
    p.trunc = trunc
    p.nlon = -1
    p.nlat = -1
    p.nlev = nlev
    p.nmember = 1
    p.precision = PREC_FP64
    p.dt = 1800.0
    p.eps_filter = 0.06
    p.raw_alpha = 0.53
    p.si_alpha = 0.5
    p.tau_diff = 6.0
    p.ndiff = 6
    p.semi_implicit = 1
    p.held_suarez = 1
    p.mass_fixer = 1
    p.stretch_a = 1.0
    p.stretch_r = 2.0
    p.sigma_t = 0.0
    p.p_top = 1000.0
    p.ps_ref = 1.0e5
    p.t_ref = 300.0
    p.hs_t_equator = 315.0
    p.hs_t_min = 200.0
    p.hs_dt_y = 60.0
    p.hs_dtheta_z = 10.0
    p.hs_sigma_b = 0.7
    p.hs_p0 = 1.0e5
    p.hs_k_a = 1.0 / (40.0 * 86400.0)
    p.hs_k_s = 1.0 / (4.0 * 86400.0)
    p.hs_k_f = 1.0 / 86400.0
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p
