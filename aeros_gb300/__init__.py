"""aeros_gb300 -- GB300-native (sm_103a) spectral dynamics path of aeros.

The compute path is the C-ABI library aeros_gb300/_lib/libaeros_gb300.so
(include/aeros_gpu.h).  This package is its Python mirror:
  spectral.AerosSHT   -- aeros_spectral transforms (scalar, vector, gradient, ...)
  dynamics.AerosDyn   -- aeros_timestep dry step (Held-Suarez), ensembles
  params              -- aeros_params and the Held-Suarez defaults
There is no CPU fallback: the classes raise if the library is not built or
no GPU is present.
"""
from .params import AerosParams, held_suarez_params, PREC_FP64, PREC_SPLIT

__all__ = ["AerosParams", "held_suarez_params", "PREC_FP64", "PREC_SPLIT", "AerosSHT", "AerosDyn", "grid_size"]


def __getattr__(name):
    if name in ("AerosSHT", "grid_size"):
        from . import spectral
        return getattr(spectral, name)
    if name == "AerosDyn":
        from .dynamics import AerosDyn
        return AerosDyn
    raise AttributeError(name)
