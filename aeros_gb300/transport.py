"""Python mirror of the tracer transport C-ABI (aeros_transport_*), the GPU
replacement of src/dynamics/aeros_transport.f90.

Arrays are numpy (host) or torch CUDA tensors (device, used in place):
u, v, q (nlev, nlat, nlon) and lnps, ps (nlat, nlon) -- the Fortran
(nlon, nlat, nlev) grids in C order, latitude north to south.
"""
import ctypes

import numpy as np

from . import _capi
from .spectral import _is_torch, _ptr


class AerosTransport:
    """aeros_transport_class: one Gaussian grid, nlev layers with p_half = a_half + b_half ps."""

    def __init__(self, trunc, a_half, b_half, vert_vanleer=False):
        a = np.ascontiguousarray(a_half, dtype=np.float64)
        b = np.ascontiguousarray(b_half, dtype=np.float64)
        if a.shape != b.shape or a.ndim != 1 or len(a) < 2:
            raise ValueError("a_half and b_half must be (nlev + 1,) arrays")
        h = ctypes.c_void_p()
        _capi.check(_capi.lib().aeros_transport_create(ctypes.byref(h), int(trunc), len(a) - 1, _ptr(a), _ptr(b)),
                    "aeros_transport_create")
        self._h = h
        n1, n2, n3 = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _capi.lib().aeros_transport_grid(h, ctypes.byref(n1), ctypes.byref(n2), ctypes.byref(n3))
        self.nlon, self.nlat, self.nlev = n1.value, n2.value, n3.value
        if vert_vanleer:
            _capi.check(_capi.lib().aeros_transport_set_vert_vanleer(h, 1), "aeros_transport_set_vert_vanleer")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _capi.lib().aeros_transport_destroy(h)
            self._h = None

    def _chk(self, x, shape, name):
        if tuple(x.shape) != shape:
            raise ValueError(f"{name} has shape {tuple(x.shape)}, expected {shape}")
        if _is_torch(x):
            import torch
            if x.dtype != torch.float64 or not x.is_contiguous():
                raise ValueError(f"{name} must be a contiguous float64 tensor")
            if x.is_cuda:
                _capi.check(_capi.lib().aeros_transport_set_stream(
                    self._h, ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)),
                    "aeros_transport_set_stream")
            return x
        return np.ascontiguousarray(x, dtype=np.float64)

    def step(self, u, v, lnps, q, dt):
        """aeros_transport_transport: advance q over dt [s]; returns q (updated in place
        for a contiguous float64 array or tensor)."""
        s3, s2 = (self.nlev, self.nlat, self.nlon), (self.nlat, self.nlon)
        u, v, lnps = self._chk(u, s3, "u"), self._chk(v, s3, "v"), self._chk(lnps, s2, "lnps")
        qq = self._chk(q, s3, "q")
        _capi.check(_capi.lib().aeros_transport_step(self._h, _ptr(u), _ptr(v), _ptr(lnps), _ptr(qq), float(dt)),
                    "aeros_transport_step")
        return qq

    def last(self):
        """(last_cfl, last_nsub) of the previous step."""
        c, n = ctypes.c_double(), ctypes.c_int()
        _capi.check(_capi.lib().aeros_transport_last(self._h, ctypes.byref(c), ctypes.byref(n)), "aeros_transport_last")
        return c.value, n.value

    def water(self, ps, q):
        """aeros_transport_water: total tracer mass [kg]."""
        ps = self._chk(ps, (self.nlat, self.nlon), "ps")
        q = self._chk(q, (self.nlev, self.nlat, self.nlon), "q")
        w = ctypes.c_double()
        _capi.check(_capi.lib().aeros_transport_water(self._h, _ptr(ps), _ptr(q), ctypes.byref(w)),
                    "aeros_transport_water")
        return w.value
