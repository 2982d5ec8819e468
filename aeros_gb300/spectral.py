"""Python mirror of aeros' spectral transform module on the GPU library.

`AerosSHT` plays the role of `aeros_sht_class` (src/aeros_spectral.f90:47-85)
with the same operations (aeros_sht_synthesis, aeros_sht_analysis, the vector
pair, the gradient, the Laplacian, the surface integral) plus the wind helpers
of aeros_vordiv (src/dynamics/aeros_vordiv.f90:82-205).

Arrays: numpy (host) or torch CUDA tensors (device, used in place).  Spectral
fields are complex128 shaped (..., nlm); grid fields float64 (..., nlat, nlon),
i.e. the reference's Fortran (nlon, nlat, ...) layout.
"""
import ctypes

import numpy as np

from . import _capi
from .params import PREC_FP64, PREC_SPLIT

try:  # torch is optional plumbing for device arrays
    import torch
except Exception:  # pragma: no cover
    torch = None


def _ptr(a):
    if torch is not None and isinstance(a, torch.Tensor):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


def _is_torch(a):
    return torch is not None and isinstance(a, torch.Tensor)


def grid_size(trunc):
    a, b = ctypes.c_int(), ctypes.c_int()
    _capi.check(_capi.lib().aeros_sht_grid_size(trunc, ctypes.byref(a), ctypes.byref(b)), "aeros_sht_grid_size")
    return a.value, b.value


class AerosSHT:
    """One configured transform (truncation + Gaussian grid) on the GPU."""

    def __init__(self, trunc, nlon=-1, nlat=-1, batch_max=64, precision=PREC_FP64):
        L = _capi.lib()
        h = ctypes.c_void_p()
        _capi.check(L.aeros_sht_create(ctypes.byref(h), trunc, nlon, nlat, batch_max), "aeros_sht_create")
        self._h = h
        self.batch_max = batch_max
        T, n1, n2, nlm = (ctypes.c_int() for _ in range(4))
        L.aeros_sht_info(h, ctypes.byref(T), ctypes.byref(n1), ctypes.byref(n2), ctypes.byref(nlm),
                         None, None, None, None)
        self.trunc, self.nlon, self.nlat, self.nlm = T.value, n1.value, n2.value, nlm.value
        self.lmax = self.mmax = self.trunc
        self.sinlat = np.zeros(self.nlat)
        self.gauss_w = np.zeros(self.nlat)
        self.l_of_lm = np.zeros(self.nlm, np.int32)
        self.m_of_lm = np.zeros(self.nlm, np.int32)
        L.aeros_sht_info(h, None, None, None, None, _ptr(self.sinlat), _ptr(self.gauss_w),
                         _ptr(self.l_of_lm), _ptr(self.m_of_lm))
        self.colat = np.arccos(self.sinlat)
        self.lon = 2.0 * np.pi * np.arange(self.nlon) / self.nlon
        if precision != PREC_FP64:
            self.set_precision(precision)

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().aeros_sht_destroy(self._h)
            self._h = None

    __del__ = close

    def set_precision(self, mode):
        _capi.check(_capi.lib().aeros_sht_set_precision(self._h, int(mode)), "aeros_sht_set_precision")
        self.precision = mode

    def lm(self, l, m):
        """1-based index as aeros_sht_lm, or -1."""
        return _capi.lib().aeros_sht_lm(self._h, l, m)

    def launch_count(self):
        c = ctypes.c_longlong()
        _capi.lib().aeros_sht_launch_count(self._h, ctypes.byref(c))
        return c.value

    # ------------------------------------------------------------------ helpers
    def _bind(self, a):
        """Run on torch's current stream when given CUDA tensors (stream order)."""
        if _is_torch(a) and a.is_cuda:
            s = torch.cuda.current_stream(a.device).cuda_stream
            if s != getattr(self, "_bound", None):
                _capi.check(_capi.lib().aeros_sht_set_stream(self._h, ctypes.c_void_p(s)), "aeros_sht_set_stream")
                self._bound = s

    def _spec_out(self, like, lead):
        if _is_torch(like):
            return torch.zeros(lead + (self.nlm,), dtype=torch.complex128, device=like.device)
        return np.zeros(lead + (self.nlm,), np.complex128)

    def _grid_out(self, like, lead):
        if _is_torch(like):
            return torch.zeros(lead + (self.nlat, self.nlon), dtype=torch.float64, device=like.device)
        return np.zeros(lead + (self.nlat, self.nlon))

    def _spec_in(self, a):
        if _is_torch(a):
            self._bind(a)
            return a.contiguous()
        return np.ascontiguousarray(a, np.complex128)

    def _grid_in(self, a):
        if _is_torch(a):
            self._bind(a)
            return a.contiguous()
        return np.ascontiguousarray(a, np.float64)

    def _nb_spec(self, c):
        return int(np.prod(tuple(c.shape[:-1]), dtype=np.int64)) if len(c.shape) > 1 else 1

    def _nb_grid(self, f):
        return int(np.prod(tuple(f.shape[:-2]), dtype=np.int64)) if len(f.shape) > 2 else 1

    # ------------------------------------------------------------------ transforms
    def synthesis(self, coeffs):
        c = self._spec_in(coeffs)
        f = self._grid_out(c, tuple(c.shape[:-1]))
        _capi.check(_capi.lib().aeros_sht_synthesis(self._h, _ptr(c), _ptr(f), self._nb_spec(c)), "aeros_sht_synthesis")
        return f

    def analysis(self, field):
        f = self._grid_in(field)
        c = self._spec_out(f, tuple(f.shape[:-2]))
        _capi.check(_capi.lib().aeros_sht_analysis(self._h, _ptr(f), _ptr(c), self._nb_grid(f)), "aeros_sht_analysis")
        return c

    def synthesis_vec(self, slm, tlm):
        s, t = self._spec_in(slm), self._spec_in(tlm)
        a, b = self._grid_out(s, tuple(s.shape[:-1])), self._grid_out(s, tuple(s.shape[:-1]))
        _capi.check(_capi.lib().aeros_sht_synthesis_vec(self._h, _ptr(s), _ptr(t), _ptr(a), _ptr(b),
                                                        self._nb_spec(s)), "aeros_sht_synthesis_vec")
        return a, b

    def analysis_vec(self, vth, vph):
        a, b = self._grid_in(vth), self._grid_in(vph)
        s, t = self._spec_out(a, tuple(a.shape[:-2])), self._spec_out(a, tuple(a.shape[:-2]))
        _capi.check(_capi.lib().aeros_sht_analysis_vec(self._h, _ptr(a), _ptr(b), _ptr(s), _ptr(t),
                                                       self._nb_grid(a)), "aeros_sht_analysis_vec")
        return s, t

    # ---- adjoints (Euclidean inner products of the arrays; m = 0 imaginary
    # parts are not degrees of freedom)
    def synthesis_ad(self, field_ad):
        """coeffs_ad = synthesis^T field_ad."""
        f = self._grid_in(field_ad)
        c = self._spec_out(f, tuple(f.shape[:-2]))
        _capi.check(_capi.lib().aeros_sht_synthesis_ad(self._h, _ptr(f), _ptr(c), self._nb_grid(f)),
                    "aeros_sht_synthesis_ad")
        return c

    def analysis_ad(self, coeffs_ad):
        """field_ad = analysis^T coeffs_ad."""
        c = self._spec_in(coeffs_ad)
        f = self._grid_out(c, tuple(c.shape[:-1]))
        _capi.check(_capi.lib().aeros_sht_analysis_ad(self._h, _ptr(c), _ptr(f), self._nb_spec(c)),
                    "aeros_sht_analysis_ad")
        return f

    def synthesis_vec_ad(self, vth_ad, vph_ad):
        a, b = self._grid_in(vth_ad), self._grid_in(vph_ad)
        s, t = self._spec_out(a, tuple(a.shape[:-2])), self._spec_out(a, tuple(a.shape[:-2]))
        _capi.check(_capi.lib().aeros_sht_synthesis_vec_ad(self._h, _ptr(a), _ptr(b), _ptr(s), _ptr(t),
                                                           self._nb_grid(a)), "aeros_sht_synthesis_vec_ad")
        return s, t

    def analysis_vec_ad(self, slm_ad, tlm_ad):
        s, t = self._spec_in(slm_ad), self._spec_in(tlm_ad)
        a, b = self._grid_out(s, tuple(s.shape[:-1])), self._grid_out(s, tuple(s.shape[:-1]))
        _capi.check(_capi.lib().aeros_sht_analysis_vec_ad(self._h, _ptr(s), _ptr(t), _ptr(a), _ptr(b),
                                                          self._nb_spec(s)), "aeros_sht_analysis_vec_ad")
        return a, b

    def gradient(self, coeffs):
        """(dF/dtheta, (1/sin theta) dF/dphi) on the unit sphere (SHsph_to_spat)."""
        c = self._spec_in(coeffs)
        a, b = self._grid_out(c, tuple(c.shape[:-1])), self._grid_out(c, tuple(c.shape[:-1]))
        _capi.check(_capi.lib().aeros_sht_gradient(self._h, _ptr(c), _ptr(a), _ptr(b), self._nb_spec(c)),
                    "aeros_sht_gradient")
        return a, b

    def laplacian(self, coeffs, inverse=False):
        c = self._spec_in(coeffs)
        c = c.clone() if _is_torch(c) else c.copy()
        _capi.check(_capi.lib().aeros_sht_laplacian(self._h, _ptr(c), int(bool(inverse)), self._nb_spec(c)),
                    "aeros_sht_laplacian")
        return c

    def surface_integral(self, field):
        f = self._grid_in(field)
        nb = self._nb_grid(f)
        out = np.zeros(nb)
        _capi.check(_capi.lib().aeros_sht_surface_integral(self._h, _ptr(f), _ptr(out), nb),
                    "aeros_sht_surface_integral")
        return out.reshape(tuple(f.shape[:-2])) if len(f.shape) > 2 else float(out[0])

    # ------------------------------------------------------------------ winds
    def uv_from_vordiv(self, vor, div):
        v_, d_ = self._spec_in(vor), self._spec_in(div)
        u, v = self._grid_out(v_, tuple(v_.shape[:-1])), self._grid_out(v_, tuple(v_.shape[:-1]))
        _capi.check(_capi.lib().aeros_uv_from_vordiv(self._h, _ptr(v_), _ptr(d_), _ptr(u), _ptr(v),
                                                     self._nb_spec(v_)), "aeros_uv_from_vordiv")
        return u, v

    def vordiv_from_uv(self, u, v):
        a, b = self._grid_in(u), self._grid_in(v)
        vo, dv = self._spec_out(a, tuple(a.shape[:-2])), self._spec_out(a, tuple(a.shape[:-2]))
        _capi.check(_capi.lib().aeros_vordiv_from_uv(self._h, _ptr(a), _ptr(b), _ptr(vo), _ptr(dv),
                                                     self._nb_grid(a)), "aeros_vordiv_from_uv")
        return vo, dv

    def grad(self, f):
        """Physical east/north gradient (aeros_gradient)."""
        c = self._spec_in(f)
        a, b = self._grid_out(c, tuple(c.shape[:-1])), self._grid_out(c, tuple(c.shape[:-1]))
        _capi.check(_capi.lib().aeros_gradient(self._h, _ptr(c), _ptr(a), _ptr(b), self._nb_spec(c)),
                    "aeros_gradient")
        return a, b


__all__ = ["AerosSHT", "grid_size", "PREC_FP64", "PREC_SPLIT"]
