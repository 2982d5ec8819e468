"""ctypes wrapper of the CPU oracle (test infrastructure only).

Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
legs.  Array conventions match the GPU library's Python mirror:
spectral fields are complex128 arrays shaped (..., nlm); grid fields are
float64 arrays shaped (..., nlat, nlon) (= Fortran (nlon, nlat, ...)).
"""
import ctypes
import os

import numpy as np

from . import build as _build

_libs = {}
_variant = "parity"


def use_variant(name: str):
    """Select the oracle build later handles use: "parity" (default; no fused
    multiply-adds, the build the tests check against) or "fast" (the timed CPU
    baseline).  Handles keep the library they were created with."""
    global _variant
    assert name in ("parity", "fast")
    _variant = name


def lib(variant=None):
    variant = variant or _variant
    L = _libs.get(variant)
    if L is None:
        path = _build.build(variant=variant)
        L = ctypes.CDLL(path)
        vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
        L.ora_sht_create.restype = vp
        L.ora_sht_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.ora_sht_destroy.argtypes = [vp]
        L.ora_dyn_create.restype = vp
        L.ora_dyn_create.argtypes = [vp, vp, vp, ctypes.c_int, ip]
        L.ora_dyn_destroy.argtypes = [vp]
        for name in ["ora_sht_info", "ora_sht_tables", "ora_sht_synthesis", "ora_sht_analysis",
                     "ora_sht_synthesis_vec", "ora_sht_analysis_vec", "ora_sht_gradient",
                     "ora_sht_laplacian", "ora_sht_surface_integral", "ora_uv_from_vordiv",
                     "ora_vordiv_from_uv", "ora_gradient", "ora_dyn_info", "ora_dyn_set_state",
                     "ora_dyn_get_state", "ora_dyn_get_old_state", "ora_dyn_set_old_state",
                     "ora_dyn_set_isothermal", "ora_dyn_set_phis", "ora_dyn_set_forcing", "ora_dyn_hs_perturb",
                     "ora_dyn_step", "ora_dyn_tendency", "ora_dyn_tendency_forced",
                     "ora_dyn_grid_rhs", "ora_dyn_diagnose", "ora_dyn_counters",
                     "ora_dyn_set_mass_target", "ora_dyn_budget", "ora_dyn_diag_accumulate",
                     "ora_dyn_diag_read", "ora_dyn_gwspeed", "ora_dyn_si_linear"]:
            getattr(L, name).restype = ctypes.c_int
        L.ora_dyn_set_isothermal.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.ora_dyn_hs_perturb.argtypes = [vp, ctypes.c_double]
        L.ora_dyn_set_forcing.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.ora_dyn_set_mass_target.argtypes = [vp, ctypes.c_double]
        L.ora_dyn_step.argtypes = [vp, ctypes.c_int]
        L.ora_grid_size.argtypes = [ctypes.c_int, ip, ip]
        L.ora_set_threads.argtypes = [ctypes.c_int]
        for name, n in (("ora_hs_teq", 3), ("ora_hs_kt", 2), ("ora_hs_kv", 1)):
            fn = getattr(L, name)
            fn.restype = ctypes.c_double
            fn.argtypes = [vp] + [ctypes.c_double] * n
        _libs[variant] = L
    return L


def truth_lib():
    L = _libs.get("truth")
    if L is None:
        L = ctypes.CDLL(_build.build(variant="truth"))
        L.truth_tendency.restype = ctypes.c_int
        L.truth_tendency.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + \
            [ctypes.c_void_p] * 3 + [ctypes.c_int] + [ctypes.c_void_p] * 8 + [ctypes.c_int]
        L.truth_digits.restype = ctypes.c_int
        _libs["truth"] = L
    return L


def truth_tendency(params, nlon, nlat, a_half, b_half, state, forced=False, phis=None, wide=True, nthreads=0):
    """Spectral tendencies (vor, div, temp, lnps) of `state` = (vor, div, temp
    (nlev, nlm), lnps (nlm)) evaluated in long double (wide) or double by the
    independent restatement in oracle/truth.cpp.  params.hs_dt_y / hs_k_a are
    the forcing used when forced."""
    vor, div, temp, lnps = (np.ascontiguousarray(a, dtype=np.complex128) for a in state)
    outs = [np.zeros_like(vor), np.zeros_like(div), np.zeros_like(temp), np.zeros_like(lnps)]
    ah = np.ascontiguousarray(a_half, dtype=np.float64)
    bh = np.ascontiguousarray(b_half, dtype=np.float64)
    ph = None if phis is None else np.ascontiguousarray(phis, dtype=np.float64)
    nth = nthreads or (os.cpu_count() or 1)
    rc = truth_lib().truth_tendency(int(bool(wide)), ctypes.cast(ctypes.pointer(params), ctypes.c_void_p),
                                    int(nlon), int(nlat), _p(ah), _p(bh), _p(ph), int(bool(forced)),
                                    _p(vor), _p(div), _p(temp), _p(lnps), *[_p(o) for o in outs], nth)
    if rc:
        raise RuntimeError(f"truth_tendency failed ({rc})")
    return tuple(outs)


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> int:
    return lib().ora_set_threads(int(n))


def hs_teq(params, p, sinlat2, coslat2):
    return lib().ora_hs_teq(ctypes.byref(params), p, sinlat2, coslat2)


def hs_kt(params, sigma, coslat4):
    return lib().ora_hs_kt(ctypes.byref(params), sigma, coslat4)


def hs_kv(params, sigma):
    return lib().ora_hs_kv(ctypes.byref(params), sigma)


def grid_size(trunc):
    a, b = ctypes.c_int(), ctypes.c_int()
    lib().ora_grid_size(trunc, ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


YEAR_SECONDS = 365.25 * 86400.0   # year_seconds, src/aeros_defs.f90:100


class OracleClock:
    """The facade's clock of src/aeros.f90:60-124,202-241 (aeros_init's
    time/time_init/nstep and aeros_update's step-count rule)."""

    def __init__(self, dt, time_init=0.0):
        self.dt = float(dt)
        self.time_init = self.time = float(time_init)   # :121-123
        self.nstep = 0                                   # :124

    def update(self, time):
        """Steps aeros_update takes to reach `time` [yr]; raises ValueError for
        an earlier time (:212-216, "cannot step backwards", stop 1)."""
        if time < self.time:
            raise ValueError("cannot step backwards")
        x = (float(time) - self.time_init) * YEAR_SECONDS / self.dt     # :220-221
        target = int(np.sign(x) * np.floor(abs(x) + 0.5))              # nint: halves away from zero
        ndo = target - self.nstep                                       # :222
        self.nstep = max(target, self.nstep)                            # :228
        self.time = float(time)                                         # :229
        return max(ndo, 0)


class OracleSHT:
    """CPU restatement of aeros_sht_class + the transforms of aeros_spectral."""

    def __init__(self, trunc, nlon=-1, nlat=-1):
        L = self._L = lib()
        self.h = L.ora_sht_create(trunc, nlon, nlat)
        T, n1, n2, nlm = (ctypes.c_int() for _ in range(4))
        L.ora_sht_info(ctypes.c_void_p(self.h), ctypes.byref(T), ctypes.byref(n1), ctypes.byref(n2),
                       ctypes.byref(nlm), None, None, None, None)
        self.trunc, self.nlon, self.nlat, self.nlm = T.value, n1.value, n2.value, nlm.value
        self.sinlat = np.zeros(self.nlat)
        self.gauss_w = np.zeros(self.nlat)
        self.l_of_lm = np.zeros(self.nlm, np.int32)
        self.m_of_lm = np.zeros(self.nlm, np.int32)
        L.ora_sht_info(ctypes.c_void_p(self.h), None, None, None, None, _p(self.sinlat),
                       _p(self.gauss_w), _p(self.l_of_lm), _p(self.m_of_lm))

    def __del__(self):
        if getattr(self, "h", None):
            self._L.ora_sht_destroy(ctypes.c_void_p(self.h))
            self.h = None

    def lm(self, l, m):
        """0-based index of (l, m) or -1 (src/aeros_spectral.f90:460-482 is 1-based)."""
        if m < 0 or m > self.trunc or l < m or l > self.trunc:
            return -1
        return (m * (2 * self.trunc + 1 - m)) // 2 + l

    def tables(self):
        P = np.zeros((self.nlm, self.nlat))
        dP = np.zeros((self.nlm, self.nlat))
        self._L.ora_sht_tables(ctypes.c_void_p(self.h), _p(P), _p(dP))
        return P, dP

    def _spec(self, shape):
        return np.zeros(shape + (self.nlm,), np.complex128)

    def _grid(self, shape):
        return np.zeros(shape + (self.nlat, self.nlon))

    def synthesis(self, c):
        c = np.ascontiguousarray(c, np.complex128)
        f = self._grid(c.shape[:-1])
        self._L.ora_sht_synthesis(ctypes.c_void_p(self.h), _p(c), _p(f), int(c.size // self.nlm))
        return f

    def analysis(self, f):
        f = np.ascontiguousarray(f, np.float64)
        c = self._spec(f.shape[:-2])
        self._L.ora_sht_analysis(ctypes.c_void_p(self.h), _p(f), _p(c), int(c.size // self.nlm))
        return c

    def synthesis_vec(self, s, t):
        s = np.ascontiguousarray(s, np.complex128)
        t = np.ascontiguousarray(t, np.complex128)
        a, b = self._grid(s.shape[:-1]), self._grid(s.shape[:-1])
        self._L.ora_sht_synthesis_vec(ctypes.c_void_p(self.h), _p(s), _p(t), _p(a), _p(b), int(s.size // self.nlm))
        return a, b

    def analysis_vec(self, vth, vph):
        vth = np.ascontiguousarray(vth, np.float64)
        vph = np.ascontiguousarray(vph, np.float64)
        s, t = self._spec(vth.shape[:-2]), self._spec(vth.shape[:-2])
        self._L.ora_sht_analysis_vec(ctypes.c_void_p(self.h), _p(vth), _p(vph), _p(s), _p(t), int(s.size // self.nlm))
        return s, t

    def gradient(self, c):
        c = np.ascontiguousarray(c, np.complex128)
        a, b = self._grid(c.shape[:-1]), self._grid(c.shape[:-1])
        self._L.ora_sht_gradient(ctypes.c_void_p(self.h), _p(c), _p(a), _p(b), int(c.size // self.nlm))
        return a, b

    def laplacian(self, c, inverse=False):
        c = np.array(c, np.complex128, copy=True, order="C")
        self._L.ora_sht_laplacian(ctypes.c_void_p(self.h), _p(c), int(bool(inverse)), int(c.size // self.nlm))
        return c

    def surface_integral(self, f):
        f = np.ascontiguousarray(f, np.float64)
        nb = int(f.size // (self.nlat * self.nlon))
        out = np.zeros(nb)
        self._L.ora_sht_surface_integral(ctypes.c_void_p(self.h), _p(f), _p(out), nb)
        return out.reshape(f.shape[:-2]) if f.ndim > 2 else out[0]

    def uv_from_vordiv(self, vor, div):
        vor = np.ascontiguousarray(vor, np.complex128)
        div = np.ascontiguousarray(div, np.complex128)
        u, v = self._grid(vor.shape[:-1]), self._grid(vor.shape[:-1])
        self._L.ora_uv_from_vordiv(ctypes.c_void_p(self.h), _p(vor), _p(div), _p(u), _p(v), int(vor.size // self.nlm))
        return u, v

    def vordiv_from_uv(self, u, v):
        u = np.ascontiguousarray(u, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        vor, div = self._spec(u.shape[:-2]), self._spec(u.shape[:-2])
        self._L.ora_vordiv_from_uv(ctypes.c_void_p(self.h), _p(u), _p(v), _p(vor), _p(div), int(vor.size // self.nlm))
        return vor, div

    def grad(self, f):
        f = np.ascontiguousarray(f, np.complex128)
        a, b = self._grid(f.shape[:-1]), self._grid(f.shape[:-1])
        self._L.ora_gradient(ctypes.c_void_p(self.h), _p(f), _p(a), _p(b), int(f.size // self.nlm))
        return a, b


class OracleDyn:
    """CPU restatement of aeros_timestep (dry Held-Suarez path), one member."""

    def __init__(self, params, a_half=None, b_half=None, nthreads=0):
        L = self._L = lib()
        rc = ctypes.c_int()
        ah = None if a_half is None else np.ascontiguousarray(a_half, np.float64)
        bh = None if b_half is None else np.ascontiguousarray(b_half, np.float64)
        self.params = params
        self.h = L.ora_dyn_create(ctypes.byref(params), _p(ah), _p(bh), int(nthreads), ctypes.byref(rc))
        if not self.h:
            raise ValueError(f"oracle dyn_create failed with status {rc.value}")
        a, b, c, d = (ctypes.c_int() for _ in range(4))
        L.ora_dyn_info(ctypes.c_void_p(self.h), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d),
                       None, None, None)
        self.nlon, self.nlat, self.nlm, self.nlev = a.value, b.value, c.value, d.value
        self.A = np.zeros(self.nlev + 1)
        self.B = np.zeros(self.nlev + 1)
        self.sigma_full = np.zeros(self.nlev)
        L.ora_dyn_info(ctypes.c_void_p(self.h), None, None, None, None, _p(self.A), _p(self.B), _p(self.sigma_full))

    def __del__(self):
        if getattr(self, "h", None):
            self._L.ora_dyn_destroy(ctypes.c_void_p(self.h))
            self.h = None

    @property
    def _h(self):
        return ctypes.c_void_p(self.h)

    def _alloc_state(self):
        return (np.zeros((self.nlev, self.nlm), np.complex128), np.zeros((self.nlev, self.nlm), np.complex128),
                np.zeros((self.nlev, self.nlm), np.complex128), np.zeros(self.nlm, np.complex128))

    def set_state(self, vor, div, temp, lnps):
        arrs = [np.ascontiguousarray(a, np.complex128) for a in (vor, div, temp, lnps)]
        self._L.ora_dyn_set_state(self._h, *[_p(a) for a in arrs])

    def get_state(self):
        s = self._alloc_state()
        self._L.ora_dyn_get_state(self._h, *[_p(a) for a in s])
        return s

    def get_old_state(self):
        s = self._alloc_state()
        self._L.ora_dyn_get_old_state(self._h, *[_p(a) for a in s])
        return s

    def set_old_state(self, vor, div, temp, lnps, nstep):
        arrs = [np.ascontiguousarray(a, np.complex128) for a in (vor, div, temp, lnps)]
        self._L.ora_dyn_set_old_state(self._h, *[_p(a) for a in arrs], int(nstep))

    def set_isothermal(self, temp=-1.0, ps=-1.0):
        self._L.ora_dyn_set_isothermal(self._h, float(temp), float(ps))

    def hs_perturb(self, amp=1.0):
        self._L.ora_dyn_hs_perturb(self._h, float(amp))

    def set_phis(self, phis):
        phis = np.ascontiguousarray(phis, np.float64)
        self._L.ora_dyn_set_phis(self._h, _p(phis))

    def set_forcing(self, dt_y, k_a):
        self._L.ora_dyn_set_forcing(self._h, float(dt_y), float(k_a))

    def step(self, n=1):
        rc = self._L.ora_dyn_step(self._h, int(n))
        if rc:
            raise RuntimeError(f"oracle step failed: {rc}")

    def tendency(self, forced=False):
        s = self._alloc_state()
        fn = self._L.ora_dyn_tendency_forced if forced else self._L.ora_dyn_tendency
        fn(self._h, *[_p(a) for a in s])
        return s

    def grid_rhs(self, forced=False):
        ng = self.nlon * self.nlat
        out = np.zeros(4 * ng * self.nlev + ng)
        self._L.ora_dyn_grid_rhs(self._h, int(bool(forced)), _p(out))
        n3 = ng * self.nlev
        shp = (self.nlev, self.nlat, self.nlon)
        return (out[:n3].reshape(shp), out[n3:2 * n3].reshape(shp), out[2 * n3:3 * n3].reshape(shp),
                out[3 * n3:4 * n3].reshape(shp), out[4 * n3:].reshape(self.nlat, self.nlon))

    def diagnose(self):
        shp = (self.nlev, self.nlat, self.nlon)
        u, v, t, ps = np.zeros(shp), np.zeros(shp), np.zeros(shp), np.zeros((self.nlat, self.nlon))
        self._L.ora_dyn_diagnose(self._h, _p(u), _p(v), _p(t), _p(ps))
        return u, v, t, ps

    def counters(self):
        n = ctypes.c_int()
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._L.ora_dyn_counters(self._h, ctypes.byref(n), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return n.value, a.value, b.value, c.value

    def set_mass_target(self, m):
        self._L.ora_dyn_set_mass_target(self._h, float(m))

    def budget(self):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._L.ora_dyn_budget(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def diag_accumulate(self):
        self._L.ora_dyn_diag_accumulate(self._h)

    def diag_read(self):
        nl, n = self.nlat, self.nlev
        out = np.zeros(7 * nl * n + 2 * nl)
        ns = ctypes.c_int()
        self._L.ora_dyn_diag_read(self._h, _p(out), ctypes.byref(ns))
        F = nl * n
        names = ["u", "v", "temp", "uv", "vt", "eke", "tvar"]
        d = {nm: out[i * F:(i + 1) * F].reshape(n, nl) for i, nm in enumerate(names)}
        d["ps"] = out[7 * F:7 * F + nl]
        d["u_sfc"] = out[7 * F + nl:]
        d["nsample"] = ns.value
        return d

    def gwspeed(self):
        c = ctypes.c_double()
        self._L.ora_dyn_gwspeed(self._h, ctypes.byref(c))
        return c.value

    def si_linear(self):
        ld = np.zeros((self.nlev, self.nlm), np.complex128)
        lt = np.zeros((self.nlev, self.nlm), np.complex128)
        lp = np.zeros(self.nlm, np.complex128)
        self._L.ora_dyn_si_linear(self._h, _p(ld), _p(lt), _p(lp))
        return ld, lt, lp
