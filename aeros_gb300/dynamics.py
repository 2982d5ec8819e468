"""Python mirror of aeros' dry time step on the GPU library.

`AerosDyn` plays the role of aeros_timestep_class + the aeros facade
(src/dynamics/aeros_timestep.f90:435-448, src/aeros.f90:64-70) for an ensemble
of `nmember` members that share truncation and levels.  State arrays are
complex128 numpy arrays (host) or torch complex128 CUDA tensors (device):
vor/div/temp (nmember, nlev, nlm), lnps (nmember, nlm); with nmember == 1 the
leading member axis may be dropped.
"""
import ctypes

import numpy as np

from . import _capi
from .params import AerosParams, held_suarez_params
from .spectral import _ptr, _is_torch

YEAR_SECONDS = 365.25 * 86400.0   # src/aeros_defs.f90:100


class AerosDyn:
    def __init__(self, params: AerosParams = None, a_half=None, b_half=None):
        self.params = params if params is not None else held_suarez_params()
        L = _capi.lib()
        h = ctypes.c_void_p()
        ah = None if a_half is None else np.ascontiguousarray(a_half, np.float64)
        bh = None if b_half is None else np.ascontiguousarray(b_half, np.float64)
        _capi.check(L.aeros_dyn_create(ctypes.byref(h), ctypes.byref(self.params),
                                       None if ah is None else _ptr(ah), None if bh is None else _ptr(bh)),
                    "aeros_dyn_create")
        self._h = h
        a, b, c, d = (ctypes.c_int() for _ in range(4))
        L.aeros_dyn_info(h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d),
                         None, None, None, None, None)
        self.nlon, self.nlat, self.nlm, self.nlev = a.value, b.value, c.value, d.value
        self.nmember = self.params.nmember
        self.A = np.zeros(self.nlev + 1)
        self.B = np.zeros(self.nlev + 1)
        self.sigma_full = np.zeros(self.nlev)
        self.sinlat = np.zeros(self.nlat)
        self.gauss_w = np.zeros(self.nlat)
        L.aeros_dyn_info(h, None, None, None, None, _ptr(self.A), _ptr(self.B), _ptr(self.sigma_full),
                         _ptr(self.sinlat), _ptr(self.gauss_w))

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().aeros_dyn_destroy(self._h)
            self._h = None

    __del__ = close

    # ------------------------------------------------------------------ state
    def _shape3(self):
        return (self.nmember, self.nlev, self.nlm)

    def _alloc(self, like=None):
        if like is not None and _is_torch(like):
            import torch
            z = lambda s: torch.zeros(s, dtype=torch.complex128, device=like.device)
        else:
            z = lambda s: np.zeros(s, np.complex128)
        return z(self._shape3()), z(self._shape3()), z(self._shape3()), z((self.nmember, self.nlm))

    @staticmethod
    def _c(a):
        if _is_torch(a):
            import torch
            if a.is_cuda:
                torch.cuda.current_stream(a.device).synchronize()
            return a.contiguous()
        return np.ascontiguousarray(a, np.complex128)

    def set_state(self, vor, div, temp, lnps):
        arrs = [self._c(x) for x in (vor, div, temp, lnps)]
        n3 = self.nmember * self.nlev * self.nlm
        for x, n in zip(arrs, (n3, n3, n3, self.nmember * self.nlm)):
            if (x.numel() if _is_torch(x) else x.size) != n:
                raise ValueError("state array has the wrong size")
        _capi.check(_capi.lib().aeros_dyn_set_state(self._h, *[_ptr(x) for x in arrs]), "aeros_dyn_set_state")

    def get_state(self, like=None, squeeze=True, out=None):
        s = self._alloc(like) if out is None else tuple(out)
        if like is not None and _is_torch(like) and like.is_cuda:
            import torch
            torch.cuda.current_stream(like.device).synchronize()
        _capi.check(_capi.lib().aeros_dyn_get_state(self._h, *[_ptr(x) for x in s]), "aeros_dyn_get_state")
        return self._squeeze(s) if squeeze else s

    def set_old_state(self, vor, div, temp, lnps, nstep):
        arrs = [self._c(x) for x in (vor, div, temp, lnps)]
        _capi.check(_capi.lib().aeros_dyn_set_old_state(self._h, *[_ptr(x) for x in arrs], int(nstep)),
                    "aeros_dyn_set_old_state")

    def get_old_state(self, squeeze=True):
        s = self._alloc()
        _capi.check(_capi.lib().aeros_dyn_get_old_state(self._h, *[_ptr(x) for x in s]), "aeros_dyn_get_old_state")
        return self._squeeze(s) if squeeze else s

    def _squeeze(self, s):
        if self.nmember == 1:
            return tuple(x[0] for x in s)
        return s

    def set_isothermal(self, temp=-1.0, ps=-1.0):
        _capi.check(_capi.lib().aeros_dyn_set_isothermal(self._h, float(temp), float(ps)), "aeros_dyn_set_isothermal")

    def hs_perturb(self, amp=1.0):
        """Deterministic Held-Suarez temperature seed (aeros_hs_perturb)."""
        _capi.check(_capi.lib().aeros_dyn_hs_perturb(self._h, float(amp)), "aeros_dyn_hs_perturb")

    def set_phis(self, phis):
        p = np.ascontiguousarray(phis, np.float64)
        _capi.check(_capi.lib().aeros_dyn_set_phis(self._h, _ptr(p)), "aeros_dyn_set_phis")

    def set_member_forcing(self, member, dt_y, k_a):
        _capi.check(_capi.lib().aeros_dyn_set_member_forcing(self._h, int(member), float(dt_y), float(k_a)),
                    "aeros_dyn_set_member_forcing")

    # ------------------------------------------------------------------ stepping
    def step(self, nsteps=1):
        _capi.check(_capi.lib().aeros_dyn_step(self._h, int(nsteps)), "aeros_dyn_step")

    def step_async(self, nsteps=1):
        """Enqueue steps (CUDA graphs) without waiting; pair with sync()."""
        _capi.check(_capi.lib().aeros_dyn_step_async(self._h, int(nsteps)), "aeros_dyn_step_async")

    def sync(self):
        _capi.check(_capi.lib().aeros_dyn_sync(self._h), "aeros_dyn_sync")

    def profile_step(self, maxk=32):
        """One real step with events between its kernels: [(name, ms), ...]."""
        ms = np.zeros(maxk)
        names = ctypes.create_string_buffer(maxk * 32)
        nk = ctypes.c_int()
        _capi.check(_capi.lib().aeros_dyn_profile_step(self._h, maxk, _ptr(ms), names, 32, ctypes.byref(nk)),
                    "aeros_dyn_profile_step")
        raw = names.raw
        out = []
        for i in range(nk.value):
            nm = raw[i * 32:(i + 1) * 32].split(b"\0", 1)[0].decode()
            out.append((nm, float(ms[i])))
        return out

    @property
    def time(self):
        """Facade clock [yr]: the time of the last aeros_dyn_update (or set_time)."""
        return self.facade_clock()[0]

    @time.setter
    def time(self, t):
        self.set_time(t)

    def set_time(self, time_init):
        """Model time at initialisation [yr] (aeros_init's time_init,
        src/aeros.f90:121-124); clears the facade's step count."""
        _capi.check(_capi.lib().aeros_dyn_set_time(self._h, float(time_init)), "aeros_dyn_set_time")

    def facade_clock(self):
        """(time [yr], steps taken through update)."""
        t, n = ctypes.c_double(), ctypes.c_int()
        _capi.check(_capi.lib().aeros_dyn_get_time(self._h, ctypes.byref(t), ctypes.byref(n)), "aeros_dyn_get_time")
        return t.value, n.value

    def update(self, time_years):
        """Advance to `time_years` with the step-count rule of aeros_update
        (src/aeros.f90:202-241): n_target = nint((t - t0) yr / dt), halves away
        from zero; an earlier time raises (the reference's "cannot step
        backwards" stop)."""
        _capi.check(_capi.lib().aeros_dyn_update(self._h, float(time_years)), "aeros_dyn_update")

    def tendency(self):
        s = self._alloc()
        _capi.check(_capi.lib().aeros_dyn_tendency(self._h, *[_ptr(x) for x in s]), "aeros_dyn_tendency")
        return self._squeeze(s)

    def tendency_forced(self):
        """Spectral tendencies with the step's forcing: Held-Suarez (when enabled)
        and the physics hook, both added on the grid at the seam."""
        s = self._alloc()
        _capi.check(_capi.lib().aeros_dyn_tendency_forced(self._h, *[_ptr(x) for x in s]),
                    "aeros_dyn_tendency_forced")
        return self._squeeze(s)

    def set_physics(self, fn, user=None):
        """Install a physics hook at the grid seam (a C function with the
        aeros_physics_fn signature: an address, or a ctypes function pointer),
        or remove it with fn=None.  The step graphs are re-captured; the hook
        enqueues its work when they are.  `user` (a ctypes object, passed by
        reference) is kept alive by the handle."""
        if fn is None:
            self._phys = None
            _capi.check(_capi.lib().aeros_dyn_set_physics(self._h, None, None), "aeros_dyn_set_physics")
            return
        addr = fn if isinstance(fn, int) else ctypes.cast(fn, ctypes.c_void_p).value
        self._phys = (fn, user)
        uptr = ctypes.cast(ctypes.byref(user), ctypes.c_void_p) if user is not None else None
        _capi.check(_capi.lib().aeros_dyn_set_physics(self._h, ctypes.c_void_p(addr), uptr),
                    "aeros_dyn_set_physics")

    def set_relaxation(self, k_drag, k_temp=0.0, t_ref=0.0):
        """The ready-made hook aeros_physics_relaxation: ae -= k_drag u,
        an -= k_drag v, dtdt -= k_temp (T - t_ref) on the grid."""
        self.set_physics(_capi.lib().aeros_physics_relaxation, _capi.AerosRelaxation(k_drag, k_temp, t_ref))

    def diagnose(self):
        shp = (self.nmember, self.nlev, self.nlat, self.nlon)
        u, v, t = np.zeros(shp), np.zeros(shp), np.zeros(shp)
        ps = np.zeros((self.nmember, self.nlat, self.nlon))
        _capi.check(_capi.lib().aeros_dyn_diagnose(self._h, _ptr(u), _ptr(v), _ptr(t), _ptr(ps)), "aeros_dyn_diagnose")
        if self.nmember == 1:
            return u[0], v[0], t[0], ps[0]
        return u, v, t, ps

    def budget(self):
        m, e, a = (np.zeros(self.nmember) for _ in range(3))
        _capi.check(_capi.lib().aeros_dyn_budget(self._h, _ptr(m), _ptr(e), _ptr(a)), "aeros_dyn_budget")
        if self.nmember == 1:
            return float(m[0]), float(e[0]), float(a[0])
        return m, e, a

    def counters(self):
        n = ctypes.c_int()
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _capi.check(_capi.lib().aeros_dyn_counters(self._h, ctypes.byref(n), ctypes.byref(a), ctypes.byref(b),
                                                   ctypes.byref(c)), "aeros_dyn_counters")
        return n.value, a.value, b.value, c.value

    def step_packed(self, now_in, old_in, nstep, nsteps=1, now_out=None, old_out=None):
        """aeros_dyn_step_packed: packed complex128 time levels (vor | div | temp | lnps,
        state_size() values each, host or CUDA) in, nsteps steps, the new X^n into
        now_out (allocated when None) and, when given, the new X^(n-1) (the
        filtered previous level) into old_out; returns now_out."""
        n = self.state_size()
        if now_out is None:
            now_out = np.empty(n, np.complex128)
        for a in (now_in, old_in, now_out) + (() if old_out is None else (old_out,)):
            if a.shape != (n,) or (not _is_torch(a) and (a.dtype != np.complex128 or not a.flags.c_contiguous)):
                raise ValueError(f"packed states are contiguous complex128 arrays of {n} values")
        _capi.check(_capi.lib().aeros_dyn_step_packed(self._h, _ptr(now_in), _ptr(old_in), int(nstep), int(nsteps),
                                                      _ptr(now_out), None if old_out is None else _ptr(old_out)),
                    "aeros_dyn_step_packed")
        return now_out

    def member_counters(self, member=0):
        """(mass_target, lnr_last, lnr_cum) of one member."""
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _capi.check(_capi.lib().aeros_dyn_member_counters(self._h, int(member), ctypes.byref(a), ctypes.byref(b),
                                                          ctypes.byref(c)), "aeros_dyn_member_counters")
        return a.value, b.value, c.value

    def set_member_counters(self, member, mass_target, lnr_last, lnr_cum):
        _capi.check(_capi.lib().aeros_dyn_set_member_counters(self._h, int(member), float(mass_target),
                                                              float(lnr_last), float(lnr_cum)),
                    "aeros_dyn_set_member_counters")

    def set_mass_target(self, mass):
        _capi.check(_capi.lib().aeros_dyn_set_mass_target(self._h, float(mass)), "aeros_dyn_set_mass_target")

    def diag_accumulate(self):
        _capi.check(_capi.lib().aeros_dyn_diag_accumulate(self._h), "aeros_dyn_diag_accumulate")

    def diag_read(self, member=0):
        nl, n = self.nlat, self.nlev
        out = np.zeros(7 * nl * n + 2 * nl)
        ns = ctypes.c_int()
        _capi.check(_capi.lib().aeros_dyn_diag_read(self._h, int(member), _ptr(out), ctypes.byref(ns)),
                    "aeros_dyn_diag_read")
        F = nl * n
        names = ["u", "v", "temp", "uv", "vt", "eke", "tvar"]
        d = {nm: out[i * F:(i + 1) * F].reshape(n, nl) for i, nm in enumerate(names)}
        d["ps"] = out[7 * F:7 * F + nl]
        d["u_sfc"] = out[7 * F + nl:]
        d["nsample"] = ns.value
        return d

    def gwspeed(self):
        c = ctypes.c_double()
        _capi.check(_capi.lib().aeros_dyn_gwspeed(self._h, ctypes.byref(c)), "aeros_dyn_gwspeed")
        return c.value

    def set_stream(self, stream_ptr):
        _capi.check(_capi.lib().aeros_dyn_set_stream(self._h, ctypes.c_void_p(stream_ptr)), "aeros_dyn_set_stream")

    def launch_count(self):
        c = ctypes.c_longlong()
        _capi.lib().aeros_dyn_launch_count(self._h, ctypes.byref(c))
        return c.value

    # ------------------------------------------------------------------ autotuner
    TUNE_KEYS = ("fs_lpb", "fs_thr", "fa_lpb", "fa_thr", "la_ct", "col_thr", "spec_warps", "col_lanes", "ls_jt",
                 "spec_cols", "sp_cps", "sp_dft_cps")

    def autotune(self, reps=3):
        """Choose launch shapes by timing whole steps; returns (ms before, ms after, shapes)."""
        b, a = ctypes.c_double(), ctypes.c_double()
        _capi.check(_capi.lib().aeros_dyn_autotune(self._h, int(reps), ctypes.byref(b), ctypes.byref(a)),
                    "aeros_dyn_autotune")
        return b.value, a.value, self.tune_shapes()

    def tune_shapes(self):
        v = np.zeros(len(self.TUNE_KEYS), np.int32)
        _capi.check(_capi.lib().aeros_dyn_tune_get(self._h, _ptr(v), len(v)), "aeros_dyn_tune_get")
        return dict(zip(self.TUNE_KEYS, (int(x) for x in v)))

    def set_tune_shapes(self, **shapes):
        """Set launch shapes by name (the others keep their values); each must
        be one the autotuner would try.  Re-captures the step graphs."""
        cur = self.tune_shapes()
        unknown = set(shapes) - set(cur)
        if unknown:
            raise KeyError(f"unknown launch shapes {sorted(unknown)}")
        cur.update(shapes)
        v = np.array([cur[k] for k in self.TUNE_KEYS], np.int32)
        _capi.check(_capi.lib().aeros_dyn_tune_set(self._h, _ptr(v), len(v)), "aeros_dyn_tune_set")

    # ------------------------------------------------------------------ adjoint
    # Packed state: vor (M, nlev, nlm) | div | temp | lnps (M, nlm), complex128.
    def pack(self, vor, div, temp, lnps):
        M = self.nmember
        parts = [np.asarray(vor, np.complex128).reshape(M, -1), np.asarray(div, np.complex128).reshape(M, -1),
                 np.asarray(temp, np.complex128).reshape(M, -1), np.asarray(lnps, np.complex128).reshape(M, -1)]
        return np.concatenate([p.ravel() for p in parts])

    def unpack(self, x):
        M, n3 = self.nmember, self.nmember * self.nlev * self.nlm
        s3 = self._shape3()
        out = (x[:n3].reshape(s3), x[n3:2 * n3].reshape(s3), x[2 * n3:3 * n3].reshape(s3),
               x[3 * n3:].reshape(M, self.nlm))
        return self._squeeze(out)

    @staticmethod
    def host_register(arr):
        """Page-lock a numpy array (aeros_host_register) so that aeros_dyn_step_packed
        takes its one-graph form with it."""
        _capi.check(_capi.lib().aeros_host_register(arr.ctypes.data_as(ctypes.c_void_p), arr.nbytes),
                    "aeros_host_register")

    @staticmethod
    def host_unregister(arr):
        _capi.check(_capi.lib().aeros_host_unregister(arr.ctypes.data_as(ctypes.c_void_p)), "aeros_host_unregister")

    def state_size(self):
        n = ctypes.c_longlong()
        _capi.check(_capi.lib().aeros_dyn_state_size(self._h, ctypes.byref(n)), "aeros_dyn_state_size")
        return n.value

    def step_ad(self, old_ad, now_ad):
        """Adjoint of the next step (state unchanged): packed adjoints of the
        post-step (old, now) slots -> packed adjoints of the pre-step slots,
        and per-member d/dk_a, d/ddT_y."""
        n = self.state_size()
        oi = np.ascontiguousarray(old_ad, np.complex128)
        ni = np.ascontiguousarray(now_ad, np.complex128)
        assert oi.size == n and ni.size == n
        oo, no = np.zeros(n, np.complex128), np.zeros(n, np.complex128)
        ka, dty = np.zeros(self.nmember), np.zeros(self.nmember)
        _capi.check(_capi.lib().aeros_dyn_step_ad(self._h, _ptr(oi), _ptr(ni), _ptr(oo), _ptr(no), _ptr(ka),
                                                  _ptr(dty)), "aeros_dyn_step_ad")
        return oo, no, ka, dty

    def window_forward(self, nsteps, ckpt_every=12):
        """Step nsteps with checkpoints; J per member (window-mean kinetic energy, J)."""
        J = np.zeros(self.nmember)
        _capi.check(_capi.lib().aeros_dyn_window_forward(self._h, int(nsteps), int(ckpt_every), _ptr(J)),
                    "aeros_dyn_window_forward")
        return J

    def window_backward(self):
        """Gradient of sum(J) w.r.t. the window's initial state (packed now, old)
        and the members' k_a, dT_y."""
        n = self.state_size()
        now, old = np.zeros(n, np.complex128), np.zeros(n, np.complex128)
        ka, dty = np.zeros(self.nmember), np.zeros(self.nmember)
        _capi.check(_capi.lib().aeros_dyn_window_backward(self._h, _ptr(now), _ptr(old), _ptr(ka), _ptr(dty)),
                    "aeros_dyn_window_backward")
        return now, old, ka, dty


class AerosGroup:
    """Several AerosDyn handles stepped by one CUDA graph launch per step.

    Members may differ in truncation and level count (e.g. 32 x T21L16,
    32 x T31L20 and 32 x T42L20).  The group fuses the handles' launches: each
    kernel of the step runs once over every handle that uses it (a ragged
    launch whose CTAs look up their handle), so the step is about one launch
    per kernel type.  With a physics hook installed (or AEROS_GROUP_FUSE=0)
    each handle's own step graph is a branch of the group's graph instead.
    Configure the handles (state, forcing) before grouping and step them only
    through the group afterwards.
    """

    def __init__(self, handles):
        self.handles = list(handles)
        arr = (ctypes.c_void_p * len(self.handles))(*[h._h.value for h in self.handles])
        g = ctypes.c_void_p()
        _capi.check(_capi.lib().aeros_group_create(ctypes.byref(g), arr, len(self.handles)), "aeros_group_create")
        self._g = g

    def close(self):
        if getattr(self, "_g", None):
            _capi.lib().aeros_group_destroy(self._g)
            self._g = None

    __del__ = close

    def set_stream(self, stream_ptr):
        _capi.check(_capi.lib().aeros_group_set_stream(self._g, ctypes.c_void_p(stream_ptr)), "aeros_group_set_stream")

    def step(self, nsteps=1):
        _capi.check(_capi.lib().aeros_group_step(self._g, int(nsteps)), "aeros_group_step")

    def step_async(self, nsteps=1):
        _capi.check(_capi.lib().aeros_group_step_async(self._g, int(nsteps)), "aeros_group_step_async")

    def sync(self):
        _capi.check(_capi.lib().aeros_group_sync(self._g), "aeros_group_sync")

    def launch_count(self):
        c = ctypes.c_longlong()
        _capi.lib().aeros_group_launch_count(self._g, ctypes.byref(c))
        return c.value

    def info(self):
        """{'fused': bool, 'kernels_startup': n, 'kernels_step': n} (launches per step)."""
        f, k0, k1 = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong()
        _capi.check(_capi.lib().aeros_group_info(self._g, ctypes.byref(f), ctypes.byref(k0), ctypes.byref(k1)),
                    "aeros_group_info")
        return {"fused": bool(f.value), "kernels_startup": k0.value, "kernels_step": k1.value}

    @property
    def nmember(self):
        return sum(h.nmember for h in self.handles)
