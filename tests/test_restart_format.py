"""Restart files: the layout of aeros_timestep_write_restart
(src/dynamics/aeros_timestep.f90:1303-1633) and a lossless round trip.  Host
code only: a stand-in handle holds the state in numpy arrays."""
import numpy as np
import pytest

pytest.importorskip("scipy")
from scipy.io import netcdf_file

from aeros_gb300.restart import read_restart, write_restart


class _Handle:
    """The slice of the AerosDyn interface the restart code uses."""

    def __init__(self, nmember=2, nlev=5, T=10, nlat=16, nlon=32, seed=0):
        rng = np.random.default_rng(seed)
        self.nmember, self.nlev, self.nlat, self.nlon = nmember, nlev, nlat, nlon
        self.nlm = (T + 1) * (T + 2) // 2
        c = lambda *s: rng.normal(size=s) + 1j * rng.normal(size=s)
        self.now = [c(nmember, nlev, self.nlm) for _ in range(3)] + [c(nmember, self.nlm)]
        self.old = [c(nmember, nlev, self.nlm) for _ in range(3)] + [c(nmember, self.nlm)]
        self.nstep = 37
        self.cnt = [[5.1e18 + e, 1e-9 * (e + 1), 3e-7 * (e + 1)] for e in range(nmember)]
        self.time = 0.25

    def get_state(self, squeeze=True):
        return [a.copy() for a in self.now]

    def get_old_state(self, squeeze=True):
        return [a.copy() for a in self.old]

    def counters(self):
        return (self.nstep, *self.cnt[0])

    def member_counters(self, member=0):
        return tuple(self.cnt[member])

    def set_state(self, *s):
        self.now = [np.array(a) for a in s]
        self.nstep = 0

    def set_old_state(self, *s):
        *arrs, nstep = s
        self.old = [np.array(a) for a in arrs]
        self.nstep = nstep

    def set_member_counters(self, member, mt, ll, lc):
        self.cnt[member] = [mt, ll, lc]


def test_layout_matches_the_reference_writer(tmp_path):
    h = _Handle()
    p = str(tmp_path / "restart.nc")
    write_restart(h, p, member=1)
    f = netcdf_file(p, "r", mmap=False)
    try:
        assert {k: f.dimensions[k] for k in ("lon", "lat", "lev", "nlm")} == \
            {"lon": h.nlon, "lat": h.nlat, "lev": h.nlev, "nlm": h.nlm}
        for k in ("lon", "lat", "lev", "nlm"):
            assert np.array_equal(f.variables[k][:], np.arange(1, f.dimensions[k] + 1))
        for k, v in (("nlm", h.nlm), ("nlev", h.nlev), ("nlon", h.nlon), ("nlat", h.nlat), ("nstep", 37),
                     ("ocn_mode", 0), ("rad_heat_present", 0), ("land_present", 0), ("seaice_present", 0),
                     ("cf_present", 0)):
            assert int(getattr(f, k)) == v
        assert float(f.time) == 0.25 and float(f.mass_target) == h.cnt[1][0]
        assert float(f.lnr_last) == h.cnt[1][1] and float(f.lnr_cum) == h.cnt[1][2]
        for prefix in ("now", "old"):
            for fld in ("vor", "div", "temp"):
                for part in ("re", "im"):
                    assert f.variables[f"{prefix}_{fld}_{part}"].dimensions == ("lev", "nlm")
            for part in ("re", "im"):
                assert f.variables[f"{prefix}_lnps_{part}"].dimensions == ("nlm",)
        assert np.array_equal(f.variables["now_temp_im"][:], h.now[2][1].imag)
        assert f.variables["qv_g"].dimensions == ("lev", "lat", "lon")
        for k in ("ocn_sst", "ocn_fnet", "rad_sw_net_sur", "rad_lw_dw_sur", "rad_sw_dw_sur", "rad_olr",
                  "rad_sw_up_toa"):
            assert f.variables[k].dimensions == ("lat", "lon")
    finally:
        f.close()


def test_round_trip_is_lossless_and_member_local(tmp_path):
    a, b = _Handle(seed=1), _Handle(seed=2)
    p = str(tmp_path / "r.nc")
    write_restart(a, p, member=0)
    keep = [x[1].copy() for x in b.now]
    t = read_restart(b, p, member=0)
    assert t == a.time and b.nstep == a.nstep and b.cnt[0] == a.cnt[0]
    for x, y in zip(b.now, a.now):
        assert np.array_equal(x[0], y[0])
    for x, y in zip(b.old, a.old):
        assert np.array_equal(x[0], y[0])
    for x, y in zip(b.now, keep):      # member 1 untouched
        assert np.array_equal(x[1], y)


def test_mismatched_grid_is_refused(tmp_path):
    p = str(tmp_path / "r.nc")
    write_restart(_Handle(nlev=5), p)
    with pytest.raises(ValueError):
        read_restart(_Handle(nlev=6), p)
