"""Restart files in the layout of the reference's aeros_timestep_write_restart /
aeros_timestep_read_restart (src/dynamics/aeros_timestep.f90:1303-1633).

The file is netCDF classic (64-bit offset), written and read with
scipy.io.netcdf_file; the reference's netCDF library reads classic files.  Its
contents follow the reference field by field:

- index dimensions lon, lat, lev, nlm, each with a coordinate variable 1..n
  (units "1"), as its nc_write_dim calls make them;
- global attributes nlm, nlev, nlon, nlat (checked on read), nstep, ocn_mode,
  rad_heat_present, land_present, seaice_present, cf_present (ints), time,
  mass_target, lnr_cum, lnr_last (doubles);
- the two spectral time levels X^n ("now") and X^(n-1) ("old") as separate
  real and imaginary parts: {now,old}_{vor,div,temp}_{re,im} (lev, nlm) and
  {now,old}_lnps_{re,im} (nlm);
- the fields the reference's reader requires of every restart even in a dry
  run, written as zeros here (this path has no moisture, ocean or radiation):
  qv_g (lev, lat, lon); ocn_sst, ocn_fnet and the cached radiative fluxes
  rad_sw_net_sur, rad_lw_dw_sur, rad_sw_dw_sur, rad_olr, rad_sw_up_toa
  (lat, lon).

Dimension order is the C order of the Fortran arrays (a Fortran (nlm, lev)
array is (lev, nlm) here), so a restart written by either side reads on the
other.  A handle with several members writes and reads one member per file.
"""
import numpy as np

from scipy.io import netcdf_file

_SPEC = ("vor", "div", "temp")
_ZERO2 = ("ocn_sst", "ocn_fnet", "rad_sw_net_sur", "rad_lw_dw_sur", "rad_sw_dw_sur", "rad_olr", "rad_sw_up_toa")


def _member(arrs, member):
    return [np.ascontiguousarray(a[member]) for a in arrs]


def write_restart(dyn, path, member=0, time=None):
    """Write member `member` of an AerosDyn handle (its X^n, X^(n-1), step count
    and mass-fixer scalars) to `path`.  `time` defaults to dyn.time [years]."""
    nlm, nlev, nlat, nlon = dyn.nlm, dyn.nlev, dyn.nlat, dyn.nlon
    now = _member(dyn.get_state(squeeze=False), member)
    old = _member(dyn.get_old_state(squeeze=False), member)
    nstep = dyn.counters()[0]
    mass_target, lnr_last, lnr_cum = dyn.member_counters(member)
    f = netcdf_file(path, "w", version=2)
    try:
        for name, n in (("lon", nlon), ("lat", nlat), ("lev", nlev), ("nlm", nlm)):
            f.createDimension(name, n)
            v = f.createVariable(name, "d", (name,))
            v[:] = np.arange(1, n + 1, dtype=np.float64)
            v.units = "1"
        for name, val in (("nlm", nlm), ("nlev", nlev), ("nlon", nlon), ("nlat", nlat), ("nstep", nstep),
                          ("ocn_mode", 0), ("rad_heat_present", 0), ("land_present", 0), ("seaice_present", 0)):
            setattr(f, name, np.int32(val))
        for name, val in (("time", dyn.time if time is None else time), ("mass_target", mass_target),
                          ("lnr_cum", lnr_cum), ("lnr_last", lnr_last)):
            setattr(f, name, np.float64(val))
        for prefix, st in (("now", now), ("old", old)):
            for fld, arr in zip(_SPEC, st[:3]):
                for part, val in (("re", arr.real), ("im", arr.imag)):
                    v = f.createVariable(f"{prefix}_{fld}_{part}", "d", ("lev", "nlm"))
                    v[:] = val
            for part, val in (("re", st[3].real), ("im", st[3].imag)):
                v = f.createVariable(f"{prefix}_lnps_{part}", "d", ("nlm",))
                v[:] = val
        v = f.createVariable("qv_g", "d", ("lev", "lat", "lon"))
        v[:] = 0.0
        v.units = "kg kg-1"
        v.long_name = "specific humidity (prognostic)"
        for name in _ZERO2:
            v = f.createVariable(name, "d", ("lat", "lon"))
            v[:] = 0.0
        f.cf_present = np.int32(0)
    finally:
        f.close()


def read_restart(dyn, path, member=0):
    """Load a restart into member `member` of an AerosDyn handle (the other
    members keep their state); returns the file's time [years] and sets
    dyn.time to it.  Raises ValueError if the file's (nlm, nlev, nlon, nlat)
    differ from the handle's, as the reference's reader stops."""
    f = netcdf_file(path, "r", mmap=False)
    try:
        want = (dyn.nlm, dyn.nlev, dyn.nlon, dyn.nlat)
        got = tuple(int(getattr(f, k)) for k in ("nlm", "nlev", "nlon", "nlat"))
        if got != want:
            raise ValueError(f"restart file metadata (nlm, nlev, nlon, nlat) = {got} does not match the model {want}")
        for k in ("land_present", "seaice_present", "cf_present", "rad_heat_present"):
            if int(getattr(f, k, 0)) != 0:
                raise ValueError(f"restart file carries state this dry path does not model ({k} = 1)")
        nstep = int(f.nstep)
        time = float(f.time)
        mt = float(f.mass_target)
        counters = (mt if mt > 0.0 else -1.0, float(f.lnr_last), float(f.lnr_cum))   # <= 0: not captured yet

        def cplx(name):   # real and imaginary parts placed as stored (keeps signed zeros)
            re, im = f.variables[name + "_re"][:], f.variables[name + "_im"][:]
            out = np.empty(re.shape, dtype=np.complex128)
            out.real, out.imag = re, im
            return out

        def spec(prefix):
            return [cplx(f"{prefix}_{fld}") for fld in _SPEC] + [cplx(f"{prefix}_lnps")]

        now, old = spec("now"), spec("old")
    finally:
        f.close()
    cur_now = [np.array(a) for a in dyn.get_state(squeeze=False)]
    cur_old = [np.array(a) for a in dyn.get_old_state(squeeze=False)]
    for full, part in zip(cur_now, now):
        full[member] = part
    for full, part in zip(cur_old, old):
        full[member] = part
    dyn.set_state(*cur_now)
    dyn.set_old_state(*cur_old, nstep)
    dyn.set_member_counters(member, *counters)
    dyn.time = time
    return time
