"""The reference's transport test cases (tests/test_transport.f90:97-181,
360-384), shared by the oracle and the GPU tests: T21 L8 grid, winds, tracer
fields and the surface pressure of each check."""
import numpy as np

P0 = 1.0e5           # src/aeros_defs.f90 (reference pressure)
R_EARTH = 6.371e6


def geometry(trunc=21, nlev=8):
    """(sinlat, gauss_w, nlon, nlat, A, B, lon, lat) from the oracle."""
    from aeros_gb300.params import held_suarez_params
    from oracle.pyoracle import OracleDyn, OracleSHT
    s = OracleSHT(trunc)
    o = OracleDyn(held_suarez_params(trunc=trunc, nlev=nlev))
    lon = 2.0 * np.pi * np.arange(s.nlon) / s.nlon
    lat = np.arcsin(s.sinlat)
    return s.sinlat.copy(), s.gauss_w.copy(), s.nlon, s.nlat, o.A.copy(), o.B.copy(), lon, lat


def set_lnps(lon, lat):
    """set_lnps (:97-111): a wavenumber-1 surface-pressure pattern."""
    return np.log(P0 * (1.0 + 0.05 * np.sin(lon)[None, :] * np.cos(lat)[:, None]))


def solid_body(lon, lat, nlev, u0):
    """solid_body (:113-134): u = u0 cos(lat), v = 0."""
    u = np.broadcast_to(u0 * np.cos(lat)[None, :, None], (nlev, len(lat), len(lon))).copy()
    return u, np.zeros_like(u)


def divergent_wind(lon, lat, nlev, u0):
    """divergent_wind (:136-158)."""
    k = (np.arange(1, nlev + 1) / nlev)[:, None, None]
    u = u0 * np.sin(lon)[None, None, :] * np.cos(lat)[None, :, None] * k
    v = np.broadcast_to(u0 * np.cos(lon)[None, None, :] * 0.5, u.shape).copy()
    return u, v


def blob(lon, lat, nlev, qbg, qamp):
    """blob (:160-181): background plus a sharp-flanked bump at the equator."""
    r2 = (lon[None, :] - np.pi) ** 2 + (lat[:, None] ** 2) * 4.0
    return np.broadcast_to(qbg + qamp * np.exp(-r2 * 6.0), (nlev, len(lat), len(lon))).copy()


def smooth_bell(lon, lat, nlev):
    """smooth_bell (:360-384): a broad cos^2 bell on the equator."""
    r = np.sqrt((lon[None, :] - np.pi) ** 2 + lat[:, None] ** 2)
    q = np.where(r < 1.2, 0.01 * np.cos(r / 1.2 * 0.5 * np.pi) ** 2, 0.0)
    return np.broadcast_to(q, (nlev, len(lat), len(lon))).copy()
