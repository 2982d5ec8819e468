"""The transport oracle against every check of the reference's own
tests/test_transport.f90 (T21 L8, dt = 1800 s): constancy under a divergent
wind, conservation, positivity, polar sub-stepping, peak retention."""
import numpy as np
import pytest

from oracle.transport_oracle import OracleTransport
from tests._transport_cases import (P0, blob, divergent_wind, geometry, set_lnps, smooth_bell, solid_body)

DT = 1800.0


@pytest.fixture(scope="module")
def geo():
    return geometry(21, 8)


def _mst(geo):
    sinlat, w, nlon, nlat, A, B, lon, lat = geo
    return OracleTransport(sinlat, w, nlon, A, B), lon, lat, len(A) - 1


def test_constancy(geo):
    """:185-209: q = 0.7 under a divergent wind stays 0.7 (< 1e-13 after 50 steps)."""
    mst, lon, lat, nlev = _mst(geo)
    lnps = set_lnps(lon, lat)
    u, v = divergent_wind(lon, lat, nlev, 40.0)
    q = np.full(u.shape, 0.7)
    for _ in range(50):
        q = mst.transport(u, v, lnps, q, DT)
    assert np.max(np.abs(q - 0.7)) < 1e-13


def test_conservation(geo):
    """:213-246: total water conserved to 1e-13 over 100 steps of solid-body rotation."""
    mst, lon, lat, nlev = _mst(geo)
    lnps = np.full((len(lat), len(lon)), np.log(P0))
    u, v = solid_body(lon, lat, nlev, 60.0)
    q = blob(lon, lat, nlev, 0.001, 0.02)
    w0 = mst.water(np.exp(lnps), q)
    for _ in range(100):
        q = mst.transport(u, v, lnps, q, DT)
    assert abs(mst.water(np.exp(lnps), q) - w0) / w0 < 1e-13


def test_positivity(geo):
    """:250-273: a zero-background blob never goes negative in 200 steps."""
    mst, lon, lat, nlev = _mst(geo)
    lnps = np.full((len(lat), len(lon)), np.log(P0))
    u, v = solid_body(lon, lat, nlev, 70.0)
    q = blob(lon, lat, nlev, 0.0, 0.02)
    qmin = q.min()
    for _ in range(200):
        q = mst.transport(u, v, lnps, q, DT)
        qmin = min(qmin, q.min())
    assert qmin >= 0.0


def test_polar_substep(geo):
    """:277-313: u = 80 m/s at every latitude forces sub-stepping; still conservative and positive."""
    mst, lon, lat, nlev = _mst(geo)
    lnps = np.full((len(lat), len(lon)), np.log(P0))
    u = np.full((nlev, len(lat), len(lon)), 80.0)
    v = np.zeros_like(u)
    q = blob(lon, lat, nlev, 0.0, 0.02)
    w0 = mst.water(np.exp(lnps), q)
    qmin = q.min()
    for _ in range(50):
        q = mst.transport(u, v, lnps, q, DT)
        qmin = min(qmin, q.min())
    assert mst.last_nsub > 1
    assert abs(mst.water(np.exp(lnps), q) - w0) / w0 < 1e-13
    assert qmin >= 0.0


def test_accuracy(geo):
    """:317-358: one full rotation of a smooth bell keeps > 70 % of its peak."""
    mst, lon, lat, nlev = _mst(geo)
    lnps = np.full((len(lat), len(lon)), np.log(P0))
    u0 = 60.0
    u, v = solid_body(lon, lat, nlev, u0)
    q = smooth_bell(lon, lat, nlev)
    peak0 = q.max()
    nrot = int(np.floor(2.0 * np.pi * 6.371e6 / u0 / DT + 0.5))
    for _ in range(nrot):
        q = mst.transport(u, v, lnps, q, DT)
    assert q.max() / peak0 > 0.70
    assert q.min() >= 0.0


def test_vertical_van_leer_keeps_the_invariants(geo):
    """The optional vertical van Leer reconstruction (vert_vanleer) keeps constancy."""
    sinlat, w, nlon, nlat, A, B, lon, lat = geo
    mst = OracleTransport(sinlat, w, nlon, A, B, vert_vanleer=True)
    lnps = set_lnps(lon, lat)
    u, v = divergent_wind(lon, lat, len(A) - 1, 40.0)
    q = np.full(u.shape, 0.7)
    for _ in range(20):
        q = mst.transport(u, v, lnps, q, DT)
    assert np.max(np.abs(q - 0.7)) < 1e-13
