"""Tracer transport on the GPU (src/dynamics/aeros_transport.f90) against the
oracle, and the reference's own checks (tests/test_transport.f90:185-358) run
through the C-ABI."""
import numpy as np
import pytest

from oracle.transport_oracle import OracleTransport
from tests._helpers import relerr
from tests._transport_cases import (P0, blob, divergent_wind, geometry, set_lnps, smooth_bell, solid_body)

pytestmark = pytest.mark.gpu
DT = 1800.0


def _pair(trunc, nlev, vl=False):
    from aeros_gb300.transport import AerosTransport
    sinlat, w, nlon, nlat, A, B, lon, lat = geometry(trunc, nlev)
    g = AerosTransport(trunc, A, B, vert_vanleer=vl)
    o = OracleTransport(sinlat, w, nlon, A, B, vert_vanleer=vl)
    assert (g.nlon, g.nlat, g.nlev) == (nlon, nlat, nlev)
    return g, o, lon, lat


def _mixed_case(lon, lat, nlev, seed):
    rng = np.random.default_rng(seed)
    u, v = divergent_wind(lon, lat, nlev, 35.0)
    u = u + solid_body(lon, lat, nlev, 25.0)[0] + rng.normal(0.0, 2.0, u.shape)
    v = v + rng.normal(0.0, 2.0, v.shape)
    q = blob(lon, lat, nlev, 0.002, 0.015) * (1.0 + 0.1 * rng.random(u.shape))
    return u, v, set_lnps(lon, lat), q


# 64 levels: the vertical kernel's largest shared-memory stage; T31: 96 longitudes, a partial
# thread block in every longitude row; 33 levels: a level count that no lane stride divides
@pytest.mark.parametrize("trunc,nlev,vl", [(21, 8, False), (42, 20, False), (21, 8, True), (21, 64, False),
                                          (21, 64, True), (31, 20, True), (21, 33, False)])
def test_matches_oracle(gpulib, trunc, nlev, vl):
    g, o, lon, lat = _pair(trunc, nlev, vl)
    u, v, lnps, q = _mixed_case(lon, lat, nlev, seed=trunc + nlev)
    qg, qo = q.copy(), q.copy()
    for n in range(6):
        qg = g.step(u, v, lnps, qg, DT)
        qo = o.transport(u, v, lnps, qo, DT)
        assert g.last()[1] == o.last_nsub
        assert abs(g.last()[0] - o.last_cfl) <= 1e-12 * o.last_cfl
        assert relerr(qg, qo) < 1e-12, n
    ps = np.exp(lnps)
    assert abs(g.water(ps, qg) - o.water(ps, qo)) <= 1e-13 * o.water(ps, qo)


def test_device_pointers_match_host(gpulib):
    import torch
    g, _, lon, lat = _pair(21, 8)
    u, v, lnps, q = _mixed_case(lon, lat, 8, seed=5)
    qh = g.step(u, v, lnps, q.copy(), DT)
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (u, v, lnps, q)]
    qd = g.step(*dev, DT)
    torch.cuda.synchronize()
    assert np.array_equal(qd.cpu().numpy(), qh)


def test_reference_checks(gpulib):
    """constancy, conservation, positivity, polar sub-stepping and accuracy, as the reference tests them."""
    g, _, lon, lat = _pair(21, 8)
    nlev, shape2 = 8, (len(lat), len(lon))
    # constancy under a divergent wind, 50 steps
    u, v = divergent_wind(lon, lat, nlev, 40.0)
    lnps = set_lnps(lon, lat)
    q = np.full(u.shape, 0.7)
    for _ in range(50):
        q = g.step(u, v, lnps, q, DT)
    assert np.max(np.abs(q - 0.7)) < 1e-13
    # conservation, 100 steps of solid-body rotation
    lnps = np.full(shape2, np.log(P0))
    ps = np.exp(lnps)
    u, v = solid_body(lon, lat, nlev, 60.0)
    q = blob(lon, lat, nlev, 0.001, 0.02)
    w0 = g.water(ps, q)
    for _ in range(100):
        q = g.step(u, v, lnps, q, DT)
    assert abs(g.water(ps, q) - w0) / w0 < 1e-13
    # positivity, 200 steps
    u, v = solid_body(lon, lat, nlev, 70.0)
    q = blob(lon, lat, nlev, 0.0, 0.02)
    qmin = q.min()
    for _ in range(200):
        q = g.step(u, v, lnps, q, DT)
        qmin = min(qmin, q.min())
    assert qmin >= 0.0
    # polar Courant: u = 80 m/s everywhere
    u = np.full((nlev,) + shape2, 80.0)
    v = np.zeros_like(u)
    q = blob(lon, lat, nlev, 0.0, 0.02)
    w0, qmin = g.water(ps, q), q.min()
    for _ in range(50):
        q = g.step(u, v, lnps, q, DT)
        qmin = min(qmin, q.min())
    assert g.last()[1] > 1
    assert abs(g.water(ps, q) - w0) / w0 < 1e-13 and qmin >= 0.0
    # accuracy: one rotation of a smooth bell keeps > 70 % of its peak
    u, v = solid_body(lon, lat, nlev, 60.0)
    q = smooth_bell(lon, lat, nlev)
    peak0 = q.max()
    for _ in range(int(np.floor(2.0 * np.pi * 6.371e6 / 60.0 / DT + 0.5))):
        q = g.step(u, v, lnps, q, DT)
    assert q.max() / peak0 > 0.70 and q.min() >= 0.0
