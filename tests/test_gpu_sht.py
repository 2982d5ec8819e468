"""GPU transform parity: the CUDA library (C-ABI) against the CPU oracle.

FP64 path bar: <= 1e-12 relative (max |gpu - oracle| / max |oracle|) on seeded
inputs, plus the reference's own transform known-answer tests
(tests/test_spectral.f90, tests/test_vordiv.f90) run on the GPU.
"""
import numpy as np
import pytest

from tests._helpers import spectrum_test, red_spectrum, relerr

pytestmark = pytest.mark.gpu

TOL = 1e-12
EPS20 = 20 * np.finfo(float).eps   # tests/test_spectral.f90:30


@pytest.fixture(scope="module", params=[21, 31, 42, 85])
def pair(request, gpulib):
    from aeros_gb300.spectral import AerosSHT
    from oracle.pyoracle import OracleSHT
    T = request.param
    return AerosSHT(T, batch_max=8), OracleSHT(T)


def test_geometry_matches(pair):
    g, o = pair
    assert (g.nlon, g.nlat, g.nlm) == (o.nlon, o.nlat, o.nlm)
    assert np.max(np.abs(g.sinlat - o.sinlat)) < 1e-15
    assert np.max(np.abs(g.gauss_w - o.gauss_w)) < 1e-15
    assert (g.l_of_lm == o.l_of_lm).all() and (g.m_of_lm == o.m_of_lm).all()


def test_scalar_synthesis_analysis(pair):
    g, o = pair
    rng = np.random.default_rng(11)
    c = red_spectrum(rng, o.l_of_lm, o.m_of_lm, (3,))
    fg, fo = g.synthesis(c), o.synthesis(c)
    assert relerr(fg, fo) < TOL
    cg, co = g.analysis(fo), o.analysis(fo)
    assert relerr(cg, co) < TOL


def test_vector_and_gradient(pair):
    g, o = pair
    rng = np.random.default_rng(12)
    s = red_spectrum(rng, o.l_of_lm, o.m_of_lm, (2,))
    t = red_spectrum(rng, o.l_of_lm, o.m_of_lm, (2,))
    s[:, 0] = 0
    t[:, 0] = 0
    ag, bg = g.synthesis_vec(s, t)
    ao, bo = o.synthesis_vec(s, t)
    assert relerr(ag, ao) < TOL and relerr(bg, bo) < TOL
    sg, tg = g.analysis_vec(ao, bo)
    so, to = o.analysis_vec(ao, bo)
    assert relerr(sg, so) < TOL and relerr(tg, to) < TOL
    gg = g.gradient(s)
    go = o.gradient(s)
    assert relerr(gg[0], go[0]) < TOL and relerr(gg[1], go[1]) < TOL


def test_winds(pair):
    g, o = pair
    rng = np.random.default_rng(13)
    vor = 1e-5 * red_spectrum(rng, o.l_of_lm, o.m_of_lm, (2,))
    div = 3e-6 * red_spectrum(rng, o.l_of_lm, o.m_of_lm, (2,))
    ug, vg = g.uv_from_vordiv(vor, div)
    uo, vo = o.uv_from_vordiv(vor, div)
    assert relerr(ug, uo) < TOL and relerr(vg, vo) < TOL
    zg, dg = g.vordiv_from_uv(uo, vo)
    zo, do = o.vordiv_from_uv(uo, vo)
    assert relerr(zg, zo) < TOL and relerr(dg, do) < TOL
    xg, yg = g.grad(vor)
    xo, yo = o.grad(vor)
    assert relerr(xg, xo) < TOL and relerr(yg, yo) < TOL


def test_reference_transform_kats(pair):
    """tests/test_spectral.f90 sections 3-6 on the GPU."""
    g, _ = pair
    c = spectrum_test(g.l_of_lm, g.m_of_lm)
    c2 = g.analysis(g.synthesis(c))
    assert relerr(c2, c) < EPS20
    one = np.ones((g.nlat, g.nlon))
    a = 6.371e6
    assert abs(g.surface_integral(one) - 4 * np.pi * a * a) / (4 * np.pi * a * a) < EPS20
    y10 = np.zeros(g.nlm, complex)
    y10[g.lm(1, 0) - 1] = 1.0
    assert abs(g.surface_integral(g.synthesis(y10))) / (4 * np.pi * a * a) < EPS20
    lap = g.laplacian(c)
    ll = g.l_of_lm * (g.l_of_lm + 1.0)
    assert np.max(np.abs(lap - c * (-ll / a ** 2))) == 0.0
    inv = g.laplacian(lap, inverse=True)
    c0 = c.copy()
    c0[0] = 0
    assert relerr(inv, c0) < 1e-12
    s = spectrum_test(g.l_of_lm, g.m_of_lm)
    s[0] = 0
    vs, vt = g.analysis_vec(*g.synthesis_vec(s, s))
    assert max(relerr(vs, s), relerr(vt, s)) < EPS20


def test_solid_body_rotation(pair):
    """tests/test_vordiv.f90:59-143: u = U0 cos(lat) -> zeta_10 = (2U0/a)/sqrt(3/4pi)."""
    g, _ = pair
    u0, a = 40.0, 6.371e6
    u = u0 * np.sqrt(1 - g.sinlat ** 2)[:, None] * np.ones((1, g.nlon))
    v = np.zeros_like(u)
    vor, div = g.vordiv_from_uv(u, v)
    expect = (2 * u0 / a) / np.sqrt(3 / (4 * np.pi))
    assert abs(vor[g.lm(1, 0) - 1].real - expect) / expect < EPS20
    assert np.max(np.abs(div)) / expect < EPS20
    rest = vor.copy()
    rest[g.lm(1, 0) - 1] = 0
    assert np.max(np.abs(rest)) / expect < 1e3 * np.finfo(float).eps
    zg = g.synthesis(vor)
    assert zg[0, 0] > 0 and zg[-1, 0] < 0


def test_device_pointers(pair):
    """Device-resident torch tensors go through the same C-ABI in place."""
    torch = pytest.importorskip("torch")
    g, o = pair
    rng = np.random.default_rng(14)
    c = red_spectrum(rng, o.l_of_lm, o.m_of_lm, (4,))
    cd = torch.from_numpy(c).cuda()
    fd = g.synthesis(cd)
    torch.cuda.synchronize()
    assert fd.is_cuda
    assert relerr(fd.cpu().numpy(), o.synthesis(c)) < TOL
    cb = g.analysis(fd)
    torch.cuda.synchronize()
    assert relerr(cb.cpu().numpy(), c) < 1e-13


def test_call_argument_errors(gpulib):
    """Per-call argument errors (batch outside 1..batch_max, null arrays, (l, m)
    outside the truncation, packed states of the wrong count) come back as
    status codes without device work, and the handles stay usable."""
    import ctypes
    from aeros_gb300 import _capi
    from aeros_gb300.spectral import AerosSHT
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    L = _capi.lib()
    s = AerosSHT(21, batch_max=2)
    c = np.zeros((3, s.nlm), np.complex128)
    f = np.zeros((3, s.nlat, s.nlon))

    def p(a):
        return a.ctypes.data_as(ctypes.c_void_p)

    assert L.aeros_sht_synthesis(s._h, p(c), p(f), 3) == _capi.ERR_ARG
    assert L.aeros_sht_synthesis(s._h, p(c), p(f), 0) == _capi.ERR_ARG
    assert L.aeros_sht_synthesis(s._h, None, p(f), 1) == _capi.ERR_ARG
    assert L.aeros_sht_analysis(s._h, p(f), None, 1) == _capi.ERR_ARG
    assert L.aeros_sht_lm(s._h, 0, 0) == 1
    assert L.aeros_sht_lm(s._h, 3, 4) == -1 and L.aeros_sht_lm(s._h, 22, 0) == -1
    c[0, 1] = 1.0
    assert L.aeros_sht_synthesis(s._h, p(c), p(f), 1) == _capi.OK
    assert np.abs(f[0]).max() > 0.0
    d = AerosDyn(held_suarez_params(trunc=21, nlev=12))
    x = np.zeros(d.state_size(), np.complex128)
    assert L.aeros_dyn_step_packed(d._h, None, p(x), 0, 1, None, None) == _capi.ERR_ARG
    assert L.aeros_dyn_step_packed(d._h, p(x), p(x), -1, 1, None, None) == _capi.ERR_ARG
    with pytest.raises(ValueError):
        d.step_packed(x[:-1], x, 0)
    d.set_isothermal(264.0, 1.0e5)
    d.step(1)
