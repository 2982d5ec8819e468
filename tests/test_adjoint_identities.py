"""The transform adjoint identities the GPU adjoints are built on, checked on
the CPU oracle (exact to rounding):
    synthesis^T = Dm analysis W^-1        analysis^T = W synthesis Dm^-1
    synthesis_vec^T = Dm L analysis_vec W^-1
    uv_from_vordiv^T = Dm a^2/L vordiv_from_uv W^-1
    vordiv_from_uv^T = W uv_from_vordiv L/a^2 Dm^-1
    (d/dx, d/dy)^T = -Dm div(vordiv_from_uv W^-1)
with W = diag(Gauss weight), Dm = diag((2 - delta_m0) nlon / 2 pi), L = diag(l(l+1)),
and the tendency analysis = vordiv_from_uv(ae, an) + L/a^2 analysis(Phi + K).
"""
import numpy as np
import pytest

from tests._helpers import red_spectrum

A = 6.371e6


def ip_s(a, b):
    return float(np.sum(a.real * b.real + a.imag * b.imag))


def ip_g(a, b):
    return float(np.sum(a * b))


@pytest.mark.parametrize("T", [21, 42])
def test_transform_adjoint_identities(T):
    from oracle.pyoracle import OracleSHT
    o = OracleSHT(T)
    L = o.l_of_lm.astype(float)
    LL = L * (L + 1)
    w = o.gauss_w[:, None]
    Dm = np.where(o.m_of_lm == 0, 1.0, 2.0) * o.nlon / (2 * np.pi)
    rng = np.random.default_rng(T)
    spec = lambda: red_spectrum(rng, o.l_of_lm, o.m_of_lm, (), slope=-1.0)
    grid = lambda: rng.standard_normal((o.nlat, o.nlon))
    errs = {}
    c, g = spec(), grid()
    x, y = ip_g(o.synthesis(c), g), ip_s(c, Dm * o.analysis(g / w))
    errs["S"] = abs(x - y) / abs(x)
    d = spec()
    x, y = ip_s(o.analysis(g), d), ip_g(g, w * o.synthesis(d / Dm))
    errs["A"] = abs(x - y) / abs(x)
    s, t, g2 = spec(), spec(), grid()
    a, b = o.synthesis_vec(s, t)
    S2, T2 = o.analysis_vec(g / w, g2 / w)
    x, y = ip_g(a, g) + ip_g(b, g2), ip_s(s, Dm * LL * S2) + ip_s(t, Dm * LL * T2)
    errs["SV"] = abs(x - y) / abs(x)
    u, v = o.uv_from_vordiv(s, t)
    zz, dd = o.vordiv_from_uv(g / w, g2 / w)
    f = np.where(L > 0, Dm * A ** 2 / np.where(L > 0, LL, 1.0), 0.0)
    x, y = ip_g(u, g) + ip_g(v, g2), ip_s(s, f * zz) + ip_s(t, f * dd)
    errs["UV"] = abs(x - y) / abs(x)
    zz, dd = o.vordiv_from_uv(g, g2)
    uu, vv = o.uv_from_vordiv(LL / A ** 2 / Dm * s, LL / A ** 2 / Dm * t)
    x, y = ip_s(zz, s) + ip_s(dd, t), ip_g(g, w * uu) + ip_g(g2, w * vv)
    errs["VD"] = abs(x - y) / abs(x)
    gx, gy = o.grad(s)
    _, dd = o.vordiv_from_uv(g / w, g2 / w)
    x, y = ip_g(gx, g) + ip_g(gy, g2), ip_s(s, -Dm * dd)
    errs["grad"] = abs(x - y) / abs(x)
    assert max(errs.values()) < 1e-13, errs


def test_tendency_analysis_structure():
    from oracle.pyoracle import OracleDyn, OracleSHT
    from aeros_gb300.params import held_suarez_params
    from tests.test_gpu_dyn import moving_state
    o = OracleDyn(held_suarez_params(trunc=21, nlev=8))
    s = OracleSHT(21)
    o.set_state(*moving_state(o, seed=3))
    ae, an, ek, dtdt, dpdt = o.grid_rhs(forced=True)
    tv, td, tt, tp = o.tendency(forced=True)
    L = s.l_of_lm.astype(float)
    zz, dd = s.vordiv_from_uv(ae, an)
    assert np.array_equal(zz, tv)
    assert np.max(np.abs(dd + L * (L + 1) / A ** 2 * s.analysis(ek) - td)) <= 1e-15 * np.max(np.abs(td))
    assert np.array_equal(s.analysis(dtdt), tt)
    assert np.array_equal(s.analysis(dpdt), tp)
