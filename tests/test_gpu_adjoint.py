"""Differentiation form: hand-written adjoints through the C-ABI.

* Transform adjoint pairs: exact dot-product tests <A x, y> = <x, A^T y>
  (relative bar 1e-12).
* One step (aeros_dyn_step_ad) at the start-up step and at a regular step:
  <y, J dx> from central differences of the forward step against <J^T y, dx>
  (relative bar 1e-6; the differences themselves are good to ~1e-9).
* The checkpointed window pair (aeros_dyn_window_forward/_backward): gradient
  of the window-mean kinetic energy with respect to the initial temperature,
  k_a and dT_y against central finite differences over an epsilon sweep
  (relative bar 1e-6), at T21L8 (24 steps, checkpoints every 6) and at the
  T42L20 window of 96 steps with checkpoints every 12.
"""
import numpy as np
import pytest

from tests._helpers import red_spectrum

pytestmark = pytest.mark.gpu


def ip_s(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.sum(a.real * b.real + a.imag * b.imag))


def ip_g(a, b):
    return float(np.sum(np.asarray(a) * np.asarray(b)))


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("T", [21, 42, 85])
def test_transform_adjoint_dot(gpulib, T):
    from aeros_gb300.spectral import AerosSHT
    h = AerosSHT(T, batch_max=4)
    rng = np.random.default_rng(T)
    L, M = h.l_of_lm, h.m_of_lm
    c = red_spectrum(rng, L, M, (3,), slope=-1.0)
    d = red_spectrum(rng, L, M, (3,), slope=-1.0)
    g1 = rng.standard_normal((3, h.nlat, h.nlon))
    g2 = rng.standard_normal((3, h.nlat, h.nlon))
    errs = {
        "synthesis": rel(ip_g(h.synthesis(c), g1), ip_s(c, h.synthesis_ad(g1))),
        "analysis": rel(ip_s(h.analysis(g1), d), ip_g(g1, h.analysis_ad(d))),
    }
    a, b = h.synthesis_vec(c, d)
    s, t = h.synthesis_vec_ad(g1, g2)
    errs["synthesis_vec"] = rel(ip_g(a, g1) + ip_g(b, g2), ip_s(c, s) + ip_s(d, t))
    s, t = h.analysis_vec(g1, g2)
    a, b = h.analysis_vec_ad(c, d)
    errs["analysis_vec"] = rel(ip_s(s, c) + ip_s(t, d), ip_g(g1, a) + ip_g(g2, b))
    print(f"T{T} dot-product tests", {k: f"{v:.1e}" for k, v in errs.items()})
    assert max(errs.values()) < 1e-12


def adjoint_initial_state(dyn, seed=2):
    """Seeded spun-up-like state: red-spectrum vorticity (amplitude 1e-5/l^2
    s^-1), divergence 0.2 of that, temperature 1 K/l about 264 K."""
    rng = np.random.default_rng(seed)
    from aeros_gb300.spectral import AerosSHT
    s = AerosSHT(dyn.params.trunc, batch_max=1)
    L, M = s.l_of_lm, s.m_of_lm
    dyn.set_isothermal(264.0, 1.0e5)
    _, _, t, lnps = dyn.get_state()
    vor = 1e-5 * red_spectrum(rng, L, M, (dyn.nlev,), slope=-2.0)
    div = 0.2 * 1e-5 * red_spectrum(rng, L, M, (dyn.nlev,), slope=-2.0)
    vor[:, 0] = 0
    div[:, 0] = 0
    t = t + red_spectrum(rng, L, M, (dyn.nlev,), slope=-1.0)
    return vor, div, t, lnps


def _weights(dyn, rng):
    """Random adjoint inputs / directions scaled to each field's magnitude."""
    from aeros_gb300.spectral import AerosSHT
    s = AerosSHT(dyn.params.trunc, batch_max=1)
    L, M = s.l_of_lm, s.m_of_lm
    f = lambda sc, shape: sc * red_spectrum(rng, L, M, shape, slope=-1.0)
    return f, (dyn.nlev,)


def _step_pair(nstep, nlev=8):
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    p = held_suarez_params(trunc=21, nlev=nlev)
    return AerosDyn(p)


# 40 levels: the 64-level column adjoint and the two-levels-per-lane spectral adjoint
@pytest.mark.parametrize("nstep,nlev", [(0, 8), (5, 8), (5, 40)])
def test_step_adjoint_fd(gpulib, nstep, nlev):
    dyn = _step_pair(nstep, nlev)
    rng = np.random.default_rng(11 + nstep)
    x_now = adjoint_initial_state(dyn, seed=3)
    f, sh = _weights(dyn, rng)
    x_old = tuple(a + b for a, b in zip(x_now, (f(1e-6, sh), f(2e-7, sh), f(0.1, sh), f(1e-3, ()))))
    dyn.set_state(*x_now)
    dyn.step(1)
    mt = dyn.counters()[1]

    def setup(old, now):
        dyn.set_state(*now)
        if nstep > 0:
            dyn.set_old_state(*old, nstep)
            dyn.set_mass_target(mt)
        else:
            dyn.set_mass_target(-1.0)

    def fwd(old, now):
        setup(old, now)
        dyn.step(1)
        return dyn.pack(*dyn.get_old_state()), dyn.pack(*dyn.get_state())

    # adjoint inputs, weighted so that every field contributes
    yo = dyn.pack(f(1e5, sh), f(5e5, sh), f(1.0, sh), f(100.0, ()))
    yn = dyn.pack(f(1e5, sh), f(5e5, sh), f(1.0, sh), f(100.0, ()))
    setup(x_old, x_now)
    xo_b, xn_b, ka_b, dty_b = dyn.step_ad(yo, yn)
    d_old = (f(1e-6, sh), f(2e-7, sh), f(0.1, sh), f(1e-3, ()))
    d_now = (f(1e-6, sh), f(2e-7, sh), f(0.1, sh), f(1e-3, ()))
    ad = ip_s(xo_b, dyn.pack(*d_old)) + ip_s(xn_b, dyn.pack(*d_now))
    best = np.inf
    for eps in (1e-3, 1e-4, 1e-5):
        op, np_ = fwd(tuple(a + eps * b for a, b in zip(x_old, d_old)), tuple(a + eps * b for a, b in zip(x_now, d_now)))
        om, nm = fwd(tuple(a - eps * b for a, b in zip(x_old, d_old)), tuple(a - eps * b for a, b in zip(x_now, d_now)))
        fd = (ip_s(yo, op - om) + ip_s(yn, np_ - nm)) / (2 * eps)
        best = min(best, rel(fd, ad))
    print(f"step adjoint at nstep={nstep}: <J^T y, dx> = {ad:.6e}, best FD relative error {best:.2e}")
    assert best < 1e-6
    if nstep == 0:   # the start-up step copies now into old: the old slot has no influence
        assert np.max(np.abs(xo_b)) == 0.0


def _window_case(trunc, nlev, nsteps, every, seed=2):
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    dyn = AerosDyn(held_suarez_params(trunc=trunc, nlev=nlev))
    x0 = adjoint_initial_state(dyn, seed=seed)

    def J(state, ka=None, dty=None):
        dyn.set_member_forcing(0, dyn.params.hs_dt_y if dty is None else dty,
                               dyn.params.hs_k_a if ka is None else ka)
        dyn.set_mass_target(-1.0)
        dyn.set_state(*state)
        return float(dyn.window_forward(nsteps, every)[0])

    j0 = J(x0)
    now_b, old_b, ka_b, dty_b = dyn.window_backward()
    return dyn, x0, J, j0, now_b, ka_b[0], dty_b[0]


def _check_window(trunc, nlev, nsteps, every):
    dyn, x0, J, j0, now_b, ka_b, dty_b = _window_case(trunc, nlev, nsteps, every)
    rng = np.random.default_rng(5)
    f, sh = _weights(dyn, rng)
    dT = f(1.0, sh)
    vb, db, tb, pb = dyn.unpack(now_b)
    ad_T = ip_s(tb, dT)
    res = {}
    best = np.inf
    for eps in (1e-2, 1e-3, 1e-4):
        jp = J((x0[0], x0[1], x0[2] + eps * dT, x0[3]))
        jm = J((x0[0], x0[1], x0[2] - eps * dT, x0[3]))
        best = min(best, rel((jp - jm) / (2 * eps), ad_T))
    res["T0"] = best
    ka0, dty0 = dyn.params.hs_k_a, dyn.params.hs_dt_y
    best = np.inf
    for r in (1e-3, 1e-4, 1e-5):
        e = r * ka0
        best = min(best, rel((J(x0, ka=ka0 + e) - J(x0, ka=ka0 - e)) / (2 * e), ka_b))
    res["k_a"] = best
    best = np.inf
    for e in (1e-1, 3e-2, 1e-2, 3e-3, 1e-3):
        best = min(best, rel((J(x0, dty=dty0 + e) - J(x0, dty=dty0 - e)) / (2 * e), dty_b))
    res["dT_y"] = best
    print(f"T{trunc}L{nlev} window {nsteps} steps (checkpoints every {every}): J = {j0:.6e} J; "
          f"dJ/dT0.dT = {ad_T:.4e}, dJ/dk_a = {ka_b:.4e}, dJ/ddT_y = {dty_b:.4e}; "
          "best FD relative errors", {k: f"{v:.1e}" for k, v in res.items()})
    assert max(res.values()) < 1e-6


def test_window_gradient_small(gpulib):
    _check_window(21, 8, 24, 6)


def test_window_gradient_many_levels(gpulib):
    _check_window(21, 40, 12, 4)


def test_window_gradient_T42L20(gpulib):
    _check_window(42, 20, 96, 12)
