"""CPU known-answer tests of the oracle, ported from the reference's own tests
(tests/test_spectral.f90, test_vordiv.f90, test_tendency.f90,
test_semiimp.f90, test_held_suarez.f90, test_timestep.f90, test_restart.f90)
plus the golden fixtures of tests/golden (numpy / scipy, independent code).
These pin the oracle before it is used as the GPU path's checker.
"""
import os

import numpy as np
import pytest

from tests._helpers import spectrum_test, red_spectrum, relerr

A = 6.371e6
EPS20 = 20 * np.finfo(float).eps
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def o21():
    from oracle.pyoracle import OracleSHT
    return OracleSHT(21)


# ---------------------------------------------------------------- grid, indexing
@pytest.mark.parametrize("T,grid", [(21, (64, 32)), (31, (96, 48)), (42, (128, 64)), (85, (256, 128)),
                                    (170, (512, 256)), (341, (1024, 512))])
def test_grid_size(T, grid):
    """src/aeros_spectral.f90:399-458; tests/test_spectral.f90:42-46."""
    from oracle.pyoracle import grid_size
    nlon, nlat = grid_size(T)
    assert (nlon, nlat) == grid
    assert nlon >= 3 * T + 1 and nlat == nlon // 2


def test_lm_table(o21):
    """tests/test_spectral.f90:48-68: m-major index, -1 outside the truncation."""
    s = o21
    assert s.nlm == 22 * 23 // 2
    for m in range(s.trunc + 1):
        for l in range(m, s.trunc + 1):
            lm = s.lm(l, m)
            assert s.l_of_lm[lm] == l and s.m_of_lm[lm] == m
    assert s.lm(s.trunc + 1, 0) == -1


# ---------------------------------------------------------------- golden fixtures
@pytest.mark.parametrize("n", [32, 48, 64, 128, 256, 512])
def test_gauss_nodes_against_numpy(n):
    from oracle.pyoracle import OracleSHT
    g = np.load(os.path.join(GOLD, f"gauss_{n}.npz"))
    T = {32: 21, 48: 31, 64: 42, 128: 85, 256: 170, 512: 341}[n]
    if n > 128:
        pytest.importorskip("numpy")
    s = OracleSHT(T)
    # fixture: 40-digit Newton (mpmath), rounded; agreement to the last bit
    assert np.max(np.abs(s.sinlat - g["x"])) <= 2.3e-16
    assert np.max(np.abs(s.gauss_w - g["w"])) <= 2.8e-17
    assert abs(s.gauss_w.sum() - 2.0) < 1e-14


@pytest.mark.parametrize("T", [21, 42])
def test_legendre_against_scipy(T):
    """Pbar_l^m (orthonormal, no Condon-Shortley phase) = scipy's Y_lm scaled."""
    from oracle.pyoracle import OracleSHT
    g = np.load(os.path.join(GOLD, f"plm_T{T}.npz"))
    s = OracleSHT(T)
    P, dP = s.tables()
    nh = s.nlat // 2
    assert np.max(np.abs(s.sinlat[:nh] - g["x"])) <= 2.3e-16
    assert np.max(np.abs(P[:, :nh] - g["P"])) < 2e-13      # scipy's own error ~1e-13
    # dPbar/dtheta against a centred difference of scipy's Pbar in theta
    from scipy.special import sph_harm_y
    th = np.arccos(s.sinlat[:4])
    h = 1e-6
    for lm in range(0, s.nlm, 37):
        l, m = int(s.l_of_lm[lm]), int(s.m_of_lm[lm])
        f = lambda t: np.real(sph_harm_y(l, m, t, 0.0)) * np.sqrt(2 * np.pi) * (-1.0) ** m
        fd = (f(th + h) - f(th - h)) / (2 * h)
        assert np.max(np.abs(dP[lm, :4] - fd)) < 1e-7 * max(1.0, np.max(np.abs(fd)))


def test_fourier_synthesis_against_direct_sum(o21):
    """SHTns real-field synthesis written out with numpy exp (no FFT)."""
    g = np.load(os.path.join(GOLD, "fourier.npz"))
    f = o21.synthesis(g["coeffs"])
    assert relerr(f, g["field"]) < 1e-13


# ---------------------------------------------------------------- transforms
def test_spectral_kats(o21):
    """tests/test_spectral.f90:70-124 and 174-207."""
    s = o21
    c = spectrum_test(s.l_of_lm, s.m_of_lm)
    assert relerr(s.analysis(s.synthesis(c)), c) < EPS20
    one = np.ones((s.nlat, s.nlon))
    assert abs(s.surface_integral(one) / (4 * np.pi * A * A) - 1) < EPS20
    y10 = np.zeros(s.nlm, complex)
    y10[s.lm(1, 0)] = 1
    assert abs(s.surface_integral(s.synthesis(y10))) / (4 * np.pi * A * A) < EPS20
    lap = s.laplacian(c)
    ll = s.l_of_lm * (s.l_of_lm + 1.0)
    assert np.max(np.abs(lap - c * (-ll / A ** 2))) == 0.0
    c0 = c.copy()
    c0[0] = 0
    assert relerr(s.laplacian(lap, inverse=True), c0) < 1e-12
    S = c.copy()
    S[0] = 0
    s2, t2 = s.analysis_vec(*s.synthesis_vec(S, S))
    assert max(relerr(s2, S), relerr(t2, S)) < EPS20


def test_measured_signs(o21):
    """src/dynamics/aeros_vordiv.f90:36-42: T_10 = 1 gives V_phi = +N sin(theta),
    S_10 = 1 gives V_theta = -N sin(theta), N = sqrt(3/4pi)."""
    s = o21
    N = np.sqrt(3 / (4 * np.pi))
    e = np.zeros(s.nlm, complex)
    e[s.lm(1, 0)] = 1
    z = np.zeros(s.nlm, complex)
    st = np.sqrt(1 - s.sinlat ** 2)[:, None]
    vth, vph = s.synthesis_vec(z, e)
    assert np.max(np.abs(vph - N * st)) < 1e-15 and np.max(np.abs(vth)) < 1e-15
    vth, vph = s.synthesis_vec(e, z)
    assert np.max(np.abs(vth + N * st)) < 1e-15


def test_solid_body_rotation(o21):
    """tests/test_vordiv.f90:59-143."""
    s = o21
    u0 = 40.0
    u = u0 * np.sqrt(1 - s.sinlat ** 2)[:, None] * np.ones((1, s.nlon))
    vor, div = s.vordiv_from_uv(u, np.zeros_like(u))
    expect = (2 * u0 / A) / np.sqrt(3 / (4 * np.pi))
    tol = 1e3 * np.finfo(float).eps          # tests/test_vordiv.f90:36
    assert abs(vor[s.lm(1, 0)].real - expect) / expect < tol
    assert np.max(np.abs(div)) / expect < tol
    z = s.synthesis(vor)
    assert np.max(np.abs(z - (2 * u0 / A) * s.sinlat[:, None])) / (2 * u0 / A) < tol
    assert z[0, 0] > 0 and z[-1, 0] < 0


def test_vordiv_round_trip_and_l0_discard(o21):
    """tests/test_vordiv.f90:145-289: channel separation, l = 0 discarded exactly."""
    s = o21
    l, m = s.l_of_lm, s.m_of_lm
    amp = np.where(l > 0, 1e-5 / np.maximum(l, 1) ** 2, 0.0)
    vor = amp * np.cos(3 * l + m) + 1j * amp * np.sin(l + 2 * m)
    div = 0.3 * amp * np.sin(l + m) + 0.3j * amp * np.cos(2 * l + m)
    vor[m == 0] = vor[m == 0].real
    div[m == 0] = div[m == 0].real
    v2, d2 = s.vordiv_from_uv(*s.uv_from_vordiv(vor, div))
    sc = max(np.max(np.abs(vor)), np.max(np.abs(div)))
    assert np.max(np.abs(v2 - vor)) / sc < 1e3 * np.finfo(float).eps
    assert np.max(np.abs(d2 - div)) / sc < 1e3 * np.finfo(float).eps
    vor0 = vor.copy()
    vor0[0] = 5.0
    u1, v1 = s.uv_from_vordiv(vor0, div)
    u2, v2_ = s.uv_from_vordiv(vor, div)
    assert np.array_equal(u1, u2) and np.array_equal(v1, v2_)
    # pure divergence: no vorticity
    v3, d3 = s.vordiv_from_uv(*s.uv_from_vordiv(np.zeros_like(div), div))
    assert np.max(np.abs(v3)) / np.max(np.abs(div)) < 1e3 * np.finfo(float).eps


# ---------------------------------------------------------------- Held-Suarez
def test_held_suarez_formulas():
    """tests/test_held_suarez.f90:88-172."""
    from oracle.pyoracle import hs_teq, hs_kt, hs_kv
    from aeros_gb300.params import held_suarez_params
    p = held_suarez_params()
    kappa = 287.05 / 1004.64
    assert abs(hs_teq(p, 1e5, 0.0, 1.0) - 315.0) < 1e-12
    assert abs(hs_teq(p, 1e5, 1.0, 0.0) - 255.0) < 1e-12
    expect = (315.0 - 60.0 * 0.5 - 10.0 * np.log(0.5) * 0.5) * 0.5 ** kappa
    assert abs(hs_teq(p, 0.5e5, 0.5, 0.5) - expect) < 1e-12
    assert abs(hs_teq(p, 1e3, 0.0, 1.0) - 200.0) < 1e-12
    assert abs(hs_kt(p, 1.0, 1.0) - p.hs_k_s) < 1e-18
    assert abs(hs_kt(p, 0.5, 1.0) - p.hs_k_a) < 1e-18
    assert abs(hs_kt(p, 1.0, 0.0) - p.hs_k_a) < 1e-18
    assert hs_kv(p, 0.5) == 0.0 and hs_kv(p, 0.7) == 0.0
    assert abs(hs_kv(p, 1.0) - p.hs_k_f) < 1e-18
    assert abs(hs_kv(p, 0.85) - 0.5 * p.hs_k_f) < 1e-18
    assert abs(1 / (p.hs_k_a * 86400) - 40) < 1e-12 and abs(1 / (p.hs_k_s * 86400) - 4) < 1e-12


# ---------------------------------------------------------------- tendencies
def _rest(o, s, topography, tiso=280.0):
    """tests/test_tendency.f90:164-213: isothermal rest state in discrete
    hydrostatic balance with its surface geopotential."""
    o.set_isothermal(tiso, 1e5)
    vor, div, t, lnps = o.get_state()
    if topography:
        lnps = lnps.copy()
        lnps[s.lm(2, 1)] = -0.06 + 0.03j
        lnps[s.lm(3, 0)] = 0.05
        lnps[s.lm(5, 3)] = 0.02 - 0.01j
    o.set_state(vor, div, t, lnps)
    phis = 287.05 * tiso * (np.log(1e5) - s.synthesis(lnps))
    o.set_phis(phis)
    return phis


# aeros_vgrid_init defaults (src/dynamics/aeros_vertical.f90:165-170) and the
# pure-sigma, zero-top variant of tests/test_tendency.f90:73,94
VG_DEFAULT = dict(stretch_a=0.4, stretch_r=2.0, sigma_t=0.2, p_top=1000.0)
VG_SIGMA0 = dict(stretch_a=0.4, stretch_r=2.0, sigma_t=0.0, p_top=0.0)


@pytest.mark.parametrize("label,kw,topo,tol,kmin", [
    ("flat, pure sigma", VG_SIGMA0, False, 1e-12, 0),
    ("topography, hybrid (default)", VG_DEFAULT, True, 1e-9, 0),
    ("topography, pure sigma, p_top = 0", VG_SIGMA0, True, 1e-9, 1),
])
def test_rest_state_tendencies_vanish(label, kw, topo, tol, kmin):
    """tests/test_tendency.f90:77-107.  The divergence and vorticity
    tendencies are scaled by max|Phi + K| / a^2 over the column (the reference
    reads its scale from the Phi + K array after the analysis has overwritten
    it, so its exact value is not reproducible)."""
    from oracle.pyoracle import OracleDyn, OracleSHT
    from aeros_gb300.params import held_suarez_params
    p = held_suarez_params(trunc=21, nlev=12, held_suarez=0, **kw)
    o, s = OracleDyn(p), OracleSHT(21)
    _rest(o, s, topo)
    ek = o.grid_rhs()[2]
    dscale = max(np.max(np.abs(ek)), 1.0) / A ** 2
    tv, td, tt, tp = o.tendency()
    assert np.max(np.abs(tv[kmin:])) / dscale < tol, label
    assert np.max(np.abs(td[kmin:])) / dscale < tol, label
    assert np.max(np.abs(tt[kmin:])) / 280.0 < tol, label
    assert np.max(np.abs(tp)) < tol, label


def reference_moving_state(o, s, tiso=280.0):
    """The sheared rotational flow of tests/test_tendency.f90:320-350."""
    nlev, nlm = o.nlev, o.nlm
    y00 = np.sqrt(4 * np.pi)
    vor = np.zeros((nlev, nlm), complex)
    div = np.zeros((nlev, nlm), complex)
    temp = np.zeros((nlev, nlm), complex)
    lnps = np.zeros(nlm, complex)
    lnps[s.lm(0, 0)] = np.log(1e5) * y00
    lnps[s.lm(2, 1)] = -0.03 + 0.01j
    for k in range(1, nlev + 1):
        temp[k - 1, s.lm(0, 0)] = tiso * y00
        temp[k - 1, s.lm(2, 0)] = -20.0 * k / nlev
        for lm in range(nlm):
            l, m = int(s.l_of_lm[lm]), int(s.m_of_lm[lm])
            if l < 1 or l > 6:
                continue
            amp = 1e-5 / (l * l) * (0.5 + 0.5 * k / nlev)
            vor[k - 1, lm] = amp * np.cos(3 * l + m) + 1j * amp * np.sin(l + 2 * m)
            div[k - 1, lm] = 0.2 * amp * np.sin(l + m) + 0.2j * amp * np.cos(2 * l + m)
            if m == 0:
                vor[k - 1, lm] = vor[k - 1, lm].real
                div[k - 1, lm] = div[k - 1, lm].real
    return vor, div, temp, lnps


def test_moving_state_conserves_mass():
    """tests/test_tendency.f90:303-396: the global mass tendency vanishes."""
    from oracle.pyoracle import OracleDyn, OracleSHT
    from aeros_gb300.params import held_suarez_params
    p = held_suarez_params(trunc=21, nlev=12, held_suarez=0, **VG_SIGMA0)
    o, s = OracleDyn(p), OracleSHT(21)
    o.set_state(*reference_moving_state(o, s))
    u = o.diagnose()[0]
    assert 1.0 < np.max(np.abs(u)) < 150.0
    dlnpsdt = o.grid_rhs()[4]
    ps = o.diagnose()[3]
    rate = s.surface_integral(ps * dlnpsdt)
    scale = s.surface_integral(np.abs(ps * dlnpsdt))
    assert abs(rate) / scale < 1e-12


# ---------------------------------------------------------------- semi-implicit
def test_gravity_wave_speed():
    """tests/test_semiimp.f90:73-111: external mode within 5% of sqrt(gamma R T),
    coordinate-independent to 1%."""
    from oracle.pyoracle import OracleDyn
    from aeros_gb300.params import held_suarez_params
    c_lamb = np.sqrt(1004.64 / (1004.64 - 287.05) * 287.05 * 300.0)
    c_sig = OracleDyn(held_suarez_params(trunc=21, nlev=20)).gwspeed()
    c_hyb = OracleDyn(held_suarez_params(trunc=21, nlev=20, stretch_a=0.4, sigma_t=0.2)).gwspeed()
    assert abs(c_hyb - c_lamb) / c_lamb < 0.05
    assert abs(c_hyb - c_sig) / c_sig < 0.01


def test_linear_operator_matches_finite_difference():
    """tests/test_semiimp.f90:167-289: L = dR about the reference rest state."""
    from oracle.pyoracle import OracleDyn, OracleSHT
    from aeros_gb300.params import held_suarez_params
    p = held_suarez_params(trunc=21, nlev=20, stretch_a=0.4, sigma_t=0.2, held_suarez=0)
    o, s = OracleDyn(p), OracleSHT(21)
    o.set_isothermal(-1, -1)                      # t_ref, ps_ref
    base = [x.copy() for x in o.get_state()]
    t0 = o.tendency()
    assert np.max(np.abs(t0[1])) < 1e-18
    l0 = o.si_linear()
    lm = s.lm(3, 2)

    def rel(a, b):
        return np.max(np.abs(a - b)) / np.max(np.abs(b))

    k = np.arange(1, 21)
    pert = [x.copy() for x in base]
    pert[2][:, lm] += 1e-2 * np.cos(k) + 0.6e-2j * np.sin(2 * k)
    o.set_state(*pert)
    t1, l1 = o.tendency(), o.si_linear()
    assert rel(t1[1] - t0[1], l1[0] - l0[0]) < 1e-6
    assert np.max(np.abs(t1[2] - t0[2])) < 1e-15
    assert np.max(np.abs(t1[3] - t0[3])) < 1e-18
    pert = [x.copy() for x in base]
    pert[3][lm] += 2e-5 - 1e-5j
    o.set_state(*pert)
    t1, l1 = o.tendency(), o.si_linear()
    assert rel(t1[1] - t0[1], l1[0] - l0[0]) < 1e-6
    assert np.max(np.abs(t1[2] - t0[2])) < 1e-15
    pert = [x.copy() for x in base]
    pert[1][:, lm] += 1e-9 * np.cos(k) + 0.7e-9j * np.sin(3 * k)
    o.set_state(*pert)
    t1, l1 = o.tendency(), o.si_linear()
    assert rel(t1[2] - t0[2], l1[1] - l0[1]) < 1e-6
    assert rel(t1[3] - t0[3], l1[2] - l0[2]) < 1e-9


# ---------------------------------------------------------------- integrator
def test_rest_state_holds():
    """tests/test_timestep.f90:232-285: a resting atmosphere stays at rest."""
    from oracle.pyoracle import OracleDyn
    from aeros_gb300.params import held_suarez_params
    p = held_suarez_params(trunc=21, nlev=12, held_suarez=0, mass_fixer=0)
    o = OracleDyn(p)
    o.set_isothermal(280.0, 1e5)
    o.step(100)
    u, v, t, ps = o.diagnose()
    assert max(np.max(np.abs(u)), np.max(np.abs(v))) < 1e-3       # m/s
    assert np.max(np.abs(ps - 1e5)) < 1e-2                          # Pa
    assert np.max(np.abs(t - 280.0)) < 1e-4                         # K


def test_hyperdiffusion_decay_of_a_zonal_mode():
    """del^6 implicit diffusion (src/dynamics/aeros_timestep.f90:1673-1726):
    a zonal vorticity mode has no dynamical tendency, so the start-up step
    divides it by exactly 1 + (dt/tau) (l(l+1)/(T(T+1)))^3."""
    from oracle.pyoracle import OracleDyn, OracleSHT
    from aeros_gb300.params import held_suarez_params
    p = held_suarez_params(trunc=21, nlev=12, held_suarez=0, mass_fixer=0)
    o, s = OracleDyn(p), OracleSHT(21)
    o.set_isothermal(280.0, 1e5)
    vor, div, t, lnps = o.get_state()
    for l in (5, 21):
        vor = np.zeros_like(vor)
        vor[:, s.lm(l, 0)] = 1e-9
        o.set_state(vor, div, t, lnps)
        o.step(1)
        fac = 1.0 / (1.0 + (1800.0 / (6 * 3600.0)) * (l * (l + 1.0) / (21 * 22.0)) ** 3)
        assert relerr(o.get_state()[0][:, s.lm(l, 0)], vor[:, s.lm(l, 0)] * fac) < 1e-12


def test_mass_fixer_restores_target():
    """src/dynamics/aeros_timestep.f90:1225-1276: mass after each fixed step
    equals the captured target."""
    from oracle.pyoracle import OracleDyn
    from aeros_gb300.params import held_suarez_params
    from tests.test_gpu_dyn import moving_state
    o = OracleDyn(held_suarez_params(trunc=21, nlev=12))
    o.set_state(*moving_state(o, seed=8))
    m0 = o.budget()[0]
    o.step(5)
    n, target, lnr_last, lnr_cum = o.counters()
    assert n == 5 and abs(target - m0) / m0 < 1e-14
    assert abs(o.budget()[0] - target) / target < 1e-13


def test_restart_split_run_bitwise():
    """tests/test_restart.f90:1-43 on the oracle."""
    from oracle.pyoracle import OracleDyn
    from aeros_gb300.params import held_suarez_params
    from tests.test_gpu_dyn import moving_state
    p = held_suarez_params(trunc=21, nlev=12)
    a = OracleDyn(p)
    st = moving_state(a, seed=9)
    a.set_state(*st)
    a.step(6)
    b = OracleDyn(p)
    b.set_state(*st)
    b.step(3)
    now, old = b.get_state(), b.get_old_state()
    n, mt, _, _ = b.counters()
    c = OracleDyn(p)
    c.set_state(*now)
    c.set_old_state(*old, n)
    c.set_mass_target(mt)
    c.step(3)
    for x, y in zip(c.get_state(), a.get_state()):
        assert np.array_equal(x, y)


def test_hs_perturb_formula():
    """aeros_hs_perturb (src/physics/aeros_held_suarez.f90:295-336): T_lm,k +=
    amp (cos(3l + 5m + k), sin(7l + 2m + 3k)) for m = 1..min(8, T),
    l = m..min(m+4, T), k = 1..nlev, added to the isothermal state."""
    from oracle.pyoracle import OracleDyn
    from aeros_gb300.params import held_suarez_params
    T, nlev, amp = 21, 5, 0.7
    o = OracleDyn(held_suarez_params(trunc=T, nlev=nlev))
    o.set_isothermal(264.0, 1.0e5)
    _, _, t0, _ = o.get_state()
    o.hs_perturb(amp)
    _, _, t1, _ = o.get_state()
    exp = t0.copy()
    for k in range(1, nlev + 1):
        for m in range(1, min(8, T) + 1):
            for l in range(m, min(m + 4, T) + 1):
                lm = m * (2 * T + 1 - m) // 2 + l
                exp[k - 1, lm] += amp * np.cos(3 * l + 5 * m + k) + 1j * amp * np.sin(7 * l + 2 * m + 3 * k)
    assert np.array_equal(t1, exp)


def _exact_half_time(time_init, k, dt):
    """A time t [yr] with (t - time_init) * year_seconds / dt == k + 0.5 exactly."""
    from oracle.pyoracle import YEAR_SECONDS
    t = time_init + (k + 0.5) * dt / YEAR_SECONDS
    for _ in range(64):
        x = (t - time_init) * YEAR_SECONDS / dt
        if x == k + 0.5:
            return t
        t = np.nextafter(t, np.inf if x < k + 0.5 else -np.inf)
    raise AssertionError("no exactly-half time found")


def test_update_step_count_rule():
    """aeros_update (src/aeros.f90:202-241): n_target = nint((t - t0) yr / dt),
    halves away from zero, steps only forward, refuses an earlier time."""
    from oracle.pyoracle import OracleClock, YEAR_SECONDS
    dt = 1800.0
    step = dt / YEAR_SECONDS
    c = OracleClock(dt, time_init=0.0)
    assert c.update(0.0) == 0 and c.nstep == 0
    assert c.update(2.49 * step) == 2 and c.nstep == 2
    t_half = _exact_half_time(0.0, 2, dt)
    assert c.update(t_half) == 1 and c.nstep == 3          # 2.5 -> 3
    assert c.update(3.49 * step) == 0 and c.nstep == 3
    assert c.update(10.0 * step) == 7 and c.nstep == 10
    with pytest.raises(ValueError):
        c.update(0.0)
    assert c.nstep == 10
    c = OracleClock(dt, time_init=0.25)                       # aeros_init's time_init
    assert c.update(0.25 + 1.2 * step) == 1 and c.nstep == 1


def test_timing_build_matches_parity_build():
    """The CPU baseline times the oracle's -ffp-contract=fast build; it computes
    the same steps as the parity build (fused multiply-adds change the last bits
    only)."""
    import oracle.pyoracle as po
    from aeros_gb300.params import held_suarez_params
    p = held_suarez_params(trunc=21, nlev=8)
    out = []
    for variant in ("fast", "parity"):
        po.use_variant(variant)
        o = po.OracleDyn(p)
        o.set_isothermal(264.0, 1.0e5)
        o.hs_perturb(1.0)
        o.step(4)
        out.append(o.get_state())
    po.use_variant("parity")
    for a, b in zip(*out):
        assert np.max(np.abs(a - b)) <= 1e-11 * np.max(np.abs(b))


def test_truth_chain_is_the_oracle_chain():
    """oracle/truth.cpp restates the tendency chain independently; in double it
    agrees with the oracle to round-off, and the oracle lies within the FP64
    round-off of the long double evaluation (1e-12 except the divergence, whose
    cancellation leaves the oracle ~1e-11 from it at T42L20)."""
    from oracle.pyoracle import OracleDyn, OracleSHT, truth_tendency
    from aeros_gb300.params import held_suarez_params
    for T, nl in ((21, 12), (42, 20)):
        p = held_suarez_params(trunc=T, nlev=nl)
        o, s = OracleDyn(p), OracleSHT(T)
        rng = np.random.default_rng(5)
        L, M = s.l_of_lm.astype(float), s.m_of_lm

        def red(shape, amp):
            x = (rng.standard_normal(shape + (len(L),)) + 1j * rng.standard_normal(shape + (len(L),))) * amp / (L + 1)
            x[..., M == 0] = x[..., M == 0].real
            return x
        o.set_isothermal(264.0, 1.0e5)
        _, _, t, lnps = o.get_state()
        vor, div = red((nl,), 1e-5), red((nl,), 2e-6)
        vor[:, 0] = div[:, 0] = 0
        st = (vor, div, t + red((nl,), 1.0), lnps + red((), 0.01))
        o.set_state(*st)
        for forced in (False, True):
            to = o.tendency(forced=forced)
            td = truth_tendency(p, s.nlon, s.nlat, o.A, o.B, st, forced=forced, wide=False)
            tw = truth_tendency(p, s.nlon, s.nlat, o.A, o.B, st, forced=forced, wide=True)
            for i in range(4):
                bar = 5e-11 if i == 1 else 1e-12
                assert relerr(to[i], tw[i]) < bar, (T, forced, i)
                assert relerr(td[i], tw[i]) < bar, (T, forced, i)
