"""GPU dynamics parity: the dry Held-Suarez step on the GPU (C-ABI) against
the CPU oracle on the same seeded inputs, and its tendencies against the
same chain evaluated in long double (oracle/truth.cpp, "truth").

Bars (max |a - b| / max |b|):
  tendencies, GPU against truth                  1e-12 for every field
  divergence tendency, GPU against truth         also no further from truth than
      the FP64 oracle is: dD/dt = div(A) - lap(Phi + K) cancels several digits,
      and the oracle (the reference's algorithm in FP64) lies 3e-12 - 1.4e-11
      from truth; the GPU analyses Phi + K less a per-level constant, which
      only the l = 0 coefficient sees (multiplied by zero in the Laplacian)
  tendencies of vorticity, temperature, ln ps,   1e-12 of max |tendency|
      GPU against oracle
  state after one step (moving state)            1e-12 for vor, T, ln ps;
                                                 1e-10 for D (carries the oracle's h dD/dt error)
  state after 10 steps                           1e-10
  mass fixer                                     target 1e-13 rel, ln r 1e-14 abs
"""
import numpy as np
import pytest

from tests._helpers import red_spectrum, relerr, truth

pytestmark = pytest.mark.gpu


def noisy_state(o, sht, temp=264.0, noise=0.1, seed=0):
    """Rest, isothermal T, ps = 1000 hPa, N(0, noise^2) K on grid T, analysed."""
    o.set_isothermal(temp, 1.0e5)
    vor, div, t, lnps = o.get_state()
    rng = np.random.default_rng(seed)
    tg = sht.synthesis(t) + rng.normal(0.0, noise, (o.nlev, o.nlat, o.nlon))
    t = sht.analysis(tg)
    return vor, div, t, lnps


def moving_state(o, seed=3):
    rng = np.random.default_rng(seed)
    from oracle.pyoracle import OracleSHT
    s = OracleSHT(o.params.trunc)
    vor = 1e-5 * red_spectrum(rng, s.l_of_lm, s.m_of_lm, (o.nlev,), slope=-1.0)
    div = 2e-6 * red_spectrum(rng, s.l_of_lm, s.m_of_lm, (o.nlev,), slope=-1.0)
    vor[:, 0] = 0
    div[:, 0] = 0
    o.set_isothermal(264.0, 1.0e5)
    _, _, t, lnps = o.get_state()
    t = t + 1.0 * red_spectrum(rng, s.l_of_lm, s.m_of_lm, (o.nlev,), slope=-1.0)
    lnps = lnps + 0.01 * red_spectrum(rng, s.l_of_lm, s.m_of_lm, (), slope=-1.0)
    return vor, div, t, lnps


def make_pair(trunc, nlev, **kw):
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    from oracle.pyoracle import OracleDyn, OracleSHT
    p = held_suarez_params(trunc=trunc, nlev=nlev, **kw)
    return AerosDyn(p), OracleDyn(p), OracleSHT(trunc)


def check_against_truth(tg, to, tt, label):
    """GPU (tg) and oracle (to) tendencies against truth (tt): every GPU field
    within 1e-12 of truth, the GPU's divergence no further from truth than the
    oracle's, and vor, T, ln ps within 1e-12 of the oracle."""
    eg = [relerr(a, b) for a, b in zip(tg, tt)]
    eo = [relerr(a, b) for a, b in zip(to, tt)]
    print(f"{label}: GPU-truth", ["%.1e" % x for x in eg], " oracle-truth", ["%.1e" % x for x in eo])
    for i in range(4):
        assert eg[i] < 1e-12, (label, i, eg[i])
    assert eg[1] <= eo[1], (label, eg[1], eo[1])
    for i in (0, 2, 3):
        assert relerr(tg[i], to[i]) < 1e-12


@pytest.mark.parametrize("trunc,nlev", [(21, 12), (31, 20), (42, 20), (21, 40), (21, 64)])
def test_adiabatic_tendency(gpulib, trunc, nlev):
    g, o, s = make_pair(trunc, nlev)
    st = moving_state(o)
    o.set_state(*st)
    g.set_state(*st)
    check_against_truth(g.tendency(), o.tendency(), truth(o, st), f"T{trunc}L{nlev} adiabatic")


def test_rest_state_tendency(gpulib):
    """tests/test_tendency.f90:77-107: resting isothermal atmosphere has no tendency."""
    g, o, s = make_pair(21, 12, held_suarez=0, p_top=0.0)
    g.set_isothermal(280.0, 1.0e5)
    tv, td, tt, tp = g.tendency()
    assert np.max(np.abs(tv)) == 0.0
    assert np.max(np.abs(td)) < 1e-12 * 1e-5
    assert np.max(np.abs(tt)) < 1e-12 and np.max(np.abs(tp)) < 1e-12


@pytest.mark.parametrize("trunc", [21, 31])
def test_hs_steps_match_oracle(gpulib, trunc):
    """Forced steps from a moving state: every term of the column is active."""
    g, o, s = make_pair(trunc, 20)
    st = moving_state(o, seed=21)
    o.set_state(*st)
    g.set_state(*st)
    o.step(1)
    g.step(1)
    sg, so = g.get_state(), o.get_state()
    assert relerr(sg[0], so[0]) < 1e-12
    assert relerr(sg[1], so[1]) < 1e-10
    assert relerr(sg[2], so[2]) < 1e-12
    assert relerr(sg[3], so[3]) < 1e-12
    o.step(9)
    g.step(9)
    for a, b in zip(g.get_state(), o.get_state()):
        assert relerr(a, b) < 1e-10
    for a, b in zip(g.get_old_state(), o.get_old_state()):
        assert relerr(a, b) < 1e-10
    ng, mg, lg, cg = g.counters()
    no, mo, lo, co = o.counters()
    assert ng == no == 10
    assert abs(mg - mo) / mo < 1e-13
    assert abs(lg - lo) < 1e-14 and abs(cg - co) < 1e-13


@pytest.mark.parametrize("nlev", [33, 40, 64])
@pytest.mark.parametrize("precision", [0, 1])
def test_many_levels_steps_match_oracle(gpulib, nlev, precision):
    """More than 32 levels (the 64-level column kernels and the two-levels-per-lane
    spectral solve): forced steps from a moving state against the oracle, with the
    bars of the 20-level case; the split form within its own 1e-10 bar."""
    g, o, s = make_pair(21, nlev, precision=precision)
    st = moving_state(o, seed=23)
    o.set_state(*st)
    g.set_state(*st)
    o.step(4)
    g.step(4)
    for a, b in zip(g.get_state(), o.get_state()):
        assert relerr(a, b) < 1e-10, nlev
    for a, b in zip(g.get_old_state(), o.get_old_state()):
        assert relerr(a, b) < 1e-10, nlev
    ng, mg, _, _ = g.counters()
    no, mo, _, _ = o.counters()
    assert ng == no == 4
    assert abs(mg - mo) / mo < 1e-13


def test_hs_rest_noise_start(gpulib):
    """Rest + 0.1 K noise (the Held-Suarez start): T and ln ps match from the
    first step; vor and D start at round-off size (dzeta/dt is analytically 0
    at rest) and are compared once populated, after 30 steps."""
    g, o, s = make_pair(21, 20)
    st = noisy_state(o, s)
    o.set_state(*st)
    g.set_state(*st)
    o.step(1)
    g.step(1)
    sg, so = g.get_state(), o.get_state()
    assert relerr(sg[2], so[2]) < 1e-12 and relerr(sg[3], so[3]) < 1e-12
    o.step(29)
    g.step(29)
    sg, so = g.get_state(), o.get_state()
    assert relerr(sg[0], so[0]) < 1e-10 and relerr(sg[1], so[1]) < 1e-10
    assert relerr(sg[2], so[2]) < 1e-12 and relerr(sg[3], so[3]) < 1e-12


def test_forced_moving_state_steps(gpulib):
    """A state with winds and ln(ps) structure: every term of the column is active."""
    g, o, s = make_pair(31, 20)
    st = moving_state(o, seed=5)
    o.set_state(*st)
    g.set_state(*st)
    o.step(3)
    g.step(3)
    for a, b in zip(g.get_state(), o.get_state()):
        assert relerr(a, b) < 1e-11


def test_diagnose_budget_zonal(gpulib):
    g, o, s = make_pair(21, 12)
    st = moving_state(o, seed=7)
    o.set_state(*st)
    g.set_state(*st)
    for a, b in zip(g.diagnose(), o.diagnose()):
        assert relerr(a, b) < 1e-12
    bg, bo = g.budget(), o.budget()
    for a, b in zip(bg, bo):
        assert abs(a - b) / abs(b) < 1e-12
    g.diag_accumulate()
    o.diag_accumulate()
    dg, do = g.diag_read(), o.diag_read()
    for k in ("u", "v", "temp", "uv", "vt", "eke", "tvar", "ps", "u_sfc"):
        assert relerr(dg[k], do[k]) < 1e-11, k


def test_ensemble_members_independent(gpulib):
    """Members stepped together equal single-member runs with the same forcing."""
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    from oracle.pyoracle import OracleDyn, OracleSHT
    p = held_suarez_params(trunc=21, nlev=16, nmember=3)
    g = AerosDyn(p)
    s = OracleSHT(21)
    states, oracles = [], []
    for e, dty in enumerate((40.0, 60.0, 80.0)):
        p1 = held_suarez_params(trunc=21, nlev=16)
        o = OracleDyn(p1)
        o.set_forcing(dty, p1.hs_k_a * (1 + 0.1 * e))
        g.set_member_forcing(e, dty, p1.hs_k_a * (1 + 0.1 * e))
        st = moving_state(o, seed=1000 + e)
        o.set_state(*st)
        states.append(st)
        oracles.append(o)
    g.set_state(*[np.stack([st[i] for st in states]) for i in range(4)])
    g.step(4)
    for o in oracles:
        o.step(4)
    gs = g.get_state()
    for e, o in enumerate(oracles):
        for a, b in zip([x[e] for x in gs], o.get_state()):
            assert relerr(a, b) < 1e-10


def test_restart_split_run_bitwise(gpulib):
    """tests/test_restart.f90: a split run equals the continuous run bit for bit."""
    g1, o, s = make_pair(21, 12)
    st = noisy_state(o, s, seed=9)
    g1.set_state(*st)
    g1.step(6)
    full = g1.get_state()
    g2, _, _ = make_pair(21, 12)
    g2.set_state(*st)
    g2.step(3)
    now, old = g2.get_state(), g2.get_old_state()
    n, mt, _, _ = g2.counters()
    g3, _, _ = make_pair(21, 12)
    g3.set_state(*now)
    g3.set_old_state(*old, nstep=n)
    g3.set_mass_target(mt)
    g3.step(3)
    for a, b in zip(g3.get_state(), full):
        assert np.array_equal(a, b)


def test_nonfinite_state_is_reported(gpulib):
    """A NaN planted in the input state comes back as AEROS_ERR_NONFINITE."""
    from aeros_gb300._capi import AerosError, ERR_NONFINITE
    g, o, s = make_pair(21, 12, mass_fixer=0)
    g.set_isothermal(264.0, 1.0e5)
    vor, div, t, lnps = g.get_state()
    t = t.copy()
    t[3, 5] = np.nan
    g.set_state(vor, div, t, lnps)
    with pytest.raises(AerosError) as ei:
        g.step(1)
    assert ei.value.code == ERR_NONFINITE
    g.set_isothermal(264.0, 1.0e5)
    g.set_state(*g.get_state())
    g.step(1)


def test_held_suarez_climate_short(gpulib):
    """A short T21L8 Held-Suarez climate (300 days, the last 100 averaged, two
    members) develops the published circulation: westerly jets near +-45 deg in
    the upper troposphere, poleward [v'T'] with its maximum low down, tropical
    surface easterlies."""
    from aeros_gb300.hs_climate import run
    r = run(trunc=21, nlev=8, days=300, spinup=200, members=2)
    print("T21L8 300-day HS summary", {k: r[k] for k in ("jet_nh", "jet_sh", "vT_max", "u_surface_tropics_min")})
    for jet in (r["jet_nh"], r["jet_sh"]):
        assert jet["u_max"] > 15.0 and 25.0 < abs(jet["lat"]) < 65.0 and jet["p_hpa"] < 500.0
    assert r["vT_max"]["value"] > 5.0 and r["vT_max"]["p_hpa"] > 600.0
    assert r["u_surface_tropics_min"] < 0.0


def test_config_T31L20_480_steps(gpulib):
    """The plain-method configuration: T31L20 Held-Suarez from rest (T = 264 K,
    ps = 1000 hPa) plus N(0, 0.1^2) K on the grid temperature (seed 0), dt =
    1800 s, 480 steps (10 days), compared with the oracle at step 1 (tendencies)
    and every 48 steps (state).  The step-1 tendencies of D, T and ln ps agree
    to the parity bars (the vorticity tendency of a rest state is round-off in
    both and is compared in absolute terms); the state difference is reported
    daily and stays below 1e-9 relative over the 10 days."""
    import os
    from oracle.pyoracle import OracleSHT, set_threads
    set_threads(os.cpu_count() or 1)
    g, o, s = make_pair(31, 20)
    o.set_isothermal(264.0, 1.0e5)
    vor, div, t, lnps = o.get_state()
    rng = np.random.default_rng(0)
    t = s.analysis(s.synthesis(t) + rng.normal(0.0, 0.1, (20, s.nlat, s.nlon)))
    g.set_state(vor, div, t, lnps)
    o.set_state(vor, div, t, lnps)
    tg, to = g.tendency(), o.tendency()
    tt = truth(o, (vor, div, t, lnps))
    assert np.max(np.abs(tg[0] - to[0])) < 1e-20
    e_div, o_div = relerr(tg[1], tt[1]), relerr(to[1], tt[1])
    e_t, e_p = relerr(tg[2], to[2]), relerr(tg[3], to[3])
    print(f"T31L20 step-1 tendencies: div {e_div:.1e} from truth (oracle {o_div:.1e})  T {e_t:.1e}  lnps {e_p:.1e}")
    assert e_t < 1e-12 and e_p < 1e-12 and e_div < 1e-12 and e_div <= o_div
    assert relerr(tg[2], tt[2]) < 1e-12 and relerr(tg[3], tt[3]) < 1e-12
    daily = []
    for day in range(10):
        g.step(48)
        o.step(48)
        daily.append(max(relerr(a, b) for a, b in zip(g.get_state()[1:], o.get_state()[1:])))
    ev = relerr(g.get_state()[0], o.get_state()[0])
    print("T31L20 daily max relative state difference (div, T, lnps):", ["%.1e" % x for x in daily],
          f"vorticity at day 10 {ev:.1e}")
    assert max(daily) < 1e-9 and ev < 1e-6


def test_hs_perturb_matches_oracle(gpulib):
    g, o, s = make_pair(42, 20)
    g.set_isothermal(264.0, 1.0e5)
    o.set_isothermal(264.0, 1.0e5)
    g.hs_perturb(1.0)
    o.hs_perturb(1.0)
    for a, b in zip(g.get_state(), o.get_state()):
        assert np.array_equal(a, b)


def test_handles_with_different_level_sets(gpulib):
    """Level and forcing constants belong to the handle: a 16-level handle
    created before a 20-level one (different sigma levels, different
    Held-Suarez sigma_b) still steps like its own oracle, and so does the
    20-level one, stepped alternately."""
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    from oracle.pyoracle import OracleDyn
    pa = held_suarez_params(trunc=21, nlev=16)
    pb = held_suarez_params(trunc=21, nlev=20)
    pb.hs_sigma_b = 0.65
    ga, oa = AerosDyn(pa), OracleDyn(pa)
    gb, ob = AerosDyn(pb), OracleDyn(pb)
    for g, o, seed in ((ga, oa, 31), (gb, ob, 32)):
        st = moving_state(o, seed=seed)
        o.set_state(*st)
        g.set_state(*st)
    for _ in range(3):
        for g, o in ((ga, oa), (gb, ob)):
            g.step(1)
            o.step(1)
    for g, o in ((ga, oa), (gb, ob)):
        for a, b in zip(g.get_state(), o.get_state()):
            assert relerr(a, b) < 1e-11
        bg, bo = g.budget(), o.budget()
        assert np.allclose(bg, bo, rtol=1e-12, atol=0)


def test_restart_file_resumes_bitwise(gpulib, tmp_path):
    """aeros_timestep_write_restart / _read_restart round trip through a file in
    the reference's layout: a fresh handle resumes bit-identically."""
    from aeros_gb300.restart import read_restart, write_restart
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    p = held_suarez_params(trunc=21, nlev=12)
    a = AerosDyn(p)
    a.set_isothermal(264.0, 1.0e5)
    a.hs_perturb(1.0)
    a.step(7)
    path = str(tmp_path / "restart.nc")
    write_restart(a, path, time=0.125)
    a.step(6)
    b = AerosDyn(p)
    assert read_restart(b, path) == 0.125
    assert b.counters()[0] == 7
    b.step(6)
    for x, y in zip(a.get_state(), b.get_state()):
        assert np.array_equal(x, y)
    assert a.counters() == b.counters()


def test_step_packed_equals_the_four_calls(gpulib):
    """aeros_dyn_step_packed == set_state + set_old_state(nstep) + step + get_state, bitwise."""
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    p = held_suarez_params(trunc=21, nlev=12)
    a = AerosDyn(p)
    a.set_isothermal(264.0, 1.0e5)
    a.hs_perturb(1.0)
    a.step(5)
    now, old, n = a.pack(*a.get_state()), a.pack(*a.get_old_state()), a.counters()[0]
    b = AerosDyn(p)
    b.set_mass_target(a.member_counters(0)[0])
    old_out = np.empty_like(now)
    out = b.step_packed(now, old, n, nsteps=3, old_out=old_out)
    a.step(3)
    assert np.array_equal(out, a.pack(*a.get_state()))
    assert np.array_equal(old_out, a.pack(*a.get_old_state()))
    assert b.counters()[0] == n + 3


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("kind", ["pinned", "registered", "device"])
def test_step_packed_one_graph_form(gpulib, kind, prec):
    """One step between pinned, registered or device buffers runs as one graph
    launch: bitwise the four-call result, through the start-up step and the
    regular one, and rebuilt when the buffers change."""
    import ctypes
    import torch
    from aeros_gb300 import _capi
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    p = held_suarez_params(trunc=21, nlev=12, nmember=2, precision=prec)
    a = AerosDyn(p)
    a.set_isothermal(264.0, 1.0e5)
    a.hs_perturb(1.0)
    n0 = a.pack(*a.get_state())
    lib = _capi.lib()
    keep = []

    def buf(x):
        if kind == "device":
            t = torch.from_numpy(np.array(x)).cuda()
            keep.append(t)
            return t
        if kind == "pinned":
            t = torch.empty(x.shape, dtype=torch.complex128, pin_memory=True)
            t.numpy()[...] = x
            keep.append(t)
            return t.numpy()
        h = np.array(x)
        _capi.check(lib.aeros_host_register(h.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(h.nbytes)),
                    "aeros_host_register")
        keep.append(h)
        return h

    def host(x):
        return x.cpu().numpy() if kind == "device" else np.array(x)

    b = AerosDyn(p)
    nw, od, out = buf(n0), buf(n0), buf(np.zeros_like(n0))
    b.step_packed(nw, od, 0, nsteps=1, now_out=out)           # start-up step: X^(n-1) = X^n on entry
    a.step(1)
    assert np.array_equal(host(out), a.pack(*a.get_state()))
    cur, prev = host(out), a.pack(*a.get_old_state())
    for it in range(4):                                         # regular steps: the outputs feed the next call
        nw2, od2, out2, old2 = buf(cur), buf(prev), buf(np.zeros_like(n0)), buf(np.zeros_like(n0))
        if it == 3:
            b.step_packed(nw2, od2, 1 + it, nsteps=1, now_out=out2)   # X^n only: another graph
            old2 = None
        else:
            b.step_packed(nw2, od2, 1 + it, nsteps=1, now_out=out2, old_out=old2)
        a.step(1)
        assert np.array_equal(host(out2), a.pack(*a.get_state()))
        if old2 is not None:
            assert np.array_equal(host(old2), a.pack(*a.get_old_state()))
            cur, prev = host(out2), host(old2)
    assert b.counters()[0] == 5
    if kind == "registered":
        for h in keep:
            _capi.check(lib.aeros_host_unregister(h.ctypes.data_as(ctypes.c_void_p)), "aeros_host_unregister")


@pytest.mark.parametrize("kind", ["pinned", "host"])
def test_step_packed_reports_nonfinite(gpulib, kind):
    """A NaN in the packed input comes back as AEROS_ERR_NONFINITE from the
    one-graph form (pinned arrays) and the copy form (pageable arrays); the next
    clean call succeeds (the flag is cleared on entry)."""
    import torch
    from aeros_gb300._capi import AerosError, ERR_NONFINITE
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    d = AerosDyn(held_suarez_params(trunc=21, nlev=12, mass_fixer=0))
    d.set_isothermal(264.0, 1.0e5)
    d.step(2)
    now, old = d.pack(*d.get_state()), d.pack(*d.get_old_state())

    def buf(x):
        if kind == "host":
            return np.array(x)
        t = torch.empty(x.shape, dtype=torch.complex128, pin_memory=True)
        t.numpy()[...] = x
        return t.numpy()

    bad = now.copy()
    bad[d.nlev * d.nlm + 7] = np.nan          # a divergence coefficient
    nw, od, out, out_old = buf(bad), buf(old), buf(np.zeros_like(now)), buf(np.zeros_like(now))
    with pytest.raises(AerosError) as ei:
        d.step_packed(nw, od, 2, 1, out, out_old)
    assert ei.value.code == ERR_NONFINITE
    nw[...] = now
    d.step_packed(nw, od, 2, 1, out, out_old)
    assert np.all(np.isfinite(out))


@pytest.mark.parametrize("trunc", [21, 42])
def test_forced_tendency_matches_oracle(gpulib, trunc):
    """aeros_dyn_tendency_forced: the adiabatic tendencies plus the Held-Suarez forcing
    added on the grid at the seam, against the oracle's forced tendency."""
    g, o, s = make_pair(trunc, 20)
    st = moving_state(o, seed=8)
    o.set_state(*st)
    g.set_state(*st)
    tg = g.tendency_forced()
    to = o.tendency(forced=True)
    check_against_truth(tg, to, truth(o, st, forced=True), f"T{trunc}L20 forced")
    ta = g.tendency()
    assert relerr(ta[2], tg[2]) > 1e-8    # the forcing is in the forced tendency
