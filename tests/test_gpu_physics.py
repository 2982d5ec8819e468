"""The physics seam (src/dynamics/aeros_tendency.f90:362-388): a hook adds its
tendencies on the grid between the adiabatic right-hand sides and the
transforms back to spectral space.

A uniform linear drag commutes with the curl and the divergence, so on the
spectral side it must appear as exactly -k zeta and -k D; a uniform Newtonian
cooling as -k (T - t_ref) with t_ref entering the (0, 0) coefficient only."""
import numpy as np
import pytest

from tests._helpers import relerr
from tests.test_gpu_dyn import make_pair, moving_state

pytestmark = pytest.mark.gpu

SQRT4PI = np.sqrt(4.0 * np.pi)


def _dyn(trunc=21, nlev=12, held_suarez=False):
    g, o, _ = make_pair(trunc, nlev, held_suarez=held_suarez)
    st = moving_state(o, seed=41)
    g.set_state(*st)
    return g, st


def test_no_hook_forced_equals_adiabatic(gpulib):
    g, _ = _dyn()
    for a, b in zip(g.tendency(), g.tendency_forced()):
        assert np.array_equal(a, b)


def test_relaxation_seam_identities(gpulib):
    g, st = _dyn()
    vor, div, tmp, lnps = st
    base = g.tendency_forced()
    kd, kt, tref = 1.0 / 86400.0, 1.0 / (4 * 86400.0), 250.0
    g.set_relaxation(kd, kt, tref)
    forced = g.tendency_forced()
    dv, dd, dt_, dp = (a - b for a, b in zip(forced, base))
    assert relerr(dv, -kd * vor) < 1e-9
    assert relerr(dd, -kd * div) < 1e-9
    expect_t = -kt * tmp.copy()
    expect_t[:, 0] += kt * tref * SQRT4PI     # (l, m) = (0, 0): the constant t_ref
    assert relerr(dt_, expect_t) < 1e-9
    assert np.array_equal(dp, np.zeros_like(dp))
    # the adiabatic entry point is unaffected by the hook
    for a, b in zip(g.tendency(), base):
        assert np.array_equal(a, b)


def test_hook_runs_in_the_step_graph(gpulib):
    ga, st = _dyn()
    gb, _ = _dyn()
    gc, _ = _dyn()
    gb.set_relaxation(0.0, 0.0, 0.0)           # a hook that adds zero
    gc.set_relaxation(1.0 / 86400.0)
    for g in (ga, gb, gc):
        g.step(3)
    sa, sb, sc = ga.get_state(), gb.get_state(), gc.get_state()
    for a, b in zip(sa, sb):
        assert np.array_equal(a, b)
    assert relerr(sc[0], sa[0]) > 1e-6          # the drag changed the vorticity
    names = [n for n, _ in gc.profile_step()]
    assert "physics" in names and names.index("physics") == names.index("column") + 1
    gc.set_physics(None)
    assert "physics" not in [n for n, _ in gc.profile_step()]


def test_adjoint_refuses_a_hook(gpulib):
    from aeros_gb300._capi import AerosError, ERR_UNSUPPORTED
    g, _ = _dyn()
    g.set_relaxation(1.0 / 86400.0)
    with pytest.raises(AerosError) as ei:
        g.window_forward(4, 2)
    assert ei.value.code == ERR_UNSUPPORTED


def test_hook_inside_an_ensemble_group(gpulib):
    """A handle's hook is part of its step graph, so a group that contains it steps
    bit-identically to the handle stepped alone."""
    from aeros_gb300.dynamics import AerosGroup
    a, _ = _dyn()
    b, _ = _dyn()
    c, _ = _dyn(trunc=31)
    for h in (a, b):
        h.set_relaxation(1.0 / 86400.0, 1.0 / (4 * 86400.0), 250.0)
    g = AerosGroup([a, c])
    g.step(3)
    b.step(3)
    for x, y in zip(a.get_state(), b.get_state()):
        assert np.array_equal(x, y)


def test_hook_in_the_packed_step(gpulib):
    """aeros_dyn_step_packed runs the hook too: between pinned arrays (one graph)
    its two new time levels equal set_state + step + get_state, bitwise."""
    import torch
    ga, st = _dyn()
    gb, _ = _dyn()
    for g in (ga, gb):
        g.set_relaxation(1.0 / 86400.0, 1.0 / (4 * 86400.0), 250.0)
        g.step(2)
    now, old, n = ga.pack(*ga.get_state()), ga.pack(*ga.get_old_state()), ga.counters()[0]

    def pinned(x):
        t = torch.empty(x.shape, dtype=torch.complex128, pin_memory=True)
        t.numpy()[...] = x
        return t.numpy()

    hn, ho, out, out_old = pinned(now), pinned(old), pinned(np.zeros_like(now)), pinned(np.zeros_like(now))
    gb.step_packed(hn, ho, n, 1, out, out_old)
    ga.step(1)
    assert np.array_equal(out, ga.pack(*ga.get_state()))
    assert np.array_equal(out_old, ga.pack(*ga.get_old_state()))
