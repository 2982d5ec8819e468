"""The facade's time rule through the C-ABI (aeros_dyn_set_time /
aeros_dyn_update / aeros_dyn_get_time) against the oracle's restatement of
aeros_update (src/aeros.f90:202-241): the number of steps taken, the facade's
step count, the clock, the half-way rounding case and the refusal to step
backwards."""
import ctypes

import numpy as np
import pytest

from tests.test_oracle_kat import _exact_half_time

pytestmark = pytest.mark.gpu


def test_update_matches_oracle_clock(gpulib):
    from aeros_gb300 import _capi
    from aeros_gb300.dynamics import AerosDyn
    from aeros_gb300.params import held_suarez_params
    from oracle.pyoracle import OracleClock, YEAR_SECONDS
    p = held_suarez_params(trunc=21, nlev=8)
    g = AerosDyn(p)
    g.set_isothermal(264.0, 1.0e5)
    g.hs_perturb(1.0)
    t0 = 0.0
    g.set_time(t0)
    o = OracleClock(p.dt, time_init=t0)
    step = p.dt / YEAR_SECONDS
    times = [t0, t0 + 2.49 * step, _exact_half_time(t0, 2, p.dt), t0 + 3.49 * step, t0 + 3.51 * step,
             t0 + 9.0 * step]
    total = 0
    for t in times:
        before = g.counters()[0]
        g.update(t)
        total += o.update(t)
        taken = g.counters()[0] - before
        assert g.counters()[0] == total, (t, taken)
        assert g.facade_clock() == (t, o.nstep)
    assert total == 9
    # an earlier time is refused and steps nothing
    n = g.counters()[0]
    rc = _capi.lib().aeros_dyn_update(g._h, ctypes.c_double(times[-2]))
    assert rc == _capi.ERR_ARG
    assert b"backwards" in _capi.lib().aeros_last_error()
    assert g.counters()[0] == n and g.facade_clock() == (times[-1], o.nstep)
    # a new initial time restarts the facade count (aeros_init's time_init)
    g.set_time(0.25)
    o = OracleClock(p.dt, time_init=0.25)
    g.update(0.25 + 1.2 * step)
    total += o.update(0.25 + 1.2 * step)
    assert g.counters()[0] == total == 10 and g.facade_clock() == (0.25 + 1.2 * step, 1)
    # the state stepped through update equals the same steps taken directly
    h = AerosDyn(p)
    h.set_isothermal(264.0, 1.0e5)
    h.hs_perturb(1.0)
    h.step(total)
    for a, b in zip(g.get_state(), h.get_state()):
        assert np.array_equal(a, b)
