"""Split precision on an ensemble large enough (T42L20 x 10 members: 81,920 grid
columns, 18,920 real spectral columns) for its ensemble kernels: the
double-float column kernel and the exact fixed-point level products of the
semi-implicit solve.  Every member
against the FP64 oracle (and the divergence tendency against the long-double
truth) at the split form's 1e-10 bar, tendencies and 5 steps, with two
different member states interleaved so that cross-talk between members shows.
The errors reached are printed (pytest -s)."""
import numpy as np
import pytest

from tests._helpers import relerr, truth

pytestmark = pytest.mark.gpu

TOL = 1e-10


def test_split_ensemble_kernels_match_oracle(gpulib):
    from aeros_gb300.params import held_suarez_params, PREC_SPLIT
    from aeros_gb300.dynamics import AerosDyn
    from oracle.pyoracle import OracleDyn
    from tests.test_gpu_dyn import moving_state
    M = 10
    g = AerosDyn(held_suarez_params(trunc=42, nlev=20, nmember=M, precision=PREC_SPLIT))
    oracles, states = [], []
    for seed in (41, 42):
        o = OracleDyn(held_suarez_params(trunc=42, nlev=20))
        st = moving_state(o, seed=seed)
        o.set_state(*st)
        oracles.append(o)
        states.append(st)
    vor, div, t, lnps = (np.stack([states[e % 2][i] for e in range(M)]) for i in range(4))
    g.set_state(vor, div, t, lnps)
    tg = g.tendency_forced()
    worst_t, worst_truth = 0.0, 0.0
    for i, o in enumerate(oracles):
        to = o.tendency(forced=True)
        tt = truth(o, states[i], forced=True)
        for e in range(i, M, 2):
            errs = [relerr(tg[f][e], to[f]) for f in range(4)]
            worst_t = max(worst_t, max(errs))
            assert max(errs) < TOL, (e, errs)
            et = relerr(tg[1][e], tt[1])
            worst_truth = max(worst_truth, et)
            assert et < TOL, (e, et)
    g.step(5)
    sg = g.get_state(squeeze=False)
    worst_s = 0.0
    for i, o in enumerate(oracles):
        o.step(5)
        so = o.get_state()
        for e in range(i, M, 2):
            errs = [relerr(sg[f][e], so[f]) for f in range(4)]
            worst_s = max(worst_s, max(errs))
            assert max(errs) < TOL, (e, errs)
    print(f"split T42L20 x {M}: tendencies {worst_t:.1e} from the oracle, divergence {worst_truth:.1e} from "
          f"truth, state after 5 steps {worst_s:.1e}")
