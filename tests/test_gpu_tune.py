"""Launch-shape autotuner: it keeps the results unchanged (every candidate
shape computes each output with the same arithmetic), never makes the step
slower than the shapes it started from, and its cache file restores the
chosen shapes in a new handle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _state(dyn, seed=7):
    from aeros_gb300.spectral import AerosSHT
    from tests._helpers import red_spectrum
    s = AerosSHT(dyn.params.trunc, batch_max=1)
    rng = np.random.default_rng(seed)
    dyn.set_isothermal(264.0, 1.0e5)
    vor, div, t, lnps = dyn.get_state(squeeze=False)
    sh = (dyn.nmember, dyn.nlev)
    vor = 1e-5 * red_spectrum(rng, s.l_of_lm, s.m_of_lm, sh, slope=-1.0)
    div = 2e-6 * red_spectrum(rng, s.l_of_lm, s.m_of_lm, sh, slope=-1.0)
    vor[..., 0] = 0
    div[..., 0] = 0
    return vor, div, t + red_spectrum(rng, s.l_of_lm, s.m_of_lm, sh, slope=-1.0), lnps


@pytest.mark.parametrize("prec", [0, 1])
def test_autotune_results_unchanged(gpulib, tmp_path, monkeypatch, prec):
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    monkeypatch.setenv("AEROS_TUNE_CACHE", str(tmp_path / "tune.txt"))
    p = held_suarez_params(trunc=31, nlev=12, nmember=4, precision=prec)
    ref, tuned = AerosDyn(p), AerosDyn(p)
    st = _state(ref)
    ref.set_state(*st)
    tuned.set_state(*st)
    before, after, shapes = tuned.autotune(reps=2)
    print(f"precision {prec}: step {before:.3f} ms -> {after:.3f} ms with", shapes)
    assert after <= before
    ref.step(6)
    tuned.step(6)
    for a, b in zip(ref.get_state(), tuned.get_state()):
        assert np.array_equal(a, b)
    fresh = AerosDyn(p)
    assert fresh.tune_shapes() == shapes
