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


@pytest.mark.parametrize("nlev,prec,si", [(20, 0, 1), (16, 1, 1), (20, 0, 0)])
def test_spectral_column_layout_same_results(gpulib, nlev, prec, si):
    """The thread-per-column spectral kernel computes every update with the
    arithmetic, in the order, of the warp-per-coefficient kernel."""
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    p = held_suarez_params(trunc=31, nlev=nlev, nmember=3, precision=prec, semi_implicit=si)
    ref, cols = AerosDyn(p), AerosDyn(p)
    st = _state(ref)
    ref.set_state(*st)
    cols.set_state(*st)
    cols.set_tune_shapes(spec_cols=1, spec_warps=2)
    assert cols.tune_shapes()["spec_cols"] == 1 and ref.tune_shapes()["spec_cols"] == 0
    ref.step(6)
    cols.step(6)
    for a, b in zip(ref.get_state(), cols.get_state()):
        rel = np.max(np.abs(a - b)) / np.max(np.abs(a))
        assert np.array_equal(a, b), f"largest relative difference {rel:.3e}"


def test_tune_set_rejects_shapes_outside_the_candidates(gpulib):
    from aeros_gb300.params import held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    from aeros_gb300._capi import AerosError
    d = AerosDyn(held_suarez_params(trunc=21, nlev=12))
    before = d.tune_shapes()
    with pytest.raises(AerosError):
        d.set_tune_shapes(spec_cols=1)      # no column-layout kernel for 12 levels
    with pytest.raises(AerosError):
        d.set_tune_shapes(spec_warps=3)
    with pytest.raises(KeyError):
        d.set_tune_shapes(warps=2)
    assert d.tune_shapes() == before
    d.set_tune_shapes(col_thr=128, col_lanes=4)
    assert d.tune_shapes()["col_lanes"] == 4


def test_split_grid_shapes_leave_results_unchanged(gpulib):
    """The split form's grid sizes (CTAs per SM of the Legendre kernels and of
    the DFT products) only decide which CTA takes which column group: the
    steps are bitwise those of the default shapes."""
    from aeros_gb300.params import held_suarez_params, PREC_SPLIT
    from aeros_gb300.dynamics import AerosDyn
    p = held_suarez_params(trunc=42, nlev=20, nmember=4, precision=PREC_SPLIT)
    ref = AerosDyn(p)
    st = _state(ref)
    ref.set_state(*st)
    ref.step(3)
    for cps, dcps in ((2, 16), (16, 2)):
        d = AerosDyn(p)
        d.set_state(*st)
        d.set_tune_shapes(sp_cps=cps, sp_dft_cps=dcps)
        assert d.tune_shapes()["sp_cps"] == cps and d.tune_shapes()["sp_dft_cps"] == dcps
        d.step(3)
        for a, b in zip(ref.get_state(), d.get_state()):
            assert np.array_equal(a, b)
    with pytest.raises(Exception):
        ref.set_tune_shapes(sp_cps=3)
