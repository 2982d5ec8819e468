"""Split-precision (Ozaki, tcgen05 bf16 digits, exact integer recombination) path
against the FP64 CPU oracle.

Bar: 1e-10 relative (max |split - oracle| / max |oracle|) for every transform
and for the step, the tolerance the split-precision form is specified to.  The
errors actually reached are printed (pytest -s) and are ~1e-14.
"""
import numpy as np
import pytest

from tests._helpers import red_spectrum, relerr

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module", params=[21, 42, 85, 170])
def pair(request, gpulib):
    from aeros_gb300.spectral import AerosSHT
    from aeros_gb300.params import PREC_SPLIT
    from oracle.pyoracle import OracleSHT
    T = request.param
    return AerosSHT(T, batch_max=6, precision=PREC_SPLIT), OracleSHT(T)


def test_split_scalar(pair):
    g, o = pair
    rng = np.random.default_rng(31)
    c = red_spectrum(rng, o.l_of_lm, o.m_of_lm, (3,))
    e1 = relerr(g.synthesis(c), o.synthesis(c))
    f = o.synthesis(c)
    e2 = relerr(g.analysis(f), o.analysis(f))
    print(f"T{o.trunc} split synthesis {e1:.2e} analysis {e2:.2e}")
    assert e1 < TOL and e2 < TOL


def test_split_vector_gradient_winds(pair):
    g, o = pair
    rng = np.random.default_rng(32)
    s = red_spectrum(rng, o.l_of_lm, o.m_of_lm, (2,))
    t = red_spectrum(rng, o.l_of_lm, o.m_of_lm, (2,))
    s[:, 0] = 0
    t[:, 0] = 0
    errs = []
    for a, b in zip(g.synthesis_vec(s, t), o.synthesis_vec(s, t)):
        errs.append(relerr(a, b))
    vth, vph = o.synthesis_vec(s, t)
    for a, b in zip(g.analysis_vec(vth, vph), o.analysis_vec(vth, vph)):
        errs.append(relerr(a, b))
    for a, b in zip(g.gradient(s), o.gradient(s)):
        errs.append(relerr(a, b))
    vor, div = 1e-5 * s, 2e-6 * t
    u, v = o.uv_from_vordiv(vor, div)
    for a, b in zip(g.uv_from_vordiv(vor, div), (u, v)):
        errs.append(relerr(a, b))
    for a, b in zip(g.vordiv_from_uv(u, v), o.vordiv_from_uv(u, v)):
        errs.append(relerr(a, b))
    print(f"T{o.trunc} split vector/gradient/winds max {max(errs):.2e}")
    assert max(errs) < TOL


def test_split_round_trip_T341(gpulib):
    """Size-independent property at the largest transform size:
    analysis(synthesis(c)) = c for a band-limited spectrum."""
    from aeros_gb300.spectral import AerosSHT
    from aeros_gb300.params import PREC_SPLIT
    g = AerosSHT(341, batch_max=2, precision=PREC_SPLIT)
    rng = np.random.default_rng(33)
    c = red_spectrum(rng, g.l_of_lm, g.m_of_lm, (2,))
    e = relerr(g.analysis(g.synthesis(c)), c)
    print(f"T341 split round trip {e:.2e}")
    assert e < TOL


def test_split_dynamics_step(gpulib):
    from aeros_gb300.params import held_suarez_params, PREC_SPLIT
    from aeros_gb300.dynamics import AerosDyn
    from oracle.pyoracle import OracleDyn
    from tests.test_gpu_dyn import moving_state
    p = held_suarez_params(trunc=42, nlev=20, precision=PREC_SPLIT)
    g = AerosDyn(p)
    o = OracleDyn(held_suarez_params(trunc=42, nlev=20))
    st = moving_state(o, seed=41)
    g.set_state(*st)
    o.set_state(*st)
    et = [relerr(a, b) for a, b in zip(g.tendency(), o.tendency())]
    g.step(5)
    o.step(5)
    es = [relerr(a, b) for a, b in zip(g.get_state(), o.get_state())]
    print("split T42L20 tendency errors", ["%.1e" % x for x in et], "state after 5 steps",
          ["%.1e" % x for x in es])
    assert max(et) < TOL and max(es) < TOL


@pytest.mark.parametrize("T,B", [(85, 240), (170, 240), (341, 30)])
def test_transform_sweep_vs_oracle(gpulib, T, B):
    """The transform sweep workload (30 levels x 8 fields at T85/T170; 30 fields
    at T341 to bound the oracle's time): seeded complex Gaussian coefficients with
    variance (l+1)^-3.  FP64 path <= 1e-12, split path <= 1e-10 against the
    oracle, forward and inverse."""
    from aeros_gb300.spectral import AerosSHT
    from aeros_gb300.params import PREC_SPLIT, PREC_FP64
    from oracle.pyoracle import OracleSHT, set_threads
    import os
    set_threads(os.cpu_count() or 1)
    o = OracleSHT(T)
    rng = np.random.default_rng(1)
    l = o.l_of_lm.astype(float)
    c = (rng.standard_normal((B, o.nlm)) + 1j * rng.standard_normal((B, o.nlm))) * (l + 1.0) ** -1.5
    c[:, o.m_of_lm == 0] = c[:, o.m_of_lm == 0].real
    fo = o.synthesis(c)
    co = o.analysis(fo)
    for prec, tol in ((PREC_FP64, 1e-12), (PREC_SPLIT, 1e-10)):
        g = AerosSHT(T, batch_max=B, precision=prec)
        es, ea = relerr(g.synthesis(c), fo), relerr(g.analysis(fo), co)
        print(f"T{T} B={B} precision {prec}: synthesis {es:.2e} analysis {ea:.2e}")
        assert es < tol and ea < tol


@pytest.mark.parametrize("T", [42, 85])
def test_split_analysis_groups_are_per_column(gpulib, T):
    """The analysis packs outputs into column groups of up to 8 sources; every
    output is computed from its own columns, so a batch's analyses equal the
    same fields analysed one at a time, bitwise, across group boundaries."""
    from aeros_gb300.spectral import AerosSHT
    from aeros_gb300.params import PREC_SPLIT
    from oracle.pyoracle import OracleSHT
    o = OracleSHT(T)
    g = AerosSHT(T, batch_max=13, precision=PREC_SPLIT)
    rng = np.random.default_rng(77)
    c = red_spectrum(rng, o.l_of_lm, o.m_of_lm, (13,))
    f = o.synthesis(c)
    batch = g.analysis(f)                       # 13 one-slot outputs: groups of 8 and 5
    for i in (0, 7, 8, 12):
        assert np.array_equal(batch[i], g.analysis(f[i:i + 1])[0])
    assert relerr(batch, o.analysis(f)) < TOL
    s = red_spectrum(rng, o.l_of_lm, o.m_of_lm, (5,))
    t = red_spectrum(rng, o.l_of_lm, o.m_of_lm, (5,))
    s[:, 0] = 0
    t[:, 0] = 0
    vth, vph = o.synthesis_vec(s, t)
    S, Tt = g.analysis_vec(vth, vph)            # 10 two-slot outputs: groups of 4, 4 and 2
    for i in (0, 2, 4):
        S1, T1 = g.analysis_vec(vth[i:i + 1], vph[i:i + 1])
        assert np.array_equal(S[i], S1[0]) and np.array_equal(Tt[i], T1[0])
    so, to = o.analysis_vec(vth, vph)
    assert relerr(S, so) < TOL and relerr(Tt, to) < TOL


@pytest.mark.parametrize("T", [21, 42])
def test_split_fourier_paths_agree(gpulib, T, monkeypatch):
    """The split form's two longitude-transform paths: double-float FFTs (the
    default) and exact-digit DFT products on the tensor cores (AEROS_SPLIT_DFT=1),
    each against the oracle, and the step tendencies of both at T42L20."""
    from aeros_gb300.spectral import AerosSHT
    from aeros_gb300.params import PREC_SPLIT, held_suarez_params
    from aeros_gb300.dynamics import AerosDyn
    from oracle.pyoracle import OracleSHT, OracleDyn
    from tests.test_gpu_dyn import moving_state
    o = OracleSHT(T)
    rng = np.random.default_rng(34)
    c = red_spectrum(rng, o.l_of_lm, o.m_of_lm, (3,))
    f = o.synthesis(c)
    res = {}
    for path in ("0", "1"):
        monkeypatch.setenv("AEROS_SPLIT_DFT", path)
        g = AerosSHT(T, batch_max=3, precision=PREC_SPLIT)
        res[path] = (g.synthesis(c), g.analysis(f))
        e1, e2 = relerr(res[path][0], f), relerr(res[path][1], o.analysis(f))
        print(f"T{T} split Fourier path AEROS_SPLIT_DFT={path}: synthesis {e1:.2e} analysis {e2:.2e}")
        assert e1 < TOL and e2 < TOL
    assert relerr(res["0"][0], res["1"][0]) < 1e-12 and relerr(res["0"][1], res["1"][1]) < 1e-12
    if T == 42:
        od = OracleDyn(held_suarez_params(trunc=42, nlev=20))
        st = moving_state(od, seed=43)
        od.set_state(*st)
        ref = od.tendency()
        for path in ("0", "1"):
            monkeypatch.setenv("AEROS_SPLIT_DFT", path)
            d = AerosDyn(held_suarez_params(trunc=42, nlev=20, precision=PREC_SPLIT))
            d.set_state(*st)
            et = [relerr(a, b) for a, b in zip(d.tendency(), ref)]
            print(f"T42L20 split tendencies, AEROS_SPLIT_DFT={path}:", ["%.1e" % x for x in et])
            assert max(et) < TOL
