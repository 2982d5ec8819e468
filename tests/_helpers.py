"""Shared input generators and error measures for the tests."""
import numpy as np


def spectrum_test(l_of_lm, m_of_lm):
    """The test spectrum of tests/test_spectral.f90:147-172 (reference):
    amp = 1/(l+1)^2, re = amp cos(3l+m), im = amp sin(l+2m), m = 0 real."""
    l = np.asarray(l_of_lm, float)
    m = np.asarray(m_of_lm, float)
    amp = 1.0 / ((l + 1.0) ** 2)
    c = amp * np.cos(3 * l + m) + 1j * amp * np.sin(l + 2 * m)
    c[np.asarray(m_of_lm) == 0] = c[np.asarray(m_of_lm) == 0].real
    return c


def red_spectrum(rng, l_of_lm, m_of_lm, shape, slope=-1.5):
    """Seeded complex Gaussian coefficients, std ~ (l+1)^slope, m = 0 real."""
    l = np.asarray(l_of_lm, float)
    amp = (l + 1.0) ** slope
    n = len(l)
    c = (rng.standard_normal(shape + (n,)) + 1j * rng.standard_normal(shape + (n,))) * amp
    c[..., np.asarray(m_of_lm) == 0] = c[..., np.asarray(m_of_lm) == 0].real
    return c


def relerr(a, b):
    """max |a - b| / max |b| (the reference tests' error measure)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def truth(o, st, forced=False):
    """Spectral tendencies of state `st` evaluated in long double by
    oracle/truth.cpp, with oracle handle o's parameters and vertical grid."""
    from oracle.pyoracle import truth_tendency
    return truth_tendency(o.params, o.nlon, o.nlat, o.A, o.B, st, forced=forced)
