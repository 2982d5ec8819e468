"""Error bound of the Newton-Raphson reciprocal the tracer-transport kernels use
for the ratios qm / dp and the van Leer harmonic mean (recip_nr in
aeros_gb300/csrc/transport.cu): from a seed r0 = (1 + d) / y with |d| <= 2^-22
(the hardware approximation rcp.approx.ftz.f64 is closer, near 2^-23), two steps
e = fma(-y, r, 1), r <- fma(r, e, r) land within an ulp of 1 / y.

Each fused multiply-add is evaluated here exactly (rational arithmetic) and
rounded once to double, as the GPU's FMA does, so the test checks the method's
bound itself, seeds at both ends of the error interval included."""
from fractions import Fraction

import numpy as np
import pytest


def _fma(a, b, c):
    """a * b + c with one rounding to double (round to nearest even, via Fraction -> float)."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _recip_nr(y, r0):
    r = r0
    for _ in range(2):
        e = _fma(-y, r, 1.0)
        r = _fma(r, e, r)
    return r


def _ulp_err(r, y):
    """|r - 1/y| in units of the last place of the double nearest 1/y."""
    exact = Fraction(1) / Fraction(y)
    ref = float(exact)
    return abs(Fraction(r) - exact) / Fraction(np.spacing(abs(ref)))


@pytest.mark.parametrize("scale", [1e-300, 1e-8, 1.0, 1e5, 1e300])
def test_two_newton_steps_within_an_ulp(scale):
    rng = np.random.default_rng(17)
    worst = 0.0
    for y0 in rng.uniform(0.5, 2.0, 200):
        y = float(y0 * scale) * (1 if rng.random() < 0.5 else -1)
        for d in (2.0 ** -22, -(2.0 ** -22), float(rng.uniform(-2.0 ** -22, 2.0 ** -22))):
            r0 = float((1 + Fraction(d)) / Fraction(y))
            worst = max(worst, float(_ulp_err(_recip_nr(y, r0), y)))
    assert worst <= 1.0, worst


def test_one_step_is_not_enough():
    """The second step is needed: after one, a seed 2^-22 off is still far outside an ulp."""
    y = 1.2345678901234567
    r0 = float((1 + Fraction(2.0 ** -22)) / Fraction(y))
    e = _fma(-y, r0, 1.0)
    r1 = _fma(r0, e, r0)
    assert _ulp_err(r1, y) > 1.0
