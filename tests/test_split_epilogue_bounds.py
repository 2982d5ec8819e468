"""The split kernels' epilogue sums Z = sum_q Y_q 2^(40 - 8 q) over the seven
shifted accumulators of (S, B) = (7, 8) digits with int32 pairs
(hi = Y0 2^8 + Y1, mid = Y2 2^8 + Y3, lo = Y4 2^8 + Y5 + (Y6 >> 8)) when the
contraction has at most 101 terms, and converts the fp32 accumulators to
integers by adding 1.5 2^23 when it has at most 36 (zsum in split_common.cuh).
Here, on the CPU, the bounds those modes rely on and the identity with the
term-by-term int64 sum, at the extremes the digit bound allows (|digit| <= 128,
so |Y_q| <= (q + 1) K 2^14)."""
import numpy as np
import pytest

pytestmark = pytest.mark.filterwarnings("ignore")

I32 = 2 ** 31


def term_sum(Y):
    z = 0
    for q, y in enumerate(Y):
        sh = 40 - 8 * q
        z += (y << sh) if sh >= 0 else (y >> (-sh))
    return z


def packed(Y, magic):
    if magic:
        v = []
        for y in Y:
            bits = int(np.array([np.float32(y) + np.float32(12582912.0)], np.float32).view(np.int32)[0])
            v.append(bits - 0x4B400000)
    else:
        v = list(Y)
    hi, mid, lo = v[0] * 256 + v[1], v[2] * 256 + v[3], v[4] * 256 + v[5] + (v[6] >> 8)
    for x in (hi, mid, lo):
        assert -I32 <= x < I32, x
    return (hi << 32) + (mid << 16) + lo


def zmode_for(Kp):
    # the kernel's rule (split_common.cuh, zmode_for<7>), on the padded contraction length
    return 2 if Kp <= 32 else (1 if Kp <= 96 else 0)


@pytest.mark.parametrize("K", [16, 32, 36, 48, 86, 96, 101])
def test_packed_sum_equals_term_sum(K):
    rng = np.random.default_rng(K)
    bound = [(q + 1) * K * 2 ** 14 for q in range(7)]
    cases = [[b for b in bound], [-b for b in bound], [(-1) ** q * b for q, b in enumerate(bound)]]
    cases += [[int(rng.integers(-b, b + 1)) for b in bound] for _ in range(2000)]
    for Y in cases:
        assert packed(Y, False) == term_sum(Y)
        if K <= 36:
            assert max(abs(y) for y in Y) <= 2 ** 22
            assert packed(Y, True) == term_sum(Y)


def test_kernel_rule_stays_inside_the_bounds():
    # every padded length the kernels use maps to a mode whose bound holds for it
    for Kp in range(16, 512, 16):
        m = zmode_for(Kp)
        if m == 2:
            assert 7 * Kp * 2 ** 14 <= 2 ** 22
        if m >= 1:
            assert 5 * Kp * 2 ** 22 + 6 * Kp * 2 ** 14 + 7 * Kp * 2 ** 6 < I32
