"""Generate tests/golden/*.npz from independent implementations (numpy, scipy).

The reference keeps no golden vectors (its tests are analytic), and its
transform engine (SHTns 3.7.5 + FFTW) is not in the tree.  These fixtures pin
the pieces of the SHTns convention that the oracle restates against
third-party code that shares nothing with it:
  gauss_N.npz     Gauss-Legendre nodes (descending) and weights, N = 32..512,
                  from mpmath.gauss_legendre-style Newton at 40 digits (mpmath
                  polynomial evaluation, independent of the oracle), rounded
  plm_T.npz       orthonormal, no-Condon-Shortley Pbar_l^m at those nodes,
                  from scipy.special.sph_harm_y (Y_lm sqrt(2 pi) (-1)^m); scipy's
                  own error at l <= 42 is ~1e-13
  fourier.npz     a grid field built directly from the SHTns synthesis formula
                  f = sum_m (2 - delta_m0) Re[sum_l a_lm Pbar_lm e^{i m lon}] / sqrt(2 pi)
                  with numpy's exp (no FFT), for the test spectrum of
                  tests/test_spectral.f90:147-172 at T21
Run:  python tests/golden/make_golden.py
"""
import os

import mpmath as mp
import numpy as np
from scipy.special import sph_harm_y

mp.mp.dps = 40

HERE = os.path.dirname(os.path.abspath(__file__))


def grid(T):
    n = 3 * T + 1
    while True:
        m = n
        if m % 2 == 0:
            for p in (2, 3, 5):
                while m % p == 0:
                    m //= p
            if m == 1:
                break
        n += 1
    return n, n // 2


def lm_table(T):
    ls, ms = [], []
    for m in range(T + 1):
        for l in range(m, T + 1):
            ls.append(l)
            ms.append(m)
    return np.array(ls), np.array(ms)


def gauss(n):
    """Gauss-Legendre nodes/weights at 40 digits (Newton on mpmath.legendre)."""
    xs, ws = [], []
    for i in range(n // 2):
        z = mp.cos(mp.pi * (i + mp.mpf(3) / 4) / (n + mp.mpf(1) / 2))
        for _ in range(100):
            p = mp.legendre(n, z)
            dp = n * (z * p - mp.legendre(n - 1, z)) / (z * z - 1)
            dz = p / dp
            z -= dz
            if abs(dz) < mp.mpf(10) ** -35:
                break
        dp = n * (z * mp.legendre(n, z) - mp.legendre(n - 1, z)) / (z * z - 1)
        xs.append(z)
        ws.append(2 / ((1 - z * z) * dp * dp))
    x = np.array([float(v) for v in xs] + [-float(v) for v in reversed(xs)])
    w = np.array([float(v) for v in ws] + [float(v) for v in reversed(ws)])
    return x, w


def pbar(T, x):
    ls, ms = lm_table(T)
    th = np.arccos(x)
    P = np.zeros((len(ls), len(x)))
    for i, (l, m) in enumerate(zip(ls, ms)):
        P[i] = np.real(sph_harm_y(l, m, th, 0.0)) * np.sqrt(2 * np.pi) * (-1.0) ** m
    return P


def main():
    for n in (32, 48, 64, 128, 256, 512):
        x, w = gauss(n)
        np.savez_compressed(os.path.join(HERE, f"gauss_{n}.npz"), x=x, w=w)
    for T in (21, 42):
        nlon, nlat = grid(T)
        x, _ = gauss(nlat)
        xn = x[: nlat // 2]
        np.savez_compressed(os.path.join(HERE, f"plm_T{T}.npz"), x=xn, P=pbar(T, xn))
    T = 21
    nlon, nlat = grid(T)
    ls, ms = lm_table(T)
    amp = 1.0 / (ls + 1.0) ** 2
    a = amp * np.cos(3 * ls + ms) + 1j * amp * np.sin(ls + 2 * ms)
    a[ms == 0] = a[ms == 0].real
    x, _ = gauss(nlat)
    P = pbar(T, x)
    lon = 2 * np.pi * np.arange(nlon) / nlon
    f = np.zeros((nlat, nlon))
    for i in range(len(ls)):
        term = np.outer(P[i], np.exp(1j * ms[i] * lon)) * a[i]
        f += (1.0 if ms[i] == 0 else 2.0) * term.real
    f /= np.sqrt(2 * np.pi)
    np.savez_compressed(os.path.join(HERE, "fourier.npz"), coeffs=a, field=f)


if __name__ == "__main__":
    main()
