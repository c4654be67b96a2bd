"""The oracle's fft991 (the pressure solver's x transform, crm/fft.F90)
against the discrete Fourier transform.

fft991 returns, for a real row x of length n, the coefficients of
numpy.fft.rfft(x) / n as [Re X_0, Im X_0, Re X_1, Im X_1, ..., Re X_n/2,
Im X_n/2] and its inverse rebuilds x.  Its trig table is computed in REAL*4
(fftrig_crm, fft.F90:247-300), so the transform agrees with the exact DFT to
single-precision accuracy and not better — the property that makes the FP64
form's bit-exact parity depend on restating those REAL*4 twiddles.
"""
import numpy as np
import pytest

import oracle

SIZES = [16, 32, 48, 64, 80, 96, 128, 256]   # radix 2, 3, 4 and 5 factors


def _forward(x):
    n = x.size
    a = np.zeros(n + 2)
    a[:n] = x
    return oracle.fft991(a, -1)


@pytest.mark.parametrize('n', SIZES)
def test_fft991_matches_the_dft(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    f = _forward(x)
    X = np.fft.rfft(x) / n
    err = max(np.max(np.abs(f[0::2] - X.real)), np.max(np.abs(f[1::2] - X.imag)))
    assert err <= 2e-6 * np.max(np.abs(X)), (n, err)


@pytest.mark.parametrize('n', SIZES)
def test_fft991_inverse_rebuilds_the_row(n):
    rng = np.random.default_rng(100 + n)
    x = rng.standard_normal(n)
    back = oracle.fft991(_forward(x), +1)
    assert np.max(np.abs(back[:n] - x)) <= 2e-6 * np.max(np.abs(x))


def test_fft991_twiddles_are_single_precision():
    """A pure cosine mode comes out with REAL*4-sized errors (1e-9..1e-6),
    not the ~1e-16 of a double-precision table."""
    n = 64
    j = np.arange(n)
    errs = []
    for k in (3, 5, 7, 11):
        f = _forward(np.cos(2 * np.pi * k * j / n))
        exact = np.zeros(n + 2)
        exact[2 * k] = 0.5
        errs.append(np.max(np.abs(f - exact)))
    assert 1e-10 < max(errs) < 1e-5, errs


def test_fft991_rejects_lengths_it_cannot_factor():
    with pytest.raises(ValueError):
        oracle.fft991(np.zeros(14 + 2), -1)          # 14 = 2 x 7
