"""Spatio-temporal spectra restatement (oracle/sts_oracle.py, following
Run/CompSTS/driver.f90) on the CPU: known answers and size-independent
properties.  Tolerances relative 1e-12 (FP64)."""
import math

import numpy as np

from oracle import sts_oracle


def test_hann_endpoints_and_symmetry():
    w = sts_oracle.hann(64)
    assert w[0] == 0.0 and abs(w[-1]) < 1e-15
    assert np.allclose(w, w[::-1], rtol=0, atol=1e-15)
    assert abs(w.max() - 1.0) < 2e-3


def test_wavenumbers_follow_the_post_processor():
    n = 8
    assert [sts_oracle.kwn(i, n) for i in range(n)] == [0, 1, 2, 3, -4, -3, -2, -1]


def test_parseval_per_mode():
    """sum_w |X|^2 = Nt sum_t |w x|^2 for every mode (DFT Parseval)."""
    rng = np.random.default_rng(3)
    nt, nx = 32, 16
    rec = rng.standard_normal((nt, nx, nx)) + 1j * rng.standard_normal((nt, nx, nx))
    s1, s2 = sts_oracle.spectra(rec)
    stsnorm = (1.0 / nt) ** 2 * (1.0 / (nx * nx)) ** 2
    wx = rec * sts_oracle.hann(nt)[:, None, None]
    direct = nt * stsnorm * (np.abs(wx) ** 2).sum(0)          # [kx, ky]
    assert np.allclose(s1.sum(0), direct[0], rtol=1e-12)
    # shells m <= nx/3 add up to the modes they contain
    k = np.array([sts_oracle.kwn(i, nx) for i in range(nx)])
    m = np.rint(np.sqrt(k[:, None] ** 2 + k[None, :] ** 2)).astype(int)
    assert np.allclose(s2.sum(0), [direct[m == j].sum() for j in range(nx // 3 + 1)], rtol=1e-12)


def test_single_frequency_mode_peaks_at_its_bin():
    """kpsi(k0, t) = exp(-2 pi i f t / Nt): the line spectrum peaks at bin f."""
    nt, nx, f = 64, 16, 5
    t = np.arange(nt)
    rec = np.zeros((nt, nx, nx), dtype=complex)
    rec[:, 0, 3] = np.exp(2j * math.pi * f * t / nt)     # FFTW_FORWARD sign -1 -> peak at +f
    s1, s2 = sts_oracle.spectra(rec)
    assert int(np.argmax(s1[:, 3])) == f
    assert np.all(s1[:, [0, 1, 2, 4]] == 0.0)
    assert int(np.argmax(s2[:, 3])) == f and np.allclose(s2[:, 3], s1[:, 3], rtol=1e-15)
