"""CPU restatement of the spatio-temporal spectra post-processor
(Run/CompSTS/driver.f90:132-265) for the records sts_gpe writes
(src/diagnostics.f90:636-695).

TEST INFRASTRUCTURE ONLY: imported by tests/, never by the product package.
PARITY UNPINNED against the reference binary (no Fortran/FFTW toolchain
here); numpy's FFT stands in for FFTW_FORWARD.
"""
from __future__ import annotations

import math

import numpy as np


def hann(nt: int) -> np.ndarray:
    """whann = half*(one - COS(tpp)), tpp = 2*pi*(i4-1)/(Ntt-1)
    (Run/CompSTS/driver.f90:194-196, 236-238)."""
    pi = 4.0 * math.atan(1.0)
    return np.array([0.5 * (1.0 - math.cos(2.0 * pi * t / (nt - 1))) for t in range(nt)])


def kwn(i: int, n: int) -> int:
    """k = (i1-1) - N*(i1/(N/2+1)) with i1 = i+1 (Run/CompSTS/driver.f90:233-235)."""
    return i - n * ((i + 1) // (n // 2 + 1))


def spectra(records: np.ndarray):
    """records[nt, nx, ny]: kpsi planes in the transposed layout [kx][ky].
    Returns (sts1d[nt, ny], sts2d[nt, nx//3 + 1]):
      sts1d[w, ky] = stsnorm |X(kx=0, ky, w)|^2          (:190-203)
      sts2d[w, m]  = sum_{nint|k| = m} stsnorm |X(k, w)|^2 (:243-255, written
                     for m = 0..INT(Nx/3), :262)
    X = FFTW_FORWARD along time of the Hann-windowed record,
    stsnorm = (1/Ntt)^2 (1/(Nx Ny))^2 (:123)."""
    nt, nx, ny = records.shape
    a, b = 1.0 / nt, 1.0 / (nx * ny)
    stsnorm = (a * a) * (b * b)
    x = records * hann(nt)[:, None, None]
    X = np.fft.fft(x, axis=0)
    P = stsnorm * np.abs(X) ** 2
    sts1d = P[:, 0, :].copy()
    nsh = nx // 3 + 1
    k1 = np.array([kwn(i, nx) for i in range(nx)])
    k2 = np.array([kwn(i, ny) for i in range(ny)])
    ksq = k1[:, None] ** 2 + k2[None, :] ** 2
    mshl = np.rint(np.sqrt(ksq.astype(float))).astype(int)   # NINT; never a half-integer
    sts2d = np.zeros((nt, nsh))
    flat_m = mshl.ravel()
    keep = flat_m < nsh
    idx = np.nonzero(keep)[0]                                 # increasing (kx, ky) order
    Pf = P.reshape(nt, -1)
    for w in range(nt):
        np.add.at(sts2d[w], flat_m[idx], Pf[w, idx])          # sequential, in mode order
    return sts1d, sts2d
