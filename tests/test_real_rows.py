"""The single-row real transforms of the FP64 x passes at 1024^2
(x1_single_body / x2_single_body in quantumvortices_gb300/csrc/vk_kernels.cuh),
restated with the kernels' expressions in numpy float64:

  k_x1: z(n) = rho(2n) + i rho(2n+1), Z = F_{L/2} z,
        rho^(k) = E(k) + W_L^k O(k), E = (Z(k) + conj Z(L/2-k))/2,
        O = -i (Z(k) - conj Z(L/2-k))/2, k in [0, K];
  k_x2: Z(k) = A(k) + conj A(L/2-k) + i (A(k) - conj A(L/2-k)) W_L^-k,
        (F^-1_{L/2} Z)(n) = p(2n) + i p(2n+1) for the real row p whose
        Hermitian spectrum A is zero for K < k < L-K.

Checked against numpy's full-length transforms to 1e-13 of the row scale.
The GPU tests check the kernels themselves against the row-pair layout and
the oracle."""
import numpy as np
import pytest


def unpack_r2c(rho, K):
    L = rho.size
    H = L // 2
    tw = np.exp(-2j * np.pi * np.arange(L) / L)
    Z = np.fft.fft(rho[0::2] + 1j * rho[1::2])
    k = np.arange(K + 1)
    zk, zm = Z[k], Z[(H - k) & (H - 1)]
    er, ei = 0.5 * (zk.real + zm.real), 0.5 * (zk.imag - zm.imag)
    o_r, o_i = 0.5 * (zk.imag + zm.imag), 0.5 * (zm.real - zk.real)
    w = tw[k]
    return (er + (w.real * o_r - w.imag * o_i)) + 1j * (ei + (w.real * o_i + w.imag * o_r))


def pack_c2r(row, L, K):
    H = L // 2
    tw = np.exp(-2j * np.pi * np.arange(L) / L)
    k = np.arange(H)
    m = H - k
    a = np.where(k <= K, row[np.minimum(k, K)], 0)
    b = np.where(m <= K, row[np.minimum(m, K)], 0)
    er, ei = a.real + b.real, a.imag - b.imag
    dr, di = a.real - b.real, a.imag + b.imag
    w = tw[k]
    o_r, o_i = dr * w.real + di * w.imag, di * w.real - dr * w.imag
    Z = (er - o_i) + 1j * (ei + o_r)
    z = np.fft.ifft(Z) * H  # unnormalised inverse
    p = np.empty(L)
    p[0::2], p[1::2] = z.real, z.imag
    return p


@pytest.mark.parametrize("L", [128, 256, 1024, 4096])
def test_single_row_forward_matches_full_transform(L):
    K = int(np.sqrt(np.floor((L / 3.0) ** 2 - 1e-9)))
    rng = np.random.default_rng(L)
    rho = rng.random(L) + 0.5
    ref = np.fft.fft(rho)[:K + 1]
    got = unpack_r2c(rho, K)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("L", [128, 256, 1024, 4096])
def test_single_row_inverse_matches_full_transform(L):
    K = int(np.sqrt(np.floor((L / 3.0) ** 2 - 1e-9)))
    rng = np.random.default_rng(L + 1)
    row = rng.normal(size=K + 1) + 1j * rng.normal(size=K + 1)
    row[0] = row[0].real
    full = np.zeros(L, complex)
    full[:K + 1] = row
    full[L - K:] = np.conj(row[1:][::-1])
    ref = np.fft.ifft(full).real * L
    got = pack_c2r(row, L, K)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
