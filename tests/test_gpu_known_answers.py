"""Exact known answers and exact properties of the GPU path (FP64),
independent of the oracle.

A plane wave A e^{ik.x} keeps a uniform density, so P_G |psi|^2 = |A|^2 and
the passes reduce to scalar maps of the amplitude:
* RK4 (src/gpe.f90:310-671): the scalar RK4 of a' = -i (alpha k^2 - Omega + g |a|^2) a;
* ARGLE (src/gpe.f90:5-224): A <- A (1 + dt (Omega - g |A|^2)) / (1 + alpha k^2 dt),
  with the residual |A_new - A_old| / (dt |A_old|) of the last step;
* diagnostics_gpe (src/diagnostics.f90:4-571): norm = |A|^2 L^2, mom = 2 alpha |A|^2 k,
  Egrad = 2 alpha^2 |A|^2 k^2, Echem = 2 alpha Omega |A|^2, Eint = alpha g |A|^4, and the
  |kpsi|^2 spectrum holds |A|^2 in the shell nint(|k|) alone.
With g = Omega = 0 every mode follows the RK4 polynomial R(z)^n of its
linear rotation, and at 1024^2 the step commutes with a shift by whole grid
points and with a quarter turn.  Bounds: 1e-12 (FP64 rounding of a few
hundred transforms of an O(1) field); the FP32 plane wave to 1e-5.
"""
import math

import numpy as np
import pytest

from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu

K = (3, -2)
A0 = 0.9 + 0.1j


def _plane_wave(n):
    x = np.arange(n) * 2 * np.pi / n
    X, Y = np.meshgrid(x, x)
    return A0 * np.exp(1j * (K[0] * X + K[1] * Y))


@pytest.mark.parametrize("n", [64, 1024])
def test_plane_wave_rk4(n):
    p = vk.params_for(n, dt=5e-4, otoc=False)
    psi0 = _plane_wave(n)
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        s.gpe_rk4(10)
        got = s.get_psi()
    k2 = K[0] ** 2 + K[1] ** 2
    f = lambda a: -1j * (p.alpha * k2 - p.omega_chem + p.gstrength * abs(a) ** 2) * a
    a, dt = A0, p.dt
    for _ in range(10):
        k1 = f(a)
        k2_ = f(a + dt / 2 * k1)
        k3 = f(a + dt / 2 * k2_)
        k4 = f(a + dt * k3)
        a = a + dt / 6 * (k1 + 2 * k2_ + 2 * k3 + k4)
    assert np.abs(got - psi0 * (a / A0)).max() < 1e-12


@pytest.mark.parametrize("n", [64, 1024])
def test_plane_wave_argle(n):
    p = vk.params_for(n, dt=1e-3, otoc=False)
    with vk.GPESolver(p) as s:
        s.set_psi(_plane_wave(n))
        r = s.argle(9)
        kp = s.get_kpsi()
    k2 = K[0] ** 2 + K[1] ** 2
    a = A0
    for _ in range(9):
        prev = a
        a = a * (1 + p.dt * (p.omega_chem - p.gstrength * abs(a) ** 2)) / (1 + p.alpha * k2 * p.dt)
    want = np.zeros((n, n), complex)
    want[K[0] % n, K[1] % n] = a * n * n
    assert np.abs(kp - want).max() < 1e-12 * n * n
    assert abs(r - abs(a - prev) / (p.dt * abs(prev))) < 1e-9 * r


def test_plane_wave_diagnostics():
    n = 64
    p = vk.params_for(n, dt=1e-3, otoc=False)
    with vk.GPESolver(p) as s:
        s.set_psi(_plane_wave(n))
        d = s.diagnostics_gpe()
    al, g, om, a2 = p.alpha, p.gstrength, p.omega_chem, abs(A0) ** 2
    k2 = K[0] ** 2 + K[1] ** 2
    want = [(d.momx, 2 * al * a2 * K[0]), (d.momy, 2 * al * a2 * K[1]), (d.egrad, 2 * al * al * a2 * k2),
            (d.echem, 2 * al * om * a2), (d.eintr, al * g * a2 * a2),
            (d.etot, 2 * al * al * a2 * k2 + al * g * a2 * a2), (d.norm, a2 * (2 * math.pi) ** 2)]
    for got, w in want:
        assert abs(got - w) <= 1e-12 * max(1.0, abs(w)), (got, w)
    shell = np.zeros(d.spec.shape[1])
    shell[int(round(math.sqrt(k2)))] = a2
    assert np.abs(d.spec[5] - shell).max() <= 1e-12


def test_linear_dispersion_without_interaction():
    """g = Omega = 0: every mode evolves by the RK4 polynomial of
    z = -i alpha k^2 dt, psi^(t_n) = R(z)^n psi^(0), R = 1 + z + z^2/2 + z^3/6 + z^4/24."""
    n = 64
    p = vk.params_for(n, dt=2e-3, otoc=False)
    p.gstrength = 0.0
    p.omega_chem = 0.0
    x = np.arange(n) * 2 * np.pi / n
    X, Y = np.meshgrid(x, x)
    rng = np.random.default_rng(5)
    psi0 = np.zeros((n, n), complex)
    for kx, ky in [(1, 2), (-3, 4), (5, -1), (0, 7)]:
        psi0 += (rng.standard_normal() + 1j * rng.standard_normal()) * np.exp(1j * (kx * X + ky * Y))
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        s.gpe_rk4(6)
        got = s.get_psi()
    kk = np.fft.fftfreq(n, 1.0 / n)
    KX, KY = np.meshgrid(kk, kk)
    z = -1j * p.alpha * (KX ** 2 + KY ** 2) * p.dt
    R = 1 + z + z * z / 2 + z ** 3 / 6 + z ** 4 / 24
    want = np.fft.ifft2(np.fft.fft2(psi0) * R ** 6)
    assert np.abs(got - want).max() < 1e-12 * np.abs(want).max()


def test_translation_equivariance_at_1024():
    """The step commutes with a shift by whole grid points (all the physics is
    in Fourier multipliers and pointwise products): 1024^2 FP64, 64 vortices,
    5 RK4 steps from psi and from psi rolled by (37, -101)."""
    n = 1024
    p = vk.params_for(n, dt=5e-4)
    psi0, _ = vk.ic_vortices(n, n, 64, seed=9, min_sep=4 * math.sqrt(2) * 2 * math.pi / n)
    shift = (37, -101)
    out = []
    for psi in (psi0, np.roll(psi0, shift, axis=(0, 1))):
        with vk.GPESolver(p) as s:
            s.set_psi(np.ascontiguousarray(psi))
            s.gpe_rk4(5)
            out.append(s.get_psi())
    a, b = np.roll(out[0], shift, axis=(0, 1)), out[1]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-12


def test_rotation_equivariance_at_1024():
    """A quarter turn of the grid commutes with the step: the kinetic operator
    and the 2/3 disk are isotropic, and the quarter turn swaps the x passes
    (real-row transforms) with the y passes (complex, transposed layout), so
    the two sides run different kernels on the same physics."""
    n = 1024
    p = vk.params_for(n, dt=5e-4)
    psi0, _ = vk.ic_vortices(n, n, 64, seed=12, min_sep=4 * math.sqrt(2) * 2 * math.pi / n)
    out = []
    for psi in (psi0, np.rot90(psi0)):
        with vk.GPESolver(p) as s:
            s.set_psi(np.ascontiguousarray(psi))
            s.gpe_rk4(5)
            out.append(s.get_psi())
    a, b = np.rot90(out[0]), out[1]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-12


def test_plane_wave_rk4_fp32():
    """The FP32 path (background density moved out of the transforms) on the
    plane wave: the scalar RK4 map to FP32 accuracy (1e-5 relative)."""
    n = 256
    p = vk.params_for(n, dt=5e-4, precision=vk.VK_PREC_FP32, otoc=False)
    psi0 = _plane_wave(n)
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        s.gpe_rk4(10)
        got = s.get_psi()
    k2 = K[0] ** 2 + K[1] ** 2
    f = lambda a: -1j * (p.alpha * k2 - p.omega_chem + p.gstrength * abs(a) ** 2) * a
    a, dt = A0, p.dt
    for _ in range(10):
        k1 = f(a)
        k2_ = f(a + dt / 2 * k1)
        k3 = f(a + dt / 2 * k2_)
        k4 = f(a + dt * k3)
        a = a + dt / 6 * (k1 + 2 * k2_ + 2 * k3 + k4)
    want = psi0 * (a / A0)
    assert np.abs(got - want).max() < 1e-5 * np.abs(want).max()
