"""The -DGPE_FRCDISP right-hand side in the oracle (src/gpe.f90:623-658), on
the CPU: known answers for the dissipation, statistics of the forcing
phases, and the forcing confined to its shell."""
import math

import numpy as np

from oracle.oracle import Oracle
from quantumvortices_gb300 import vk


def _oracle(n=32, dt=1e-3):
    return Oracle.from_vk_params(vk.params_for(n, dt=dt))


def test_hypoviscosity_decays_a_single_mode_exactly():
    """g = 0 (no nonlinearity), one mode k = (1, 0): the RHS is
    (-i(alpha k^2 - Omega) - vishypo k^-16) c, so RK4 multiplies c by the
    degree-4 Taylor polynomial of exp(z dt) per step."""
    n, dt, nu = 32, 1e-3, 0.7
    p = vk.params_for(n, dt=dt)
    p.gstrength = 0.0
    o = Oracle.from_vk_params(p)
    k = np.zeros((n, n), dtype=complex)
    k[1, 0] = 2.0                                   # kx = 1, ky = 0
    o.set_kpsi(k)
    o.set_psi(o.fft_inverse(k), otoc=False)
    o.set_frcdisp(True, vishypo=nu)
    steps = 20
    o.gpe_rk4(steps)
    z = (-1j * (p.alpha * 1.0 - p.omega_chem) - nu) * dt
    r = 1 + z + z ** 2 / 2 + z ** 3 / 6 + z ** 4 / 24
    got = o.get_kpsi()[1, 0]
    assert abs(got - 2.0 * r ** steps) <= 1e-13 * abs(got)


def test_forcing_is_confined_to_its_shell_and_phases_are_uniform():
    """psi = 0, g = 0: after one step only kf1^2 <= k^2 <= kf2^2 modes are
    non-zero; the first-stage forcing phases are uniform on [0, 2 pi)."""
    n, dt = 64, 1e-3
    p = vk.params_for(n, dt=dt)
    p.gstrength = 0.0
    o = Oracle.from_vk_params(p)
    o.set_psi(np.zeros((n, n), dtype=complex), otoc=False)
    o.set_frcdisp(True, famp=1.0, kf1=3.0, kf2=9.0, seed=11)
    o.gpe_rk4(1)
    kp = o.get_kpsi()
    k = np.array([i if i < n // 2 else i - n for i in range(n)])
    ksq = k[:, None] ** 2 + k[None, :] ** 2
    shell = (ksq >= 9) & (ksq <= 81)
    assert np.all(kp[~shell] == 0) and np.all(np.abs(kp[shell]) > 0)
    ph = np.angle(kp[shell])
    hist, _ = np.histogram(ph, bins=8, range=(-math.pi, math.pi))
    expected = shell.sum() / 8
    chi2 = ((hist - expected) ** 2 / expected).sum()
    assert chi2 < 24.3, (hist, chi2)              # 7 dof, p ~ 0.001


def test_hyperviscosity_damps_high_modes_more():
    n = 32
    o = _oracle(n)
    psi, _ = vk.ic_vortices(n, n, 4, seed=2)
    o.set_psi(psi)
    o.set_frcdisp(True, vishype=1e-18)
    k0 = o.get_kpsi()
    o.gpe_rk4(5)
    k1 = o.get_kpsi()
    o2 = _oracle(n)
    o2.set_psi(psi)
    o2.gpe_rk4(5)
    k2 = o2.get_kpsi()
    kk = np.array([i if i < n // 2 else i - n for i in range(n)])
    hi = (kk[:, None] ** 2 + kk[None, :] ** 2) >= 64
    assert np.linalg.norm(k1[hi]) < np.linalg.norm(k2[hi])
    assert np.isfinite(k0).all()


def test_counterflow_on_a_plane_wave_is_a_chemical_potential_shift():
    """g = 0, psi = exp(i k.x): grad psi = i k psi, so the counterflow term
    -i v.grad psi = (v.k) psi and one ARGLE step multiplies the mode by
    (1 + dt (v.k + Omega)) / (1 + alpha k^2 dt)  (src/gpe.f90:135-145, 199-203)."""
    n, dt = 32, 1e-3
    p = vk.params_for(n, dt=dt)
    p.gstrength = 0.0
    o = Oracle.from_vk_params(p)
    x = np.arange(n) * 2 * math.pi / n
    kx, ky = 2, -3
    psi = np.exp(1j * (kx * x[None, :] + ky * x[:, None]))
    o.set_psi(psi, otoc=False)
    vnx, vny = 0.3, -0.7
    o.set_argle_flow(2, vnx, vny)
    steps = 5
    o.argle(steps)
    f = (1 + dt * (vnx * kx + vny * ky + p.omega_chem)) / (1 + p.alpha * (kx * kx + ky * ky) * dt)
    want = n * n * f ** steps
    got = o.get_kpsi()[kx % n, ky % n]
    assert abs(got - want) <= 1e-12 * abs(want)


def test_advection_velocity_field_is_taylor_green():
    """The advection term with psi = 1 (grad psi = 0) is -(1/4)(1/alpha)|u|^2,
    |u|^2 = sin^2 x cos^2 y + cos^2 x sin^2 y: one step from psi = 1 with
    g = 0 changes kpsi by dt * F[-(1/4)(1/alpha)|u|^2] / (1 + alpha k^2 dt)."""
    n, dt = 32, 1e-3
    p = vk.params_for(n, dt=dt)
    p.gstrength = 0.0
    o = Oracle.from_vk_params(p)
    o.set_psi(np.ones((n, n), dtype=complex), otoc=False)
    o.set_argle_flow(1)
    k0 = o.get_kpsi()
    o.argle(1)
    x = np.arange(n) * 2 * math.pi / n
    X, Y = np.meshgrid(x, x)
    u2 = (np.sin(X) * np.cos(Y)) ** 2 + (np.cos(X) * np.sin(Y)) ** 2
    nhat = np.fft.fft2(-0.25 / p.alpha * u2).T
    k = np.array([i if i < n // 2 else i - n for i in range(n)])
    denom = 1 + p.alpha * (k[:, None] ** 2 + k[None, :] ** 2) * dt
    want = (k0 + dt * (nhat + p.omega_chem * k0)) / denom
    assert np.abs(o.get_kpsi() - want).max() <= 1e-12 * np.abs(want).max()


def test_sgle_chemical_potential_ode_on_a_uniform_state():
    """No noise (oneybeta = 0), psi = a: norm = a^2 Lx Ly, so one step sets
    omega = chempot0 - dt nuN (a^2 - 1) (src/gpe.f90:264) and the k = 0 mode
    follows a' = a + dt (-g a^3 + omega a) (src/gpe.f90:211)."""
    n, dt, a, nun, mu0 = 32, 1e-3, 1.3, 5.0, 0.8
    p = vk.params_for(n, dt=dt)
    o = Oracle.from_vk_params(p)
    o.set_psi(np.full((n, n), a, dtype=complex), otoc=False)
    o.set_sgle(True, oneybeta=0.0, nuN=nun, chempot0=mu0)
    o.argle(1)
    om = mu0 - dt * nun * (a * a - 1.0)
    assert abs(o.chempot - om) <= 1e-13 * abs(om)
    want = a + dt * (-p.gstrength * a ** 3 + om * a)
    assert abs(o.get_kpsi()[0, 0] / (n * n) - want) <= 1e-13 * abs(want)


def test_sgle_noise_statistics_and_truncation():
    """psi = 0, g = 0, nuN = 0: one step leaves kpsi = sqrt(dt) F[noise]
    (2/3 mask) / (1 + alpha k^2 dt); E|F[noise]|^2 = 2 amp^2 nx ny with
    amp = sqrt(oneybeta/(2 alpha))/sqrt(dvol).  With self-truncation every
    k^2 > ktrunc^2 is zero."""
    n, dt, beta = 64, 1e-3, 0.5
    p = vk.params_for(n, dt=dt)
    p.gstrength = 0.0
    o = Oracle.from_vk_params(p)
    o.set_psi(np.zeros((n, n), dtype=complex), otoc=False)
    o.set_sgle(True, oneybeta=beta, nuN=0.0, chempot0=0.0, seed=5)
    o.argle(1)
    k = np.array([i if i < n // 2 else i - n for i in range(n)])
    ksq = k[:, None] ** 2 + k[None, :] ** 2
    kept = ksq < (n / 3.0) ** 2
    den = 1 + p.alpha * ksq * dt
    fz = o.get_kpsi() * den / math.sqrt(dt)
    assert np.all(fz[~kept] == 0)
    dvol = (2 * math.pi / n) ** 2
    amp2 = beta / (2 * p.alpha) / dvol
    ratio = np.mean(np.abs(fz[kept]) ** 2) / (2 * amp2 * n * n)
    assert abs(ratio - 1.0) < 0.05, ratio
    o2 = Oracle.from_vk_params(p)
    o2.set_psi(np.zeros((n, n), dtype=complex), otoc=False)
    o2.set_sgle(True, oneybeta=beta, chempot0=0.0, selftrunc=True, ktrunc=6.0, seed=5)
    o2.argle(1)
    kp = o2.get_kpsi()
    assert np.all(kp[ksq > 36] == 0) and np.all(kp[ksq <= 36] != 0)
