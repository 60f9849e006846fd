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
