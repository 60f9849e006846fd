"""Gaussian particles coupled to the GPE: GPU against the CPU FP64 oracle
(which follows src/gpe_particle.f90 with its 4 FFTs per particle and stage;
the GPU takes all forces from one Parseval pass).

Tolerances: psi relative L2 1e-12; particle positions/velocities 1e-12
absolute (O(1) values); forces 1e-9 relative to the largest force.
"""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle
from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu


def _params(n, npart, dt=1e-3, prec=vk.VK_PREC_FP64):
    dx = 2 * math.pi / n
    d = 2.0 * math.sqrt(2.0) * dx            # ppotd = 2 -> d = 2 xi
    mass = 5.0 * math.pi * d * d             # M = 5 rho0 pi d^2
    return vk.params_for(n, dt=dt, precision=prec, n_particles=npart, ppotd=2.0, ppotv0=10.0, gp_mass_part=mass)


def _state(n, npart, seed=4, nv=4, prec=vk.VK_PREC_FP64, dt=1e-3):
    p = _params(n, npart, dt, prec)
    psi0, _ = vk.ic_vortices(n, n, nv, seed=seed)
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, 2 * np.pi, (npart, 2))
    vel = rng.normal(0, 0.1, (npart, 2))
    f0 = np.zeros((npart, 2))
    f0[0] = [0.05, -0.02]
    s = vk.GPESolver(p)
    s.set_psi(psi0)
    s.particles_set(pos, vel, f0)
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0, otoc=True)
    o.particles_set(pos, vel, f0)
    return s, o, p


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_forces_match_oracle():
    s, o, _ = _state(64, 4)
    d = s.diagnostics_gpe()
    sc, _ = o.diagnostics()
    _, _, frc = s.particles_get()
    _, _, ofrc = o.particles_get()
    assert np.abs(frc - ofrc).max() <= 1e-9 * np.abs(ofrc).max()
    assert abs(d.eppot - sc[7]) <= 1e-11 * abs(sc[7])
    assert abs(d.eobj_kin - sc[8]) <= 1e-13 * abs(sc[8])
    assert d.esrep == sc[9] == 0.0  # no force evaluation has run yet (gpdeltaE unset)
    d2 = s.diagnostics_gpe()
    sc2, _ = o.diagnostics()
    assert abs(d2.esrep - sc2[9]) <= 1e-12 * abs(sc2[9]) and sc2[9] != 0.0
    s.close()


def test_rk4_with_particles_parity():
    s, o, _ = _state(64, 4)
    s.gpe_rk4(10)
    o.gpe_rk4(10)
    assert rel(s.get_psi(), o.get_psi()) < 1e-12
    pos, vel, _ = s.particles_get()
    opos, ovel, _ = o.particles_get()
    assert np.abs(pos - opos).max() < 1e-12
    assert np.abs(vel - ovel).max() < 1e-12
    s.close()


def test_argle_with_particles_parity():
    s, o, _ = _state(64, 3)
    s.argle(10)
    o.argle(10)
    assert rel(s.get_kpsi(), o.get_kpsi()) < 1e-12
    s.close()


def test_single_particle_in_uniform_fluid_feels_only_external_force():
    n = 64
    p = _params(n, 1)
    s = vk.GPESolver(p)
    s.set_psi(np.ones((n, n), complex))
    f0 = np.array([[0.3, -0.1]])
    s.particles_set(np.array([[1.0, 2.0]]), np.zeros((1, 2)), f0)
    s.diagnostics_gpe()
    _, _, frc = s.particles_get()
    assert np.abs(frc - f0).max() < 1e-12
    s.close()


def test_mirror_pair_equal_and_opposite():
    n = 64
    p = _params(n, 2)
    x = np.arange(n) * 2 * np.pi / n
    X, Y = np.meshgrid(x, x)
    psi = 1.0 + 0.2 * np.cos(X) + 0j       # symmetric about x = 0 and x = pi
    s = vk.GPESolver(p)
    s.set_psi(psi)
    pos = np.array([[np.pi - 0.7, 1.3], [np.pi + 0.7, 1.3]])
    s.particles_set(pos, np.zeros((2, 2)), np.zeros((2, 2)))
    s.diagnostics_gpe()
    _, _, frc = s.particles_get()
    assert abs(frc[0, 0] + frc[1, 0]) <= 1e-10 * abs(frc[0, 0])
    assert abs(frc[0, 1] - frc[1, 1]) <= 1e-12
    s.close()


def test_particles_1024_sixteen_particles_rk4_smoke():
    n = 1024
    p = _params(n, 16, dt=5e-4)
    psi0, _ = vk.ic_vortices(n, n, 64, seed=2, min_sep=4 * math.sqrt(2) * 2 * math.pi / n)
    rng = np.random.default_rng(2)
    s = vk.GPESolver(p)
    s.set_psi(psi0)
    s.particles_set(rng.uniform(0, 2 * np.pi, (16, 2)), rng.normal(0, 0.1, (16, 2)), np.zeros((16, 2)))
    s.gpe_rk4(20)
    pos, vel, _ = s.particles_get()
    assert np.isfinite(pos).all() and np.isfinite(vel).all() and np.isfinite(s.get_psi()).all()
    s.close()


def test_particles_fp32_bulk():
    """FP32 bulk path with particles: psi within 1e-5 and positions within
    1e-6 of the FP64 oracle after 20 steps."""
    s, o, _ = _state(64, 4, prec=vk.VK_PREC_FP32)
    s.gpe_rk4(20)
    o.gpe_rk4(20)
    assert rel(s.get_psi(), o.get_psi()) < 1e-5
    pos, _, _ = s.particles_get()
    opos, _, _ = o.particles_get()
    assert np.abs(pos - opos).max() < 1e-6
    s.close()


def test_two_particle_repulsion_closed_form():
    """Two particles in a uniform fluid (grad rho = 0: no fluid force) feel
    the short-range repulsion of src/gpe_particle.f90:378-427 alone:
    -384 dE pi^12 r0^12 / L^12 sin(dq) / (-3 + cos dqx + cos dqy)^7, with the
    single-precision literal dE = 0.062, r0 = 4 xi and L = 2 pi."""
    n = 64
    p = _params(n, 2)
    s = vk.GPESolver(p)
    s.set_psi(np.ones((n, n), complex))
    q = np.array([[1.0, 2.0], [1.9, 1.4]])
    s.particles_set(q, np.zeros((2, 2)), np.zeros((2, 2)))
    s.diagnostics_gpe()
    _, _, frc = s.particles_get()
    s.close()
    rf = 384.0 * float(np.float32(0.062)) * math.pi ** 12 * (4.0 * p.xi) ** 12 / (2 * math.pi) ** 12
    dq = q[0] - q[1]
    f01 = -rf * np.sin(dq) / (-3 + math.cos(dq[0]) + math.cos(dq[1])) ** 7
    assert np.abs(frc[0] - f01).max() <= 1e-12 * np.abs(f01).max()
    assert np.abs(frc[1] + f01).max() <= 1e-12 * np.abs(f01).max()
