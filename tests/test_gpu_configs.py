"""GPU against the CPU FP64 oracle on the benchmark configurations at their own
sizes (the smaller parity tests live in test_gpu_parity.py and
test_gpu_particles.py).

* 1024^2 with 16 Gaussian particles (V0 = 10, d = 2 xi, M = 5 pi d^2,
  64 vortices, dt = 5e-4): the oracle takes 4 FFTs per particle and stage
  (src/gpe_particle.f90:219-324), the GPU one Parseval pass for all of them.
  psi relative L2 <= 1e-12, positions and velocities <= 1e-12 absolute; on
  the final state (diagnostics), forces <= 1e-9 of the largest force and the
  particle potential and kinetic energies <= 1e-11 / 1e-12 relative.
* ARGLE with renormalisation (argle_renorm = 1) at 128^2 and 1024^2:
  kpsi <= 1e-12 and the norm dvol/(nx ny) sum|kpsi|^2 equal to
  Nparticle = rho_avg Lx Ly to 1e-12.
* 4096^2 plain FP64 RK4 with 1024 vortices (dt = 5e-4): psi <= 1e-12 after
  two steps.
"""
import math
import os

import numpy as np
import pytest

from oracle.oracle import Oracle
from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu

TWO_PI = 2.0 * math.pi


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _particle_params(n, npart, dt):
    dx = TWO_PI / n
    d = 2.0 * math.sqrt(2.0) * dx            # ppotd = 2: d = 2 xi
    mass = 5.0 * math.pi * d * d             # M = 5 rho0 pi d^2
    return vk.params_for(n, dt=dt, n_particles=npart, ppotd=2.0, ppotv0=10.0, gp_mass_part=mass)


def test_particles_1024_sixteen_particles_vs_oracle():
    n, npart, steps = 1024, 16, 3
    p = _particle_params(n, npart, 5e-4)
    psi0, _ = vk.ic_vortices(n, n, 64, seed=2, min_sep=4 * math.sqrt(2) * TWO_PI / n)
    rng = np.random.default_rng(2)
    pos0 = rng.uniform(0, TWO_PI, (npart, 2))
    vel0 = rng.normal(0, 0.1, (npart, 2))
    f0 = np.zeros((npart, 2))
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        s.particles_set(pos0, vel0, f0)
        s.gpe_rk4(steps)
        got = s.get_psi()
        pos, vel, _ = s.particles_get()
        d = s.diagnostics_gpe()          # evaluates the forces on the final state
        _, _, frc = s.particles_get()
    o = Oracle.from_vk_params(p, threads=os.cpu_count())
    o.set_psi(psi0, otoc=True, k_otoc=p.k_otoc_gp, eps_otoc=p.eps_otoc_gp)
    o.particles_set(pos0, vel0, f0)
    o.gpe_rk4(steps)
    opos, ovel, _ = o.particles_get()
    assert rel(got, o.get_psi()) < 1e-12
    assert np.abs(pos - opos).max() < 1e-12
    assert np.abs(vel - ovel).max() < 1e-12
    sc, _ = o.diagnostics()
    _, _, ofrc = o.particles_get()
    assert np.abs(ofrc).max() > 0.0
    assert np.abs(frc - ofrc).max() <= 1e-9 * np.abs(ofrc).max()
    assert abs(d.eppot - sc[7]) <= 1e-11 * abs(sc[7])
    assert abs(d.eobj_kin - sc[8]) <= 1e-12 * abs(sc[8])


@pytest.mark.parametrize("n,steps", [(128, 50), (1024, 10)])
def test_argle_renormalisation_vs_oracle(n, steps):
    p = vk.params_for(n, dt=1e-3 if n == 128 else 5e-4, argle_renorm=True)
    psi0, _ = vk.ic_vortices(n, n, 8 if n == 128 else 64, seed=9)
    psi0 = 0.8 * psi0  # start away from the target norm
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        r_gpu = s.argle(steps)
        kpsi = s.get_kpsi()
    o = Oracle.from_vk_params(p, threads=os.cpu_count())
    assert o.p.renorm == 1
    o.set_psi(psi0, otoc=True, k_otoc=p.k_otoc_gp, eps_otoc=p.eps_otoc_gp)
    r_ref = o.argle(steps)
    assert rel(kpsi, o.get_kpsi()) < 1e-12
    assert abs(r_gpu - r_ref) <= 1e-9 * r_ref
    dvol = (TWO_PI / n) ** 2
    norm = dvol / (n * n) * float(np.sum(np.abs(kpsi) ** 2))
    assert abs(norm - TWO_PI * TWO_PI) <= 1e-12 * TWO_PI * TWO_PI


def test_rk4_parity_fp64_4096_with_1024_vortices():
    n, steps = 4096, 2
    p = vk.params_for(n, dt=5e-4)
    with vk.GPESolver(p) as s:
        s.set_psi_vortices(1024, seed=5, min_sep=4 * math.sqrt(2) * TWO_PI / n)
        psi0 = s.get_psi()   # the state after set_psi (OTOC band limit applied)
        kpsi0 = s.get_kpsi()
        s.gpe_rk4(steps)
        got = s.get_psi()
    o = Oracle.from_vk_params(p, threads=os.cpu_count())
    o.set_psi(psi0, otoc=False)   # psi0 is already band-limited
    assert rel(o.get_kpsi(), kpsi0) < 1e-13
    o.gpe_rk4(steps)
    assert rel(got, o.get_psi()) < 1e-12
