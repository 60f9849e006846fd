"""RK4 pass kernels by programmatic dependent launch (the default): each pass
kernel waits for its predecessor to complete before it touches a field, so
the result is that of plain launches (VK_PDL=0) bit for bit.  Covered: the
FP32 and FP64 steps at 1024^2 (graph replays), ARGLE (the pass kernels
between plain launches), and the particle step, where plain kernels sit
between the pass kernels.
"""
import math

import numpy as np
import pytest

from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu


def _psi0(n, nv=64):
    psi, _ = vk.ic_vortices(n, n, nv, seed=13, min_sep=4 * math.sqrt(2) * 2 * math.pi / n)
    return psi


def _rk4_argle(monkeypatch, pdl, n, prec):
    monkeypatch.setenv("VK_PDL", "1" if pdl else "0")
    psi0 = _psi0(n)
    with vk.GPESolver(vk.params_for(n, dt=5e-4, precision=prec)) as s:
        s.set_psi(psi0)
        s.gpe_rk4(12)
        a = s.get_psi()
        s.set_psi(psi0)
        r = s.argle(4)
        return a, s.get_kpsi(), r


@pytest.mark.parametrize("prec", [vk.VK_PREC_FP32, vk.VK_PREC_FP64])
def test_pdl_equals_plain_launches(monkeypatch, prec):
    a, ka, ra = _rk4_argle(monkeypatch, True, 1024, prec)
    b, kb, rb = _rk4_argle(monkeypatch, False, 1024, prec)
    assert np.isfinite(a).all()
    assert np.array_equal(a, b) and np.array_equal(ka, kb) and ra == rb


def _particles(monkeypatch, pdl):
    monkeypatch.setenv("VK_PDL", "1" if pdl else "0")
    n, npart = 256, 4
    dx = 2 * math.pi / n
    d = 2.0 * math.sqrt(2.0) * dx
    p = vk.params_for(n, dt=1e-3, n_particles=npart, ppotd=2.0, ppotv0=10.0, gp_mass_part=5.0 * math.pi * d * d)
    rng = np.random.default_rng(3)
    with vk.GPESolver(p) as s:
        s.set_psi(_psi0(n, 8))
        s.particles_set(rng.uniform(0, 2 * np.pi, (npart, 2)), rng.normal(0, 0.1, (npart, 2)), np.zeros((npart, 2)))
        s.gpe_rk4(6)
        pos, vel, _ = s.particles_get()
        return s.get_psi(), pos, vel


def test_pdl_particle_step_equals_plain_launches(monkeypatch):
    a, pa, va = _particles(monkeypatch, True)
    b, pb, vb = _particles(monkeypatch, False)
    assert np.array_equal(a, b) and np.array_equal(pa, pb) and np.array_equal(va, vb)
