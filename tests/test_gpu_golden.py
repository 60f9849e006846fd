"""The GPU path against the committed golden fixtures (oracle outputs made
by tests/golden/make_golden.py), through the C ABI.

Tolerances as the FP64 parity bar: psi/kpsi relative L2 1e-12 after <= 100
steps, 1e-10 after 2000 steps; scalars 1e-12 relative (1e-10 after 2000
steps); spectra 1e-10; vortex counts exact; particle positions and
velocities 1e-12 absolute, forces 1e-9 of the largest.  The FP32 bulk path:
psi relative L2 <= 1e-5 after 100 steps."""
import os

import numpy as np
import pytest

from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SC = ("momx", "momy", "egrad", "echem", "eintr", "etot", "norm", "eppot", "eobj_kin", "esrep")


def load(name):
    return np.load(os.path.join(GOLD, f"{name}.npz"))


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def scal(d):
    return np.array([getattr(d, k) for k in SC])


def test_gpu_rk4_64():
    g = load("rk4_64")
    s = vk.GPESolver(vk.params_for(64, dt=1e-3))
    s.set_psi(g["psi0"])
    s.gpe_rk4(100)
    assert rel(s.get_psi(), g["psi"]) < 1e-12
    assert rel(s.get_kpsi(), g["kpsi"]) < 1e-12
    d = s.diagnostics_gpe()
    assert np.allclose(scal(d)[:7], g["scalars"][:7], rtol=1e-12, atol=1e-15)
    assert rel(d.spec, g["spec"]) < 1e-10
    assert tuple(d.nvort) == tuple(g["nvort"])
    s.close()


def test_gpu_fp32_rk4_64():
    g = load("rk4_64")
    s = vk.GPESolver(vk.params_for(64, dt=1e-3, precision=vk.VK_PREC_FP32))
    s.set_psi(g["psi0"])
    s.gpe_rk4(100)
    assert rel(s.get_psi(), g["psi"]) < 1e-5
    s.close()


def test_gpu_argle_64():
    g = load("argle_64")
    s = vk.GPESolver(vk.params_for(64, dt=1e-3))
    s.set_psi(g["psi0"])
    res = [s.argle(50) for _ in range(4)]
    assert np.allclose(res, g["residuals"], rtol=1e-10, atol=0)
    assert rel(s.get_kpsi(), g["kpsi"]) < 1e-12
    s.close()


def test_gpu_particles_64():
    import sys
    sys.path.insert(0, GOLD)
    from make_golden import part_params
    g = load("part_64")
    s = vk.GPESolver(part_params(64, 4))
    s.set_psi(g["psi0"])
    s.particles_set(g["pos0"], g["vel0"], g["f0ext"])
    s.gpe_rk4(50)
    d = s.diagnostics_gpe()
    pos, vel, frc = s.particles_get()
    assert rel(s.get_psi(), g["psi"]) < 1e-12
    assert np.abs(pos - g["pos"]).max() < 1e-12 and np.abs(vel - g["vel"]).max() < 1e-12
    assert np.abs(frc - g["frc"]).max() <= 1e-9 * np.abs(g["frc"]).max()
    assert np.allclose(scal(d)[:9], g["scalars"][:9], rtol=1e-11, atol=1e-15)
    s.close()


def test_gpu_c1_128():
    g = load("c1_128")
    s = vk.GPESolver(vk.params_for(128, dt=1e-3))
    s.set_psi(g["psi0"])
    r = s.argle(1000)
    assert abs(r - float(g["argle_residual"])) <= 1e-10 * abs(r)
    for i in range(10):
        s.gpe_rk4(100)
        d = s.diagnostics_gpe()
        assert np.allclose(scal(d)[:7], g["scalars"][i][:7], rtol=1e-10, atol=1e-14), i
        assert tuple(d.nvort) == tuple(g["nvort"][i])
    assert rel(d.spec, g["spec"]) < 1e-10
    assert rel(s.get_psi(), g["psi"]) < 1e-10
    s.close()
