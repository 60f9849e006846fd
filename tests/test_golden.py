"""The committed golden fixtures (tests/golden/*.npz, made by
tests/golden/make_golden.py from the CPU FP64 oracle) against the oracle
and the host initial-state generator, on the CPU.  The fixtures pin the
oracle against regressions (the reference has no golden vectors of its
own; parity with the reference binary is unpinned).

Tolerances (relative L2 unless stated): fields 1e-12 after <= 100 steps and
1e-10 after 2000 steps (the fixtures may come from another CPU's libm);
spectra 1e-10; vortex counts exact."""
import os

import numpy as np
import pytest

from oracle.oracle import Oracle
from quantumvortices_gb300 import vk

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, f"{name}.npz"))


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


@pytest.mark.parametrize("name,nv,seed", [("rk4_64", 8, 3), ("argle_64", 12, 5), ("part_64", 4, 4),
                                          ("c1_128", 8, 1)])
def test_host_initial_state_matches_fixture(name, nv, seed):
    g = load(name)
    n = g["psi0"].shape[0]
    psi0, _ = vk.ic_vortices(n, n, nv, seed=seed)
    assert rel(psi0, g["psi0"]) < 1e-12


def test_oracle_rk4_64():
    g = load("rk4_64")
    o = Oracle.from_vk_params(vk.params_for(64, dt=1e-3))
    o.set_psi(g["psi0"])
    o.gpe_rk4(100)
    assert rel(o.get_psi(), g["psi"]) < 1e-12
    assert rel(o.get_kpsi(), g["kpsi"]) < 1e-12
    sc, spec = o.diagnostics()
    assert np.allclose(sc, g["scalars"], rtol=1e-12, atol=1e-15)
    assert rel(spec, g["spec"]) < 1e-10
    assert tuple(o.count_vortices()) == tuple(g["nvort"])


def test_oracle_argle_64():
    g = load("argle_64")
    o = Oracle.from_vk_params(vk.params_for(64, dt=1e-3))
    o.set_psi(g["psi0"])
    res = [o.argle(50) for _ in range(4)]
    assert np.allclose(res, g["residuals"], rtol=1e-10, atol=0)
    assert rel(o.get_kpsi(), g["kpsi"]) < 1e-12


def test_oracle_particles_64():
    import sys
    sys.path.insert(0, GOLD)
    from make_golden import part_params
    g = load("part_64")
    o = Oracle.from_vk_params(part_params(64, 4))
    o.set_psi(g["psi0"])
    o.particles_set(g["pos0"], g["vel0"], g["f0ext"])
    o.gpe_rk4(50)
    sc, _ = o.diagnostics()
    pos, vel, frc = o.particles_get()
    assert rel(o.get_psi(), g["psi"]) < 1e-12
    assert np.abs(pos - g["pos"]).max() < 1e-12 and np.abs(vel - g["vel"]).max() < 1e-12
    assert np.abs(frc - g["frc"]).max() <= 1e-10 * np.abs(g["frc"]).max()
    assert np.allclose(sc, g["scalars"], rtol=1e-11, atol=1e-15)


def test_oracle_c1_128():
    g = load("c1_128")
    o = Oracle.from_vk_params(vk.params_for(128, dt=1e-3))
    o.set_psi(g["psi0"])
    r = o.argle(1000)
    assert abs(r - float(g["argle_residual"])) <= 1e-10 * abs(r)
    for i in range(10):
        o.gpe_rk4(100)
        sc, spec = o.diagnostics()
        assert np.allclose(sc, g["scalars"][i], rtol=1e-10, atol=1e-14), i
        assert tuple(o.count_vortices()) == tuple(g["nvort"][i])
    assert rel(spec, g["spec"]) < 1e-10
    assert rel(o.get_psi(), g["psi"]) < 1e-10
