"""Generates the golden fixtures in this folder from the CPU FP64 oracle.

    python tests/golden/make_golden.py

The reference (Fortran + FFTW 3.3.8 + MPI) cannot be built here and has no
tests or golden vectors of its own, so these fixtures hold the oracle's
outputs (oracle/vk_oracle.c, a line-by-line restatement of src/gpe.f90,
src/diagnostics.f90 and src/gpe_particle.f90) on seeded inputs.  They pin
the oracle and the GPU path against regressions; they are not reference
outputs.  Inputs are stored with the outputs, so the fixtures do not depend
on the product's initial-state generator.

Cases (the benchmark equation: xi = sqrt(2) dx, alpha = dx, g = Omega = 1/(2 dx)):
  c1_128    128^2, 8 vortices (seed 1), ARGLE 1000 steps then RK4 1000 steps
            at dt = 1e-3, scalars + spectra + vortex counts every 100 RK4
            steps; the final psi in full.
  rk4_64    64^2, 8 vortices (seed 3), OTOC-masked start, RK4 100 steps at
            dt = 1e-3 (psi and kpsi in full), then diagnostics.
  argle_64  64^2, 12 vortices (seed 5), ARGLE 200 steps at dt = 1e-3 with the
            residual after every 50 steps; kpsi in full.
  part_64   64^2, 4 vortices (seed 4) + 4 Gaussian particles (V0 = 10, d = 2 xi,
            M = 5 pi d^2), RK4 50 steps at dt = 1e-3: psi, particle state,
            forces and the particle energies.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle  # noqa: E402
from quantumvortices_gb300 import vk  # noqa: E402


def part_params(n, npart, dt=1e-3):
    dx = 2 * math.pi / n
    d = 2.0 * math.sqrt(2.0) * dx
    return vk.params_for(n, dt=dt, n_particles=npart, ppotd=2.0, ppotv0=10.0, gp_mass_part=5.0 * math.pi * d * d)


def part_inputs(npart, seed=4):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, 2 * np.pi, (npart, 2))
    vel = rng.normal(0, 0.1, (npart, 2))
    f0 = np.zeros((npart, 2))
    f0[0] = [0.05, -0.02]
    return pos, vel, f0


def c1_128():
    n = 128
    p = vk.params_for(n, dt=1e-3)
    psi0, pos = vk.ic_vortices(n, n, 8, seed=1)
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0)
    resid = o.argle(1000)
    scal, nvort = [], []
    for _ in range(10):
        o.gpe_rk4(100)
        sc, spec = o.diagnostics()
        scal.append(sc)
        nvort.append(o.count_vortices())
    return dict(psi0=psi0, vortex_pos=pos, argle_residual=resid, scalars=np.array(scal), spec=spec,
                nvort=np.array(nvort, dtype=np.int32), psi=o.get_psi())


def rk4_64():
    n = 64
    p = vk.params_for(n, dt=1e-3)
    psi0, _ = vk.ic_vortices(n, n, 8, seed=3)
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0)
    o.gpe_rk4(100)
    sc, spec = o.diagnostics()
    return dict(psi0=psi0, psi=o.get_psi(), kpsi=o.get_kpsi(), scalars=sc, spec=spec,
                nvort=np.array(o.count_vortices(), dtype=np.int32))


def argle_64():
    n = 64
    p = vk.params_for(n, dt=1e-3)
    psi0, _ = vk.ic_vortices(n, n, 12, seed=5)
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0)
    res = [o.argle(50) for _ in range(4)]
    return dict(psi0=psi0, residuals=np.array(res), kpsi=o.get_kpsi())


def part_64():
    n, npart = 64, 4
    p = part_params(n, npart)
    psi0, _ = vk.ic_vortices(n, n, 4, seed=4)
    pos, vel, f0 = part_inputs(npart)
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0)
    o.particles_set(pos, vel, f0)
    o.gpe_rk4(50)
    sc, _ = o.diagnostics()
    qp, qv, qf = o.particles_get()
    return dict(psi0=psi0, pos0=pos, vel0=vel, f0ext=f0, psi=o.get_psi(), pos=qp, vel=qv, frc=qf, scalars=sc)


CASES = {"c1_128": c1_128, "rk4_64": rk4_64, "argle_64": argle_64, "part_64": part_64}


def main():
    for name, fn in CASES.items():
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **fn())
        print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()
