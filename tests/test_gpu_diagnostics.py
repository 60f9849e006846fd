"""diagnostics_gpe on the GPU against the CPU FP64 oracle.

Tolerances (FP64 path): scalars 1e-12 relative, each of the six shell
spectra 1e-10 relative to that spectrum's largest shell, vortex counts
exact.  FP32 bulk: scalars 1e-5, spectra 1e-4.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu


def _setup(n, steps=0, argle=0, prec=vk.VK_PREC_FP64, nv=8, seed=3, otoc=True):
    p = vk.params_for(n, dt=1e-3, precision=prec, otoc=otoc)
    psi0, _ = vk.ic_vortices(n, n, nv, seed=seed)
    s = vk.GPESolver(p)
    s.set_psi(psi0)
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0, otoc=otoc)
    if argle:
        s.argle(argle)
        o.argle(argle)
    if steps:
        s.gpe_rk4(steps)
        o.gpe_rk4(steps)
    return s, o


def _check(s, o, tol_s, tol_sp):
    d = s.diagnostics_gpe()
    sc, spec = o.diagnostics()
    got = [d.momx, d.momy, d.egrad, d.echem, d.eintr, d.etot, d.norm]
    scale = max(abs(sc[2]), abs(sc[4]), 1.0)
    for j, g in enumerate(got):
        assert abs(g - sc[j]) <= tol_s * max(abs(sc[j]), 1e-3 * scale), (j, g, sc[j])
    for j in range(6):
        ref = spec[j]
        assert np.abs(d.spec[j] - ref).max() <= tol_sp * np.abs(ref).max(), j
    return d


@pytest.mark.parametrize("n", [64, 256])
def test_diagnostics_fp64_after_rk4(n):
    s, o = _setup(n, steps=20)
    d = _check(s, o, 1e-12, 1e-10)
    assert d.nvort == o.count_vortices()
    s.close()


def test_diagnostics_fp64_unmasked_state_after_argle():
    s, o = _setup(128, argle=10, otoc=False)
    _check(s, o, 1e-12, 1e-10)
    s.close()


def test_diagnostics_1024_and_vortex_count():
    s, o = _setup(1024, steps=5, nv=64, seed=9)
    d = _check(s, o, 1e-12, 1e-10)
    assert d.nvort == o.count_vortices()
    assert d.nvort[0] == d.nvort[1]
    s.close()


def test_diagnostics_fp32():
    s, o = _setup(128, steps=20, prec=vk.VK_PREC_FP32)
    _check(s, o, 1e-5, 1e-4)
    s.close()


def test_quantglobal_sums():
    s, o = _setup(64, steps=5)
    d = s.diagnostics_gpe()
    _, spec = o.diagnostics()
    ekint, ekini, ekinc, equnt, eintr, n0 = d.quantglobal()
    assert abs(ekint - spec[0, 1:].sum()) <= 1e-10 * abs(ekint)
    assert abs(eintr - spec[4, :].sum()) <= 1e-10 * abs(eintr)
    assert abs(n0 - spec[5, 0]) <= 1e-10 * abs(n0)
    s.close()


def test_diagnostics_4096_fp64_largest_grid():
    """The largest grid (4096^2, nshell = 2897, histogram of K + 3 shells in
    shared memory beside two 4096-point rows): GPU diagnostics of a
    1024-vortex state against the oracle's."""
    import os
    n = 4096
    p = vk.params_for(n, dt=5e-4)
    with vk.GPESolver(p) as s:
        s.set_psi_vortices(1024, seed=5, min_sep=4 * np.sqrt(2) * 2 * np.pi / n)
        psi = s.get_psi()
        o = Oracle.from_vk_params(p, threads=os.cpu_count())
        o.set_psi(psi, otoc=False)
        o.set_kpsi(s.get_kpsi())
        _check(s, o, 1e-12, 1e-10)
