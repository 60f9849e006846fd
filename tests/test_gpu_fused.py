"""Persistent RK4 stage kernel (FP32 at 1024^2): each stage is one
cooperative launch with bounded grid-wide barriers between its four passes.

* It runs the same pass bodies as the four pass kernels (VK_FUSED=0), so the
  two give the same field bit for bit, through the first stage (psi read
  directly) and the CUDA-graph replays of the later steps.
* A barrier wait that runs out (VK_SPIN_LIMIT=0: a CTA gives up on its first
  poll, before the last CTA has arrived) is reported as an error status at
  the next synchronising call, and the GPU stays usable.
"""
import math

import numpy as np
import pytest

from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu

N = 1024


def _psi0():
    psi, _ = vk.ic_vortices(N, N, 64, seed=8, min_sep=4 * math.sqrt(2) * 2 * math.pi / N)
    return psi


def _run(monkeypatch, fused, steps, psi0):
    monkeypatch.setenv("VK_FUSED", "1" if fused else "0")
    with vk.GPESolver(vk.params_for(N, dt=5e-4, precision=vk.VK_PREC_FP32)) as s:
        s.set_psi(psi0)
        n0 = s.launches
        s.gpe_rk4(steps)
        launches = s.launches - n0
        return s.get_psi(), s.get_kpsi(), launches


def test_fused_stage_equals_four_pass_kernels(monkeypatch):
    psi0 = _psi0()
    a, ka, la = _run(monkeypatch, True, 20, psi0)
    b, kb, lb = _run(monkeypatch, False, 20, psi0)
    assert np.array_equal(a, b) and np.array_equal(ka, kb)
    # one launch per stage plus the final inverse x pass, against four per stage
    assert la == 4 * 20 + 1 and lb == 16 * 20 + 1


def test_fused_stage_barrier_timeout_is_reported(monkeypatch):
    psi0 = _psi0()
    monkeypatch.setenv("VK_FUSED", "1")
    monkeypatch.setenv("VK_SPIN_LIMIT", "0")
    with vk.GPESolver(vk.params_for(N, dt=5e-4, precision=vk.VK_PREC_FP32)) as s:
        s.set_psi(psi0)
        s.gpe_rk4(2)
        with pytest.raises(vk.VkError, match="gave up waiting at grid barrier"):
            s.get_psi()
        with pytest.raises(vk.VkError, match="VK_E_STATE"):
            s.gpe_rk4(1)          # the field was invalidated
        s.set_psi(psi0)           # the context itself still works
        assert np.isfinite(s.get_psi()).all()
    monkeypatch.delenv("VK_SPIN_LIMIT")
    a, _, _ = _run(monkeypatch, True, 3, psi0)
    b, _, _ = _run(monkeypatch, False, 3, psi0)
    assert np.array_equal(a, b)
