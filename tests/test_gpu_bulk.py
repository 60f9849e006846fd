"""FP64 bulk row loads: the y passes (k_y1, k_y2_rk4) and the single-row
CTAs of k_x1 bring their rows into shared memory by bulk copies
(cp.async.bulk completing on an mbarrier, vk_bulk.cuh).

* Bulk loads (the default) and element-wise loads (VK_BULK=0) fill shared
  memory with the same values, so they give the same field bit for bit,
  through RK4 (pruned rows, the CUDA-graph replays) and ARGLE, at 1024^2
  (single-row x passes) and 256^2 (row-pair x passes, bulk y passes only).
* A wait for the bulk loads that runs out (VK_SPIN_LIMIT=0: every CTA gives
  up before its first poll, then waits, bounded, for its copies in flight)
  is reported as an error status at the next synchronising call, and the
  GPU stays usable.
"""
import math

import numpy as np
import pytest

from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu


def _psi0(n):
    psi, _ = vk.ic_vortices(n, n, 16 if n < 512 else 64, seed=21, min_sep=4 * math.sqrt(2) * 2 * math.pi / n)
    return psi


def _run(monkeypatch, bulk, n, psi0, rk4=6, argle=3):
    monkeypatch.setenv("VK_BULK", "1" if bulk else "0")
    with vk.GPESolver(vk.params_for(n, dt=5e-4)) as s:
        s.set_psi(psi0)
        s.gpe_rk4(rk4)
        a = s.get_psi()
        s.set_psi(psi0)
        r = s.argle(argle)
        return a, s.get_kpsi(), r


@pytest.mark.parametrize("n", [1024, 256])
def test_bulk_and_elementwise_loads_agree_bitwise(monkeypatch, n):
    psi0 = _psi0(n)
    a, ka, ra = _run(monkeypatch, True, n, psi0)
    b, kb, rb = _run(monkeypatch, False, n, psi0)
    assert np.isfinite(a).all() and np.isfinite(ka).all()
    assert np.array_equal(a, b) and np.array_equal(ka, kb) and ra == rb


def test_bulk_load_timeout_is_reported(monkeypatch):
    n = 1024
    psi0 = _psi0(n)
    monkeypatch.setenv("VK_SPIN_LIMIT", "0")
    with vk.GPESolver(vk.params_for(n, dt=5e-4)) as s:
        s.set_psi(psi0)
        s.gpe_rk4(1)
        with pytest.raises(vk.VkError, match="bulk row loads"):
            s.get_psi()
        with pytest.raises(vk.VkError, match="VK_E_STATE"):
            s.gpe_rk4(1)          # the field was invalidated
        s.set_psi(psi0)           # the context itself still works
        assert np.isfinite(s.get_psi()).all()
    monkeypatch.delenv("VK_SPIN_LIMIT")
    a, _, _ = _run(monkeypatch, True, n, psi0, rk4=2, argle=1)
    b, _, _ = _run(monkeypatch, False, n, psi0, rk4=2, argle=1)
    assert np.array_equal(a, b)
