"""Spatio-temporal spectra on the GPU (vk_sts_*) against the CPU
restatement of Run/CompSTS/driver.f90 (oracle/sts_oracle.py) fed with the
same kpsi records read back through vk_get_kpsi.

Tolerance: relative 1e-12 of the largest entry (FP64 arithmetic on identical
records; the FFT rounding differs)."""
import numpy as np
import pytest

from oracle import sts_oracle
from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu


def _run(n, nt, every, prec=vk.VK_PREC_FP64, nv=8):
    s = vk.GPESolver(vk.params_for(n, dt=1e-3, precision=prec))
    psi0, _ = vk.ic_vortices(n, n, nv, seed=9)
    s.set_psi(psi0)
    s.sts_begin(nt)
    rec = np.empty((nt, n, n), dtype=np.complex128)
    for t in range(nt):
        s.gpe_rk4(every)
        s.sts_record()
        rec[t] = s.get_kpsi()
    assert s.sts_count == nt
    g1, g2 = s.sts_spectra()
    assert s.sts_count == 0
    s.close()
    return g1, g2, rec


def close(a, b, tol=1e-12):
    return float(np.abs(a - b).max() / np.abs(b).max()) < tol


@pytest.mark.parametrize("n,nt,every", [(64, 64, 5), (128, 256, 2)])
def test_sts_matches_oracle(n, nt, every):
    g1, g2, rec = _run(n, nt, every)
    r1, r2 = sts_oracle.spectra(rec)
    assert g1.shape == r1.shape and g2.shape == r2.shape
    assert close(g1, r1) and close(g2, r2)


def test_sts_fp32_records():
    g1, g2, rec = _run(64, 32, 4, prec=vk.VK_PREC_FP32)
    r1, r2 = sts_oracle.spectra(rec)
    assert close(g1, r1) and close(g2, r2)


def test_sts_state_errors():
    s = vk.GPESolver(vk.params_for(32, dt=1e-3))
    with pytest.raises(vk.VkError, match="VK_E_STATE"):
        s.sts_record()                      # no ring yet
    with pytest.raises(vk.VkError, match="VK_E_INVALID"):
        s.sts_begin(100)                    # not a power of two
    s.sts_begin(16)
    with pytest.raises(vk.VkError, match="VK_E_STATE"):
        s.sts_spectra()                     # ring not full
    for _ in range(16):
        s.sts_record()
    with pytest.raises(vk.VkError, match="VK_E_STATE"):
        s.sts_record()                      # ring full
    s.sts_spectra()
    s.sts_end()
    s.close()
