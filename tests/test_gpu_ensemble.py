"""Batched ensembles of uneven grid sizes against single-field solvers and
the CPU FP64 oracle.  Member fields run the same device bodies as the
single-field kernels, so an ensemble member must match a single-field run
of the same member to rounding (1e-14) and the oracle to the parity bar."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _members(sizes, prec):
    ps, psis = [], []
    for i, n in enumerate(sizes):
        ps.append(vk.params_for(n, dt=1e-3, precision=prec))
        psi, _ = vk.ic_vortices(n, n, 16 + 2 * (i % 8), seed=100 + i)
        psis.append(psi)
    return ps, psis


@pytest.mark.parametrize("prec", [vk.VK_PREC_FP64, vk.VK_PREC_FP32])
def test_ensemble_members_match_single_field(prec):
    sizes = [128, 256, 512, 256, 128, 1024]
    ps, psis = _members(sizes, prec)
    with vk.Ensemble(ps) as e:
        assert "x1:" in e.report
        for m, psi in enumerate(psis):
            e.set_psi(m, psi)
        e.gpe_rk4(12)
        for m, (p, psi) in enumerate(zip(ps, psis)):
            with vk.GPESolver(p) as s:
                s.set_psi(psi)
                s.gpe_rk4(12)
                tol = 1e-14 if prec == vk.VK_PREC_FP64 else 1e-6
                assert rel(e.get_psi(m), s.get_psi()) < tol


def test_ensemble_fp64_members_vs_oracle():
    sizes = [256, 512, 128]
    ps, psis = _members(sizes, vk.VK_PREC_FP64)
    with vk.Ensemble(ps) as e:
        for m, psi in enumerate(psis):
            e.set_psi(m, psi)
        e.gpe_rk4(100)
        for m, (p, psi) in enumerate(zip(ps, psis)):
            o = Oracle.from_vk_params(p)
            o.set_psi(psi, otoc=True)
            o.gpe_rk4(100)
            assert rel(e.get_psi(m), o.get_psi()) < 1e-12


def test_ensemble_fp32_config_shape_sample_vs_oracle():
    """The benchmark ensemble: 192 x 256^2 + 48 x 512^2 in one ensemble,
    FP32 bulk; a sample of members is checked against the FP64 oracle."""
    sizes = [256] * 192 + [512] * 48
    ps, psis = _members(sizes, vk.VK_PREC_FP32)
    with vk.Ensemble(ps) as e:
        for m, psi in enumerate(psis):
            e.set_psi(m, psi)
        e.gpe_rk4(100)
        for m in (0, 97, 191, 192, 239):
            o = Oracle.from_vk_params(vk.params_for(sizes[m], dt=1e-3))
            o.set_psi(psis[m], otoc=True)
            o.gpe_rk4(100)
            assert rel(e.get_psi(m), o.get_psi()) < 1e-5


@pytest.mark.parametrize("prec", [vk.VK_PREC_FP64, vk.VK_PREC_FP32])
def test_persistent_stage_kernel_equals_pass_kernels(prec, monkeypatch):
    """VK_FUSED=1 makes the ensemble step with kb_stage (one cooperative launch
    per RK4 stage over every member, bounded grid barriers), VK_FUSED=0 with
    the four pass kernels: the same device bodies on the same tiles' columns
    and rows, so the members agree bit for bit."""
    sizes = [128, 256, 512, 256]
    ps, psis = _members(sizes, prec)
    out = {}
    for flag in ("1", "0"):
        monkeypatch.setenv("VK_FUSED", flag)
        with vk.Ensemble(ps) as e:
            assert ("-> persistent" if flag == "1" else "-> pass kernels") in e.report
            for m, psi in enumerate(psis):
                e.set_psi(m, psi)
            e.gpe_rk4(6)
            out[flag] = [e.get_psi(m) for m in range(len(sizes))]
    for a, b in zip(out["1"], out["0"]):
        assert np.array_equal(a, b)
