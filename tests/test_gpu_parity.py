"""GPU path (libvk kernels through the C ABI) against the CPU FP64 oracle.

Tolerances: FP64 path psi / kpsi relative L2 <= 1e-12 after 100 RK4 steps
(the stated parity bar); FFT round trips <= 1e-13; the FP32 bulk path
<= 1e-5 relative L2 against the FP64 oracle after 100 steps.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _pair(n, ny=None, dt=1e-3, prec=vk.VK_PREC_FP64, otoc=True, nv=8, seed=1):
    ny = ny or n
    p = vk.params_for(n, ny, dt=dt, precision=prec, otoc=otoc)
    psi0, _ = vk.ic_vortices(n, ny, nv, seed=seed)
    s = vk.GPESolver(p)
    s.set_psi(psi0)
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0, otoc=otoc, k_otoc=p.k_otoc_gp, eps_otoc=p.eps_otoc_gp)
    return s, o, psi0


@pytest.mark.parametrize("nx,ny", [(16, 16), (32, 32), (64, 64), (128, 128), (256, 256), (512, 512),
                                   (1024, 1024), (2048, 2048), (64, 32), (32, 128)])
def test_forward_fft_and_state_upload(nx, ny):
    s, o, psi0 = _pair(nx, ny, otoc=False, nv=4)
    assert rel(s.get_kpsi(), o.get_kpsi()) < 1e-13
    assert np.array_equal(s.get_psi(), psi0)
    s.close()


@pytest.mark.parametrize("n", [64, 4096])
def test_otoc_band_limit(n):
    s, o, _ = _pair(n, nv=8)
    assert rel(s.get_psi(), o.get_psi()) < 1e-13
    assert rel(s.get_kpsi(), o.get_kpsi()) < 1e-13
    s.close()


@pytest.mark.parametrize("n,steps", [(128, 100), (256, 50)])
def test_rk4_parity_fp64(n, steps):
    s, o, _ = _pair(n, nv=8)
    s.gpe_rk4(steps)
    o.gpe_rk4(steps)
    assert rel(s.get_psi(), o.get_psi()) < 1e-12
    assert rel(s.get_kpsi(), o.get_kpsi()) < 1e-12
    s.close()


def test_rk4_parity_fp64_1024():
    s, o, _ = _pair(1024, dt=5e-4, nv=64, seed=11)
    s.gpe_rk4(100)
    o.gpe_rk4(100)
    assert rel(s.get_psi(), o.get_psi()) < 1e-12
    s.close()


def test_x_single_rows_equal_row_pairs_1024(monkeypatch):
    """The FP64 x passes at nx = 1024 run one real row per CTA (half-length
    complex transforms); VK_XSPLIT=0 selects the row-pair transforms.  Both
    layouts agree to rounding through RK4, ARGLE and the diagnostics."""
    p = vk.params_for(1024, dt=5e-4)
    psi0, _ = vk.ic_vortices(1024, 1024, 32, seed=4)
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("VK_XSPLIT", flag)
        with vk.GPESolver(p) as s:
            s.set_psi(psi0)
            r = s.argle(10)
            s.gpe_rk4(20)
            out.append((s.get_psi(), r, s.diagnostics_gpe().etot))
    assert rel(out[0][0], out[1][0]) < 1e-13
    assert abs(out[0][1] - out[1][1]) <= 1e-12 * abs(out[1][1])
    assert abs(out[0][2] - out[1][2]) <= 1e-12 * abs(out[1][2])


def test_x_single_rows_nonsquare_1024_by_256():
    s, o, _ = _pair(1024, 256, nv=8, seed=6)
    s.argle(5)
    o.argle(5)
    s.gpe_rk4(10)
    o.gpe_rk4(10)
    assert rel(s.get_psi(), o.get_psi()) < 1e-12
    s.close()


def test_rk4_without_otoc_uses_raw_psi_first_stage():
    s, o, _ = _pair(64, otoc=False, nv=4)
    s.gpe_rk4(10)
    o.gpe_rk4(10)
    assert rel(s.get_psi(), o.get_psi()) < 1e-12
    s.close()


def test_rk4_split_calls_equal_one_call():
    a, _, psi0 = _pair(128, nv=8)
    b, _, _ = _pair(128, nv=8)
    a.gpe_rk4(5)
    b.gpe_rk4(3)
    b.gpe_rk4(2)
    assert rel(a.get_psi(), b.get_psi()) < 1e-15
    a.close()
    b.close()


def test_rk4_nonsquare():
    s, o, _ = _pair(64, 128, nv=6)
    s.gpe_rk4(20)
    o.gpe_rk4(20)
    assert rel(s.get_psi(), o.get_psi()) < 1e-12
    s.close()


def test_argle_parity_and_residual():
    s, o, _ = _pair(128, nv=8)
    r_gpu = s.argle(100)
    r_ref = o.argle(100)
    assert rel(s.get_kpsi(), o.get_kpsi()) < 1e-12
    assert rel(s.get_psi(), o.get_psi()) < 1e-12  # psi is the stale start-of-step field
    assert abs(r_gpu - r_ref) / r_ref < 1e-9
    s.close()


def test_argle_then_rk4():
    s, o, _ = _pair(128, nv=8, otoc=False)
    s.argle(30)
    o.argle(30)
    s.gpe_rk4(30)
    o.gpe_rk4(30)
    assert rel(s.get_psi(), o.get_psi()) < 1e-12
    s.close()


def test_set_kpsi_path():
    n = 64
    p = vk.params_for(n)
    rng = np.random.default_rng(2)
    k = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    s = vk.GPESolver(p)
    s.set_kpsi(k)
    o = Oracle.from_vk_params(p)
    assert rel(s.get_psi(), o.fft_inverse(k)) < 1e-13
    s.close()


def test_fp32_bulk_error_vs_fp64_oracle():
    s, o, _ = _pair(128, nv=8, prec=vk.VK_PREC_FP32)
    s.gpe_rk4(100)
    o.gpe_rk4(100)
    err = rel(s.get_psi(), o.get_psi())
    assert err < 1e-5, err
    s.close()


@pytest.mark.parametrize("n", [512, 1024, 2048])
def test_fp32_forward_fft(n):
    """The FP32 transforms (1024: the warp-per-row four-step transform)
    against numpy's FP64 FFT: relative L2 <= 1e-6."""
    p = vk.params_for(n, precision=vk.VK_PREC_FP32, otoc=False)
    psi0, _ = vk.ic_vortices(n, n, 8, seed=2)
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        ref = np.fft.fft2(psi0).T                      # transposed Fourier layout [kx][ky]
        assert rel(s.get_kpsi(), ref) < 1e-6
        s.set_kpsi(ref)                                # F^-1 through the FP32 inverse passes
        assert rel(s.get_psi(), psi0) < 1e-6


def test_fp32_1024_rk4_vs_fp64():
    """FP32 bulk at 1024^2 (warp-per-row transforms) against the FP64 path
    after 100 RK4 steps: relative L2 <= 5e-6."""
    out = {}
    for prec in (vk.VK_PREC_FP64, vk.VK_PREC_FP32):
        with vk.GPESolver(vk.params_for(1024, dt=5e-4, precision=prec)) as s:
            s.set_psi_vortices(64, seed=1, min_sep=4 * np.sqrt(2) * 2 * np.pi / 1024)
            s.gpe_rk4(100)
            out[prec] = s.get_psi()
    assert rel(out[vk.VK_PREC_FP32], out[vk.VK_PREC_FP64]) < 5e-6


def test_state_errors():
    p = vk.params_for(32)
    s = vk.GPESolver(p)
    with pytest.raises(vk.VkError, match="VK_E_STATE"):
        s.gpe_rk4(1)
    bad = np.ones((32, 32), complex)
    bad[3, 4] = np.nan
    with pytest.raises(vk.VkError, match="VK_E_NUMERIC"):
        s.set_psi(bad)
    s.close()
    # a field large enough for the threaded scan: Inf in the last imaginary part
    with vk.GPESolver(vk.params_for(1024)) as s:
        big = np.ones((1024, 1024), complex)
        big[-1, -1] = complex(1.0, np.inf)
        with pytest.raises(vk.VkError, match="VK_E_NUMERIC"):
            s.set_psi(big)
        big[-1, -1] = 1.0
        s.set_psi(big)


def test_kernel_launch_count_and_timing():
    s, _, _ = _pair(64, nv=4)
    n0 = s.launches
    s.timing_begin()
    s.gpe_rk4(2)
    t = s.timing_end()
    assert s.launches - n0 == 2 * 16 + 1
    assert {"k_x1", "k_y1", "k_x2", "k_y2_rk4"} <= set(t)
    assert t["k_x2"][1] == 8
    s.close()


def test_device_vortex_ic_matches_host():
    n = 128
    p = vk.params_for(n, otoc=False)
    psi_h, pos_h = vk.ic_vortices(n, n, 16, seed=21, min_sep=0.3)
    with vk.GPESolver(p) as s:
        pos_d = s.set_psi_vortices(16, seed=21, min_sep=0.3)
        assert np.array_equal(pos_d, pos_h)
        assert rel(s.get_psi(), psi_h) < 1e-13


def test_4096_fp32_vs_fp64_with_1024_vortices():
    """One 4096^2 field with 1024 vortices, FP32 bulk
    against plain FP64 after 100 RK4 steps."""
    n = 4096
    out = {}
    for prec in (vk.VK_PREC_FP64, vk.VK_PREC_FP32):
        with vk.GPESolver(vk.params_for(n, dt=5e-4, precision=prec)) as s:
            s.set_psi_vortices(1024, seed=5, min_sep=4 * np.sqrt(2) * 2 * np.pi / n)
            s.gpe_rk4(100)
            out[prec] = s.get_psi()
    assert np.isfinite(out[vk.VK_PREC_FP64]).all()
    assert rel(out[vk.VK_PREC_FP32], out[vk.VK_PREC_FP64]) < 1e-5


@pytest.mark.parametrize("prec", [vk.VK_PREC_FP64, vk.VK_PREC_FP32])
def test_async_dump_is_the_field_at_the_dump_point(prec):
    """vk_dump_begin snapshots psi in step order; steps issued afterwards do
    not change what vk_dump_wait returns (bitwise equal to get_psi there)."""
    n = 128
    psi0, _ = vk.ic_vortices(n, n, 8, seed=3)
    with vk.GPESolver(vk.params_for(n, dt=1e-3, precision=prec)) as s, \
            vk.GPESolver(vk.params_for(n, dt=1e-3, precision=prec)) as r:
        s.set_psi(psi0)
        r.set_psi(psi0)
        s.gpe_rk4(7)
        r.gpe_rk4(7)
        s.dump_begin()
        s.gpe_rk4(30)                  # runs while the copy is in flight
        got = s.dump_wait()
        assert np.array_equal(got, r.get_psi())
        with pytest.raises(vk.VkError, match="VK_E_STATE"):
            s.dump_wait()              # nothing in flight
        s.dump_begin()
        r.gpe_rk4(30)
        assert np.array_equal(s.dump_wait(), r.get_psi())


def test_rk4_parity_fp64_2048():
    """2048^2 (radix plan 16-16-8, two rows per x-pass CTA): ten RK4 steps
    against the oracle, relative L2 <= 1e-12."""
    import os
    n = 2048
    p = vk.params_for(n, dt=5e-4)
    psi0, _ = vk.ic_vortices(n, n, 16, seed=4)
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        s.gpe_rk4(10)
        got = s.get_psi()
    o = Oracle.from_vk_params(p, threads=os.cpu_count())
    o.set_psi(psi0, otoc=True, k_otoc=p.k_otoc_gp, eps_otoc=p.eps_otoc_gp)
    o.gpe_rk4(10)
    assert rel(got, o.get_psi()) < 1e-12
