"""The -DGPE_FRCDISP right-hand side (src/gpe.f90:623-658) on the GPU
against the oracle: same forcing-phase stream (counter-based), so FP64
parity is the plain path's bar, psi relative L2 <= 1e-12 after 50 steps;
FP32 bulk <= 1e-5."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu

# stable at 64^2 / 128^2 with dt = 1e-3: vishype k^16 dt < 1 for k^2 <= k2max
CASES = [dict(vishypo=0.5), dict(vishype=1e-25), dict(famp=0.5, kf1=2.0, kf2=5.0, seed=7),
         dict(vishypo=0.3, vishype=1e-26, famp=0.2, kf1=3.0, kf2=6.0, seed=3)]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [64, 128])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_frcdisp_matches_oracle(n, case):
    kw = CASES[case]
    p = vk.params_for(n, dt=1e-3)
    psi0, _ = vk.ic_vortices(n, n, 8, seed=4)
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        s.set_variant(frcdisp=True, **kw)
        s.gpe_rk4(20)
        s.gpe_rk4(30)                   # split calls: the phase counter carries over
        got = s.get_psi()
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0)
    o.set_frcdisp(True, **kw)
    o.gpe_rk4(50)
    assert rel(got, o.get_psi()) < 1e-12


def test_frcdisp_fp32_and_reset():
    kw = CASES[3]
    n = 128
    p32 = vk.params_for(n, dt=1e-3, precision=vk.VK_PREC_FP32)
    psi0, _ = vk.ic_vortices(n, n, 8, seed=4)
    o = Oracle.from_vk_params(vk.params_for(n, dt=1e-3))
    o.set_psi(psi0)
    o.set_frcdisp(True, **kw)
    o.gpe_rk4(50)
    with vk.GPESolver(p32) as s:
        s.set_psi(psi0)
        s.set_variant(frcdisp=True, **kw)
        s.gpe_rk4(50)
        assert rel(s.get_psi(), o.get_psi()) < 1e-5
        s.set_variant(frcdisp=False)    # back to the plain equations
        s.set_psi(psi0)
        s.gpe_rk4(10)
        o2 = Oracle.from_vk_params(vk.params_for(n, dt=1e-3))
        o2.set_psi(psi0)
        o2.gpe_rk4(10)
        assert rel(s.get_psi(), o2.get_psi()) < 1e-5


def test_unbuilt_variant_flags_are_rejected():
    with vk.GPESolver(vk.params_for(32)) as s:
        v = vk.VkVariant()
        v.flags = 64                    # not a branch
        with pytest.raises(vk.VkError, match="VK_E_INVALID"):
            vk._check(s.lib.vk_set_variant(s._h, vk.C.byref(v)), "vk_set_variant")


@pytest.mark.parametrize("n", [64, 256])
@pytest.mark.parametrize("flow,vel", [("counterflow", (0.3, -0.2)), ("advection", (0.0, 0.0))])
def test_argle_flow_matches_oracle(n, flow, vel):
    p = vk.params_for(n, dt=1e-3)
    psi0, _ = vk.ic_vortices(n, n, 8, seed=6)
    mode = {"advection": 1, "counterflow": 2}[flow]
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        s.set_variant(flow=flow, vnx=vel[0], vny=vel[1])
        r1 = s.argle(20)
        r2 = s.argle(30)
        got = s.get_kpsi()
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0)
    o.set_argle_flow(mode, *vel)
    o.argle(20)
    ro = o.argle(30)
    assert rel(got, o.get_kpsi()) < 1e-12
    assert abs(r2 - ro) <= 1e-9 * abs(ro) and np.isfinite(r1)


def test_argle_flow_fp32():
    n = 128
    psi0, _ = vk.ic_vortices(n, n, 8, seed=6)
    o = Oracle.from_vk_params(vk.params_for(n, dt=1e-3))
    o.set_psi(psi0)
    o.set_argle_flow(1)
    o.argle(50)
    with vk.GPESolver(vk.params_for(n, dt=1e-3, precision=vk.VK_PREC_FP32)) as s:
        s.set_psi(psi0)
        s.set_variant(flow="advection")
        s.argle(50)
        assert rel(s.get_kpsi(), o.get_kpsi()) < 1e-5


def test_flow_rejections():
    with vk.GPESolver(vk.params_for(32)) as s:
        v = vk.VkVariant()
        v.flags = vk.VK_VAR_ADVECTION | vk.VK_VAR_COUNTERFLOW
        with pytest.raises(vk.VkError, match="VK_E_INVALID"):
            vk._check(s.lib.vk_set_variant(s._h, vk.C.byref(v)), "vk_set_variant")


SGLE = dict(oneybeta=0.05, nuN=2.0, seed=13)


def _sgle_pair(n, prec=vk.VK_PREC_FP64, flow=None, selftrunc=False):
    p = vk.params_for(n, dt=1e-3, precision=prec)
    kw = dict(SGLE, chempot0=p.gstrength * 0.9)
    psi0, _ = vk.ic_vortices(n, n, 8, seed=8)
    o = Oracle.from_vk_params(vk.params_for(n, dt=1e-3))
    o.set_psi(psi0)
    o.set_sgle(True, selftrunc=selftrunc, ktrunc=n / 4, **kw)
    if flow:
        o.set_argle_flow(2, 0.2, 0.1)
    s = vk.GPESolver(p)
    s.set_psi(psi0)
    s.set_variant(sgle=True, selftrunc=selftrunc, ktrunc=n / 4,
                  flow="counterflow" if flow else None, vnx=0.2, vny=0.1, **kw)
    return s, o


@pytest.mark.parametrize("n", [64, 128])
@pytest.mark.parametrize("flow,trunc", [(None, False), (None, True), ("counterflow", False)])
def test_sgle_matches_oracle(n, flow, trunc):
    s, o = _sgle_pair(n, flow=flow, selftrunc=trunc)
    s.argle(10)
    s.argle(20)                           # split calls: noise counter and omega carry over
    o.argle(30)
    assert rel(s.get_kpsi(), o.get_kpsi()) < 1e-12
    assert abs(s.chempot - o.chempot) <= 1e-12 * abs(o.chempot)
    d = s.diagnostics_gpe()
    sc, _ = o.diagnostics()
    assert abs(d.echem - sc[3]) <= 1e-11 * abs(sc[3])
    s.close()


def test_sgle_fp32():
    s, o = _sgle_pair(128, prec=vk.VK_PREC_FP32)
    s.argle(30)
    o.argle(30)
    assert rel(s.get_kpsi(), o.get_kpsi()) < 1e-5
    assert abs(s.chempot - o.chempot) <= 1e-6 * abs(o.chempot)
    s.close()


def test_variants_nonsquare_grid():
    """nx != ny (128 x 64): forced-dissipative RK4, counterflow ARGLE and SGLE
    against the oracle."""
    nx, ny = 128, 64
    psi0, _ = vk.ic_vortices(nx, ny, 8, seed=2)
    p = vk.params_for(nx, ny, dt=1e-3)
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        s.set_variant(frcdisp=True, vishypo=0.3, famp=0.2, kf1=2.0, kf2=5.0, seed=9)
        s.gpe_rk4(20)
        got = s.get_psi()
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0)
    o.set_frcdisp(True, vishypo=0.3, famp=0.2, kf1=2.0, kf2=5.0, seed=9)
    o.gpe_rk4(20)
    assert rel(got, o.get_psi()) < 1e-12
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        s.set_variant(flow="counterflow", vnx=0.3, vny=-0.1, sgle=True, oneybeta=0.05, nuN=1.0,
                      chempot0=p.gstrength, seed=4)
        s.argle(20)
        got = s.get_kpsi()
        mu = s.chempot
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0)
    o.set_argle_flow(2, 0.3, -0.1)
    o.set_sgle(True, oneybeta=0.05, nuN=1.0, chempot0=p.gstrength, seed=4)
    o.argle(20)
    assert rel(got, o.get_kpsi()) < 1e-12
    assert abs(mu - o.chempot) <= 1e-12 * abs(o.chempot)


def test_argle_residual_of_a_zero_field_is_zero():
    with vk.GPESolver(vk.params_for(32, dt=1e-3, otoc=False)) as s:
        s.set_psi(np.zeros((32, 32), dtype=complex))
        assert s.argle(3) == 0.0
