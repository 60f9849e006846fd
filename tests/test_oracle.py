"""The CPU FP64 oracle against independent answers (no GPU).

Parity with the reference binary is unpinned (no Fortran/FFTW here and no
reference tests), so the oracle is pinned by: numpy's FFT, exact
known answers of the equation (plane waves under RK4 and ARGLE, uniform
states, linear dispersion, particles in a uniform state), and an independent
numpy restatement of one RK4 step, one ARGLE step and the diagnostics.
"""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle
from quantumvortices_gb300 import vk


@pytest.mark.parametrize("nx,ny", [(16, 16), (32, 64), (64, 32), (128, 128), (256, 256)])
def test_fft_matches_numpy(nx, ny):
    rng = np.random.default_rng(nx * 7 + ny)
    o = Oracle(nx, ny)
    a = rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))
    f = o.fft_forward(a)
    ref = np.fft.fft2(a).T  # reference layout kpsi[kx][ky]
    assert np.abs(f - ref).max() / np.abs(ref).max() < 1e-15
    back = o.fft_inverse(f)
    assert np.abs(back - a).max() < 1e-14


def test_grid_constants():
    # nshell = int(1.414*Nx/2.0d0)+1 with a single-precision 1.414 (src/mod_grid.f90:77)
    for n, want in [(128, 91), (256, 181), (512, 362), (1024, 724), (4096, 2896)]:
        assert vk.nshell(n) == want
    from oracle.oracle import lib
    assert [lib().vko_kwn(8, i) for i in range(1, 9)] == [0, 1, 2, 3, -4, -3, -2, -1]


def _grid(n):
    x = np.arange(n) * 2 * np.pi / n
    return np.meshgrid(x, x)


def _plane_wave_rk4(al, g, om, dt, k2, nsteps):
    f = lambda a: -1j * (al * k2 - om + g * abs(a) ** 2) * a
    a = 1.0 + 0j
    for _ in range(nsteps):
        k1 = f(a); k2_ = f(a + dt / 2 * k1); k3 = f(a + dt / 2 * k2_); k4 = f(a + dt * k3)
        a = a + dt / 6 * (k1 + 2 * k2_ + 2 * k3 + k4)
    return a


@pytest.mark.parametrize("k", [(3, -2), (0, 5), (-7, 0)])
def test_plane_wave_rk4_known_answer(k):
    """A plane wave keeps |psi|=1 on the grid; RK4 then reduces to the scalar ODE."""
    n = 32
    p = vk.params_for(n, dt=1e-3)
    o = Oracle.from_vk_params(p)
    X, Y = _grid(n)
    psi0 = np.exp(1j * (k[0] * X + k[1] * Y))
    o.set_psi(psi0)
    o.gpe_rk4(7)
    a = _plane_wave_rk4(p.alpha, p.gstrength, p.omega_chem, p.dt, k[0] ** 2 + k[1] ** 2, 7)
    assert np.abs(o.get_psi() - a * psi0).max() < 1e-13


@pytest.mark.parametrize("k", [(2, 1), (0, -6)])
def test_plane_wave_argle_known_answer(k):
    """ARGLE on a plane wave A e^{ik.x} (src/gpe.f90:5-224): |psi|^2 is uniform,
    so P_G rho = |A|^2 and N^ = -g |A|^2 psi^, and each step is the scalar
    recurrence A <- A (1 + dt (Omega - g |A|^2)) / (1 + alpha k^2 dt); the
    residual is |A_new - A_old| / (dt |A_old|) of the last step."""
    n = 32
    p = vk.params_for(n, dt=1e-3)
    o = Oracle.from_vk_params(p)
    X, Y = _grid(n)
    a0 = 0.7 + 0.2j
    psi0 = a0 * np.exp(1j * (k[0] * X + k[1] * Y))
    o.set_psi(psi0, otoc=False)
    r = o.argle(9)
    a, k2 = a0, k[0] ** 2 + k[1] ** 2
    for _ in range(9):
        prev = a
        a = a * (1 + p.dt * (p.omega_chem - p.gstrength * abs(a) ** 2)) / (1 + p.alpha * k2 * p.dt)
    kp = o.get_kpsi()  # [kx][ky], unnormalised
    expect = np.zeros((n, n), complex)
    expect[k[0] % n, k[1] % n] = a * n * n
    assert np.abs(kp - expect).max() < 1e-12 * n * n
    assert abs(r - abs(a - prev) / (p.dt * abs(prev))) < 1e-9 * r


def test_plane_wave_diagnostics_known_answer():
    """diagnostics_gpe (src/diagnostics.f90:4-571) of A e^{ik.x}: the box
    averages are exact, so norm = |A|^2 L^2, mom = 2 alpha |A|^2 k,
    Egrad = 2 alpha^2 |A|^2 k^2, Echem = 2 alpha Omega |A|^2,
    Eint = alpha g |A|^4 (P_G keeps the uniform density), Etot = Egrad + Eint,
    and the |kpsi|^2 spectrum holds |A|^2 in the shell nint(|k|) alone."""
    n = 32
    p = vk.params_for(n, dt=1e-3)
    o = Oracle.from_vk_params(p)
    X, Y = _grid(n)
    a0, k = 0.8 - 0.3j, (3, -4)
    o.set_psi(a0 * np.exp(1j * (k[0] * X + k[1] * Y)), otoc=False)
    sc, spec = o.diagnostics()
    al, g, om, a2 = p.alpha, p.gstrength, p.omega_chem, abs(a0) ** 2
    k2 = k[0] ** 2 + k[1] ** 2
    want = {0: 2 * al * a2 * k[0], 1: 2 * al * a2 * k[1], 2: 2 * al * al * a2 * k2, 3: 2 * al * om * a2,
            4: al * g * a2 * a2, 5: 2 * al * al * a2 * k2 + al * g * a2 * a2, 6: a2 * (2 * math.pi) ** 2}
    for i, w in want.items():
        assert abs(sc[i] - w) <= 1e-12 * max(1.0, abs(w)), i
    shell = np.zeros(spec.shape[1])
    shell[int(round(math.sqrt(k2)))] = a2
    assert np.abs(spec[5] - shell).max() <= 1e-12


def _uniform_with_particles(pos, f0):
    n = 64
    dx = 2 * math.pi / n
    d = 2.0 * math.sqrt(2.0) * dx
    p = vk.params_for(n, dt=1e-3, n_particles=len(pos), ppotd=2.0, ppotv0=10.0, gp_mass_part=5.0 * math.pi * d * d)
    o = Oracle.from_vk_params(p)
    o.set_psi(np.ones((n, n), complex), otoc=False)
    o.particles_set(np.asarray(pos, float), np.zeros((len(pos), 2)), np.asarray(f0, float))
    return o, p


def test_particle_in_uniform_condensate_feels_only_its_external_force():
    """grad rho = 0 in a uniform state, so the fluid force of
    translate_particle_potential (src/gpe_particle.f90:219-324) vanishes and a
    single particle (no repulsion) feels exactly f0ext."""
    o, _ = _uniform_with_particles([[1.3, 4.1]], [[0.05, -0.02]])
    assert np.abs(o.particle_forces() - np.array([[0.05, -0.02]])).max() < 1e-13


def test_two_particle_repulsion_known_answer():
    """Two particles in a uniform state: the forces are the short-range
    repulsion of src/gpe_particle.f90:378-427 alone, equal and opposite, with
    the closed form -384 dE pi^12 r0^12 / L^12 sin(dq) / (-3 + cos dqx + cos dqy)^7
    (dE the single-precision literal 0.062, r0 = 4 xi, L = 2 pi)."""
    q = np.array([[1.0, 2.0], [1.9, 1.4]])
    o, p = _uniform_with_particles(q, np.zeros((2, 2)))
    f = o.particle_forces()
    de = float(np.float32(0.062))
    rf = 384.0 * de * math.pi ** 12 * (4.0 * p.xi) ** 12 / (2 * math.pi) ** 12
    dq = q[0] - q[1]
    den = (-3 + math.cos(dq[0]) + math.cos(dq[1])) ** 7
    f01 = -rf * np.sin(dq) / den
    assert np.abs(f[0] + f[1]).max() < 1e-12 * np.abs(f01).max()
    assert np.abs(f[0] - f01).max() < 1e-12 * np.abs(f01).max()


def test_uniform_state_stationary():
    n = 32
    p = vk.params_for(n, dt=1e-3)
    o = Oracle.from_vk_params(p)
    o.set_psi(np.ones((n, n), complex))
    o.gpe_rk4(5)
    assert np.abs(o.get_psi() - 1).max() < 1e-14
    o2 = Oracle.from_vk_params(p)
    o2.set_psi(np.ones((n, n), complex))
    r = o2.argle(5)
    assert np.abs(o2.get_kpsi()[0, 0] - n * n) < 1e-10
    assert r < 1e-12


def test_linear_dispersion_g0():
    n = 32
    p = vk.params_for(n, dt=2e-3)
    o = Oracle(n, n, dt=p.dt, alpha=p.alpha, gstrength=0.0, omega_chem=0.0)
    X, Y = _grid(n)
    rng = np.random.default_rng(5)
    kpsi = np.zeros((n, n), complex)
    modes = [(1, 2), (-3, 4), (5, -1)]
    psi0 = np.zeros((n, n), complex)
    for kx, ky in modes:
        c = rng.standard_normal() + 1j * rng.standard_normal()
        psi0 += c * np.exp(1j * (kx * X + ky * Y))
    o.set_psi(psi0)
    o.gpe_rk4(4)
    ref = np.zeros((n, n), complex)
    f = np.fft.fft2(psi0)
    kk = np.fft.fftfreq(n, 1.0 / n)
    KX, KY = np.meshgrid(kk, kk)
    z = -1j * p.alpha * (KX ** 2 + KY ** 2) * p.dt
    R = 1 + z + z * z / 2 + z ** 3 / 6 + z ** 4 / 24
    ref = np.fft.ifft2(f * R ** 4)
    assert np.abs(o.get_psi() - ref).max() < 1e-13


# ---------------------------------------------------------------- numpy restatement

def _np_setup(nx):
    k = np.array([(i - 1) - nx * (i // (nx // 2 + 1)) for i in range(1, nx + 1)])
    K1, K2 = np.meshgrid(k, k, indexing="ij")  # [kx][ky]
    ksq = K1 ** 2 + K2 ** 2
    mask = ksq.astype(float) >= (nx / 3.0) ** 2
    return K1, K2, ksq, mask


def _F(a):
    return np.fft.fft2(a).T


def _Fi(f):
    return np.fft.ifft2(f.T)


def _np_rhs(psi, kpsi, p, nx):
    K1, K2, ksq, mask = _np_setup(nx)
    rho = np.abs(psi) ** 2 + 0j
    r = _F(rho)
    tmp1 = (p.alpha * ksq - p.omega_chem) * kpsi
    r[mask] = 0
    pg = _Fi(r)
    nl = _F(p.gstrength * pg * psi)
    out = (-1j) * (tmp1 + nl)
    out[mask] = 0
    return out


def _np_rk4(psi, kpsi, p, nx):
    _, _, _, mask = _np_setup(nx)
    kpsi = kpsi.copy()
    kpsi[mask] = 0
    s1, s2 = kpsi.copy(), np.zeros_like(kpsi)
    dt = p.dt
    for c1, c2 in [(dt / 2, dt / 6), (dt / 2, dt / 3), (dt, dt / 3), (None, dt / 6)]:
        k = _np_rhs(psi, kpsi, p, nx)
        s2 = s2 + c2 * k
        kpsi = s1 + c1 * k if c1 is not None else s1 + s2
        kpsi[mask] = 0
        psi = _Fi(kpsi)
    return psi, kpsi


def test_rk4_matches_numpy_restatement():
    n = 32
    p = vk.params_for(n, dt=1e-3)
    psi0, _ = vk.ic_vortices(n, n, 4, seed=3)
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0, otoc=False)
    o.gpe_rk4(1)
    psi, kpsi = _np_rk4(psi0, _F(psi0), p, n)
    assert np.abs(o.get_psi() - psi).max() < 1e-13
    assert np.abs(o.get_kpsi() - kpsi).max() / np.abs(kpsi).max() < 1e-13


def test_argle_matches_numpy_restatement():
    n = 32
    p = vk.params_for(n, dt=1e-3)
    psi0, _ = vk.ic_vortices(n, n, 4, seed=4)
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0, otoc=False)
    r = o.argle(1)
    K1, K2, ksq, mask = _np_setup(n)
    kpsi = _F(psi0)
    psi = _Fi(kpsi)
    rh = _F(np.abs(psi) ** 2 + 0j)
    rh[mask] = 0
    nl = _F(-p.gstrength * _Fi(rh) * psi)
    new = (kpsi + p.dt * (nl + p.omega_chem * kpsi)) / (1 + p.alpha * ksq * p.dt)
    assert np.abs(o.get_kpsi() - new).max() / np.abs(new).max() < 1e-13
    want = np.linalg.norm(new - kpsi) / (p.dt * np.linalg.norm(kpsi))
    assert abs(r - want) / want < 1e-10


def test_diagnostics_matches_numpy_restatement():
    n = 32
    p = vk.params_for(n, dt=1e-3)
    psi0, _ = vk.ic_vortices(n, n, 4, seed=5)
    o = Oracle.from_vk_params(p)
    o.set_psi(psi0, otoc=True)
    sc, spec = o.diagnostics()
    psi, kpsi = o.get_psi(), o.get_kpsi()
    K1, K2, ksq, mask = _np_setup(n)
    al, g, om = p.alpha, p.gstrength, p.omega_chem
    dx = 2 * np.pi / n
    dvol, area = dx * dx, (2 * np.pi) ** 2
    gx, gy = _Fi(1j * K1 * kpsi), _Fi(1j * K2 * kpsi)
    momx = 2 * al * np.sum(np.imag(np.conj(psi) * gx)) * dvol / area
    r = _F(np.abs(psi) ** 2 + 0j)
    r[mask] = 0
    pg = _Fi(r)
    egrad = 2 * al * np.sum(al * (np.abs(gx) ** 2 + np.abs(gy) ** 2)) * dvol / area
    eintr = 2 * al * np.sum(0.5 * g * np.abs(pg) * np.abs(psi) ** 2) * dvol / area
    norm = np.sum(np.abs(psi) ** 2) * dvol
    for got, want in [(sc[0], momx), (sc[2], egrad), (sc[4], eintr), (sc[6], norm)]:
        assert abs(got - want) <= 1e-12 * max(1.0, abs(want))
    # spectra
    sm = float(np.float32(1e-30))
    wx = np.conj(psi) * gx / (np.abs(psi) + sm)
    wy = np.conj(psi) * gy / (np.abs(psi) + sm)
    aa1, aa2 = _F(2 * al * wx.imag + 0j), _F(2 * al * wy.imag + 0j)
    ee1, ee2 = _F(wx.real + 0j), _F(wy.real + 0j)
    k2f = ksq.astype(float)
    with np.errstate(divide="ignore", invalid="ignore"):
        bb = np.where(ksq == 0, 0, -1j * (K1 / k2f) * aa1 - 1j * (K2 / k2f) * aa2)
    cc1, cc2 = 1j * K1 * bb, 1j * K2 * bb
    en = (1.0 / (n * n)) ** 2
    mshl = np.rint(np.sqrt(k2f)).astype(int)
    ns = vk.nshell(n)
    want = np.zeros((6, ns + 1))
    terms = [0.5 * en * (abs(aa1) ** 2 + abs(aa2) ** 2), 0.5 * en * (abs(aa1 - cc1) ** 2 + abs(aa2 - cc2) ** 2),
             0.5 * en * (abs(cc1) ** 2 + abs(cc2) ** 2), en * (abs(ee1) ** 2 + abs(ee2) ** 2) * 2 * al * al,
             en * abs(r) ** 2 * 0.5 * g * 2 * al, en * abs(kpsi) ** 2]
    for j, t in enumerate(terms):
        t = np.where(mask, 0, t)
        np.add.at(want[j], mshl.ravel(), t.ravel())
    assert np.abs(spec - want).max() <= 1e-12 * np.abs(want).max()


def test_vortex_count_of_seeded_state():
    n = 128
    psi0, _ = vk.ic_vortices(n, n, 8, seed=1)
    o = Oracle(n)
    o.set_psi(psi0, otoc=False)
    assert o.count_vortices() == (4, 4)


def test_nn_oracle_gradient_by_finite_differences():
    """The CPU restatement of the warm-start network: exact-arithmetic
    gradient against central differences."""
    from oracle import nn_oracle as nn
    nn.EXACT = True
    try:
        base, levels, H = 16, 2, 8
        rng = np.random.default_rng(0)
        n = sum(co * 9 * ci + co for ci, co, _ in nn.layers(base, levels))
        params = rng.standard_normal(n) * 0.2
        inp = rng.standard_normal((3, H, H))
        tgt = rng.standard_normal((2, H, H))
        loss, g = nn.loss_grad(params, inp, tgt, base, levels)
        idx = rng.choice(n, 12, replace=False)
        for i in idx:
            e = np.zeros(n)
            e[i] = 1e-6
            lp, _ = nn.loss_grad(params + e, inp, tgt, base, levels)
            lm, _ = nn.loss_grad(params - e, inp, tgt, base, levels)
            fd = (lp - lm) / 2e-6
            assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])
    finally:
        nn.EXACT = False


def test_oracle_ic_and_parameters_match_the_product():
    """The oracle's own vortex IC and parameter derivation (used by the
    benchmark's reference arm, which loads no product library) give the
    product's state and parameters."""
    import math
    from oracle import oracle as orc
    from quantumvortices_gb300 import vk
    for n, nv, seed, ms in [(64, 8, 3, 0.3), (256, 64, 1, 4 * math.sqrt(2) * 2 * math.pi / 256)]:
        a, pa = orc.ic_vortices(n, n, nv, seed, min_sep=ms)
        b, pb = vk.ic_vortices(n, n, nv, seed, min_sep=ms)
        assert np.array_equal(pa, pb)
        assert np.abs(a - b).max() < 1e-13
    p = vk.params_for(128, dt=1e-3, n_particles=3, gp_mass_part=2.0)
    d = orc.derived_params(128, dt=1e-3, n_particles=3, gp_mass_part=2.0)
    for k in ("alpha", "gstrength", "omega_chem", "xi", "ppot_v0", "ppot_d", "gp_mass_part", "dt"):
        assert getattr(p, k) == d[k], k
