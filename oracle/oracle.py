"""ctypes wrapper of the CPU FP64 oracle (oracle/vk_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.
PARITY UNPINNED against the reference binary (see vk_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libvk_oracle.so")


class VkoParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("n_particles", C.c_int32), ("renorm", C.c_int32),
        ("dt", C.c_double), ("alpha", C.c_double), ("gstrength", C.c_double), ("omega_chem", C.c_double),
        ("disp_factor", C.c_double), ("xi", C.c_double), ("ppot_v0", C.c_double), ("ppot_d", C.c_double),
        ("gp_mass_part", C.c_double),
    ]


def build() -> str:
    subprocess.run(["sh", os.path.join(HERE, "build_oracle.sh")], check=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        dp, vp = C.POINTER(C.c_double), C.c_void_p
        ip = C.POINTER(C.c_int32)
        for name, res, args in [
            ("vko_create", vp, [C.POINTER(VkoParams)]), ("vko_destroy", None, [vp]),
            ("vko_nshell", C.c_int32, [C.c_int32]), ("vko_kalias", C.c_double, [C.c_int32]),
            ("vko_kwn", C.c_int32, [C.c_int32, C.c_int32]),
            ("vko_fft_forward", None, [vp, dp, dp]), ("vko_fft_inverse", None, [vp, dp, dp]),
            ("vko_set_psi", None, [vp, dp, C.c_int32, C.c_double, C.c_double]),
            ("vko_get_psi", None, [vp, dp]), ("vko_get_kpsi", None, [vp, dp]), ("vko_set_kpsi", None, [vp, dp]),
            ("vko_gpe_rk4", None, [vp, C.c_int32]), ("vko_argle", None, [vp, C.c_int32, dp]),
            ("vko_diagnostics", None, [vp, dp, dp]),
            ("vko_particles_set", None, [vp, dp, dp, dp]), ("vko_particles_get", None, [vp, dp, dp, dp]),
            ("vko_particle_forces", None, [vp, dp]),
            ("vko_count_vortices", None, [vp, ip, ip]), ("vko_set_threads", None, [C.c_int32]),
            ("vko_set_frcdisp", None, [vp, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_uint64]),
            ("vko_set_argle_flow", None, [vp, C.c_int32, C.c_double, C.c_double]),
            ("vko_set_sgle", None, [vp, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_double,
                                    C.c_uint64]),
            ("vko_chempot", C.c_double, [vp]),
            ("vko_ic_vortices", C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_double, C.c_double,
                                            dp, dp]),
        ]:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _d(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """FP64 CPU state; same layouts as the product (psi[ny,nx], kpsi[nx,ny])."""

    def __init__(self, nx, ny=None, dt=1e-3, alpha=0.5, gstrength=1.0, omega_chem=1.0, disp_factor=0.0,
                 xi=0.0, n_particles=0, ppot_v0=0.0, ppot_d=1.0, gp_mass_part=1.0, renorm=False, threads=None):
        ny = ny or nx
        self.nx, self.ny = nx, ny
        p = VkoParams(nx, ny, n_particles, int(renorm), dt, alpha, gstrength, omega_chem, disp_factor, xi,
                      ppot_v0, ppot_d, gp_mass_part)
        self.p = p
        L = lib()
        if threads:
            L.vko_set_threads(int(threads))
        self._h = L.vko_create(C.byref(p))
        self.nshell = int(L.vko_nshell(nx))

    @classmethod
    def from_vk_params(cls, vp, renorm=None, threads=None):
        return cls(int(vp.nx), int(vp.ny), vp.dt, vp.alpha, vp.gstrength, vp.omega_chem, vp.disp_factor, vp.xi,
                   int(vp.n_particles), vp.ppot_v0, vp.ppot_d, vp.gp_mass_part,
                   bool(vp.argle_renorm) if renorm is None else renorm, threads)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().vko_destroy(self._h)
            self._h = None

    def fft_forward(self, phys):
        a = np.ascontiguousarray(phys, dtype=np.complex128)
        out = np.empty((self.nx, self.ny), dtype=np.complex128)
        lib().vko_fft_forward(self._h, _d(a.view(np.float64)), _d(out.view(np.float64)))
        return out

    def fft_inverse(self, four):
        a = np.ascontiguousarray(four, dtype=np.complex128)
        out = np.empty((self.ny, self.nx), dtype=np.complex128)
        lib().vko_fft_inverse(self._h, _d(a.view(np.float64)), _d(out.view(np.float64)))
        return out

    def set_psi(self, psi, otoc=True, k_otoc=1.8, eps_otoc=1e-4):
        a = np.ascontiguousarray(psi, dtype=np.complex128)
        lib().vko_set_psi(self._h, _d(a.view(np.float64)), int(otoc), k_otoc, eps_otoc)

    def set_kpsi(self, kpsi):
        a = np.ascontiguousarray(kpsi, dtype=np.complex128)
        lib().vko_set_kpsi(self._h, _d(a.view(np.float64)))

    def get_psi(self):
        out = np.empty((self.ny, self.nx), dtype=np.complex128)
        lib().vko_get_psi(self._h, _d(out.view(np.float64)))
        return out

    def get_kpsi(self):
        out = np.empty((self.nx, self.ny), dtype=np.complex128)
        lib().vko_get_kpsi(self._h, _d(out.view(np.float64)))
        return out

    def gpe_rk4(self, n=1):
        lib().vko_gpe_rk4(self._h, n)

    def argle(self, n=1):
        r = C.c_double()
        lib().vko_argle(self._h, n, C.byref(r))
        return float(r.value)

    def diagnostics(self):
        sc = np.zeros(10)
        spec = np.zeros((6, self.nshell + 1))
        lib().vko_diagnostics(self._h, _d(sc), _d(spec))
        return sc, spec

    def particles_set(self, pos, vel, f0ext):
        a, b, c = (np.ascontiguousarray(x, dtype=np.float64) for x in (pos, vel, f0ext))
        lib().vko_particles_set(self._h, _d(a), _d(b), _d(c))

    def particles_get(self):
        P = int(self.p.n_particles)
        pos, vel, frc = np.zeros((P, 2)), np.zeros((P, 2)), np.zeros((P, 2))
        lib().vko_particles_get(self._h, _d(pos), _d(vel), _d(frc))
        return pos, vel, frc

    def particle_forces(self):
        P = int(self.p.n_particles)
        frc = np.zeros((P, 2))
        lib().vko_particle_forces(self._h, _d(frc))
        return frc

    def set_frcdisp(self, on=True, vishypo=0.0, vishype=0.0, famp=0.0, kf1=0.0, kf2=0.0, seed=1):
        """-DGPE_FRCDISP terms of gpe_rhs (gpe.f90:623-658)."""
        lib().vko_set_frcdisp(self._h, int(on), vishypo, vishype, famp, kf1, kf2, seed)

    def set_argle_flow(self, mode, vnx=0.0, vny=0.0):
        """ARGLE flow terms (gpe.f90:78-146): 1 advection, 2 counterflow."""
        lib().vko_set_argle_flow(self._h, int(mode), vnx, vny)

    def set_sgle(self, on=True, oneybeta=0.0, nuN=0.0, chempot0=1.0, selftrunc=False, ktrunc=0.0, seed=1):
        """-DGPE_SGLE noise and chemical potential ODE (gpe.f90:149-274)."""
        lib().vko_set_sgle(self._h, int(on), oneybeta, nuN, chempot0, int(selftrunc), ktrunc, seed)

    @property
    def chempot(self):
        return float(lib().vko_chempot(self._h))

    def count_vortices(self):
        a, b = C.c_int32(), C.c_int32()
        lib().vko_count_vortices(self._h, C.byref(a), C.byref(b))
        return int(a.value), int(b.value)


def derived_params(nx, ny=None, dt=1e-3, xi_in=2.0 ** 0.5, csound=1.0, rho_avg=1.0, n_particles=0, ppotd=2.0,
                   ppotv0=10.0, gp_mass_part=0.0, renorm=False):
    """Keyword arguments of Oracle for a namelist (restates set_grid,
    src/mod_grid.f90:79-82, and the derived physics, src/driver.f90:362-370,
    391-392): xi = xi_in*dx, alpha = csound*xi*sqrt(rho_avg/2),
    g = csound^2/(2 alpha), omega = g, V0 <- ppotV0*g, d <- ppotd*xi."""
    ny = ny or nx
    dx = 2.0 * np.pi / nx
    xi = xi_in * dx
    alpha = csound * xi * np.sqrt(rho_avg / 2.0)
    g = csound * csound / (2.0 * alpha)
    return dict(nx=nx, ny=ny, dt=dt, alpha=alpha, gstrength=g, omega_chem=g, disp_factor=0.0, xi=xi,
                n_particles=n_particles, ppot_v0=ppotv0 * g, ppot_d=ppotd * xi, gp_mass_part=gp_mass_part,
                renorm=renorm)


def ic_vortices(nx, ny, n_vort, seed, xi0=None, min_sep=0.0):
    """Seeded neutral vortex state (vko_ic_vortices); xi0 defaults to
    sqrt(2)*dx.  Returns (psi[ny, nx], positions[n_vort, 2])."""
    if xi0 is None:
        xi0 = 2.0 ** 0.5 * 2.0 * np.pi / nx
    psi = np.empty((ny, nx), dtype=np.complex128)
    pos = np.empty((max(n_vort, 1), 2))
    rc = lib().vko_ic_vortices(nx, ny, n_vort, seed, xi0, min_sep, _d(psi.view(np.float64)), _d(pos))
    if rc != 0:
        raise ValueError("vko_ic_vortices: invalid arguments or the vortices cannot be placed")
    return psi, pos[:n_vort]
