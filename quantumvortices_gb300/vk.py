"""Python host binding of libvk (the C ABI in include/vk.h).

Mirrors the reference's call surface for the 2D GPE hot path:

=======================  ===============================================
this module              reference (paths relative to the project root)
=======================  ===============================================
``read_namelists``       namelist reads, src/driver.f90:147-215
``derive_params``        set_grid + derived physics, src/mod_grid.f90:63-101,
                         src/driver.f90:360-396
``GPESolver``            state of src/mod_fft.f90 (psi, kpsi, ...)
``GPESolver.set_psi``    restart_from_argle_data + ic_OTOC_gpe,
                         src/initial_config.f90:630-771, :295-368
``GPESolver.gpe_rk4``    gpe_rk4 / gpe_rhs, src/gpe.f90:310-671
``GPESolver.argle``      ARGLE(time), src/gpe.f90:5-224
``GPESolver.diagnostics_gpe``  diagnostics_gpe, src/diagnostics.f90:4-571
``io_fields``/``read_wf``      src/io_fields.f90:1-66 file layout
=======================  ===============================================

There is no CPU fallback: if libvk.so is missing or no CUDA device is
present, construction raises.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libvk.so")

VK_OK = 0
VK_PREC_FP64 = 0
VK_PREC_FP32 = 1
ERRORS = {-1: "VK_E_INVALID", -2: "VK_E_CUDA", -3: "VK_E_NOMEM", -4: "VK_E_IO", -5: "VK_E_STATE",
          -6: "VK_E_NUMERIC"}


class VkParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("precision", C.c_int32), ("otoc", C.c_int32),
        ("dt", C.c_double), ("alpha", C.c_double), ("gstrength", C.c_double), ("omega_chem", C.c_double),
        ("disp_factor", C.c_double), ("xi", C.c_double), ("k_otoc_gp", C.c_double), ("eps_otoc_gp", C.c_double),
        ("n_particles", C.c_int32), ("argle_renorm", C.c_int32),
        ("ppot_v0", C.c_double), ("ppot_d", C.c_double), ("gp_mass_part", C.c_double),
        ("reserved", C.c_int32 * 8),
    ]


class VkNamelist(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("dt_fix", C.c_double),
        ("xi", C.c_double), ("csound", C.c_double), ("rho_avg", C.c_double), ("disp_factor", C.c_double),
        ("k_otoc_gp", C.c_double), ("eps_otoc_gp", C.c_double),
        ("gp_n_obj", C.c_int32),
        ("gp_mass_part", C.c_double), ("ppotd", C.c_double), ("ppotv0", C.c_double), ("ppotthick", C.c_double),
        ("maxiter", C.c_int32), ("fsteps", C.c_int32), ("ssteps", C.c_int32), ("gsteps", C.c_int32),
        ("nrst", C.c_int32), ("sprst", C.c_int32), ("strst", C.c_int32), ("ststeps", C.c_int32),
        ("famp_gp", C.c_double), ("kf1_gp", C.c_double), ("kf2_gp", C.c_double),
        ("vishypo_gp", C.c_double), ("vishype_gp", C.c_double), ("vnx", C.c_double), ("vny", C.c_double),
        ("oneybeta", C.c_double), ("nun", C.c_double), ("chempot0", C.c_double), ("ktrunc", C.c_double),
        ("nsplit_orignal", C.c_int32), ("nsplit_current", C.c_int32),
    ]


VK_VAR_FRCDISP = 1
VK_VAR_ADVECTION = 2
VK_VAR_COUNTERFLOW = 4
VK_VAR_SGLE = 8
VK_VAR_SELFTRUNC = 16


class VkVariant(C.Structure):
    """vk_variant: run-time selection of the reference's compile-time branches."""
    _fields_ = [
        ("flags", C.c_int32), ("pad", C.c_int32),
        ("vishypo_gp", C.c_double), ("vishype_gp", C.c_double),
        ("famp_gp", C.c_double), ("kf1_gp", C.c_double), ("kf2_gp", C.c_double),
        ("vnx", C.c_double), ("vny", C.c_double),
        ("oneybeta", C.c_double), ("nuN", C.c_double), ("chempot0", C.c_double), ("ktrunc", C.c_double),
        ("seed", C.c_uint64), ("reserved", C.c_int32 * 8),
    ]


class VkError(RuntimeError):
    pass


_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Loads libvk.so (built in-tree by ``quantumvortices_gb300._build``)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise VkError(f"libvk.so not built ({p}); run __graft_entry__.build()")
    lib = C.CDLL(p)
    dp = C.POINTER(C.c_double)
    vp = C.c_void_p
    sig = {
        "vk_init": (C.c_int, [C.POINTER(VkParams), C.POINTER(vp)]),
        "vk_finalize": (C.c_int, [vp]),
        "vk_set_psi": (C.c_int, [vp, dp]),
        "vk_set_kpsi": (C.c_int, [vp, dp]),
        "vk_get_psi": (C.c_int, [vp, dp]),
        "vk_get_kpsi": (C.c_int, [vp, dp]),
        "vk_gpe_rk4": (C.c_int, [vp, C.c_int32]),
        "vk_argle": (C.c_int, [vp, C.c_int32, dp]),
        "vk_diagnostics": (C.c_int, [vp, dp, dp, C.POINTER(C.c_int32)]),
        "vk_particles_set": (C.c_int, [vp, dp, dp, dp]),
        "vk_particles_get": (C.c_int, [vp, dp, dp, dp]),
        "vk_get_stream": (C.c_int, [vp, C.POINTER(vp)]),
        "vk_kernel_launches": (C.c_int, [vp, C.POINTER(C.c_int64)]),
        "vk_last_error": (C.c_char_p, []),
        "vk_timing_begin": (C.c_int, [vp]),
        "vk_timing_end": (C.c_int, [vp, C.c_int32, C.c_char_p, dp, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
        "vk_read_namelists": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(VkNamelist)]),
        "vk_params_derive": (C.c_int, [C.POINTER(VkNamelist), C.c_int32, C.c_int32, C.POINTER(VkParams)]),
        "vk_nshell": (C.c_int32, [C.c_int32]),
        "vk_write_wf": (C.c_int, [C.c_char_p, C.c_int32, C.c_double, C.c_double, C.c_int32, C.c_int32, dp]),
        "vk_read_wf": (C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.POINTER(C.c_int32), dp, dp, dp]),
        "vk_read_wf_split": (C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32), dp, dp,
                                       dp]),
        "vk_ic_vortices": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_double, C.c_double, dp, dp]),
        "vk_set_psi_vortices": (C.c_int, [vp, C.c_int32, C.c_uint64, C.c_double, C.c_double, dp]),
        "vk_ens_init": (C.c_int, [C.POINTER(VkParams), C.c_int32, C.POINTER(vp)]),
        "vk_ens_finalize": (C.c_int, [vp]),
        "vk_ens_set_psi": (C.c_int, [vp, C.c_int32, dp]),
        "vk_ens_get_psi": (C.c_int, [vp, C.c_int32, dp]),
        "vk_ens_gpe_rk4": (C.c_int, [vp, C.c_int32]),
        "vk_ens_report": (C.c_int, [vp, C.c_char_p, C.c_int32]),
        "vk_ens_get_stream": (C.c_int, [vp, C.POINTER(vp)]),
        "vk_ens_kernel_launches": (C.c_int, [vp, C.POINTER(C.c_int64)]),
        "vk_set_variant": (C.c_int, [vp, C.POINTER(VkVariant)]),
        "vk_get_chempot": (C.c_int, [vp, dp]),
        "vk_dump_begin": (C.c_int, [vp]),
        "vk_dump_wait": (C.c_int, [vp, dp]),
        "vk_variant_derive": (C.c_int, [C.POINTER(VkNamelist), C.c_int32, C.c_uint64, C.POINTER(VkVariant)]),
        "vk_sts_begin": (C.c_int, [vp, C.c_int32]),
        "vk_sts_record": (C.c_int, [vp]),
        "vk_sts_count": (C.c_int, [vp, C.POINTER(C.c_int32)]),
        "vk_sts_spectra": (C.c_int, [vp, dp, dp]),
        "vk_sts_end": (C.c_int, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _check(rc: int, what: str) -> None:
    if rc != VK_OK:
        msg = load_library().vk_last_error()
        raise VkError(f"{what}: {ERRORS.get(rc, rc)}: {msg.decode() if msg else ''}")


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def solver_len_class(nx: int, ny: int) -> int:
    """Row-length class of an nx x ny grid (vk::solver_len_class): the first of
    the sets {16..128}, {128..512}, {256..1024}, {512..2048}, {1024..4096}
    (powers of two) holding both lengths, or -1 (vk_init rejects such grids)."""
    sets = [(16, 128), (128, 512), (256, 1024), (512, 2048), (1024, 4096)]
    for c, (lo, hi) in enumerate(sets):
        if lo <= nx <= hi and lo <= ny <= hi:
            return c
    return -1


def nshell(nx: int) -> int:
    """nshell = int(1.414*Nx/2.0d0)+1 (src/mod_grid.f90:77)."""
    return int(load_library().vk_nshell(nx))


def read_namelists(parameter_txt: str | None, parameter_gpe_txt: str | None) -> VkNamelist:
    nl = VkNamelist()
    a = parameter_txt.encode() if parameter_txt else None
    b = parameter_gpe_txt.encode() if parameter_gpe_txt else None
    _check(load_library().vk_read_namelists(a, b, C.byref(nl)), "vk_read_namelists")
    return nl


def derive_params(nl: VkNamelist, precision: int = VK_PREC_FP64, otoc: bool = True) -> VkParams:
    p = VkParams()
    _check(load_library().vk_params_derive(C.byref(nl), precision, int(otoc), C.byref(p)), "vk_params_derive")
    return p


def derive_variant(nl: VkNamelist, flags: int, seed: int = 1) -> VkVariant:
    """vk_variant from the namelists (&gpforceparam, &gphypvis, &gpcounterflow,
    &gpfiniteT, &selftruncation) for the VK_VAR_* flags."""
    v = VkVariant()
    _check(load_library().vk_variant_derive(C.byref(nl), flags, seed, C.byref(v)), "vk_variant_derive")
    return v


def params_for(nx: int, ny: int | None = None, dt: float = 1e-3, precision: int = VK_PREC_FP64,
               otoc: bool = True, xi_in: float = math.sqrt(2.0), n_particles: int = 0, ppotd: float = 2.0,
               ppotv0: float = 10.0, gp_mass_part: float = 0.0, argle_renorm: bool = False) -> VkParams:
    """Parameters of the benchmark equation in the reference's parametrisation.

    csound = rho_avg = 1 and xi = xi_in*dx with xi_in = sqrt(2) (healing length
    sqrt(2)*dx) give alpha = dx and g = Omega = 1/(2 dx) (src/driver.f90:362-370),
    i.e. i dpsi/dt = -alpha lap psi + g |psi|^2 psi - g psi.  With lengths in
    units of 2*dx and times in units of 1/g this is i dpsi/dtau = -1/2 lap psi
    + |psi|^2 psi - psi (g = rho0 = mu = 1), healing length 1/sqrt(2)."""
    ny = ny or nx
    nl = VkNamelist()
    nl.nx, nl.ny, nl.dt_fix = nx, ny, dt
    nl.csound, nl.rho_avg, nl.disp_factor = 1.0, 1.0, 0.0
    nl.xi = xi_in
    nl.k_otoc_gp, nl.eps_otoc_gp = 1.8, 1.0e-4
    nl.gp_n_obj, nl.ppotd, nl.ppotv0, nl.gp_mass_part = n_particles, ppotd, ppotv0, gp_mass_part
    p = derive_params(nl, precision, otoc)
    p.argle_renorm = int(argle_renorm)
    return p


def write_wf(path: str, psi: np.ndarray, iopoint: int = 0, time: float = 0.0, dt: float = 0.0) -> None:
    """io_fields file (src/io_fields.f90:42-49): psi[ny, nx] complex128."""
    a = np.ascontiguousarray(psi, dtype=np.complex128)
    ny, nx = a.shape
    _check(load_library().vk_write_wf(path.encode(), iopoint, time, dt, nx, ny, _dptr(a.view(np.float64))),
           "vk_write_wf")


def read_wf(path: str, nx: int, ny: int):
    a = np.empty((ny, nx), dtype=np.complex128)
    io = C.c_int32()
    t = C.c_double()
    d = C.c_double()
    _check(load_library().vk_read_wf(path.encode(), nx, ny, C.byref(io), C.byref(t), C.byref(d),
                                      _dptr(a.view(np.float64))), "vk_read_wf")
    return a, int(io.value), float(t.value), float(d.value)


def read_wf_split(prefix: str, nsplit: int, nx: int, ny: int):
    """A field written as nsplit files <prefix>p<j>.dat (src/io_fields.f90:121-146);
    returns (psi[ny, nx], iopoint, time, dt)."""
    psi = np.empty((ny, nx), dtype=np.complex128)
    io, t, d = C.c_int32(), C.c_double(), C.c_double()
    _check(load_library().vk_read_wf_split(prefix.encode(), nsplit, nx, ny, C.byref(io), C.byref(t), C.byref(d),
                                           _dptr(psi.view(np.float64))), "vk_read_wf_split")
    return psi, int(io.value), float(t.value), float(d.value)


def ic_vortices(nx: int, ny: int, n_vort: int, seed: int, xi0: float | None = None, min_sep: float = 0.0):
    """Seeded neutral N-vortex state (new component; no reference counterpart).
    xi0 defaults to sqrt(2)*dx.  Returns (psi[ny, nx], positions[n_vort, 2])."""
    if xi0 is None:
        xi0 = math.sqrt(2.0) * 2.0 * math.pi / nx
    psi = np.empty((ny, nx), dtype=np.complex128)
    pos = np.empty((max(n_vort, 1), 2), dtype=np.float64)
    _check(load_library().vk_ic_vortices(nx, ny, n_vort, seed, xi0, min_sep, _dptr(psi.view(np.float64)),
                                          _dptr(pos)), "vk_ic_vortices")
    return psi, pos[:n_vort]


@dataclass
class Diagnostics:
    momx: float
    momy: float
    egrad: float
    echem: float
    eintr: float
    etot: float
    norm: float
    eppot: float
    eobj_kin: float
    esrep: float
    spec: np.ndarray          # spec_gp(0:nshell, 1:6) as [6, nshell+1]
    nvort: tuple[int, int]

    def quantglobal(self):
        """quantglobal_gpe sums (src/diagnostics.f90:588-592): ekint, ekini, ekinc,
        equnt over shells 1..nshell, eintr over 0..nshell, and n0 = spec(0,6)."""
        s = self.spec
        return (s[0, 1:].sum(), s[1, 1:].sum(), s[2, 1:].sum(), s[3, 1:].sum(), s[4, :].sum(), s[5, 0])


class GPESolver:
    """One GPU state of the 2D GPE stepper (one CUDA stream)."""

    def __init__(self, params: VkParams):
        self.lib = load_library()
        self.params = params
        self.nx, self.ny = int(params.nx), int(params.ny)
        self.nshell = nshell(self.nx)
        h = C.c_void_p()
        _check(self.lib.vk_init(C.byref(params), C.byref(h)), "vk_init")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _check(self.lib.vk_finalize(self._h), "vk_finalize")
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_psi(self, psi: np.ndarray) -> None:
        a = np.ascontiguousarray(psi, dtype=np.complex128)
        assert a.shape == (self.ny, self.nx)
        _check(self.lib.vk_set_psi(self._h, _dptr(a.view(np.float64))), "vk_set_psi")

    def set_psi_vortices(self, n_vort: int, seed: int, xi0: float | None = None, min_sep: float = 0.0):
        """Seeded vortex state computed on the GPU (same as ic_vortices), then set_psi."""
        if xi0 is None:
            xi0 = math.sqrt(2.0) * 2.0 * math.pi / self.nx
        pos = np.empty((max(n_vort, 1), 2))
        _check(self.lib.vk_set_psi_vortices(self._h, n_vort, seed, xi0, min_sep, _dptr(pos)), "vk_set_psi_vortices")
        return pos[:n_vort]

    def set_kpsi(self, kpsi: np.ndarray) -> None:
        a = np.ascontiguousarray(kpsi, dtype=np.complex128)
        assert a.shape == (self.nx, self.ny)
        _check(self.lib.vk_set_kpsi(self._h, _dptr(a.view(np.float64))), "vk_set_kpsi")

    def get_psi(self, out: np.ndarray | None = None) -> np.ndarray:
        a = out if out is not None else np.empty((self.ny, self.nx), dtype=np.complex128)
        _check(self.lib.vk_get_psi(self._h, _dptr(a.view(np.float64))), "vk_get_psi")
        return a

    def get_kpsi(self, out: np.ndarray | None = None) -> np.ndarray:
        a = out if out is not None else np.empty((self.nx, self.ny), dtype=np.complex128)
        _check(self.lib.vk_get_kpsi(self._h, _dptr(a.view(np.float64))), "vk_get_kpsi")
        return a

    def gpe_rk4(self, nsteps: int = 1) -> None:
        _check(self.lib.vk_gpe_rk4(self._h, nsteps), "vk_gpe_rk4")

    def argle(self, nsteps: int = 1) -> float:
        r = C.c_double()
        _check(self.lib.vk_argle(self._h, nsteps, C.byref(r)), "vk_argle")
        return float(r.value)

    def diagnostics_gpe(self) -> Diagnostics:
        sc = np.zeros(10)
        spec = np.zeros((6, self.nshell + 1))
        nv = (C.c_int32 * 2)()
        _check(self.lib.vk_diagnostics(self._h, _dptr(sc), _dptr(spec), nv), "vk_diagnostics")
        return Diagnostics(*[float(v) for v in sc], spec=spec, nvort=(int(nv[0]), int(nv[1])))

    def particles_set(self, pos, vel, f0ext) -> None:
        a, b, c = (np.ascontiguousarray(x, dtype=np.float64) for x in (pos, vel, f0ext))
        _check(self.lib.vk_particles_set(self._h, _dptr(a), _dptr(b), _dptr(c)), "vk_particles_set")

    def particles_get(self):
        P = int(self.params.n_particles)
        pos, vel, frc = np.zeros((P, 2)), np.zeros((P, 2)), np.zeros((P, 2))
        _check(self.lib.vk_particles_get(self._h, _dptr(pos), _dptr(vel), _dptr(frc)), "vk_particles_get")
        return pos, vel, frc

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        _check(self.lib.vk_get_stream(self._h, C.byref(s)), "vk_get_stream")
        return int(s.value or 0)

    def timing_begin(self) -> None:
        """Bracket every following kernel launch with CUDA events on the context stream."""
        _check(self.lib.vk_timing_begin(self._h), "vk_timing_begin")

    def timing_end(self) -> dict:
        """Returns {kernel tag: (total ms, launches)} since timing_begin()."""
        cap = 64
        tags = C.create_string_buffer(24 * cap)
        ms = np.zeros(cap)
        cnt = np.zeros(cap, dtype=np.int64)
        n = C.c_int32()
        _check(self.lib.vk_timing_end(self._h, cap, tags, _dptr(ms), cnt.ctypes.data_as(C.POINTER(C.c_int64)),
                                      C.byref(n)), "vk_timing_end")
        raw = tags.raw
        out = {}
        for j in range(min(n.value, cap)):
            name = raw[24 * j:24 * j + 24].split(b"\0", 1)[0].decode()
            out[name] = (float(ms[j]), int(cnt[j]))
        return out

    @property
    def launches(self) -> int:
        n = C.c_int64()
        _check(self.lib.vk_kernel_launches(self._h, C.byref(n)), "vk_kernel_launches")
        return int(n.value)

    def set_variant(self, frcdisp: bool = False, vishypo: float = 0.0, vishype: float = 0.0, famp: float = 0.0,
                    kf1: float = 0.0, kf2: float = 0.0, seed: int = 1, flow: str | None = None,
                    vnx: float = 0.0, vny: float = 0.0, sgle: bool = False, oneybeta: float = 0.0,
                    nuN: float = 0.0, chempot0: float = 0.0, selftrunc: bool = False, ktrunc: float = 0.0) -> None:
        """-DGPE_FRCDISP: hypo/hyperviscosity and random-phase shell forcing in
        every RK4 right-hand side (src/gpe.f90:623-658); kf in units of kdx.
        flow = "advection" / "counterflow": the ARGLE flow terms
        (src/gpe.f90:78-146), counterflow velocity (vnx, vny).  sgle: the
        finite-temperature ARGLE (noise + chemical potential ODE from chempot0,
        src/gpe.f90:149-274), selftrunc: zero k^2 > ktrunc^2."""
        v = VkVariant()
        v.flags = (VK_VAR_FRCDISP if frcdisp else 0) | {None: 0, "advection": VK_VAR_ADVECTION,
                                                        "counterflow": VK_VAR_COUNTERFLOW}[flow]
        v.flags |= (VK_VAR_SGLE if sgle else 0) | (VK_VAR_SELFTRUNC if selftrunc else 0)
        v.oneybeta, v.nuN, v.chempot0, v.ktrunc = oneybeta, nuN, chempot0, ktrunc
        v.vishypo_gp, v.vishype_gp, v.famp_gp, v.kf1_gp, v.kf2_gp = vishypo, vishype, famp, kf1, kf2
        v.vnx, v.vny = vnx, vny
        v.seed = seed
        _check(self.lib.vk_set_variant(self._h, C.byref(v)), "vk_set_variant")

    def dump_begin(self) -> None:
        """Start an asynchronous copy of the current psi (vk_dump_begin)."""
        _check(self.lib.vk_dump_begin(self._h), "vk_dump_begin")

    def dump_wait(self) -> np.ndarray:
        """psi[ny, nx] of the last dump_begin (blocks until its copy is done)."""
        a = np.empty((self.ny, self.nx), dtype=np.complex128)
        _check(self.lib.vk_dump_wait(self._h, _dptr(a.view(np.float64))), "vk_dump_wait")
        return a

    def apply_variant(self, v: VkVariant) -> None:
        """vk_set_variant with a ready vk_variant (see derive_variant)."""
        _check(self.lib.vk_set_variant(self._h, C.byref(v)), "vk_set_variant")

    @property
    def chempot(self) -> float:
        """Current omega_chem (evolves under the SGLE variant)."""
        x = C.c_double()
        _check(self.lib.vk_get_chempot(self._h, C.byref(x)), "vk_get_chempot")
        return float(x.value)

    # spatio-temporal spectra (sts_gpe + the Run/CompSTS post-processor)
    def sts_begin(self, nt: int) -> None:
        """Device ring for nt kpsi records (nt a power of two, 16..4096)."""
        self._sts_nt = int(nt)
        _check(self.lib.vk_sts_begin(self._h, int(nt)), "vk_sts_begin")

    def sts_record(self) -> None:
        """Appends the current kpsi (sts_gpe, every ststeps)."""
        _check(self.lib.vk_sts_record(self._h), "vk_sts_record")

    @property
    def sts_count(self) -> int:
        n = C.c_int32()
        _check(self.lib.vk_sts_count(self._h, C.byref(n)), "vk_sts_count")
        return int(n.value)

    def sts_spectra(self):
        """(sts1d[nt, ny], sts2d[nt, nx//3 + 1]) of the full ring; consumes it."""
        nt = self._sts_nt
        a = np.empty((nt, self.ny))
        b = np.empty((nt, self.nx // 3 + 1))
        _check(self.lib.vk_sts_spectra(self._h, _dptr(a), _dptr(b)), "vk_sts_spectra")
        return a, b

    def sts_end(self) -> None:
        _check(self.lib.vk_sts_end(self._h), "vk_sts_end")


class Ensemble:
    """Independent fields of uneven sizes stepped together (batched
    persistent kernels, one CUDA graph per RK4 step)."""

    def __init__(self, params: list):
        self.lib = load_library()
        self.params = list(params)
        arr = (VkParams * len(self.params))(*self.params)
        h = C.c_void_p()
        _check(self.lib.vk_ens_init(arr, len(self.params), C.byref(h)), "vk_ens_init")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _check(self.lib.vk_ens_finalize(self._h), "vk_ens_finalize")
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_psi(self, m: int, psi: np.ndarray) -> None:
        a = np.ascontiguousarray(psi, dtype=np.complex128)
        p = self.params[m]
        assert a.shape == (p.ny, p.nx)
        _check(self.lib.vk_ens_set_psi(self._h, m, _dptr(a.view(np.float64))), "vk_ens_set_psi")

    def get_psi(self, m: int) -> np.ndarray:
        p = self.params[m]
        a = np.empty((p.ny, p.nx), dtype=np.complex128)
        _check(self.lib.vk_ens_get_psi(self._h, m, _dptr(a.view(np.float64))), "vk_ens_get_psi")
        return a

    def gpe_rk4(self, nsteps: int = 1) -> None:
        _check(self.lib.vk_ens_gpe_rk4(self._h, nsteps), "vk_ens_gpe_rk4")

    @property
    def report(self) -> str:
        buf = C.create_string_buffer(2048)
        _check(self.lib.vk_ens_report(self._h, buf, 2048), "vk_ens_report")
        return buf.value.decode()

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        _check(self.lib.vk_ens_get_stream(self._h, C.byref(s)), "vk_ens_get_stream")
        return int(s.value or 0)

    @property
    def launches(self) -> int:
        n = C.c_int64()
        _check(self.lib.vk_ens_kernel_launches(self._h, C.byref(n)), "vk_ens_kernel_launches")
        return int(n.value)
