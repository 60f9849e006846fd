"""Host-side checks of libvk (no GPU): exports, parameter derivation,
namelist parsing, the wf file format, error paths and the vortex IC."""
import math
import os
import re
import struct

import numpy as np
import pytest

from quantumvortices_gb300 import vk

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(vk_\w+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    lib = vk.load_library()
    names = _declared_symbols()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_params_mapping():
    n = 128
    dx = 2 * math.pi / n
    p = vk.params_for(n, dt=1e-3)
    assert abs(p.xi - math.sqrt(2) * dx) < 1e-16
    assert abs(p.alpha - dx) < 1e-16 and abs(p.gstrength - 1 / (2 * dx)) < 1e-12
    assert p.omega_chem == p.gstrength
    # ppotV0 -> V0*g, ppotd -> d*xi (src/driver.f90:391-392)
    q = vk.params_for(n, n_particles=16, ppotd=2.0, ppotv0=10.0, gp_mass_part=3.0)
    assert abs(q.ppot_v0 - 10 * q.gstrength) < 1e-12 and abs(q.ppot_d - 2 * q.xi) < 1e-16
    assert q.n_particles == 16 and q.gp_mass_part == 3.0


def test_namelist_parsing(tmp_path):
    a = tmp_path / "parameter.txt"
    a.write_text("! Parameters\n&ckprst\nnrst = 0   ! restart\nsprst = 0\nstrst = 2\n/\n&resolution\nNx=256\n"
                 "Ny=128\nNz=64\n/\n&fileparam\nnsplit_orignal = 4\nnsplit_current = 1\n/\n&tparam\ndt_fix=1.0d-3  ! step\nmaxiter=400000\nfsteps=1000\nssteps=1000\n"
                 "gsteps=100\nststeps=20     ! kpsi 1d-line output frequency\n/\n")
    b = tmp_path / "parameter_gpe.txt"
    b.write_text("&gpparam\nxi=1.0d0 !\ncsound=1.0d0 !\nrho_avg=1.0d0 !\ndisp_factor=0.0d0 !\n/\n"
                 "&gpparticle\ngp_N_obj = 16 !\ngp_mass_part = 100.0d0 !\nppotd = 2.0d0\nppotV0 = 10.0d0 !\n/\n"
                 "&gpotoc\nk_otoc_gp = 1.8d0 !\neps_otoc_gp = 1.0d0-4 !\n/\n"
                 "&gpforceparam\nfamp_gp = 0.5d0\nkf1_gp = 2.0d0\nkf2_gp = 4.0d0\n/\n"
                 "&gphypvis\nnhypvis1_gp = 8\nvishype_gp = 1.0d-20\n/\n&gpcounterflow\nvnx = 0.25d0\nvny = -0.5d0\n/\n"
                 "&gpfiniteT\noneybeta = 0.1d0\nnuN = 3.0d0\nchempot0 = 0.9d0\n/\n&selftruncation\nktrunc = 40.0d0\n/\n")
    nl = vk.read_namelists(str(a), str(b))
    assert (nl.nx, nl.ny, nl.maxiter, nl.fsteps, nl.gsteps) == (256, 128, 400000, 1000, 100)
    assert (nl.strst, nl.ststeps) == (2, 20)
    assert (nl.famp_gp, nl.kf1_gp, nl.kf2_gp, nl.vishype_gp) == (0.5, 2.0, 4.0, 1e-20)
    assert (nl.vnx, nl.vny, nl.oneybeta, nl.nun, nl.chempot0, nl.ktrunc) == (0.25, -0.5, 0.1, 3.0, 0.9, 40.0)
    assert (nl.nsplit_orignal, nl.nsplit_current) == (4, 1)
    v = vk.derive_variant(nl, vk.VK_VAR_FRCDISP | vk.VK_VAR_SGLE, seed=7)
    assert (v.flags, v.kf1_gp, v.kf2_gp, v.nuN, v.chempot0, v.seed) == (9, 2.0, 4.0, 3.0, 0.9, 7)
    assert nl.dt_fix == 1e-3 and nl.gp_n_obj == 16 and nl.ppotv0 == 10.0
    p = vk.derive_params(nl)
    dx = 2 * math.pi / 256
    assert abs(p.xi - dx) < 1e-18
    assert abs(p.alpha - dx * math.sqrt(0.5)) < 1e-18
    assert abs(p.gstrength - 1.0 / (2 * p.alpha)) < 1e-12
    assert abs(p.ppot_v0 - 10 * p.gstrength) < 1e-12 and abs(p.ppot_d - 2 * dx) < 1e-15
    with pytest.raises(vk.VkError):
        vk.read_namelists(str(tmp_path / "missing.txt"), None)
    nl.nx = 100
    with pytest.raises(vk.VkError):
        vk.derive_params(nl)


def test_wf_file_layout_round_trip(tmp_path):
    nx, ny = 16, 8
    rng = np.random.default_rng(0)
    psi = rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))
    path = str(tmp_path / "wf3p1.dat")
    vk.write_wf(path, psi, iopoint=3, time=0.25, dt=1e-3)
    raw = open(path, "rb").read()
    # record 1: marker 20, int32 iopoint, real64 time, real64 dt, marker 20
    assert struct.unpack("<i", raw[:4])[0] == 20 and struct.unpack("<i", raw[24:28])[0] == 20
    assert struct.unpack("<idd", raw[4:24]) == (3, 0.25, 1e-3)
    rec = 16 * nx
    assert len(raw) == 28 + ny * (rec + 8)
    off = 28
    for y in range(ny):
        assert struct.unpack("<i", raw[off:off + 4])[0] == rec
        row = np.frombuffer(raw[off + 4:off + 4 + rec], dtype=np.complex128)
        assert np.array_equal(row, psi[y])
        off += rec + 8
    back, io, t, d = vk.read_wf(path, nx, ny)
    assert np.array_equal(back, psi) and (io, t, d) == (3, 0.25, 1e-3)


def test_wf_errors(tmp_path):
    nx, ny = 16, 8
    psi = np.ones((ny, nx), complex)
    path = str(tmp_path / "wf0p1.dat")
    vk.write_wf(path, psi)
    with pytest.raises(vk.VkError, match="VK_E_IO"):
        vk.read_wf(str(tmp_path / "nope.dat"), nx, ny)
    with pytest.raises(vk.VkError, match="VK_E_IO"):  # wrong record length
        vk.read_wf(path, nx * 2, ny)
    raw = open(path, "rb").read()
    open(path, "wb").write(raw[: len(raw) - 100])  # truncated
    with pytest.raises(vk.VkError, match="truncated"):
        vk.read_wf(path, nx, ny)


def test_init_rejects_bad_parameters():
    p = vk.params_for(64)
    p.nx = 100
    with pytest.raises(vk.VkError, match="VK_E_INVALID"):
        vk.GPESolver(p)
    p = vk.params_for(64)
    p.dt = float("nan")
    with pytest.raises(vk.VkError, match="VK_E_INVALID"):
        vk.GPESolver(p)
    p = vk.params_for(64)
    p.precision = 7
    with pytest.raises(vk.VkError, match="VK_E_INVALID"):
        vk.GPESolver(p)
    # grids whose rows fall in different length classes are rejected before
    # any device work
    p = vk.params_for(64, 2048)
    with pytest.raises(vk.VkError, match="row-length class"):
        vk.GPESolver(p)


def test_solver_len_classes():
    assert vk.solver_len_class(16, 128) == 0 and vk.solver_len_class(128, 64) == 0
    assert [vk.solver_len_class(n, n) for n in (256, 512, 1024, 2048, 4096)] == [1, 1, 2, 3, 4]
    assert vk.solver_len_class(1024, 256) == 2 and vk.solver_len_class(4096, 1024) == 4
    assert vk.solver_len_class(64, 256) == -1 and vk.solver_len_class(16, 4096) == -1


def test_ic_vortices_periodic_and_seeded():
    n = 64
    a, pos = vk.ic_vortices(n, n, 8, seed=7)
    b, pos2 = vk.ic_vortices(n, n, 8, seed=7)
    assert np.array_equal(a, b) and np.array_equal(pos, pos2)
    c, _ = vk.ic_vortices(n, n, 8, seed=8)
    assert not np.array_equal(a, c)
    assert np.all(np.abs(a) <= 1.0)
    with pytest.raises(vk.VkError):
        vk.ic_vortices(n, n, 7, seed=1)  # a non-neutral set cannot be periodic
    # minimum separation respected (periodic distance)
    _, p3 = vk.ic_vortices(n, n, 16, seed=2, min_sep=0.5)
    d = p3[:, None, :] - p3[None, :, :]
    d = (d + np.pi) % (2 * np.pi) - np.pi
    dist = np.sqrt((d ** 2).sum(-1)) + np.eye(16) * 10
    assert dist.min() >= 0.5


def test_split_restart_files_regroup(tmp_path):
    """A field written by 4 ranks (y slabs, src/io_fields.f90 -DIOEVERYPROC)
    reads back as one field; ny not a multiple of nsplit is rejected."""
    nx, ny, ns = 16, 32, 4
    rng = np.random.default_rng(3)
    psi = rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))
    for j in range(ns):
        vk.write_wf(str(tmp_path / f"wf7p{j + 1}.dat"), psi[j * ny // ns:(j + 1) * ny // ns], iopoint=7,
                    time=0.5, dt=1e-3)
    got, io, t, d = vk.read_wf_split(str(tmp_path / "wf7"), ns, nx, ny)
    assert np.array_equal(got, psi) and io == 7 and t == 0.5 and d == 1e-3
    with pytest.raises(vk.VkError):
        vk.read_wf_split(str(tmp_path / "wf7"), 3, nx, ny)
    with pytest.raises(vk.VkError):
        vk.read_wf_split(str(tmp_path / "missing"), ns, nx, ny)
