"""The C++ host driver (driver + solve loop) end to end on the GPU: it reads
the namelists and restart/wf/wf0p1.dat, steps, and writes the reference's
files; values are checked against the Python API on the same inputs."""
import math
import os
import re
import subprocess

import numpy as np
import pytest

from quantumvortices_gb300 import _build, vk

pytestmark = pytest.mark.gpu

E156 = r"\s*-?0\.\d{6}E[+-]\d{2}"


def _write_inputs(d, n, dt, maxiter, fsteps, gsteps, ssteps, npart=0):
    (d / "parameter.txt").write_text(
        f"&ckprst\nnrst = 0\nsprst = 0\n/\n&resolution\nNx={n}\nNy={n}\n/\n"
        f"&tparam\ndt_fix={dt:.6e}\nmaxiter={maxiter}\nfsteps={fsteps}\nssteps={ssteps}\ngsteps={gsteps}\n/\n")
    dx = 2 * math.pi / n
    gpe = "&gpparam\nxi=1.4142135623730951d0\ncsound=1.0d0\nrho_avg=1.0d0\ndisp_factor=0.0d0\n/\n"
    gpe += "&gpotoc\nk_otoc_gp = 1.8d0\neps_otoc_gp = 1.0d-4\n/\n"
    if npart:
        mass = 5 * math.pi * (2 * math.sqrt(2) * dx) ** 2
        gpe += f"&gpparticle\ngp_N_obj = {npart}\ngp_mass_part = {mass:.16e}\nppotd = 2.0d0\nppotV0 = 10.0d0\n/\n"
    (d / "parameter_gpe.txt").write_text(gpe)
    (d / "restart" / "wf").mkdir(parents=True)
    psi, _ = vk.ic_vortices(n, n, 8, seed=3)
    vk.write_wf(str(d / "restart" / "wf" / "wf0p1.dat"), psi)
    return psi


def test_driver_rk4_outputs(tmp_path):
    n, dt = 128, 1e-3
    psi0 = _write_inputs(tmp_path, n, dt, maxiter=20, fsteps=10, gsteps=5, ssteps=10)
    r = subprocess.run([_build.DRIVER], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for f in ["data/wf/wf0p1.dat", "data/wf/wf1p1.dat", "data/wf/wf2p1.dat", "spectra/spec0.dat",
              "spectra/spec1.dat", "spectra/spec2.dat", "run_info.dat"]:
        assert (tmp_path / f).exists(), f
    e1 = (tmp_path / "data/energy1.dat_nrst0").read_text().splitlines()
    assert len(e1) == 5 and all(re.fullmatch(f"({E156}){{5}}", ln) for ln in e1)
    spec = (tmp_path / "spectra/spec2.dat").read_text().splitlines()
    assert len(spec) == vk.nshell(n) and all(re.fullmatch(f"({E156}){{7}}", ln) for ln in spec)
    # same run through the Python API
    p = vk.params_for(n, dt=dt)
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        s.gpe_rk4(20)
        d = s.diagnostics_gpe()
        field, io, t, dtf = vk.read_wf(str(tmp_path / "data/wf/wf2p1.dat"), n, n)
        assert io == 2 and abs(t - 20 * dt) < 1e-12 and dtf == dt
        assert np.array_equal(field, s.get_psi())
    last = [float(v) for v in e1[-1].split()]
    for got, want in zip(last[1:], [d.egrad, d.echem, d.eintr, d.etot]):
        assert abs(got - want) <= 1e-5 * abs(want)


def test_driver_refuses_missing_restart(tmp_path):
    _write_inputs(tmp_path, 64, 1e-3, 2, 1, 1, 1)
    os.remove(tmp_path / "restart/wf/wf0p1.dat")
    r = subprocess.run([_build.DRIVER], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "restart" in r.stderr


def test_driver_argle_with_particles(tmp_path):
    n = 64
    _write_inputs(tmp_path, n, 1e-3, maxiter=6, fsteps=3, gsteps=3, ssteps=3, npart=2)
    part = tmp_path / "restart" / "part"
    part.mkdir()
    (part / "gppos.dat_nrst0").write_text("0 0.0 1.0 2.0\n0 0.0 4.0 3.5\n")
    (part / "gpvel.dat_nrst0").write_text("0 0.0 0.1 0.0\n0 0.0 0.0 -0.1\n")
    (part / "gpf0ext.dat_nrst0").write_text("0 0.0 0.0 0.0\n0 0.0 0.0 0.0\n")
    r = subprocess.run([_build.DRIVER, "--argle"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    res = (tmp_path / "data/argle_residual.dat_nrst0").read_text().splitlines()
    assert len(res) == 2
    assert (tmp_path / "data/gpobj_frc_2.dat_nrst0").exists()
    eg = (tmp_path / "data/egpobj.dat_nrst0").read_text().splitlines()
    assert len(eg) == 3 and all(re.fullmatch(f"({E156}){{4}}", ln) for ln in eg)


def _read_records(path, rec_len):
    """Fortran sequential-unformatted records of complex128."""
    raw = open(path, "rb").read()
    out, i = [], 0
    while i < len(raw):
        m = int(np.frombuffer(raw[i:i + 4], dtype=np.int32)[0])
        assert m == rec_len * 16
        out.append(np.frombuffer(raw[i + 4:i + 4 + m], dtype=np.complex128))
        assert int(np.frombuffer(raw[i + 4 + m:i + 8 + m], dtype=np.int32)[0]) == m
        i += m + 8
    return np.array(out)


def test_driver_sts_path(tmp_path):
    """--sts NT: the sts_gpe record files every ststeps and, once NT records
    are held, the spectra of Run/CompSTS (checked against the oracle fed
    with the driver's own record files)."""
    from oracle import sts_oracle
    n, dt, nt, ststeps = 64, 1e-3, 16, 3
    _write_inputs(tmp_path, n, dt, maxiter=(nt - 1) * ststeps, fsteps=1000, gsteps=1000, ssteps=1000)
    txt = (tmp_path / "parameter.txt").read_text().replace("gsteps=1000\n", f"gsteps=1000\nststeps={ststeps}\n")
    (tmp_path / "parameter.txt").write_text(txt)
    r = subprocess.run([_build.DRIVER, "--sts", str(nt)], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    t = (tmp_path / "data/sts_time.dat_nrst0").read_text().split()
    assert len(t) == nt and abs(float(t[-1]) - (nt - 1) * ststeps * dt) < 1e-9
    line = _read_records(tmp_path / "data/sts1d/kpsi_x0_nrst0.dat", n)
    plane = _read_records(tmp_path / "data/sts2d/kpsi_nrst0p1.dat", n * n)
    assert line.shape == (nt, n) and plane.shape == (nt, n * n)
    assert np.array_equal(line, plane[:, :n])            # kx = 0 is the first row of kpsi[kx][ky]
    r1, r2 = sts_oracle.spectra(plane.reshape(nt, n, n))
    g1 = np.loadtxt(tmp_path / "data/sts1d_kx0_nrst0.dat")
    g2 = np.loadtxt(tmp_path / "data/sts2d_nrst0.dat")
    assert g1.shape == r1.shape and g2.shape == r2.shape
    assert np.abs(g1 - r1).max() <= 1e-12 * np.abs(r1).max()
    assert np.abs(g2 - r2).max() <= 1e-12 * np.abs(r2).max()


def test_driver_sgle_argle_and_counterflow(tmp_path):
    """--argle --sgle --counterflow: the branches come from &gpfiniteT and
    &gpcounterflow; data/cpot_sgle.dat_nrst0 gets (time, omega_chem) every
    fsteps, equal to the Python API's run of the same variant."""
    n, dt = 64, 1e-3
    psi0 = _write_inputs(tmp_path, n, dt, maxiter=30, fsteps=10, gsteps=10, ssteps=10)
    with open(tmp_path / "parameter_gpe.txt", "a") as f:
        f.write("&gpfiniteT\noneybeta = 0.05d0\nnuN = 2.0d0\nchempot0 = 7.5d0\n/\n"
                "&gpcounterflow\nvnx = 0.2d0\nvny = 0.1d0\n/\n")
    r = subprocess.run([_build.DRIVER, "--argle", "--sgle", "--counterflow"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rows = [[float(v) for v in ln.split()] for ln in (tmp_path / "data/cpot_sgle.dat_nrst0").read_text().splitlines()]
    assert len(rows) == 3
    nl = vk.read_namelists(str(tmp_path / "parameter.txt"), str(tmp_path / "parameter_gpe.txt"))
    p = vk.derive_params(nl)
    with vk.GPESolver(p) as s:
        s.set_psi(psi0)
        s.apply_variant(vk.derive_variant(nl, vk.VK_VAR_SGLE | vk.VK_VAR_COUNTERFLOW, seed=1))
        for t, om in rows:
            s.argle(10)
            assert abs(om - s.chempot) <= 1e-5 * abs(s.chempot)
        field, *_ = vk.read_wf(str(tmp_path / "data/wf/wf3p1.dat"), n, n)
        assert np.array_equal(field, s.get_psi())


def test_driver_regroups_split_restart(tmp_path):
    """&fileparam nsplit_orignal = 4: the restart field is read from
    restart/wf/wf0p1..p4.dat; the run equals one from the joined field."""
    n, dt = 64, 1e-3
    psi0 = _write_inputs(tmp_path, n, dt, maxiter=10, fsteps=10, gsteps=10, ssteps=10)
    (tmp_path / "restart/wf/wf0p1.dat").unlink()
    for j in range(4):
        vk.write_wf(str(tmp_path / f"restart/wf/wf0p{j + 1}.dat"), psi0[j * n // 4:(j + 1) * n // 4])
    txt = (tmp_path / "parameter.txt").read_text().replace("&resolution", "&fileparam\nnsplit_orignal = 4\n"
                                                           "nsplit_current = 1\n/\n&resolution")
    (tmp_path / "parameter.txt").write_text(txt)
    r = subprocess.run([_build.DRIVER], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    with vk.GPESolver(vk.params_for(n, dt=dt)) as s:
        s.set_psi(psi0)
        s.gpe_rk4(10)
        field, *_ = vk.read_wf(str(tmp_path / "data/wf/wf1p1.dat"), n, n)
        assert np.array_equal(field, s.get_psi())
