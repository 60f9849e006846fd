"""The FP64 pass bodies of quantumvortices_gb300/csrc/vk_kernels.cuh, built on the
host with a one-thread geometry (tests/kernel_bodies_host.cpp), against numpy
restatements of each pass:

  x1  Ta[y][kx] (|kx| <= K kept) -> psi = F^-1_x Ta / N^2, Tb[kx][y] = F_x |psi|^2, kx <= K
  x2  Tc[y][kx <= K] (Hermitian half) -> p = F^-1_x Tc / N^2, Td[kx][y] = F_x (SIGN g p psi)
  y1  Tb[kx][y] -> F_y, 2/3 disk mask, F^-1_y -> Tc[y][kx]
  y2  Td rows |kx| <= K -> F_y -> RK4 right-hand side and stage update (src/gpe.f90:366-489,
      609-669) -> kpsi, str1, str2, Ta[y][kx] = F^-1_y kpsi
  y2a all rows of Td -> F_y -> the ARGLE update (src/gpe.f90:181-222)
      kpsi <- (kpsi + dt (N^ + Omega kpsi)) / (1 + alpha k^2 dt), Ta = F^-1_y kpsi, and the
      per-row sums |new - old|^2, |old|^2, |new|^2 of the residual
  x2p the RK4 x2 pass with a potential: Td = F_x ((g p + V) psi)

The x passes run both layouts the GPU uses: row pairs (two real rows per
complex transform) and single rows (a half-length complex transform).
Bound: 1e-12 of the largest output (FP64 rounding of a few transforms)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "quantumvortices_gb300", "csrc")
ALPHA, G, OMEGA, DT, PREFAC = 0.0123, 15.5, 15.5, 1e-3, complex(-0.1, -1.0)


def k2max_of(n):
    ka2 = (n / 3.0) ** 2
    k = int(np.floor(ka2)) + 1
    while k > 0 and k >= ka2:
        k -= 1
    return k


def consts(n):
    k2 = k2max_of(n)
    K = int(np.sqrt(k2))
    while (K + 1) ** 2 <= k2:
        K += 1
    while K * K > k2:
        K -= 1
    return k2, K, (K + 2) & ~1


def kwn(n):
    i = np.arange(n)
    return np.where(i < n // 2, i, i - n)


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    cxx = shutil.which("g++")
    inc = next((os.path.join(d, "include") for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda")
                if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h"))), None)
    if not cxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    out = str(tmp_path_factory.mktemp("kb") / "kernel_bodies_host")
    subprocess.run([cxx, "-std=c++17", "-O1", "-w", "-fpermissive", "-I", inc, "-I", CSRC, "-o", out,
                    os.path.join(HERE, "kernel_bodies_host.cpp")], check=True)
    return out


def run(exe, d, *args):
    subprocess.run([exe, *map(str, args), str(d)], check=True, timeout=300)


def put(d, name, a):
    np.ascontiguousarray(a, dtype=np.complex128).tofile(os.path.join(d, name))


def get(d, name, shape):
    return np.fromfile(os.path.join(d, name), dtype=np.complex128).reshape(shape)


def close(a, b, tol=1e-12):
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300)


def rand(rng, shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


@pytest.mark.parametrize("L,ny", [(128, 64), (256, 32), (1024, 16)])
@pytest.mark.parametrize("layout", ["pair", "single"])
def test_x1(exe, tmp_path, L, ny, layout):
    _, K, _ = consts(L)
    rng = np.random.default_rng(L + ny)
    Ta = rand(rng, (ny, L))
    put(tmp_path, "Ta.bin", Ta)
    run(exe, tmp_path, "x1", L, ny, layout)
    kept = np.abs(kwn(L)) <= K
    psi = np.fft.ifft(np.where(kept, Ta, 0), axis=1) * L / (L * ny)
    tb = np.fft.fft(np.abs(psi) ** 2, axis=1)[:, :K + 1].T
    assert close(get(tmp_path, "psi.bin", (ny, L)), psi)
    assert close(get(tmp_path, "Tb.bin", (K + 1, ny)), tb)


@pytest.mark.parametrize("L,ny", [(128, 64), (1024, 16)])
@pytest.mark.parametrize("layout", ["pair", "single"])
@pytest.mark.parametrize("sign", [1, -1])
def test_x2(exe, tmp_path, L, ny, layout, sign):
    _, K, pk = consts(L)
    rng = np.random.default_rng(3 * L + ny + sign)
    Tc = np.zeros((ny, pk), complex)
    Tc[:, :K + 1] = rand(rng, (ny, K + 1))
    Tc[:, 0] = Tc[:, 0].real  # the kx = 0 column of a real row's spectrum is real
    psi = rand(rng, (ny, L))
    put(tmp_path, "Tc.bin", Tc)
    put(tmp_path, "psi.bin", psi)
    run(exe, tmp_path, "x2", L, ny, layout, sign)
    full = np.zeros((ny, L), complex)
    full[:, :K + 1] = Tc[:, :K + 1]
    full[:, L - K:] = np.conj(Tc[:, 1:K + 1][:, ::-1])
    p = np.fft.ifft(full, axis=1).real * L / (L * ny)
    td = np.fft.fft(sign * G * p * psi, axis=1).T
    got = get(tmp_path, "Td.bin", (L, ny))
    rows = np.abs(kwn(L)) <= K if sign > 0 else np.ones(L, bool)  # RK4 keeps |kx| <= K only
    assert close(got[rows], td[rows])


@pytest.mark.parametrize("L", [128, 256])
def test_y1(exe, tmp_path, L):
    k2, K, pk = consts(L)
    rng = np.random.default_rng(5 * L)
    Tb = rand(rng, (K + 1, L))
    put(tmp_path, "Tb.bin", Tb)
    run(exe, tmp_path, "y1", L)
    F = np.fft.fft(Tb, axis=1)
    ksq = np.arange(K + 1)[:, None] ** 2 + kwn(L)[None, :] ** 2
    tc = (np.fft.ifft(np.where(ksq <= k2, F, 0), axis=1) * L).T
    assert close(get(tmp_path, "Tc.bin", (L, pk))[:, :K + 1], tc)


@pytest.mark.parametrize("stage", [1, 2, 3, 4])
def test_y2_rk4(exe, tmp_path, stage):
    L = 128
    k2, K, _ = consts(L)
    rng = np.random.default_rng(7 + stage)
    Td, kpsi, s1, s2 = (rand(rng, (L, L)) for _ in range(4))
    for name, a in (("Td.bin", Td), ("kpsi.bin", kpsi), ("str1.bin", s1), ("str2.bin", s2)):
        put(tmp_path, name, a)
    run(exe, tmp_path, "y2", L, stage)
    rows = np.nonzero(np.abs(kwn(L)) <= K)[0]
    k1 = kwn(L)[rows][:, None]
    ksq = k1 ** 2 + kwn(L)[None, :] ** 2
    disk = ksq <= k2
    nh = np.fft.fft(Td[rows], axis=1)
    ps = kpsi[rows]
    rhs = PREFAC * ((ALPHA * ksq - OMEGA) * ps + nh)
    c2 = DT / 6.0 if stage in (1, 4) else DT / 6.0 * 2.0
    c1 = DT if stage == 3 else DT * 0.5
    e1, e2 = s1[rows].copy(), s2[rows].copy()
    if stage == 1:
        e1 = np.where(disk, ps, e1)
        e2 = np.where(disk, c2 * rhs, e2)
        nw = ps + c1 * rhs
    else:
        s2n = s2[rows] + c2 * rhs
        if stage < 4:
            e2 = np.where(disk, s2n, e2)
            nw = s1[rows] + c1 * rhs
        else:
            nw = s1[rows] + s2n
    nw = np.where(disk, nw, 0)
    ta = (np.fft.ifft(nw, axis=1) * L).T
    assert close(get(tmp_path, "kpsi.bin", (L, L))[rows], nw)
    assert close(get(tmp_path, "str1.bin", (L, L))[rows], e1)
    assert close(get(tmp_path, "str2.bin", (L, L))[rows], e2)
    assert close(get(tmp_path, "Ta.bin", (L, L))[:, rows], ta)


def test_y2_argle_with_residual_sums(exe, tmp_path):
    L = 128
    rng = np.random.default_rng(11)
    Td, kpsi = rand(rng, (L, L)), rand(rng, (L, L))
    put(tmp_path, "Td.bin", Td)
    put(tmp_path, "kpsi.bin", kpsi)
    run(exe, tmp_path, "y2a", L)
    ksq = kwn(L)[:, None] ** 2 + kwn(L)[None, :] ** 2
    nh = np.fft.fft(Td, axis=1)
    new = (kpsi + DT * (nh + OMEGA * kpsi)) / (1.0 + ALPHA * ksq * DT)
    assert close(get(tmp_path, "kpsi.bin", (L, L)), new)
    assert close(get(tmp_path, "Ta.bin", (L, L)), (np.fft.ifft(new, axis=1) * L).T)
    part = np.fromfile(os.path.join(tmp_path, "part.bin")).reshape(L, 3)
    ref = np.stack([np.sum(np.abs(new - kpsi) ** 2, axis=1), np.sum(np.abs(kpsi) ** 2, axis=1),
                    np.sum(np.abs(new) ** 2, axis=1)], axis=1)
    assert np.abs(part - ref).max() <= 1e-12 * np.abs(ref).max()


def test_x2_with_potential(exe, tmp_path):
    L, ny = 128, 32
    _, K, pk = consts(L)
    rng = np.random.default_rng(13)
    Tc = np.zeros((ny, pk), complex)
    Tc[:, :K + 1] = rand(rng, (ny, K + 1))
    Tc[:, 0] = Tc[:, 0].real
    psi = rand(rng, (ny, L))
    vpot = rng.random((ny, L))
    put(tmp_path, "Tc.bin", Tc)
    put(tmp_path, "psi.bin", psi)
    vpot.tofile(os.path.join(tmp_path, "vpot.bin"))
    run(exe, tmp_path, "x2p", L, ny)
    full = np.zeros((ny, L), complex)
    full[:, :K + 1] = Tc[:, :K + 1]
    full[:, L - K:] = np.conj(Tc[:, 1:K + 1][:, ::-1])
    p = np.fft.ifft(full, axis=1).real * L / (L * ny)
    td = np.fft.fft((G * p + vpot) * psi, axis=1).T
    rows = np.abs(kwn(L)) <= K
    assert close(get(tmp_path, "Td.bin", (L, ny))[rows], td[rows])
