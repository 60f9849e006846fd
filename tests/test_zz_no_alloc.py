"""The allocation-free forward 2D FFT (vk_fft2d_forward_noalloc).

It exists for callers that cannot call cudaMalloc, e.g. a Fortran code whose
device arrays belong to an OpenACC / OpenMP-offload runtime: they pass device
pointers and the library uses a built-in device array as scratch.  The test
calls it through the C ABI twice in a row on different inputs and checks each
result against an independent transform, numpy.fft.fft2 transposed to the
Fourier layout kpsi[kx][ky], within the FFT tolerance of the other GPU tests
(1e-13 relative), and against the allocating entry point (vk_set_psi +
vk_get_kpsi).  The shapes include rows of 2048 and 4096 points, whose passes
need more than 48 KB of shared memory.  This file is named to be collected
last.
"""
import ctypes as C

import numpy as np
import pytest

from quantumvortices_gb300 import vk

pytestmark = pytest.mark.gpu

# (nx, ny); the last three reach the built-in limit of 262144 points and need
# the raised shared-memory limit (x rows of 2048 and 4096, y rows of 4096).
SHAPES = [(64, 64), (512, 512), (128, 32), (2048, 128), (4096, 64), (64, 4096)]


def _noalloc_fn():
    lib = vk.load_library()
    f = lib.vk_fft2d_forward_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]
    return f


def _allocating_kpsi(psi):
    ny, nx = psi.shape
    p = vk.params_for(nx, ny, otoc=False)
    with vk.GPESolver(p) as s:
        s.set_psi(psi)
        return s.get_kpsi()


@pytest.mark.parametrize("nx,ny", SHAPES)
def test_noalloc_forward_fft_matches_numpy(nx, ny):
    torch = pytest.importorskip("torch")
    f = _noalloc_fn()
    rng = np.random.default_rng(nx + 3 * ny)
    stream = torch.cuda.current_stream()
    for call in range(2):  # two calls in a row share the built-in scratch
        psi = rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))
        d_in = torch.from_numpy(psi.view(np.float64).copy()).cuda()
        d_out = torch.empty(2 * nx * ny, dtype=torch.float64, device="cuda")
        rc = f(d_in.data_ptr(), d_out.data_ptr(), nx, ny, stream.cuda_stream)
        assert rc == 0, vk.load_library().vk_last_error()
        stream.synchronize()
        got = d_out.cpu().numpy().view(np.complex128).reshape(nx, ny)
        want = np.fft.fft2(psi).T  # kpsi[kx][ky], unnormalised forward (sign -1)
        err = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert err < 1e-13, (call, err)
        if vk.solver_len_class(nx, ny) >= 0:
            alloc = _allocating_kpsi(psi)
            assert np.linalg.norm(got - alloc) / np.linalg.norm(alloc) < 1e-13


def test_noalloc_rejects_sizes_beyond_scratch():
    torch = pytest.importorskip("torch")
    f = _noalloc_fn()
    d = torch.empty(2 * 1024 * 1024, dtype=torch.float64, device="cuda")
    rc = f(d.data_ptr(), d.data_ptr(), 1024, 1024, None)
    assert rc == -1  # VK_E_INVALID
    assert b"exceeds" in vk.load_library().vk_last_error()
    rc = f(d.data_ptr(), d.data_ptr(), 100, 64, None)
    assert rc == -1
