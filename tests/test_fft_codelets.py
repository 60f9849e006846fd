"""The row-FFT arithmetic (quantumvortices_gb300/csrc/vk_fft.cuh) on the host:
the radix-2/4/8/16 codelets with their fused rotation butterflies, the
first butterfly layer with fused table twiddles, and whole Stockham
transforms of 32 to 2048 points (radix-16, -8 and -4 plans; half-length
transforms on the table of the full length) against a direct long-double
DFT.  Bound: 4e-15 of the largest output in FP64 (a few ulp per stage),
2e-6 in FP32.  The GPU runs the same code; the GPU tests check it there
against the oracle."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "quantumvortices_gb300", "csrc")


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path_factory.mktemp("fft") / "fft_codelets_host")
    subprocess.run([cxx, "-std=c++17", "-O1", "-w", "-I", inc, "-I", CSRC, "-o", exe,
                    os.path.join(HERE, "fft_codelets_host.cpp")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    rows = {}
    for line in out.splitlines():
        name, err, mx = line.split()
        rows[name] = (float(err), float(mx))
    return rows


def test_all_cases_ran(results):
    assert len(results) == 27


@pytest.mark.parametrize("kind", ["dft", "tw"])
def test_codelets_match_direct_dft(results, kind):
    for name, (err, mx) in results.items():
        if name.startswith(kind):
            assert err <= 4e-15 * mx, (name, err, mx)


def test_fp64_transforms_match_direct_dft(results):
    for name, (err, mx) in results.items():
        if name.startswith("f64_"):
            assert err <= 4e-15 * mx, (name, err, mx)


def test_fp32_transforms_match_direct_dft(results):
    for name, (err, mx) in results.items():
        if name.startswith("f32_"):
            assert err <= 2e-6 * mx, (name, err, mx)
