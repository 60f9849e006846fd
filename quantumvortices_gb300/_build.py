"""In-tree build of libvk.so (CUDA for sm_103a + host C++).

Each translation unit compiles in its own process (in parallel); objects go
to quantumvortices_gb300/_build/, the library to quantumvortices_gb300/libvk.so.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libvk.so")
DRIVER = os.path.join(PKG, "vikshobha_gb300")

# (source, object tag, extra flags).  The solver is compiled once per precision
# and row-length class, the ensemble once per precision: the compilations run
# in parallel, and no single one dominates the build.
CU_UNITS = ([("vk_solver_tu.cu", f"f{32 if fp32 else 64}.c{c}", [f"-DVK_TU_FP32={fp32}", f"-DVK_TU_CLASS={c}"])
             for fp32 in (0, 1) for c in range(5)]
            + [("vk_ens.cu", f"f{32 if fp32 else 64}", [f"-DVK_ENS_FP32={fp32}"]) for fp32 in (0, 1)]
            + [(s, "", []) for s in ("vk_common.cu", "vk_noalloc.cu", "vk_nn.cu", "vk_sts.cu")])
CPP_SRCS = ["vk_api.cpp", "vk_host.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp",
                     "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-fno-fast-math"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(PKG, "..", "include", "vk.h"))
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile every source that changed and link libvk.so; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    cxx = os.environ.get("CXX", "g++")
    cmds, objs = [], []
    for s, tag, extra in CU_UNITS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT_DIR, s + (f".{tag}" if tag else "") + ".o")
        objs.append(obj)
        if _stale(obj, src):
            cmds.append([nvcc, *NVCC_FLAGS, *extra, "-c", src, "-o", obj])
    for s in CPP_SRCS:
        src, obj = os.path.join(CSRC, s), os.path.join(OUT_DIR, s + ".o")
        objs.append(obj)
        if _stale(obj, src):
            cmds.append([cxx, *CXX_FLAGS, "-c", src, "-o", obj])
    if cmds:
        # longest compilations first
        cmds.sort(key=lambda c: (0 if "vk_solver_tu.cu" in " ".join(c) else 1))
        with ThreadPoolExecutor(max_workers=jobs or min(os.cpu_count() or 8, len(cmds))) as ex:
            list(ex.map(_run, cmds))
    if cmds or not os.path.exists(LIB):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"])
    drv_src = os.path.join(CSRC, "vk_driver.cpp")
    if not os.path.exists(DRIVER) or os.path.getmtime(DRIVER) < max(os.path.getmtime(drv_src), os.path.getmtime(LIB)):
        _run([cxx, "-O2", "-std=c++17", "-pthread", "-o", DRIVER, drv_src, "-L" + PKG, "-lvk", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
