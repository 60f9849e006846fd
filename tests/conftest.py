import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libvk kernels)")
    # Build the product library and the oracle once per session if missing.
    from quantumvortices_gb300 import _build
    lib = _build.LIB
    if not os.path.exists(lib):
        _build.build()
    from oracle import oracle
    if not os.path.exists(oracle.LIB):
        oracle.build()
