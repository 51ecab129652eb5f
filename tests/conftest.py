"""Test configuration: the `gpu` marker and shared fixtures.

`-m "not gpu"` runs the oracle against the reference's golden outputs, the
host logic and the C-ABI load/export checks (no GPU needed); `-m gpu` runs
the parity tests, which call the CUDA library through its C ABI and compare
with the oracle on the same seeded inputs.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libtracer_gpu.so")


def _gpu_present() -> bool:
    try:
        import ctypes
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                rt = ctypes.CDLL(name)
                break
            except OSError:
                rt = None
        if rt is None:
            import torch
            return torch.cuda.is_available()
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree if needed; a GPU run fails loudly
    when it cannot be built or loaded (no fallback)."""
    if not _gpu_present():
        pytest.skip("no CUDA device visible")
    from tracer_code_gb300 import build, load_library
    build.build()
    return load_library()


@pytest.fixture(scope="session")
def golden():
    import json
    import numpy as np
    d = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(d, "golden.json")) as f:
        g = json.load(f)
    z = np.load(os.path.join(d, "trestart_200.npz"))
    g["T"] = z["T"]
    g["SF"] = z["SF"]
    g["zg"] = z["zg"]
    g["xg"] = z["xg"]
    return g
