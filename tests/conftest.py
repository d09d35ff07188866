import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "gpu-physics-engine_gb300"))
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def gpe_mod():
    """The engine binding; builds libgpe.so when it is missing (nvcc cross-compiles without a GPU)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("gpe_build", ROOT / "gpu-physics-engine_gb300" / "build.py")
    build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(build)
    build.build()
    import gpe

    return gpe


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle

    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def cuda_ok():
    import ctypes

    try:
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        import glob

        cands = glob.glob("/usr/local/cuda/lib64/libcudart.so*")
        if not cands:
            pytest.fail("libcudart not found")
        rt = ctypes.CDLL(cands[0])
    n = ctypes.c_int(0)
    rc = rt.cudaGetDeviceCount(ctypes.byref(n))
    if rc != 0 or n.value == 0:
        pytest.fail("no CUDA device visible (GPU tests must run on a GPU)")
    return True
