"""Shared fixtures.  `-m "not gpu"` runs on any machine (oracle, host logic, ABI);
`-m gpu` needs a CUDA device and the in-tree libgammaray_gpu.so."""
from __future__ import annotations

import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "libgammaray_ref.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built CUDA library")


def build_oracle():
    srcs = [os.path.join(ORACLE_DIR, f) for f in os.listdir(ORACLE_DIR) if f.endswith((".hpp", ".cpp"))]
    if not os.path.exists(ORACLE_LIB) or max(os.path.getmtime(s) for s in srcs) > os.path.getmtime(ORACLE_LIB):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return ORACLE_LIB


@pytest.fixture(scope="session")
def oracle():
    from gammaray_gb300 import _abi

    return _abi.Lib(build_oracle())


def _gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    """The CUDA library.  A GPU test must not silently pass without it."""
    if not _gpu_available():
        pytest.skip("no CUDA device")
    import gammaray_gb300

    if not os.path.exists(gammaray_gb300.LIB_PATH):
        from gammaray_gb300 import build

        build.build()
    return gammaray_gb300.load()
