"""Shared pytest configuration.

Tests marked ``gpu`` need a CUDA device and the built native library; the
rest run on a CPU-only machine (oracle vs golden vectors, host logic, the
C ABI's argument checking and exported symbols).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built native library")


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def native():
    """The native library, built in-tree if stale (no CPU fallback)."""
    from masterthesis_gb300 import build
    build.build_library()
    import masterthesis_gb300 as M
    M.lib()
    return M


@pytest.fixture(scope="session")
def gpu(native):
    import ctypes
    cudart = None
    for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
        try:
            cudart = ctypes.CDLL(name)
            break
        except OSError:
            continue
    n = ctypes.c_int(0)
    if cudart is None or cudart.cudaGetDeviceCount(ctypes.byref(n)) != 0 or n.value < 1:
        pytest.fail("no CUDA device visible: gpu tests need a GPU")
    return native
