"""Test configuration: import paths, the `gpu` marker and shared fixtures.

Tests marked `gpu` need a CUDA device and call the product through its C
ABI; everything else runs on CPU (oracle checks, host logic, library load
and export checks).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "flashvector-gpu_gb300", ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the product's kernels)")


def load_golden(name: str):
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def built_lib():
    """Builds libfvgb300.so if needed (nvcc cross-compiles without a GPU)."""
    import build as fv_build  # flashvector-gpu_gb300/build.py

    return fv_build.build()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fvgb300  # noqa: F401
    from fvgb300 import _lib

    _lib.lib()  # the product must load; no fallback
    return torch
