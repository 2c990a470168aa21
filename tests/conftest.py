"""Test configuration: import paths and the `gpu` marker.

Tests marked ``gpu`` need a CUDA device and the built libkpmgb; everything
else runs on a CPU-only machine.
"""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "kpm.jl_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libkpmgb")


def relerr(a, b) -> float:
    """Norm-wise relative difference, the semantics of Julia's isapprox(rtol)."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = max(np.linalg.norm(a), np.linalg.norm(b))
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


@pytest.fixture(scope="session")
def built_lib():
    """Build libkpmgb.so (nvcc) once per session and return its path."""
    from kpm_gb300 import build
    return build.build()
