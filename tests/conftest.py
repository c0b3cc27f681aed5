"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on
the CPU.  The CUDA library and the oracle are built once per session."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from regcm_gb300 import build
    build.build_all()
    yield


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    if den == 0.0:
        return num
    return num / den
