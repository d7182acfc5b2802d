"""Shared test setup: import paths for the package and the oracle, the `gpu`
marker, and small grid factories."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "conservativeregridding.jl_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda():
    if not gpu_available():
        pytest.skip("no CUDA device")
    import torch

    torch.cuda.init()
    return torch.device("cuda", 0)


def c1_grids():
    """2 deg source, 3 deg destination shifted by +0.7 lon / +0.4 lat, lat edges clamped."""
    from crg import grids

    src = grids.lonlat_regular(2.0, 2.0)
    dst = grids.lonlat_grid(0.7 + 3 * np.arange(121), np.clip(-89.6 + 3 * np.arange(61), -90, 90))
    return dst, src
