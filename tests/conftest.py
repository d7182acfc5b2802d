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


def cell_centres(g):
    """Normalised mean of each cell's corners (unit vectors)."""
    t, nv = g.cell_table()
    c = np.zeros((t.shape[0], 3))
    for k in range(t.shape[1]):
        c += np.where((k < nv)[:, None], t[:, k], 0.0)
    return c / np.linalg.norm(c, axis=1, keepdims=True)


def sh_fields(centres, nfields, lmax, seed, noise):
    """nfields fields sum_{l <= lmax, m} a_lm Ybar_lm + noise * U[0, 1) at the
    unit vectors `centres`: real spherical harmonics, fully normalised
    associated Legendre functions by the standard three-term recurrence,
    a_lm ~ N(0, 1).  Returns (nfields, n) float64."""
    rng = np.random.default_rng(seed)
    z = np.clip(centres[:, 2], -1.0, 1.0)
    s = np.sqrt((1.0 - z) * (1.0 + z))
    lon = np.arctan2(centres[:, 1], centres[:, 0])
    n = len(z)
    out = np.zeros((nfields, n))
    pmm = np.ones(n)
    for m in range(lmax + 1):
        if m > 0:
            pmm = pmm * s * np.sqrt((2 * m + 1) / (2 * m))
        L = lmax - m + 1
        P = np.empty((L, n))
        P[0] = pmm
        if L > 1:
            P[1] = np.sqrt(2 * m + 3) * z * pmm
        for l in range(m + 2, lmax + 1):
            a = np.sqrt((4 * l * l - 1) / (l * l - m * m))
            b = np.sqrt(((l - 1) ** 2 - m * m) / (4 * (l - 1) ** 2 - 1))
            P[l - m] = a * (z * P[l - m - 1] - b * P[l - m - 2])
        out += (rng.standard_normal((nfields, L)) @ P) * np.cos(m * lon)
        if m > 0:
            out += (rng.standard_normal((nfields, L)) @ P) * np.sin(m * lon)
    return out + noise * rng.uniform(0.0, 1.0, size=(nfields, n))
