"""Synthetic grids of the five measured configurations, seeded, so that the
benchmark and the parity tests build exactly the same inputs.

- small FP64:     2-degree lon-lat -> 3-degree lon-lat shifted by (+0.7, +0.4)
                  degrees, latitude edges clamped to the poles (7,200 <- 16,200 cells)
- precision:      C48 equiangular cubed sphere -> 1-degree lon-lat (64,800 <- 13,824)
- batches:        32 (dst, src) pairs of jittered global lon-lat grids, resolution
                  exp(U[ln 0.4, ln 4]) degrees per side, vertices moved by
                  U(-0.2, 0.2) cell widths (re-drawn until every cell is convex),
                  K = round(exp(U[0, ln 512])) fields per pair
- derivatives:    jittered C96 cubed sphere (+-0.15 cell widths, seed 11) <- 1-degree lon-lat
- large:          HEALPix nside 256 nested (786,432 pixels) <-> 0.25-degree lon-lat (1,036,800)
"""
from __future__ import annotations

import numpy as np

from . import grids


def small_fp64():
    """(dst, src) of the small FP64 case."""
    src = grids.lonlat_regular(2.0, 2.0)
    dst = grids.lonlat_grid(0.7 + 3 * np.arange(121), np.clip(-89.6 + 3 * np.arange(61), -90, 90))
    return dst, src


def precision():
    """(dst, src) of the precision case: C48 -> 1 degree."""
    return grids.lonlat_regular(1.0, 1.0), grids.cubed_sphere(48)


def jittered_lonlat(rng, res_deg: float, jitter: float = 0.2):
    """A global lon-lat grid of about `res_deg` degrees with its vertices moved
    by U(-jitter, jitter) cell widths, drawn again until every cell is convex."""
    nx, ny = int(round(360.0 / res_deg)), int(round(180.0 / res_deg))
    while True:
        g = grids.lonlat_jittered(nx, ny, jitter, int(rng.integers(1 << 31)))
        if grids.convex_cells(g).all():
            return g


def batch_pairs(seed: int = 20250, npairs: int = 32):
    """The batched case: `npairs` (dst, src) pairs and the field count of each."""
    rng = np.random.default_rng(seed)
    pairs, ks = [], []
    for _ in range(npairs):
        r = np.exp(rng.uniform(np.log(0.4), np.log(4.0), size=2))
        pairs.append((jittered_lonlat(rng, r[0]), jittered_lonlat(rng, r[1])))
        ks.append(int(round(np.exp(rng.uniform(0.0, np.log(512.0))))))
    return pairs, ks


def derivatives():
    """(dst, src) of the differentiation case: jittered C96 <- 1 degree."""
    return grids.cubed_sphere(96, jitter=0.15, seed=11), grids.lonlat_regular(1.0, 1.0)


def large(nside: int = 256, dlon: float = 0.25):
    """(HEALPix, lon-lat) of the large case; R = Regridder(HEALPix, lon-lat)."""
    return grids.healpix_grid(nside, "nested"), grids.lonlat_regular(dlon, dlon)


def cell_centres(g) -> np.ndarray:
    """Normalised sum of each cell's first four corners (unit vectors, (n, 3))."""
    t, _ = g.cell_table()
    c = t[:, :4].sum(axis=1)
    return c / np.linalg.norm(c, axis=1, keepdims=True)


def harmonic_fields(centres, nfields: int, lmax: int, seed: int, noise: float, device):
    """`nfields` fields sum_{l <= lmax, m} c_lm Ybar_lm + N(0, noise) at the unit
    vectors `centres`, c_lm ~ N(0, 1) / (lmax + 1): fully normalised real
    spherical harmonics by the standard three-term recurrence in the associated
    Legendre functions, evaluated with torch on `device` in FP64.  Returns a
    (nfields, n) FP32 tensor."""
    import torch

    gen = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.as_tensor(centres, dtype=torch.float64, device=device)
    z = x[:, 2].clamp(-1, 1)
    s = torch.sqrt((1 - z) * (1 + z))
    lon = torch.atan2(x[:, 1], x[:, 0])
    n = x.shape[0]
    out = torch.zeros((n, nfields), dtype=torch.float64, device=device)
    scale = 1.0 / (lmax + 1)
    pmm = torch.ones(n, dtype=torch.float64, device=device)
    for m in range(lmax + 1):
        if m > 0:
            pmm = pmm * s * np.sqrt((2 * m + 1) / (2 * m))
        L = lmax - m + 1
        P = torch.empty((n, L), dtype=torch.float64, device=device)
        P[:, 0] = pmm
        if L > 1:
            P[:, 1] = np.sqrt(2 * m + 3) * z * pmm
        for l in range(m + 2, lmax + 1):
            a = np.sqrt((4 * l * l - 1) / (l * l - m * m))
            b = np.sqrt(((l - 1) ** 2 - m * m) / (4 * (l - 1) ** 2 - 1))
            P[:, l - m] = a * (z * P[:, l - m - 1] - b * P[:, l - m - 2])
        ca = torch.randn((L, nfields), generator=gen, dtype=torch.float64).to(device) * scale
        out += (P @ ca) * torch.cos(m * lon)[:, None]
        if m > 0:
            cb = torch.randn((L, nfields), generator=gen, dtype=torch.float64).to(device) * scale
            out += (P @ cb) * torch.sin(m * lon)[:, None]
    out += noise * torch.randn((n, nfields), generator=gen, dtype=torch.float64).to(device)
    return out.T.contiguous().float()
