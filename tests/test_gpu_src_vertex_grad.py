"""Derivatives of regrid! with respect to the SOURCE grid's vertices
(src_area_grad: crg_area_grad of the regridder built the other way round),
checked against central finite differences of

    L(s, W) = sum_i w_i d_i^2,   d = regrid(R(W), s) = (A s) ./ a,

with destination = a C96 equiangular cubed sphere whose face-interior
vertices are jittered by U(-0.15, 0.15) cell widths and source = the
1-degree lon-lat grid (W its vertices), w and s ~ N(0, 1) (seeded),
h = 1e-7 degrees, at 100 coordinates (50 interior lon-lat vertices x
longitude, latitude); plus the exact shoelace gradient on the plane.  The
reference has no derivatives; the finite differences are of the GPU build,
whose areas match the oracle bit for bit elsewhere.
"""
from __future__ import annotations

import numpy as np
import pytest

from crg import Regridder, grids, lonlat_tangents, regrid_, regrid_pullback, split_points, src_area_grad

pytestmark = pytest.mark.gpu

NE = 96
H = 1e-7


def _apply(R, s):
    d = np.zeros(R.shape[0])
    regrid_(d, R, s)
    return d


def _lonlat(p):
    return np.degrees(np.arctan2(p[1], p[0])), np.degrees(np.arcsin(np.clip(p[2], -1.0, 1.0)))


def _moved(g, b, j, i, lon, lat):
    blocks = [blk.copy() for blk in g.blocks]
    blocks[b][j, i] = grids.unit_sphere_from_geographic(np.array([lon]), np.array([lat]))[0]
    return grids.Grid("curvilinear", g.manifold, blocks=blocks, full_sphere=g.full_sphere)


def _interior_lonlat_vertices(rng, n):
    """(j, i) of n distinct interior vertices of the 1-degree grid, none on a
    meridian at a multiple of 45 degrees (the cubed sphere's unjittered face
    edges lie on the meridians at 45 + 90 k degrees; a source edge on one of
    them makes the areas kinked there, where central differences average the
    two one-sided derivatives)."""
    picks = set()
    while len(picks) < n:
        j, i = int(rng.integers(1, 180)), int(rng.integers(1, 360))
        if i % 45:
            picks.add((j, i))
    return sorted(picks)


def test_source_vertex_gradient_matches_central_differences(cuda):
    dst = grids.cubed_sphere(NE, jitter=0.15, seed=11)
    src = grids.lonlat_regular(1.0, 1.0)
    R = Regridder(dst, src, normalize=True)
    rng = np.random.default_rng(2025)
    s = rng.standard_normal(R.shape[1])
    w = rng.standard_normal(R.shape[0])
    d = _apply(R, s)
    _, _, w_bar = regrid_pullback(R, dst, src, s, 2.0 * w * d, wrt_src=True)
    assert w_bar.shape == (len(src.points_flat()), 3)
    g_blk = split_points(src, w_bar)[0]
    an, fd = [], []
    for j, i in _interior_lonlat_vertices(np.random.default_rng(7), 50):
        p = src.blocks[0][j, i]
        t_lon, t_lat = lonlat_tangents(p[None, :])
        lon, lat = _lonlat(p)
        for t, dl, dphi in ((t_lon[0], H, 0.0), (t_lat[0], 0.0, H)):
            an.append(float(g_blk[j, i] @ t))
            dp = _apply(Regridder(dst, _moved(src, 0, j, i, lon + dl, lat + dphi), normalize=True), s)
            dm = _apply(Regridder(dst, _moved(src, 0, j, i, lon - dl, lat - dphi), normalize=True), s)
            fd.append(float(np.sum(w * (dp * dp - dm * dm)) / (2 * H)))
    an, fd = np.array(an), np.array(fd)
    assert len(an) == 100
    scale = np.max(np.abs(an))
    assert scale > 0
    err = np.abs(fd - an)
    assert np.all(err <= 1e-6 * scale + 1e-4 * np.abs(an)), (np.max(err), scale)


def test_source_vertex_gradient_reuses_a_swapped_regridder(cuda):
    """Passing Regridder(src, dst) gives the same numbers as building it inside."""
    dst, src = grids.cubed_sphere(12, jitter=0.15, seed=5), grids.lonlat_regular(6.0, 6.0)
    rng = np.random.default_rng(1)
    u, s = rng.standard_normal(dst.ncells), rng.standard_normal(src.ncells)
    a = src_area_grad(dst, src, u, s)
    b = src_area_grad(dst, src, u, s, swapped=Regridder(src, dst))
    assert a.shape == (len(src.points_flat()), 3)
    # shared corners accumulate with atomics: equal to rounding, not bit for bit
    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(a))


def test_source_vertex_gradient_on_the_plane(cuda):
    """One destination square [0,2]^2 over four unit source squares: A_0k is
    the area of source cell k, so d A_00 / dW at the shared corner (1, 1)
    (the third vertex of the ring of cell 0 = [0,1]^2, counter-clockwise) is the
    shoelace gradient (y[k+1] - y[k-1], x[k-1] - x[k+1]) / 2 = (0.5, 0.5);
    summed over the four cells it vanishes (an interior vertex of a tiling
    that lies inside the destination cell)."""
    dst = grids.regular_grid([0.0, 2.0], [0.0, 2.0])
    src = grids.regular_grid([0.0, 1.0, 2.0], [0.0, 1.0, 2.0])
    pts = src.points_flat()
    k = int(np.flatnonzero((pts[:, 0] == 1.0) & (pts[:, 1] == 1.0))[0])
    g = src_area_grad(dst, src, np.ones(1), np.array([1.0, 0.0, 0.0, 0.0]))
    assert g.shape == (9, 2)
    assert np.allclose(g[k], [0.5, 0.5], atol=1e-14)
    g4 = src_area_grad(dst, src, np.ones(1), np.ones(4))
    assert np.allclose(g4[k], [0.0, 0.0], atol=1e-14)
