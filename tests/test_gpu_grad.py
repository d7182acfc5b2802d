"""Differentiation of regrid!: the pullback with respect to the source field
(crg_apply_adjoint) and to the destination vertices (crg_area_grad), checked
against central finite differences of

    L(s, V) = sum_i w_i d_i^2,   d = regrid(R(V), s) = (A s) ./ a,

with destination = a C96 equiangular cubed sphere whose face-interior
vertices are jittered by U(-0.15, 0.15) cell widths and source = the
1-degree lon-lat grid, w and s ~ N(0, 1) (seeded), h = 1e-7, at 200 source
values and 200 vertex coordinates (100 face-interior vertices x longitude,
latitude).  The reference has no derivatives, so finite differences of the
GPU build itself (whose areas are pinned against the oracle elsewhere) are
the check, plus two exact invariants: the total area of a tiling of the
sphere does not move with any interior vertex.
"""
from __future__ import annotations

import numpy as np
import pytest

from crg import Regridder, area_grad, grids, lonlat_tangents, regrid_, regrid_pullback, split_points

pytestmark = pytest.mark.gpu

NE = 96
H = 1e-7


def _c4():
    dst = grids.cubed_sphere(NE, jitter=0.15, seed=11)
    src = grids.lonlat_regular(1.0, 1.0)
    return dst, src


def _apply(R, s):
    d = np.zeros(R.shape[0])
    regrid_(d, R, s)
    return d


def _interior_points(rng, n):
    """(block, j, i) of n distinct face-interior vertices."""
    picks = set()
    while len(picks) < n:
        picks.add((int(rng.integers(6)), int(rng.integers(1, NE)), int(rng.integers(1, NE))))
    return sorted(picks)


def _lonlat(p):
    return np.degrees(np.arctan2(p[1], p[0])), np.degrees(np.arcsin(np.clip(p[2], -1.0, 1.0)))


def _moved(dst, b, j, i, lon, lat):
    blocks = [blk.copy() for blk in dst.blocks]
    blocks[b][j, i] = grids.unit_sphere_from_geographic(np.array([lon]), np.array([lat]))[0]
    return grids.Grid("curvilinear", dst.manifold, blocks=blocks, full_sphere=True)


@pytest.fixture(scope="module")
def c4(cuda):
    dst, src = _c4()
    R = Regridder(dst, src, normalize=True)
    rng = np.random.default_rng(2024)
    s = rng.standard_normal(R.shape[1])
    w = rng.standard_normal(R.shape[0])
    d = _apply(R, s)
    s_bar, v_bar = regrid_pullback(R, dst, src, s, 2.0 * w * d)
    return dict(dst=dst, src=src, R=R, s=s, w=w, d=d, s_bar=s_bar, v_bar=v_bar, rng=rng)


def test_source_gradient_matches_central_differences(c4):
    R, s, w, d = c4["R"], c4["s"], c4["w"], c4["d"]
    js = c4["rng"].choice(R.shape[1], size=200, replace=False)
    an = c4["s_bar"][js]
    fd = np.empty(len(js))
    for k, j in enumerate(js):
        sp, sm = s.copy(), s.copy()
        sp[j] += H
        sm[j] -= H
        dp, dm = _apply(R, sp), _apply(R, sm)
        fd[k] = np.sum(w * (dp * dp - dm * dm)) / (2 * H)
    scale = np.max(np.abs(an))
    assert np.all(np.abs(fd - an) <= 1e-6 * scale + 1e-5 * np.abs(an)), np.max(np.abs(fd - an))


def test_vertex_gradient_matches_central_differences(c4):
    dst, src, s, w = c4["dst"], c4["src"], c4["s"], c4["w"]
    per_block = split_points(dst, c4["v_bar"])
    pts = _interior_points(np.random.default_rng(99), 100)
    an, fd = [], []
    for b, j, i in pts:
        p = dst.blocks[b][j, i]
        t_lon, t_lat = lonlat_tangents(p[None, :])
        g = per_block[b][j, i]
        lon, lat = _lonlat(p)
        for t, dl, dphi in ((t_lon[0], H, 0.0), (t_lat[0], 0.0, H)):
            an.append(float(g @ t))
            Rp = Regridder(_moved(dst, b, j, i, lon + dl, lat + dphi), src, normalize=True)
            Rm = Regridder(_moved(dst, b, j, i, lon - dl, lat - dphi), src, normalize=True)
            dp, dm = _apply(Rp, s), _apply(Rm, s)
            fd.append(float(np.sum(w * (dp * dp - dm * dm)) / (2 * H)))
    an, fd = np.array(an), np.array(fd)
    assert len(an) == 200
    scale = np.max(np.abs(an))
    err = np.abs(fd - an)
    assert np.all(err <= 1e-6 * scale + 1e-4 * np.abs(an)), (np.max(err), scale)


def test_total_areas_do_not_move_with_interior_vertices(cuda):
    """d(sum_i a_i)/dV and d(sum_ij A_ij)/dV vanish at face-interior vertices
    (the cells tile the sphere, 4 pi whatever the interior vertices do)."""
    dst, src = grids.cubed_sphere(24, jitter=0.15, seed=3), grids.lonlat_regular(4.0, 4.0)
    R = Regridder(dst, src)
    nd, ns = R.shape
    ga = split_points(dst, area_grad(R, dst, src, area_weight=np.ones(nd)))
    gA = split_points(dst, area_grad(R, dst, src, row_weight=np.ones(nd), src_field=np.ones(ns)))
    for b in range(6):
        inner = dst.blocks[b][1:-1, 1:-1].reshape(-1, 3)
        t_lon, t_lat = lonlat_tangents(inner)
        for g in (ga[b][1:-1, 1:-1].reshape(-1, 3), gA[b][1:-1, 1:-1].reshape(-1, 3)):
            # per-vertex derivatives are ~1e-3 sr/degree; their cancellation leaves rounding only
            assert np.max(np.abs(np.sum(g * t_lon, axis=1))) < 1e-12
            assert np.max(np.abs(np.sum(g * t_lat, axis=1))) < 1e-12


def test_area_grad_on_the_plane(cuda):
    """Planar unit squares: the shared corner (1, 1) of a 2 x 2 grid is the
    third vertex of the lower-left cell and the fourth of the lower-right one;
    the shoelace gradient of a counter-clockwise polygon at vertex k is
    (y[k+1] - y[k-1], x[k-1] - x[k+1]) / 2."""
    dst = grids.regular_grid([0.0, 1.0, 2.0], [0.0, 1.0, 2.0])
    src = grids.regular_grid([0.0, 2.0], [0.0, 2.0])
    R = Regridder(dst, src)
    # cells (i, j) numbered i + 2 j: [0,1]x[0,1], [1,2]x[0,1], [0,1]x[1,2], [1,2]x[1,2]
    g = area_grad(R, dst, src, area_weight=np.array([1.0, 0.0, 0.0, 0.0]))
    pts = dst.points_flat()
    k = int(np.flatnonzero((pts[:, 0] == 1.0) & (pts[:, 1] == 1.0))[0])
    assert np.allclose(g[k], [0.5, 0.5], atol=1e-14)
    # the second cell lies inside the single source cell: A_10 moves like its area
    g2 = area_grad(R, dst, src, row_weight=np.array([0.0, 1.0, 0.0, 0.0]), src_field=np.ones(1))
    assert np.allclose(g2[k], [-0.5, 0.5], atol=1e-14)
    # all four cells together: (1, 1) is interior, the total area does not move
    g4 = area_grad(R, dst, src, area_weight=np.ones(4))
    assert np.allclose(g4[k], [0.0, 0.0], atol=1e-14)
