"""The oracle's forward-mode (dual-number) area derivatives, pinned on the
CPU: exact shoelace gradients on the plane, and central finite differences
of the oracle's own build on the sphere (curvilinear and polygon grids).
These derivatives are the reference values of the GPU's crg_area_grad
(tests/test_gpu_vertex_grad_oracle.py).  The reference has no derivatives,
and its build does not accept dual numbers (it writes Float64 buffers), so
the oracle stands in for "ForwardDiff through the CPU path"."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from crg import grids, lonlat_tangents

H = 1e-5  # degrees


def _loss(dst, src, u, s, c):
    R = oracle.OracleRegridder(dst, src)
    return float(u @ (R.intersections @ s) + c @ R.dst_areas)


def _lonlat(p):
    return np.degrees(np.arctan2(p[1], p[0])), np.degrees(np.arcsin(np.clip(p[2], -1.0, 1.0)))


def _unit(lon, lat):
    return grids.unit_sphere_from_geographic(np.array([lon]), np.array([lat]))[0]


def test_planar_shoelace_gradients_are_exact():
    dst = grids.regular_grid([0.0, 1.0, 2.0], [0.0, 1.0, 2.0])
    src = grids.regular_grid([0.0, 2.0], [0.0, 2.0])
    R = oracle.OracleRegridder(dst, src)
    pts = dst.points_flat()
    k = int(np.flatnonzero((pts[:, 0] == 1.0) & (pts[:, 1] == 1.0))[0])
    g = oracle.area_grad(R, dst, src, area_weight=np.array([1.0, 0.0, 0.0, 0.0]))
    assert g.shape == (9, 2)
    assert np.array_equal(g[k], [0.5, 0.5])
    g2 = oracle.area_grad(R, dst, src, row_weight=np.array([0.0, 1.0, 0.0, 0.0]), src_field=np.ones(1))
    assert np.array_equal(g2[k], [-0.5, 0.5])
    g4 = oracle.area_grad(R, dst, src, area_weight=np.ones(4))
    assert np.array_equal(g4[k], [0.0, 0.0])


@pytest.fixture(scope="module")
def sphere_case():
    dst = grids.cubed_sphere(4, jitter=0.15, seed=3)
    src = grids.lonlat_jittered(12, 6, 0.2, seed=1)
    rng = np.random.default_rng(5)
    u, s, c = rng.standard_normal(dst.ncells), rng.standard_normal(src.ncells), rng.standard_normal(dst.ncells)
    R = oracle.OracleRegridder(dst, src)
    return dst, src, u, s, c, oracle.area_grad(R, dst, src, u, s, c)


def test_curvilinear_gradient_matches_central_differences(sphere_case):
    dst, src, u, s, c, g = sphere_case
    assert g.shape == (6 * 25, 3)
    rng = np.random.default_rng(9)
    an, fd = [], []
    for _ in range(12):
        b, j, i = int(rng.integers(6)), int(rng.integers(1, 4)), int(rng.integers(1, 4))
        p = dst.blocks[b][j, i]
        lon, lat = _lonlat(p)
        t_lon, t_lat = lonlat_tangents(p[None, :])
        slot = b * 25 + j * 5 + i
        for t, dl, dp in ((t_lon[0], H, 0.0), (t_lat[0], 0.0, H)):
            an.append(float(g[slot] @ t))
            vals = []
            for sgn in (1.0, -1.0):
                blocks = [blk.copy() for blk in dst.blocks]
                blocks[b][j, i] = _unit(lon + sgn * dl, lat + sgn * dp)
                vals.append(_loss(grids.Grid("curvilinear", dst.manifold, blocks=blocks, full_sphere=True), src, u, s, c))
            fd.append((vals[0] - vals[1]) / (2 * H))
    an, fd = np.array(an), np.array(fd)
    scale = np.max(np.abs(an))
    assert scale > 0
    assert np.all(np.abs(an - fd) <= 1e-7 * scale + 1e-6 * np.abs(an)), np.max(np.abs(an - fd)) / scale


def test_shared_corners_accumulate_and_interior_totals_vanish(sphere_case):
    """Summed over the cells that share a face-interior vertex, the total area
    of the tiling does not move (d sum_i a_i / dV = 0 there)."""
    dst, src, *_ = sphere_case
    R = oracle.OracleRegridder(dst, src)
    g = oracle.area_grad(R, dst, src, area_weight=np.ones(dst.ncells))
    for b in range(6):
        inner = dst.blocks[b][1:-1, 1:-1].reshape(-1, 3)
        gi = g[b * 25:(b + 1) * 25].reshape(5, 5, 3)[1:-1, 1:-1].reshape(-1, 3)
        t_lon, t_lat = lonlat_tangents(inner)
        assert np.max(np.abs(np.sum(gi * t_lon, axis=1))) < 1e-14
        assert np.max(np.abs(np.sum(gi * t_lat, axis=1))) < 1e-14


def test_polygon_grid_gradient_matches_central_differences():
    dst = grids.healpix_grid(2)
    src = grids.lonlat_jittered(10, 5, 0.2, seed=4)
    rng = np.random.default_rng(6)
    u, s, c = rng.standard_normal(dst.ncells), rng.standard_normal(src.ncells), rng.standard_normal(dst.ncells)
    g = oracle.area_grad(oracle.OracleRegridder(dst, src), dst, src, u, s, c)
    assert g.shape == dst.cells.shape
    an, fd = [], []
    for _ in range(8):
        cell, k = int(rng.integers(dst.ncells)), int(rng.integers(4))
        p = dst.cells[cell, k]
        lon, lat = _lonlat(p)
        if abs(lat) > 80.0:  # the longitude tangent degenerates at the poles
            continue
        t_lon, t_lat = lonlat_tangents(p[None, :])
        for t, dl, dp in ((t_lon[0], H, 0.0), (t_lat[0], 0.0, H)):
            an.append(float(g[cell, k] @ t))
            vals = []
            for sgn in (1.0, -1.0):
                cells = dst.cells.copy()
                cells[cell, k] = _unit(lon + sgn * dl, lat + sgn * dp)
                moved = grids.Grid("cells", dst.manifold, cells=cells, nverts=dst.nverts, healpix=dst.healpix)
                vals.append(_loss(moved, src, u, s, c))
            fd.append((vals[0] - vals[1]) / (2 * H))
    an, fd = np.array(an), np.array(fd)
    assert len(an) >= 8
    scale = np.max(np.abs(an))
    assert np.all(np.abs(an - fd) <= 1e-7 * scale + 1e-6 * np.abs(an)), np.max(np.abs(an - fd)) / scale
