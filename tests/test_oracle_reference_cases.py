"""More of the reference's own known answers, on the oracle (the GPU build
equals the oracle bit for bit, tests/test_gpu_parity.py):

- test/regridding.jl:9-41: every (dst, src) pair of FlatNoTree polygon lists
  is tried and only positive areas are kept;
- test/usecases/oceananigans.jl:15-28: 1-degree -> 4-degree lon-lat
  upscaling of the cell-centre longitude keeps the plain mean exactly (==),
  and the transpose keeps it to rtol 1e-5;
- test/trees/quadtree_cursors.jl:55-80, :179-205: the dual tree search of a
  lon-lat grid against itself finds every (i, i);
- examples/healpix.jl:33-40: HEALPix nside 64 (ring order) <- 1-degree
  lon-lat conserves the area-weighted integral to rtol 1e-15 (a seeded
  uniform field stands in for the example's analytic field).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from crg import grids


def _square(x0, y0):
    return [(x0, y0), (x0 + 1.0, y0), (x0 + 1.0, y0 + 1.0), (x0, y0 + 1.0), (x0, y0)]


def test_every_flat_pair_is_tried_and_only_positive_areas_kept():
    dst = grids.polygon_grid([_square(0.0, 0.0) for _ in range(2)])
    src = grids.polygon_grid([_square(0.0, 0.0) for _ in range(3)])
    R = oracle.OracleRegridder(dst, src)
    assert R.intersections.shape == (2, 3)
    assert R.nnz == 6 and np.all(R.nzval == 1.0)
    # cells that only share an edge or a corner intersect with area exactly 0: no entry
    touching = grids.polygon_grid([_square(1.0, 0.0), _square(1.0, 1.0), _square(0.0, 1.0)])
    R0 = oracle.OracleRegridder(grids.polygon_grid([_square(0.0, 0.0)]), touching)
    assert R0.nnz == 0


def test_latlong_upscaling_keeps_the_mean():
    fine, coarse = grids.lonlat_regular(1.0, 1.0), grids.lonlat_regular(4.0, 4.0)
    R = oracle.OracleRegridder(coarse, fine)
    x = np.tile(0.5 + np.arange(360.0), 180)  # cell-centre longitude, cell i + 360 j
    d = R.apply(x)
    assert d.mean() == x.mean()
    y = np.random.default_rng(0).random(coarse.ncells)
    s = R.apply(y, transpose=True)
    assert abs(s.mean() - y.mean()) <= 1e-5 * abs(y.mean())


@pytest.mark.parametrize("nx,ny", [(4, 4), (16, 16), (13, 17)])
def test_self_query_finds_every_diagonal_pair(nx, ny):
    g = grids.lonlat_grid(np.linspace(-180.0, 180.0, nx + 1), np.linspace(-90.0, 90.0, ny + 1))
    pairs = set(map(tuple, oracle.candidates(g, g).tolist()))
    assert all((i, i) in pairs for i in range(nx * ny))
    assert len(pairs) >= nx * ny


def test_healpix_integral_is_conserved():
    hp, ll = grids.healpix_grid(64, order="ring"), grids.lonlat_regular(1.0, 1.0)
    R = oracle.OracleRegridder(hp, ll)
    f = np.random.default_rng(1).random(ll.ncells)
    h = R.apply(f)
    rs = np.asarray(R.intersections.sum(axis=1)).ravel()
    cs = np.asarray(R.intersections.sum(axis=0)).ravel()
    assert np.allclose(rs, R.dst_areas, rtol=np.sqrt(np.finfo(float).eps), atol=0)
    assert np.allclose(cs, R.src_areas, rtol=np.sqrt(np.finfo(float).eps), atol=0)
    a, b = np.sum(h * R.dst_areas), np.sum(f * R.src_areas)
    assert abs(a - b) <= 1e-15 * max(abs(a), abs(b))
