"""The intersection matrix is symmetric in its two grids: A(dst, src) equals
A(src, dst) transposed, up to rounding.

A_ij is the area of cell i of one grid intersected with cell j of the other,
the same set whichever grid is clipped against which.  The source-vertex
cotangent relies on it: it is crg_area_grad of the regridder built the other
way round (crg/grad.py src_area_grad).  The two builds clip in opposite roles,
so their entries differ by rounding only: every entry agrees to 1e-14 of the
largest, an entry present in one build only is a rounding-level sliver, and
each grid's cell areas (one routine per cell, whatever its role) are equal bit
for bit."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import c1_grids
from crg import grids

PAIRS = {
    "lonlat2_lonlat3_shifted": c1_grids,
    "healpix8_lonlat10": lambda: (grids.healpix_grid(8), grids.lonlat_regular(10.0, 10.0)),
    "jittered_cs4_lonlat15": lambda: (grids.cubed_sphere(4, jitter=0.2, seed=3), grids.lonlat_regular(15.0, 15.0)),
}


def _entries(A):
    A = A.tocoo()
    return {(int(i), int(j)): float(v) for i, j, v in zip(A.row, A.col, A.data)}


@pytest.mark.parametrize("name", sorted(PAIRS))
def test_swapped_build_is_the_transpose(name):
    dst, src = PAIRS[name]()
    fwd, swp = oracle.OracleRegridder(dst, src), oracle.OracleRegridder(src, dst)
    a, b = _entries(fwd.intersections), _entries(swp.intersections.T)
    top = max(abs(v) for v in a.values())
    both = a.keys() & b.keys()
    assert len(both) >= 0.95 * max(len(a), len(b))  # the rest are slivers, bounded below
    assert max(abs(a[k] - b[k]) for k in both) <= 1e-14 * top
    one = [abs(a.get(k, 0.0) + b.get(k, 0.0)) for k in a.keys() ^ b.keys()]
    assert max(one, default=0.0) <= 1e-15 * top  # slivers of meridian-sharing cells only
    assert np.array_equal(fwd.dst_areas, swp.src_areas) and np.array_equal(fwd.src_areas, swp.dst_areas)
