"""Host-side logic of the Python mirror (CPU only): grid builders, manifold
promotion, N-D stride flattening and the argument errors regrid! raises before
any device work (src/regridder/regrid.jl:242-245, :289-296)."""
from __future__ import annotations

import numpy as np
import pytest

from crg import grids
from crg.regridder import (ArgumentError, DimensionMismatch, Regridder, _flat_field_stride, as_grid, promote,
                           regrid_)


def test_lonlat_ring_and_index_order():
    g = grids.lonlat_regular(90.0, 90.0)
    t, nv = g.cell_table()
    assert t.shape == (8, 4, 3) and (nv == 4).all()
    # cell (i, j) = i + j*nx, ring p(i,j), p(i+1,j), p(i+1,j+1), p(i,j+1)
    p = g.blocks[0]
    assert np.array_equal(t[1 + 1 * 4], [p[1, 1], p[1, 2], p[2, 2], p[2, 1]])
    # degree-exact poles coincide
    assert np.array_equal(p[-1, 0], [0.0, 0.0, 1.0]) and np.array_equal(p[-1, 3], p[-1, 0])


def test_cubed_sphere_faces_ccw_and_offsets():
    g = grids.cubed_sphere(4)
    assert g.ncells == 6 * 16 and len(g.blocks) == 6
    t, _ = g.cell_table()
    # counter-clockwise seen from outside: (b-a) x (c-a) points outward
    a, b, c = t[:, 0], t[:, 1], t[:, 2]
    assert (np.einsum("ij,ij->i", np.cross(b - a, c - a), a) > 0).all()


def test_jittered_seam_and_poles():
    g = grids.lonlat_jittered(36, 18, 0.2, 7)
    p = g.blocks[0]
    assert np.allclose(p[:, 0], p[:, -1], atol=1e-15)
    assert np.allclose(p[0, :, 2], -1.0) and np.allclose(p[-1, :, 2], 1.0)


def test_polygon_grid_and_promotion():
    sq = [[(0, 0), (1, 0), (1, 1), (0, 1), (0, 0)]]
    tri = [[(0, 0), (1, 0), (0, 1)]]
    g = as_grid(sq + tri)
    assert g.kind == "cells" and list(g.nverts) == [4, 3]
    s = grids.lonlat_regular(30.0, 30.0)
    d, s2 = promote(g, s)
    assert d.manifold == "spherical" and s2 is s
    assert np.allclose(d.cells[0, 1], grids.unit_sphere_from_geographic(1.0, 0.0))


def test_flat_field_stride():
    a = np.zeros((5, 3, 4))  # C order strides (12, 4, 1)
    assert _flat_field_stride(a.shape, (12, 4, 1), 0) == 1
    assert _flat_field_stride(a.shape, (12, 4, 1), 2) == 4
    assert _flat_field_stride(a.shape, (12, 4, 1), 1) is None
    assert _flat_field_stride((7,), (1,), 0) == 0


def _fake_regridder(nd, ns):
    return Regridder(None, None, _view=dict(_h=None, _transposed=False, info={"n_dst": nd, "n_src": ns, "nnz": 0},
                                            _areas=[(np.ones(nd), np.ones(ns))], _temps=[None], _csc=[None],
                                            dst_space=None, src_space=None))


def test_regrid_argument_errors():
    R = _fake_regridder(9, 4)
    with pytest.raises(ArgumentError, match="dims=3 is out of range"):
        regrid_(np.zeros((9, 3)), R, np.zeros((4, 3)), dims=3)
    with pytest.raises(DimensionMismatch, match="ranks must match"):
        regrid_(np.zeros((9, 3, 2)), R, np.zeros((4, 3)))
    with pytest.raises(DimensionMismatch, match="non-spatial axes must match"):
        regrid_(np.zeros((9, 3)), R, np.zeros((4, 2)))
    with pytest.raises(DimensionMismatch):
        regrid_(np.zeros(8), R, np.zeros(4))
    with pytest.raises(ArgumentError, match="same element type"):
        regrid_(np.zeros(9, np.float32), R, np.zeros(4))


def test_transpose_view_swaps_areas_and_temps():
    R = _fake_regridder(9, 4)
    R._h = type("H", (), {"ptr": 0})()
    # transpose() retains through the library; emulate the view bookkeeping only
    view = dict(R.__dict__)
    view["_transposed"] = True  # the area and work-vector properties swap with the flag
    T = Regridder(None, None, _view=view)
    assert T.shape == (4, 9)
    assert T.src_areas is R.dst_areas and T.dst_areas is R.src_areas
    assert T.src_temp is R.dst_temp and T.dst_temp is R.src_temp


def test_esmf_file_round_trip(tmp_path):
    """ESMF weight-file layout of save_esmf_weights (the reference's NCDatasets
    extension): dimensions, variables, 1-based indices, global attributes."""
    from scipy.io import netcdf_file

    from crg.esmf import load_esmf_weights, write_esmf_file

    w = {"S": np.array([0.5, 0.5, 1.0]), "row": np.array([1, 2, 2]), "col": np.array([1, 1, 2]),
         "frac_a": np.ones(2), "frac_b": np.ones(2), "area_a": np.array([2.0, 1.0]), "area_b": np.array([1.0, 2.0])}
    path = write_esmf_file(tmp_path / "w.nc", w, "src", "dst", src_shape=(2, 1), dst_shape=(1, 2))
    f = load_esmf_weights(path)
    assert np.array_equal(f["matrix"].toarray(), [[0.5, 0.0], [0.5, 1.0]])
    for k in w:
        assert np.array_equal(f[k], w[k])
    with netcdf_file(path, "r", mmap=False) as ds:
        assert set(ds.dimensions) == {"n_s", "n_a", "n_b"}
        assert ds.normalization == b"destarea" and ds.source_grid == b"src"
        assert list(ds.destination_grid_shape) == [1, 2]


def test_convex_cells():
    """The convexity check the jittered workloads rely on (the spherical clip
    needs convex destination cells): regular, HEALPix and the C4 jittered
    C96 grid are convex; pole cells with a repeated corner count as convex; a
    dart (a concave quadrilateral) does not, in either orientation."""
    assert grids.convex_cells(grids.lonlat_regular(5.0, 5.0)).all()
    assert grids.convex_cells(grids.healpix_grid(8)).all()
    assert grids.convex_cells(grids.cubed_sphere(96, jitter=0.15, seed=11)).all()
    assert grids.convex_cells(grids.lonlat_jittered(90, 45, 0.2, seed=4)).all()
    dart = [(0.0, 0.0), (2.0, 1.0), (0.0, 2.0), (0.7, 1.0)]
    g = grids.polygon_grid([dart, dart[::-1], [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0)]])
    assert grids.convex_cells(g).tolist() == [False, False, True]
    sph = grids.polygon_grid([grids.unit_sphere_from_geographic(np.array([x for x, _ in dart]),
                                                                np.array([y for _, y in dart]))],
                             grids.SPHERICAL)
    assert not grids.convex_cells(sph)[0]
