"""The ESMF weight file against the reference's own test of its writer
(test/extensions/ncdatasets.jl): schema, values and optional attributes, on
the same two planar grids that tile [0, 2] x [0, 2] (2 x 2 unit squares; a
diamond and four corner triangles -- the README example).

The weight arrays are formed from the oracle's matrix as the reference's
save_esmf_weights forms them (ext/ConservativeRegriddingNCDatasetsExt.jl:
27-33): findnz order, S = A_ij / dst_area_i, frac_a = column sums / source
areas, frac_b = row sums / destination areas.  The GPU's crg_get_esmf_weights
is compared with the oracle in tests/test_gpu_esmf.py; this file checks the
file the writer makes from such arrays."""
from __future__ import annotations

import json

import numpy as np
import scipy.sparse as sp
from scipy.io import netcdf_file

import oracle
from conftest import GOLDEN
from crg import grids
from crg.esmf import load_esmf_weights, write_esmf_file


def _reference_arrays():
    g = json.loads((GOLDEN / "readme_planar.json").read_text())["readme"]
    O = oracle.OracleRegridder(grids.polygon_grid(g["dst"]), grids.polygon_grid(g["src"]), normalize=False)
    A = O.intersections.tocsc()
    A.sort_indices()
    coo = A.tocoo()  # CSC order: by column, rows ascending (findnz)
    order = np.lexsort((coo.row, coo.col))
    row, col, vals = coo.row[order] + 1, coo.col[order] + 1, coo.data[order]
    w = {"S": vals / O.dst_areas[row - 1], "row": row.astype(np.int64), "col": col.astype(np.int64),
         "frac_a": np.asarray(A.sum(axis=0)).ravel() / O.src_areas,
         "frac_b": np.asarray(A.sum(axis=1)).ravel() / O.dst_areas,
         "area_a": O.src_areas.copy(), "area_b": O.dst_areas.copy()}
    return O, A, w


def test_schema(tmp_path):
    O, A, w = _reference_arrays()
    path = write_esmf_file(tmp_path / "w.nc", w)
    with netcdf_file(path, "r", mmap=False) as ds:
        assert ds.dimensions == {"n_s": A.nnz, "n_a": len(O.src_areas), "n_b": len(O.dst_areas)}
        sizes = {"S": A.nnz, "row": A.nnz, "col": A.nnz, "frac_a": len(O.src_areas), "frac_b": len(O.dst_areas),
                 "area_a": len(O.src_areas), "area_b": len(O.dst_areas)}
        for v, n in sizes.items():
            assert ds.variables[v].shape == (n,)
        assert ds.normalization == b"destarea"
        assert ds.source_grid == b"source" and ds.destination_grid == b"destination"
        for absent in ("created_at", "source_grid_shape", "destination_grid_shape"):
            assert not hasattr(ds, absent)


def test_values(tmp_path):
    O, A, w = _reference_arrays()
    f = load_esmf_weights(write_esmf_file(tmp_path / "w.nc", w))
    assert np.allclose(f["area_a"], O.src_areas) and np.allclose(f["area_b"], O.dst_areas)
    rebuilt = sp.csr_matrix((f["S"] * O.dst_areas[f["row"] - 1], (f["row"] - 1, f["col"] - 1)), shape=A.shape)
    assert np.allclose(rebuilt.toarray(), A.toarray())
    assert np.allclose(f["frac_a"], np.asarray(A.sum(axis=0)).ravel() / O.src_areas)
    assert np.allclose(f["frac_b"], np.asarray(A.sum(axis=1)).ravel() / O.dst_areas)
    # both grids tile [0, 2] x [0, 2]: full coverage
    assert np.allclose(f["frac_a"], 1.0, rtol=0, atol=1e-12) and np.allclose(f["frac_b"], 1.0, rtol=0, atol=1e-12)


def test_optional_attributes(tmp_path):
    _, _, w = _reference_arrays()
    path = write_esmf_file(tmp_path / "w.nc", w, src_grid_name="era5_0.25deg", dst_grid_name="c90",
                           src_shape=(720, 361), dst_shape=(90, 90, 6), created_at="2026-04-21T00:00:00")
    with netcdf_file(path, "r", mmap=False) as ds:
        assert ds.source_grid == b"era5_0.25deg" and ds.destination_grid == b"c90"
        assert ds.created_at == b"2026-04-21T00:00:00"
        assert list(ds.source_grid_shape) == [720, 361]
        assert list(ds.destination_grid_shape) == [90, 90, 6]
