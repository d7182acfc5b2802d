"""ESMF offline weights (the reference's save_esmf_weights,
ext/ConservativeRegriddingNCDatasetsExt.jl): the arrays follow the oracle's
CSC bit for bit, a written file reads back, its matrix applies like
regrid!, and pairs that both cover the sphere have fractions 1 to machine
precision."""
from __future__ import annotations

import numpy as np
import oracle
import pytest
from conftest import c1_grids

from crg import Regridder, esmf_weights, grids, load_esmf_weights, regrid_, save_esmf_weights

pytestmark = pytest.mark.gpu


def test_esmf_weights_match_oracle_and_round_trip(cuda, tmp_path):
    dst, src = c1_grids()
    R = Regridder(dst, src)
    O = oracle.OracleRegridder(dst, src)
    w = esmf_weights(R)
    # CSC order: source column ascending, destination row ascending inside it (findnz)
    col = np.repeat(np.arange(O.ns), np.diff(O.colptr)) + 1
    assert np.array_equal(w["col"], col)
    assert np.array_equal(w["row"], O.rowval + 1)
    assert np.array_equal(w["S"], O.nzval / O.dst_areas[O.rowval])
    assert np.array_equal(w["area_a"], O.src_areas) and np.array_equal(w["area_b"], O.dst_areas)
    A = O.intersections
    assert np.allclose(w["frac_a"], np.asarray(A.sum(axis=0)).ravel() / O.src_areas, rtol=1e-14, atol=0)
    assert np.allclose(w["frac_b"], np.asarray(A.sum(axis=1)).ravel() / O.dst_areas, rtol=1e-14, atol=0)
    # the shifted destination starts at -89.6 degrees: source cells below it are partly uncovered
    assert np.min(w["frac_a"]) < 0.97 and np.max(np.abs(w["frac_b"] - 1.0)) < 1e-12
    # two grids covering the whole sphere: every fraction is 1 to machine precision
    wf = esmf_weights(Regridder(grids.healpix_grid(16), grids.lonlat_regular(4.0, 4.0)))
    assert np.max(np.abs(wf["frac_a"] - 1.0)) < 1e-12 and np.max(np.abs(wf["frac_b"] - 1.0)) < 1e-12

    path = save_esmf_weights(tmp_path / "w.nc", R, src_grid_name="lonlat2", dst_grid_name="lonlat3_shifted",
                             src_shape=(180, 90), dst_shape=(120, 60))
    f = load_esmf_weights(path)
    for k in ("S", "row", "col", "frac_a", "frac_b", "area_a", "area_b"):
        assert np.array_equal(f[k], w[k].astype(f[k].dtype)), k
    s = np.random.default_rng(3).standard_normal(R.shape[1])
    d = np.zeros(R.shape[0])
    regrid_(d, R, s)
    assert np.allclose(f["matrix"] @ s, d, rtol=1e-13, atol=1e-13)
