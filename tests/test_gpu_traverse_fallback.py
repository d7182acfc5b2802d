"""The dual traversal's fallback.  Its levels run back to back on the device
into buffers of a fixed capacity; when a frontier does not fit, the build
restarts the traversal with a per-level host loop that grows its buffers.
CRG_TRAVERSE_CAPACITY (read at every build) shrinks the capacity so that this
path runs; the matrices must be identical to the ones of the normal path and
to the oracle's (the candidate search only decides which pairs get clipped,
src/regridder/intersection_areas.jl:48-65)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import c1_grids
from crg import Regridder, grids, workloads
from test_gpu_parity import assert_parity

pytestmark = pytest.mark.gpu

PAIRS = {
    "small_fp64": c1_grids,
    "lonlat4_to_healpix16": lambda: (grids.healpix_grid(16), grids.lonlat_regular(4.0, 4.0)),
    "jittered_cs_to_lonlat2": lambda: (grids.cubed_sphere(16, jitter=0.15, seed=5), grids.lonlat_regular(2.0, 2.0)),
    "large": workloads.large,
}


@pytest.mark.parametrize("cap", [1, 1000, 40000])
@pytest.mark.parametrize("name", list(PAIRS))
def test_traversal_fallback_same_matrix(cuda, monkeypatch, name, cap):
    dst, src = PAIRS[name]()
    R0 = Regridder(dst, src, normalize=True)
    monkeypatch.setenv("CRG_TRAVERSE_CAPACITY", str(cap))
    R1 = Regridder(dst, src, normalize=True)
    monkeypatch.delenv("CRG_TRAVERSE_CAPACITY")
    assert R1.info["n_candidates"] == R0.info["n_candidates"]
    for a, b in zip(R0.csc_arrays(), R1.csc_arrays()):
        assert np.array_equal(a, b)
    assert np.array_equal(R0.dst_areas, R1.dst_areas) and np.array_equal(R0.src_areas, R1.src_areas)
    if name != "large" and cap == 1:
        assert_parity(R1, oracle.OracleRegridder(dst, src, normalize=True))
