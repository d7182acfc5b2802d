"""The GPU area gradient (crg_area_grad, and src_area_grad through the
swapped build) against the oracle's forward-mode derivatives of its own clip
and area (oracle.area_grad, pinned by finite differences in
tests/test_oracle_grad.py).  Both run the same value sequence, so they agree
to rounding: the GPU adds the shared-corner contributions with atomics in no
fixed order, so the bound is relative to the largest entry, not bit for bit.
Curvilinear and polygon (HEALPix) destinations on the sphere, and the plane."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from crg import Regridder, area_grad, grids, src_area_grad

pytestmark = pytest.mark.gpu

CASES = {
    "cs12_from_lonlat_jittered": lambda: (grids.cubed_sphere(12, jitter=0.15, seed=7),
                                          grids.lonlat_jittered(36, 18, 0.2, seed=2)),
    "healpix8_from_lonlat_jittered": lambda: (grids.healpix_grid(8), grids.lonlat_jittered(60, 30, 0.2, seed=3)),
    "lonlat_jittered_from_cs8": lambda: (grids.lonlat_jittered(30, 15, 0.2, seed=5),
                                         grids.cubed_sphere(8, jitter=0.1, seed=1)),
    "planar": lambda: (grids.regular_grid(np.linspace(0.0, 3.0, 7), np.linspace(0.0, 2.0, 5)),
                       grids.regular_grid(np.linspace(-0.3, 3.2, 5), np.linspace(-0.15, 2.35, 4))),
}


def _close(got, want):
    assert got.shape == want.shape
    scale = np.max(np.abs(want))
    assert scale > 0
    err = np.max(np.abs(got - want))
    assert err <= 1e-12 * scale, (err, scale)


@pytest.mark.parametrize("name", sorted(CASES))
def test_destination_vertex_gradient_matches_oracle_duals(cuda, name):
    dst, src = CASES[name]()
    rng = np.random.default_rng(17)
    u, s, c = rng.standard_normal(dst.ncells), rng.standard_normal(src.ncells), rng.standard_normal(dst.ncells)
    R = Regridder(dst, src)
    want = oracle.area_grad(oracle.OracleRegridder(dst, src), dst, src, u, s, c)
    _close(area_grad(R, dst, src, row_weight=u, src_field=s, area_weight=c), want)
    # the two terms alone
    _close(area_grad(R, dst, src, area_weight=c), oracle.area_grad(oracle.OracleRegridder(dst, src), dst, src,
                                                                    area_weight=c))


@pytest.mark.parametrize("name", sorted(CASES))
def test_source_vertex_gradient_matches_oracle_duals(cuda, name):
    dst, src = CASES[name]()
    rng = np.random.default_rng(23)
    u, s = rng.standard_normal(dst.ncells), rng.standard_normal(src.ncells)
    want = oracle.area_grad(oracle.OracleRegridder(src, dst), src, dst, row_weight=s, src_field=u)
    _close(src_area_grad(dst, src, u, s), want)
