"""Grid families on the CPU (oracle): folded (tripolar, RightCenterFolded)
grids -- the synthetic fold row has cell i and cell nx+1-i equal; with the
partner slots as ghosts the oracle regrids a constant exactly in both
directions, ghosts get nothing, and the library's host-side fold mirror
fills them -- and RingGrids full grids and reordered cell numberings."""
from __future__ import annotations

import numpy as np
import pytest
import oracle

from crg import grids, mirror_fold_

NX, NY = 16, 10


def test_fold_row_cells_pair_up():
    g = grids.folded_lonlat(NX, NY, 72.0)
    t, _ = g.cell_table()
    row = t[(NY - 1) * NX:]
    for i in range(NX):
        a = {tuple(np.round(p, 15)) for p in row[i]}
        b = {tuple(np.round(p, 15)) for p in row[NX - 1 - i]}
        assert a == b
    gh = grids.fold_ghosts(g)
    ghosts = np.flatnonzero(gh.nverts == 0)
    expect = (NY - 1) * NX + np.setdiff1d(np.arange(NX), grids.fold_primaries(NX) - 1)
    assert np.array_equal(ghosts, expect)


def test_oracle_constant_fields_through_a_fold():
    gh = grids.fold_ghosts(grids.folded_lonlat(NX, NY, 72.0))
    hp = grids.healpix_grid(4)
    O = oracle.OracleRegridder(hp, gh, normalize=True)   # folded source
    ghosts = np.flatnonzero(gh.nverts == 0)
    assert np.all(O.src_areas[ghosts] == 0.0)
    assert np.all(np.diff(O.colptr)[ghosts] == 0)         # ghost columns are empty
    assert abs(O.src_areas.sum() - O.dst_areas.sum()) < 1e-12 * O.dst_areas.sum()
    assert np.allclose(O.apply(np.ones(gh.ncells)), 1.0, atol=1e-10)
    B = oracle.OracleRegridder(gh, hp, normalize=True)   # folded destination
    d = B.apply(np.ones(hp.ncells))
    assert np.all(np.isnan(d[ghosts]))                    # 0 / 0 before the mirror, as in the reference
    mirror_fold_(d, NX, NY)
    assert np.allclose(d, 1.0, atol=1e-10)


def test_ring_grids_constant_and_mean():
    """RingGrids full grids (test/usecases/fullclenshaw.jl): a constant stays
    constant (atol 1e-10) and the area-weighted mean of a smooth field is
    conserved; cells are numbered ring by ring from the north."""
    src, dst = grids.full_clenshaw_grid(12), grids.full_clenshaw_grid(18)
    t, _ = dst.cell_table()
    centres = t.sum(axis=1)
    assert centres[0, 2] > 0 and centres[-1, 2] < 0             # first ring north, last ring south
    O = oracle.OracleRegridder(dst, src, normalize=True)
    assert np.allclose(O.apply(np.ones(src.ncells)), 1.0, atol=1e-10)
    ts, _ = src.cell_table()
    c = ts.sum(axis=1)
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    f = 2.0 + c[:, 2] + 0.5 * c[:, 0] * c[:, 1]
    d = O.apply(f)
    assert abs(d @ O.dst_areas - f @ O.src_areas) <= 1e-13 * abs(f @ O.src_areas)
    G = oracle.OracleRegridder(grids.full_gaussian_grid(16), src, normalize=True)
    assert np.allclose(G.apply(np.ones(src.ncells)), 1.0, atol=1e-10)


def test_reorder_cells_permutes_the_matrix():
    a, b = grids.lonlat_regular(10.0, 10.0), grids.healpix_grid(4)
    order = np.random.default_rng(1).permutation(a.ncells)
    O = oracle.OracleRegridder(b, a)
    P = oracle.OracleRegridder(b, grids.reorder_cells(a, order))
    assert np.array_equal(P.intersections.toarray(), O.intersections.toarray()[:, order])


@pytest.mark.parametrize("nx,ny", [(8, 5), (12, 2), (16, 4)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_mirror_fold_host_path(nx, ny, dtype):
    """crg_mirror_fold on host fields (a host copy, no device needed) against
    the reference's rule (ext/ConservativeRegriddingOceananigansExt.jl:221-240):
    on the fold row, the primaries r = 1..Nx/4 and Nx/2+1..Nx/2+Nx/4 (1-based)
    are copied into their partners Nx+1-r; every other cell is untouched.
    1-D fields, and 2-D fields with the cells along either axis."""
    from crg import mirror_fold_

    rng = np.random.default_rng(nx * ny)
    nq, nh, off = nx // 4, nx // 2, (ny - 1) * nx
    prim = [r for r in range(1, nx + 1) if r <= nq or nh < r <= nh + nq]

    def expect(col):
        out = col.copy()
        for r in prim:
            out[off + nx - r] = col[off + r - 1]
        return out

    f = rng.standard_normal(nx * ny).astype(dtype)
    want = expect(f)
    mirror_fold_(f, nx, ny)
    assert np.array_equal(f, want)
    cm = rng.standard_normal((nx * ny, 3)).astype(dtype)  # cells along dims 1
    want = np.stack([expect(cm[:, k]) for k in range(3)], axis=1)
    mirror_fold_(cm, nx, ny, dims=1)
    assert np.array_equal(cm, want)
    fm = rng.standard_normal((3, nx * ny)).astype(dtype)  # cells along dims 2
    want = np.stack([expect(fm[k]) for k in range(3)])
    mirror_fold_(fm, nx, ny, dims=2)
    assert np.array_equal(fm, want)


def test_mirror_fold_refuses_unpaired_fold_rows():
    """With nx not a multiple of 4 the rule above leaves fold-row cells without
    a partner (nx = 10: cells 3 and 8), so such a fold is refused."""
    from crg import ArgumentError, mirror_fold_

    with pytest.raises(ArgumentError, match="multiple of 4"):
        mirror_fold_(np.zeros(30), 10, 3)
    with pytest.raises(ArgumentError, match="cells along dims"):
        mirror_fold_(np.zeros(31), 8, 4)


def test_rotated_lonlat_is_a_rigid_rotation():
    """grids.rotated_lonlat (an Oceananigans RotatedLatitudeLongitudeGrid
    covering the sphere): the pole rows meet exactly at the requested pole and
    its antipode, the seam column repeats column 0, the cells have the regular
    grid's areas (rotation keeps great-circle cells congruent), they tile the
    sphere, and the default pole gives the regular grid bit for bit."""
    g = grids.rotated_lonlat(10.0, 10.0, (70.0, 55.0))
    pole = grids.unit_sphere_from_geographic(70.0, 55.0)
    b = g.blocks[0]
    assert np.all(b[-1] == pole) and np.all(b[0] == -pole)
    assert np.array_equal(b[:, 0], b[:, -1])
    assert g.full_sphere and grids.convex_cells(g).all()
    assert np.array_equal(grids.rotated_lonlat(10.0, 10.0).blocks[0], grids.lonlat_regular(10.0, 10.0).blocks[0])
    O = oracle.OracleRegridder(grids.healpix_grid(8), g)
    O0 = oracle.OracleRegridder(grids.healpix_grid(8), grids.lonlat_regular(10.0, 10.0))
    assert np.allclose(O.src_areas, O0.src_areas, rtol=1e-14, atol=0)
    assert abs(O.src_areas.sum() - 4 * np.pi) < 1e-12
