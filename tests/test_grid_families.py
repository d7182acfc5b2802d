"""Grid families on the CPU (oracle): folded (tripolar, RightCenterFolded)
grids -- the synthetic fold row has cell i and cell nx+1-i equal; with the
partner slots as ghosts the oracle regrids a constant exactly in both
directions, ghosts get nothing, and the library's host-side fold mirror
fills them -- and RingGrids full grids and reordered cell numberings."""
from __future__ import annotations

import numpy as np
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
