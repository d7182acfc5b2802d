"""SE <-> FV regridders on the GPU (crg_build_se_to_fv / crg_build_fv_to_se)
against the oracle's restatement: identical sparsity, values and areas (bit
for bit: the same operations in the same order), node positions and weights,
then the reference's use-case invariants at the GPU (test/usecases/climacore.jl):
constants preserved to 1e-10 in both directions, the SE -> FV integral
conserved to 1e-12, the SE -> FV -> SE round trip, and the weighted DSS of
regrid! into an SE field."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from crg import ArgumentError, Regridder, SpectralElementSpace, grids, regrid_, regrid_field_

pytestmark = pytest.mark.gpu

CASES = {
    # (SE space, FV grid, triangle rule degree or None)
    "C8_nq4_lonlat4": lambda: (SpectralElementSpace.cubed_sphere(8, 4), grids.lonlat_regular(4.0, 4.0), None),
    "C6_nq3_healpix8": lambda: (SpectralElementSpace.cubed_sphere(6, 3), grids.healpix_grid(8), None),
    "C5_nq2_lonlat7": lambda: (SpectralElementSpace.cubed_sphere(5, 2), grids.lonlat_regular(7.0, 7.0), None),
    "C4_nq5_lonlat6": lambda: (SpectralElementSpace.cubed_sphere(4, 5), grids.lonlat_regular(6.0, 6.0), None),
    # nq above 5 runs the generic kernel; the default degree 2 (nq - 1) would exceed 8
    "C3_nq6_deg8_lonlat9": lambda: (SpectralElementSpace.cubed_sphere(3, 6), grids.lonlat_regular(9.0, 9.0), 8),
    "C7j_nq4_deg5_cs9": lambda: (SpectralElementSpace.cubed_sphere(7, 4, jitter=0.15, seed=4),
                                 grids.cubed_sphere(9, jitter=0.1, seed=5), 5),
}


def _oracle(space, fv, se_is_dst, degree):
    return oracle.OracleSERegridder(fv, space.elements, space.nq, se_is_dst, degree=degree or 0,
                                    radius=space.radius)


def _same(R, O):
    colptr, rowval, nzval = R.csc_arrays()
    assert np.array_equal(colptr, O.colptr)
    assert np.array_equal(rowval, O.rowval)
    assert np.array_equal(nzval, O.nzval), np.max(np.abs(nzval - O.nzval))
    assert np.array_equal(R.dst_areas, O.dst_areas)
    assert np.array_equal(R.src_areas, O.src_areas)


@pytest.mark.parametrize("case", list(CASES))
def test_se_to_fv_matches_oracle(cuda, case):
    space, fv, degree = CASES[case]()
    R = Regridder(fv, space, triangle_quad_degree=degree)
    assert R.shape == (fv.ncells, space.nnodes)
    _same(R, _oracle(space, fv, False, degree))


@pytest.mark.parametrize("case", list(CASES))
def test_fv_to_se_matches_oracle(cuda, case):
    space, fv, degree = CASES[case]()
    R = Regridder(space, fv, triangle_quad_degree=degree)
    assert R.shape == (space.nnodes, fv.ncells)
    _same(R, _oracle(space, fv, True, degree))


def test_radius_and_given_node_weights(cuda):
    space = SpectralElementSpace.cubed_sphere(6, 4, radius=6371.0)
    fv = grids.lonlat_regular(5.0, 5.0)
    R = Regridder(fv, space)
    _same(R, _oracle(space, fv, False, None))
    assert abs(R.src_areas.sum() / (4 * np.pi * 6371.0**2) - 1.0) < 1e-5
    # the same weights handed in (as from ClimaCore's weighted_jacobian) give the same matrices
    given = SpectralElementSpace(space.elements, 4, node_weights=space.node_weights(), radius=6371.0)
    for a, b in zip(Regridder(space, fv).csc_arrays(), Regridder(given, fv).csc_arrays()):
        assert np.array_equal(a, b)


def test_node_positions_and_weights(cuda):
    space = SpectralElementSpace.cubed_sphere(5, 4)
    pts, w = space.node_positions(), space.node_weights()
    g = space.elements
    for f in range(6):
        b = g.blocks[f]
        for j in range(5):
            for i in range(5):
                e = f * 25 + i + 5 * j
                c = np.array([b[j, i], b[j, i + 1], b[j + 1, i + 1], b[j + 1, i]])
                op, ow = oracle.se_nodes(c, 4)
                assert np.array_equal(pts[e * 16:(e + 1) * 16], op)
                assert np.array_equal(w[e * 16:(e + 1) * 16], ow)
    assert np.allclose(np.linalg.norm(pts, axis=1), 1.0, atol=1e-14)


@pytest.fixture(scope="module")
def c16(cuda):
    return SpectralElementSpace.cubed_sphere(16, 4), grids.lonlat_regular(1.0, 1.0)


def test_constants_and_conservation(c16):
    space, fv = c16
    R = Regridder(fv, space)
    d = np.zeros(fv.ncells)
    regrid_(d, R, np.ones(space.nnodes))
    assert np.max(np.abs(d - 1.0)) < 1e-10
    src_integral = np.sum(np.asarray(R.intersections.sum(axis=0)).ravel())
    assert abs(src_integral / (4 * np.pi) - 1.0) < 1e-12
    assert abs(np.sum(d * R.dst_areas) / src_integral - 1.0) < 1e-12
    Q = Regridder(space, fv)
    e = np.zeros(space.nnodes)
    regrid_(e, Q, np.ones(fv.ncells))
    assert np.max(np.abs(e - 1.0)) < 1e-10


def test_roundtrip_and_dss(c16):
    import torch

    space, fv = c16
    fwd, bwd = Regridder(fv, space), Regridder(space, fv)
    p = space.node_positions()
    lat = np.degrees(np.arcsin(np.clip(p[:, 2], -1, 1)))
    fvv = np.zeros(fv.ncells)
    regrid_(fvv, fwd, lat)
    # SE integral (node weights) against the FV integral, as the reference's round-trip test
    se_integral = np.sum(space.node_weights() * lat)
    assert abs(np.sum(fvv * fwd.dst_areas) - se_integral) <= 1e-2 * abs(se_integral) + 1e-6
    back = torch.zeros(space.nnodes, dtype=torch.float64, device="cuda")
    regrid_field_(back, bwd, torch.from_numpy(fvv).cuda())
    b = back.cpu().numpy()
    ptr, nodes = space.dss_groups()
    assert len(ptr) > 1
    for g in range(len(ptr) - 1):  # shared nodes agree after the weighted DSS
        vals = b[nodes[ptr[g]:ptr[g + 1]]]
        assert np.all(vals == vals[0])
    # a continuous field is left as it is (up to rounding); FP32 fields too
    before = torch.from_numpy(lat.astype(np.float32)).cuda()
    after = before.clone()
    space.dss_(after)
    assert torch.allclose(after, before, atol=1e-4, rtol=0)
    assert np.max(np.abs(b - lat)) < 5.0  # 1-degree cells: the projection is close to the field


def test_multi_field_dss_layouts(c16):
    import torch

    space, _ = c16
    gen = torch.Generator(device="cuda").manual_seed(3)
    f = torch.randn((space.nnodes, 5), generator=gen, device="cuda", dtype=torch.float64)
    g = f.T.contiguous()
    space.dss_(f, dims=1)
    space.dss_(g, dims=2)
    assert torch.equal(f, g.T)
    ptr, nodes = space.dss_groups()
    w = space.node_weights()
    fr = np.random.default_rng(3).standard_normal((space.nnodes, 5))
    want = fr.copy()
    for k in range(len(ptr) - 1):
        idx = nodes[ptr[k]:ptr[k + 1]]
        want[idx] = (w[idx, None] * fr[idx]).sum(axis=0) / w[idx].sum()
    got = fr.copy()
    space.dss_(got, dims=1)
    assert np.allclose(got, want, rtol=1e-13, atol=1e-13)


def test_errors(cuda):
    space = SpectralElementSpace.cubed_sphere(3, 4)
    fv = grids.lonlat_regular(10.0, 10.0)
    with pytest.raises(ArgumentError, match="degree 9"):
        Regridder(fv, space, triangle_quad_degree=9)
    with pytest.raises(ArgumentError, match="degree 10"):
        Regridder(fv, SpectralElementSpace.cubed_sphere(3, 6))  # default 2 (nq - 1) = 10
    tri = grids.Grid("cells", grids.SPHERICAL, cells=_triangles())
    with pytest.raises(ArgumentError, match="4 vertices"):
        Regridder(fv, SpectralElementSpace(tri, 3))


def _triangles():
    v = np.eye(3)
    return np.array([[v[0], v[1], v[2]], [v[0], v[2], -v[1]]])
