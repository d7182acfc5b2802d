"""Spectral-element pieces of the oracle, pinned by the reference's own known
answers for its ClimaCore extension and triangle rules (no GPU):

- triangle rules integrate x^a y^b exactly up to their degree, weights sum to
  the triangle's area (test/triangle_quadrature.jl:5-20);
- Lagrange basis: Kronecker delta at the nodes, partition of unity off them
  (test/usecases/climacore.jl:15-49);
- the inverse element map returns the GLL coordinates of every node, on all
  faces (test/extensions/climacore.jl:63-92);
- the node weights sum to the sphere's area (test/extensions/climacore.jl:33-41);
- over an element itself, sum_ij b = the element's area
  (test/extensions/climacore.jl:114-141);
- SE -> FV preserves constants to 1e-10 and conserves the integral to 1e-12;
  FV -> SE preserves constants to 1e-10 (test/usecases/climacore.jl:87-100,
  :128-170).
"""
from __future__ import annotations

from math import factorial

import numpy as np
import pytest

import oracle
from crg import ArgumentError, Regridder, SpectralElementSpace, grids


def _corners(g, f, i, j):
    b = g.blocks[f]
    return np.array([b[j, i], b[j, i + 1], b[j + 1, i + 1], b[j + 1, i]])


@pytest.mark.parametrize("n", range(2, 13))
def test_gll_nodes_and_weights(n):
    from numpy.polynomial import legendre as L

    x, w = oracle.se_gll(n)
    c = np.zeros(n)
    c[-1] = 1.0
    inner = np.sort(L.legroots(L.legder(c)).real) if n > 2 else np.zeros(0)
    assert np.allclose(x, np.r_[-1.0, inner, 1.0], atol=1e-14, rtol=0)
    assert np.array_equal(x, -x[::-1]) and np.array_equal(w, w[::-1])
    # exact for polynomials of degree 2n - 3
    for k in range(2 * n - 2):
        assert abs(np.sum(w * x**k) - (2.0 / (k + 1) if k % 2 == 0 else 0.0)) < 1e-13


@pytest.mark.parametrize("degree", range(1, 9))
def test_triangle_rules_exact(degree):
    tl, tw = oracle.se_tri_rule(degree)
    assert abs(0.5 * tw.sum() - 0.5) < 1e-12
    assert np.allclose(tl.sum(axis=1), 1.0, atol=1e-14)
    for a in range(degree + 1):
        for b in range(degree + 1 - a):
            got = 0.5 * np.sum(tw * tl[:, 1] ** a * tl[:, 2] ** b)
            assert abs(got - factorial(a) * factorial(b) / factorial(a + b + 2)) < 1e-10


def test_triangle_rule_degree_range():
    assert len(oracle.se_tri_rule(0)[1]) == 1  # below 1: the degree-1 rule
    with pytest.raises(ValueError):
        oracle.se_tri_rule(9)


def test_lagrange_basis():
    x, _ = oracle.se_gll(4)
    for p in range(4):
        assert np.allclose(oracle.se_lagrange(4, x[p]), np.eye(4)[p], atol=1e-12)
    for t in (-0.7, -0.3, 0.0, 0.42, 0.91):
        assert abs(oracle.se_lagrange(4, t).sum() - 1.0) < 1e-12


def test_inverse_map_roundtrip_all_faces():
    ne, nq = 4, 4
    g = grids.cubed_sphere(ne)
    x, _ = oracle.se_gll(nq)
    for f in range(6):
        for i, j in ((0, 0), (3, 3), (1, 2), (2, 1)):
            c = _corners(g, f, i, j)
            pts, _ = oracle.se_nodes(c, nq)
            for a, b in ((0, 0), (nq - 1, nq - 1), (1, 2), (2, 1)):
                xi, eta = oracle.se_inverse(c, pts[a + b * nq])
                assert abs(xi - x[a]) < 1e-10 and abs(eta - x[b]) < 1e-10


def test_node_weights_sum_to_sphere_area():
    ne, nq = 16, 3
    g = grids.cubed_sphere(ne)
    tot = 0.0
    for f in range(6):
        for j in range(ne):
            for i in range(ne):
                tot += oracle.se_nodes(_corners(g, f, i, j), nq, radius=6371.0)[1].sum()
    assert abs(tot / (4 * np.pi * 6371.0**2) - 1.0) < 1e-5


def test_sum_b_over_an_element_is_its_area():
    g = grids.cubed_sphere(4)
    for f in range(6):
        c = _corners(g, f, 0, 0)
        B = oracle.se_poly_b(c, c, 4)
        assert abs(B.sum() / oracle.cell_area(c) - 1.0) < 1e-10


@pytest.fixture(scope="module")
def latlon1():
    return grids.lonlat_regular(1.0, 1.0)


def test_se_to_fv_constant_and_conservation(latlon1):
    R = oracle.OracleSERegridder(latlon1, grids.cubed_sphere(16), 4, se_is_dst=False)
    s = np.ones(R.ns)
    d = R.apply(s)
    assert np.max(np.abs(d - 1.0)) < 1e-10
    src_integral = np.sum(np.asarray(R.intersections.sum(axis=0)).ravel() * s)
    assert abs(src_integral / (4 * np.pi) - 1.0) < 1e-12
    assert abs(np.sum(d * R.dst_areas) / src_integral - 1.0) < 1e-12


def test_fv_to_se_constant(latlon1):
    R = oracle.OracleSERegridder(latlon1, grids.cubed_sphere(16), 4, se_is_dst=True)
    d = R.apply(np.ones(R.ns))
    assert np.max(np.abs(d - 1.0)) < 1e-10
    assert np.all(R.dst_areas == 1.0)


def test_se_to_se_is_rejected():
    s = SpectralElementSpace.cubed_sphere(2, 3)
    with pytest.raises(ArgumentError, match="SE → SE"):
        Regridder(s, s)


@pytest.mark.parametrize("ne,nq", [(2, 3), (3, 4), (4, 5)])
def test_dss_groups_match_the_cubed_sphere_topology(ne, nq):
    """The host's grouping of coincident nodes (the DSS of ClimaCore's
    weighted_dss!, ext/ConservativeRegriddingClimaCoreExt.jl:709-715), fed the
    oracle's node positions: a cubed sphere with ne x ne elements per face and
    nq x nq nodes per element has 6 ne^2 (nq-1)^2 + 2 distinct points; shared
    edge nodes come in pairs, element corners in fours, and the 8 cube corners
    in threes."""
    from crg import SpectralElementSpace

    space = SpectralElementSpace.cubed_sphere(ne, nq)
    cells, _ = space.elements.cell_table()
    space._points = np.concatenate([oracle.se_nodes(c, nq)[0] for c in cells])
    ptr, nodes = space.dss_groups()
    sizes = np.diff(ptr)
    assert space.nnodes - int(np.sum(sizes - 1)) == 6 * ne * ne * (nq - 1) ** 2 + 2
    assert set(sizes.tolist()) <= {2, 3, 4}
    # Euler: the element mesh has 6 ne^2 + 2 vertices (8 of valence 3) and 12 ne^2 edges
    assert int(np.sum(sizes == 3)) == 8
    assert int(np.sum(sizes == 4)) == 6 * ne * ne - 6
    assert int(np.sum(sizes == 2)) == 12 * ne * ne * (nq - 2)
    assert len(np.unique(nodes)) == len(nodes)
    for g in range(len(sizes)):
        members = nodes[ptr[g]:ptr[g + 1]]
        assert np.all(np.diff(members) > 0)
        p = space._points[members]
        assert np.max(np.abs(p - p[0])) < 1e-9
