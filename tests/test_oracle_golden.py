"""The oracle against the reference's known answers and independent
high-precision values (CPU only).  This pins the oracle before the CUDA kernels
are compared with it."""
from __future__ import annotations

import json
import sys

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, c1_grids
from crg import grids


def _load(name):
    return json.loads((GOLDEN / name).read_text())


def test_readme_known_answer():
    """README.md:52-80: every intersection of the 2x2 squares with the diamond and
    triangles is exactly 0.5; areas [0.5,0.5,2,0.5,0.5] and [1,1,1,1]."""
    g = _load("readme_planar.json")["readme"]
    R = oracle.OracleRegridder(grids.polygon_grid(g["dst"]), grids.polygon_grid(g["src"]), normalize=False)
    assert np.array_equal(R.intersections.toarray(), np.array(g["matrix"]))
    assert np.array_equal(R.src_areas, g["src_areas"])
    assert np.array_equal(R.dst_areas, g["dst_areas"])


def test_simple_jl_exact_conservation():
    """test/usecases/simple.jl:30-51: row/col sums == cell areas and the mean is
    conserved exactly, forward and back."""
    g = _load("readme_planar.json")["simple_jl"]
    R = oracle.OracleRegridder(grids.polygon_grid(g["dst"]), grids.polygon_grid(g["src"]), normalize=False)
    A = R.intersections
    area1 = np.asarray(A.sum(axis=1)).ravel()
    area2 = np.asarray(A.sum(axis=0)).ravel()
    assert np.array_equal(area1, g["dst_areas"]) and np.array_equal(area1, R.dst_areas)
    assert np.array_equal(area2, g["src_areas"]) and np.array_equal(area2, R.src_areas)
    v2 = np.array(g["values_on_src"], float)
    v1 = A @ v2 / area1
    assert np.sum(v1 * area1) == np.sum(v2 * area2)
    back = A.T @ v1 / area2
    assert np.sum(back * area2) == np.sum(v2 * area2)


def test_sphere_areas_vs_mpmath():
    g = _load("sphere_areas.json")
    for name, c in g["polygons"].items():
        a = oracle.cell_area(np.array(c["verts"]))
        ref = float(c["area"])
        assert abs(a - ref) <= 1e-14 * ref, name
    for name, c in g["pairs"].items():
        a = oracle.pair_area(np.array(c["src"]), np.array(c["dst"]))
        ref = float(c["area"])
        assert abs(a - ref) <= 1e-14 * max(ref, 1e-300) or (ref == 0 and a <= 0), name


def test_atan2_accuracy():
    rng = np.random.default_rng(1)
    y = np.concatenate([rng.normal(size=2000), 10.0 ** rng.uniform(-20, 3, 2000) * rng.choice([-1, 1], 2000)])
    x = np.concatenate([rng.normal(size=2000), 10.0 ** rng.uniform(-20, 3, 2000) * rng.choice([-1, 1], 2000)])
    for a, b in zip(y, x):
        r = oracle.atan2(a, b)
        ref = np.arctan2(a, b)
        assert abs(r - ref) <= 4 * np.spacing(abs(ref)) + 1e-300


def test_healpix_geometry():
    """HEALPix tree shape and indices (test/extensions/healpix.jl:16-107): 12
    nside^2 pixels, a permutation for ring order, 4 corners per pixel."""
    for nside in (1, 2, 4, 16):
        pix = np.arange(12 * nside * nside)
        ring = grids.healpix_nest2ring(nside, pix)
        assert np.array_equal(np.sort(ring), pix)
        c_np = grids.healpix_corners_nested(nside, pix)
        for p in pix[:: max(1, len(pix) // 97)]:
            assert np.array_equal(c_np[p], oracle.healpix_corners(nside, p))
            assert ring[p] == oracle.healpix_nest2ring(nside, p)
        assert np.allclose(np.linalg.norm(c_np, axis=-1), 1.0, atol=1e-15)
    g = grids.healpix_grid(8)
    R = oracle.OracleRegridder(g, g)
    assert abs(R.dst_areas.sum() - 4 * np.pi) < 1e-12


CASES = {
    "C1_lonlat2_to_lonlat3_shifted": c1_grids,
    "lonlat4_to_healpix16": lambda: (grids.healpix_grid(16), grids.lonlat_regular(4.0, 4.0)),
    "lonlat4_to_healpix8_ring": lambda: (grids.healpix_grid(8, "ring"), grids.lonlat_regular(4.0, 4.0)),
    "lonlat4_to_cs12": lambda: (grids.cubed_sphere(12), grids.lonlat_regular(4.0, 4.0)),
    "cs8_to_lonlat5": lambda: (grids.lonlat_regular(5.0, 5.0), grids.cubed_sphere(8)),
    "jittered": lambda: (grids.lonlat_jittered(60, 30, 0.2, 3), grids.lonlat_jittered(90, 45, 0.2, 4)),
    "rotated_lonlat10_pole70_55_to_healpix8": lambda: (grids.healpix_grid(8),
                                                       grids.rotated_lonlat(10.0, 10.0, (70.0, 55.0))),
}


@pytest.mark.parametrize("name", list(CASES))
def test_tree_search_is_complete(name):
    """The restated dual DFS over the reference's trees finds every pair with
    positive area that an exhaustive cap test finds (quadtree_cursors.jl:55-80
    style completeness)."""
    dst, src = CASES[name]()
    Rt = oracle.OracleRegridder(dst, src, use_tree=True)
    Re = oracle.OracleRegridder(dst, src, use_tree=False)
    assert Rt.nnz > 0 and Rt.overflows == 0
    assert np.array_equal(Rt.colptr, Re.colptr)
    assert np.array_equal(Rt.rowval, Re.rowval)
    assert np.array_equal(Rt.nzval, Re.nzval)


@pytest.mark.parametrize("name", list(CASES))
def test_area_agreement(name):
    """Row sums of A equal the destination cell areas and column sums the source
    cell areas where the other grid covers the cell (ConservativeRegriddingTestHelpers
    test_intersection_areas_agree, rtol = sqrt(eps))."""
    dst, src = CASES[name]()
    R = oracle.OracleRegridder(dst, src)
    A = R.intersections
    rs = np.asarray(A.sum(axis=1)).ravel()
    cs = np.asarray(A.sum(axis=0)).ravel()
    if dst.full_sphere and src.full_sphere:
        assert np.allclose(rs, R.dst_areas, rtol=np.sqrt(np.finfo(float).eps), atol=0)
        assert np.allclose(cs, R.src_areas, rtol=np.sqrt(np.finfo(float).eps), atol=0)
        assert abs(R.dst_areas.sum() - 4 * np.pi) < 1e-11
    else:
        assert np.allclose(rs, R.dst_areas, rtol=np.sqrt(np.finfo(float).eps), atol=0)
        assert np.all(cs <= R.src_areas * (1 + 1e-12))


def test_constant_field_and_conservation():
    """Constant fields stay constant (test/usecases/fullclenshaw.jl:19-31,
    atol 1e-10) and the area-weighted total is conserved (rtol 1e-10), forward
    and through the transpose."""
    dst, src = grids.healpix_grid(16), grids.lonlat_regular(4.0, 4.0)
    R = oracle.OracleRegridder(dst, src, normalize=True)
    d = R.apply(np.ones(R.ns))
    assert np.max(np.abs(d - 1)) < 1e-10
    s = R.apply(np.ones(R.nd), transpose=True)
    assert np.max(np.abs(s - 1)) < 1e-10
    rng = np.random.default_rng(0)
    f = rng.random(R.ns)
    d = R.apply(f)
    assert abs(np.sum(d * R.dst_areas) - np.sum(f * R.src_areas)) <= 1e-10 * abs(np.sum(f * R.src_areas))


def test_normalize_divides_by_max():
    dst, src = c1_grids()
    R0 = oracle.OracleRegridder(dst, src, normalize=False)
    R1 = oracle.OracleRegridder(dst, src, normalize=True)
    m = R0.nzval.max()
    assert np.array_equal(R1.nzval, R0.nzval / m)
    assert np.array_equal(R1.dst_areas, R0.dst_areas / m)
    assert R1.nzval.max() == 1.0


def test_disjoint_grids_have_empty_matrix():
    a = grids.polygon_grid([[(0, 0), (1, 0), (1, 1), (0, 1)]])
    b = grids.polygon_grid([[(5, 5), (6, 5), (6, 6), (5, 6)], [(2, 2), (3, 2), (3, 3)]])
    R = oracle.OracleRegridder(a, b)
    assert R.nnz == 0
    assert np.array_equal(R.colptr, [0, 0, 0])


def _ring_centres(nside):
    """Pixel centres in ring order from the ring-scheme closed forms of
    Gorski et al. (2005), ApJ 622:759, section 4: polar caps z = +-(1 - i^2 /
    (3 N^2)), phi = (j - 1/2) pi / (2 i); equatorial belt z = 4/3 - 2 i / (3 N),
    phi = (j - f) pi / (2 N) with f = 1 for odd i + N, else 1/2."""
    N = nside
    npix, ncap = 12 * N * N, 2 * N * (N - 1)
    z, phi = np.empty(npix), np.empty(npix)
    for r in range(npix):
        if r < ncap:
            i = (1 + int(np.sqrt(1 + 2 * r))) // 2
            j = r + 1 - 2 * i * (i - 1)
            z[r], phi[r] = 1 - i * i / (3.0 * N * N), (j - 0.5) * np.pi / (2 * i)
        elif r < npix - ncap:
            i = (r - ncap) // (4 * N) + N
            j = (r - ncap) % (4 * N) + 1
            f = 1.0 if (i + N) % 2 else 0.5
            z[r], phi[r] = 4.0 / 3.0 - 2.0 * i / (3.0 * N), (j - f) * np.pi / (2 * N)
        else:
            q = npix - r
            i = (1 + int(np.sqrt(2 * q - 1))) // 2
            j = 4 * i + 1 - (q - 2 * i * (i - 1))
            z[r], phi[r] = -1 + i * i / (3.0 * N * N), (j - 0.5) * np.pi / (2 * i)
    s = np.sqrt((1 - z) * (1 + z))
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)


@pytest.mark.parametrize("nside", [1, 2, 4, 8, 16])
def test_healpix_face_map_and_ring_order_match_the_published_centres(nside):
    """The face map that places the corners, evaluated at the middle of each
    nested pixel (face coordinates (ix + 1/2, iy + 1/2) / N), and the
    nested -> ring permutation, reproduce the published ring-order pixel
    centres: the corner geometry is pinned independently of its two codings."""
    pix = np.arange(12 * nside * nside)
    ix, iy, face = grids.healpix_nest2xyf(nside, pix)
    mid = grids._hp_loc2vec((ix + 0.5) / nside, (iy + 0.5) / nside, face)
    ring = grids.healpix_nest2ring(nside, pix)
    want = _ring_centres(nside)[ring]
    assert np.max(np.abs(mid - want)) < 1e-13


def test_healpix_base_pixel_corners():
    """nside 1: the 12 base pixels have 14 distinct corners -- the poles,
    z = +-2/3 at longitudes 0, 90, 180, 270 and z = 0 at 45 + 90 k -- and each
    pixel lists them north, west, south, east (z of N >= W, E >= S)."""
    c = grids.healpix_corners_nested(1, np.arange(12))
    pts = np.unique(np.round(c.reshape(-1, 3), 12), axis=0)
    want = [(0.0, 0.0, 1.0), (0.0, 0.0, -1.0)]
    s = np.sqrt(1 - 4.0 / 9.0)
    for k in range(4):
        a = np.pi / 2 * k
        want += [(s * np.cos(a), s * np.sin(a), 2.0 / 3.0), (s * np.cos(a), s * np.sin(a), -2.0 / 3.0),
                 (np.cos(a + np.pi / 4), np.sin(a + np.pi / 4), 0.0)]
    want = np.unique(np.round(np.array(want), 12), axis=0)
    assert pts.shape == (14, 3) and np.allclose(pts, want, atol=1e-12)
    z = c[:, :, 2]
    assert np.all(z[:, 0] >= z[:, 1] - 1e-15) and np.all(z[:, 0] >= z[:, 3] - 1e-15)
    assert np.all(z[:, 2] <= z[:, 1] + 1e-15) and np.all(z[:, 2] <= z[:, 3] + 1e-15)


@pytest.mark.parametrize("ne", [1, 3, 12])
def test_cubed_sphere_cell_areas_match_the_gnomonic_closed_form(ne):
    """Equiangular gnomonic cells are bounded by great circles (gnomonic
    lines), so their solid angle is exact in closed form: with x = tan(alpha),
    y = tan(beta) and W(x, y) = atan(x y / sqrt(1 + x^2 + y^2)), a cell is
    W(x2, y2) - W(x1, y2) - W(x2, y1) + W(x1, y1).  Evaluated in 40-digit
    arithmetic, it pins the cubed-sphere generator and the oracle's polygon
    area together.  The corners are rounded to doubles, which moves a cell's
    area by about one ulp per cell width (the oracle's area of the rounded
    corners is itself within 2e-16 of exact), hence the bound grows with ne."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 40
    g = grids.cubed_sphere(ne)
    R = oracle.OracleRegridder(g, g)
    t = [mpmath.tan(-mpmath.pi / 4 + k * mpmath.pi / (2 * ne)) for k in range(ne + 1)]
    W = lambda x, y: mpmath.atan(x * y / mpmath.sqrt(1 + x * x + y * y))
    face = np.array([float(W(t[i + 1], t[j + 1]) - W(t[i], t[j + 1]) - W(t[i + 1], t[j]) + W(t[i], t[j]))
                     for j in range(ne) for i in range(ne)])
    want = np.tile(face, 6)
    assert np.max(np.abs(R.dst_areas - want) / want) < 5e-16 * max(ne, 2)


def _sph_polygon(rng, centre, radius, n, ccw=True):
    """Convex spherical polygon: n points at angular distance ~radius around
    `centre`, in increasing angle (counter-clockwise seen from outside)."""
    c = centre / np.linalg.norm(centre)
    u = np.cross(c, [0.0, 0.0, 1.0] if abs(c[2]) < 0.9 else [1.0, 0.0, 0.0])
    u /= np.linalg.norm(u)
    v = np.cross(c, u)
    th = np.sort(rng.uniform(0.0, 2.0 * np.pi, n))
    p = np.cos(radius) * c[None] + np.sin(radius) * (np.cos(th)[:, None] * u + np.sin(th)[:, None] * v)
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    return p if ccw else p[::-1].copy()


def test_random_spherical_pairs_vs_mpmath():
    """The oracle's spherical clip + area against the 60-digit clip and
    Girard area of tests/golden/make_golden.py on 120 random convex pairs
    (3 to 8 vertices, 0.01 to 0.5 rad across, either orientation)."""
    pytest.importorskip("mpmath")
    sys.path.insert(0, str(GOLDEN))
    import make_golden as mg

    rng = np.random.default_rng(21)
    overlapping = 0
    for trial in range(120):
        c1 = rng.standard_normal(3)
        r1, r2 = rng.uniform(0.01, 0.5), rng.uniform(0.01, 0.5)
        c2 = c1 / np.linalg.norm(c1) + rng.uniform(-1, 1, 3) * (r1 + r2)
        s = _sph_polygon(rng, c1, r1, int(rng.integers(3, 9)), bool(rng.integers(2)))
        d = _sph_polygon(rng, c2, r2, int(rng.integers(3, 9)), bool(rng.integers(2)))
        got = oracle.pair_area(s, d)
        res = mg.mp_clip(s.tolist(), d.tolist())
        want = float(mg.girard_area_mp(res)) if len(res) >= 3 else 0.0
        overlapping += want > 0
        scale = oracle.cell_area(s)
        assert abs(got - want) <= 1e-14 * scale, (trial, got, want)
    assert overlapping >= 40


def test_pole_rows_conserve_area():
    """45-degree cells against 0.5-degree cells: both grids have a pole row whose
    cells carry the pole twice (sind(90) = 1 exactly, cosd(90) = 0).  Side values
    that the exact sign settles to about DBL_MIN at both ends of an edge make
    crossing weights whose combination underflows; the crossing is rescaled
    first, so every cell's intersections still add up to its area (before the
    rescaling one 0.5-degree pole cell lost all of it, and 22 entries)."""
    dst, src = grids.lonlat_regular(45.0, 45.0), grids.lonlat_regular(0.5, 0.5)
    R = oracle.OracleRegridder(dst, src, normalize=False)
    assert R.nnz == 261768 and np.isfinite(R.nzval).all()
    rows = np.zeros(R.nd)
    cols = np.zeros(R.ns)
    np.add.at(rows, R.rowval, R.nzval)
    np.add.at(cols, np.repeat(np.arange(R.ns), np.diff(R.colptr)), R.nzval)
    assert np.max(np.abs(rows - R.dst_areas) / R.dst_areas) < 1e-12
    assert np.max(np.abs(cols - R.src_areas) / R.src_areas) < 1e-12
    assert abs(R.nzval.sum() - 4 * np.pi) < 1e-11
