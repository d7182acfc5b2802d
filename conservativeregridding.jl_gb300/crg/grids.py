"""Grid descriptions handed to the regridder.

ConservativeRegridding.jl turns its inputs into trees with ``Trees.treeify``
(src/trees/interfaces.jl:94-129): vertex matrices become a
``CellBasedGrid`` under a ``TopDownQuadtreeCursor`` (src/trees/grids.jl:57-85),
lon-lat ocean grids are wrapped in ``KnownFullSphereExtentWrapper``
(ext/ConservativeRegriddingOceananigansExt.jl:242-264), cubed spheres become a
``CubedSphereToplevelTree`` of six index-offset quadtrees
(ext/ConservativeRegriddingClimaCoreExt.jl:43-94) and HEALPix maps a 12-face
nested tree whose cells are the pixel corner quadrilaterals
(ext/ConservativeRegriddingHealpixExt.jl:76-90, :159-167).

Here a :class:`Grid` carries the same information as plain arrays:

* ``kind='curvilinear'``: one or more blocks of ``(nx+1) x (ny+1)`` points
  (stored as arrays of shape ``(ny+1, nx+1, dim)``, so point ``(i, j)`` is
  ``block[j, i]``); cell ``(i, j)`` of block ``b`` has the 0-based index
  ``offset_b + i + j*nx`` and the ring ``p(i,j), p(i+1,j), p(i+1,j+1), p(i,j+1)``.
* ``kind='cells'``: a ``(ncells, maxv, dim)`` table of ring vertices with an
  optional vertex count per cell (HEALPix pixels, explicit polygons).

The builders below generate the synthetic grids used by the tests and the
benchmark: regular and shifted lon-lat grids, jittered lon-lat grids, the
equiangular gnomonic cubed sphere and HEALPix.
"""
from __future__ import annotations

import dataclasses
from typing import Optional, Sequence

import numpy as np

SPHERICAL = "spherical"
PLANAR = "planar"


# ----------------------------------------------------------------- coordinates

def sincosd(x):
    """sin and cos of angles in degrees, exact at multiples of 90 degrees.

    The reference converts geographic points with GeometryOps'
    ``UnitSphereFromGeographic`` (src/trees/grids.jl:195,246); degree-exact
    trigonometry makes the pole vertices of lon-lat grids coincide exactly.
    """
    x = np.asarray(x, dtype=np.float64)
    r = np.remainder(x, 360.0)
    q = np.round(r / 90.0)
    d = np.deg2rad(r - 90.0 * q)
    s, c = np.sin(d), np.cos(d)
    q = q.astype(np.int64) % 4
    sin = np.select([q == 0, q == 1, q == 2, q == 3], [s, c, -s, -c])
    cos = np.select([q == 0, q == 1, q == 2, q == 3], [c, -s, -c, s])
    return sin, cos


def unit_sphere_from_geographic(lon, lat):
    """(lon, lat) in degrees -> unit vectors of shape (..., 3)."""
    slon, clon = sincosd(lon)
    slat, clat = sincosd(lat)
    return np.stack([clat * clon, clat * slon, slat], axis=-1)


# ----------------------------------------------------------------- grid type

@dataclasses.dataclass
class Grid:
    kind: str                       # 'curvilinear' | 'cells'
    manifold: str                   # 'spherical' | 'planar'
    blocks: Optional[list] = None   # curvilinear: list of (ny+1, nx+1, dim) arrays
    cells: Optional[np.ndarray] = None   # cells: (ncells, maxv, dim)
    nverts: Optional[np.ndarray] = None  # cells: (ncells,) int32 or None
    full_sphere: bool = False       # root extent is the whole sphere (KnownFullSphereExtentWrapper)
    healpix: Optional[tuple] = None  # (nside, nested) for HEALPix grids
    name: str = ""

    def __post_init__(self):
        if self.kind == "curvilinear":
            self.blocks = [np.ascontiguousarray(b, dtype=np.float64) for b in self.blocks]
        else:
            self.cells = np.ascontiguousarray(self.cells, dtype=np.float64)
            if self.nverts is not None:
                self.nverts = np.ascontiguousarray(self.nverts, dtype=np.int32)

    @property
    def dim(self) -> int:
        return 3 if self.manifold == SPHERICAL else 2

    @property
    def ncells(self) -> int:
        if self.kind == "curvilinear":
            return int(sum((b.shape[0] - 1) * (b.shape[1] - 1) for b in self.blocks))
        return int(self.cells.shape[0])

    @property
    def block_shapes(self):
        """[(nx, ny)] per block."""
        return [(b.shape[1] - 1, b.shape[0] - 1) for b in self.blocks]

    def points_flat(self) -> np.ndarray:
        """All block points back to back, i fastest inside a block (made once per grid)."""
        flat = self.__dict__.get("_flat")
        if flat is None:
            if len(self.blocks) == 1:
                flat = np.ascontiguousarray(self.blocks[0].reshape(-1, self.dim), np.float64)
            else:
                flat = np.ascontiguousarray(np.concatenate([b.reshape(-1, self.dim) for b in self.blocks], axis=0),
                                            np.float64)
            self.__dict__["_flat"] = flat
        return flat

    def cell_table(self) -> tuple[np.ndarray, np.ndarray]:
        """(ncells, maxv, dim) ring vertices and (ncells,) vertex counts."""
        if self.kind == "cells":
            nv = self.nverts if self.nverts is not None else np.full(self.ncells, self.cells.shape[1], np.int32)
            return self.cells, nv
        out = []
        for b in self.blocks:
            p00 = b[:-1, :-1]
            p10 = b[:-1, 1:]
            p11 = b[1:, 1:]
            p01 = b[1:, :-1]
            quad = np.stack([p00, p10, p11, p01], axis=2)  # (ny, nx, 4, dim)
            out.append(quad.reshape(-1, 4, self.dim))
        t = np.concatenate(out, axis=0)
        return t, np.full(t.shape[0], 4, np.int32)

    def to_spherical(self) -> "Grid":
        """Planar (lon, lat) degrees -> unit sphere (the manifold promotion of
        Regridder(dst, src), src/regridder/regridder.jl:109-117)."""
        if self.manifold == SPHERICAL:
            return self
        if self.kind == "curvilinear":
            blocks = [unit_sphere_from_geographic(b[..., 0], b[..., 1]) for b in self.blocks]
            return Grid("curvilinear", SPHERICAL, blocks=blocks, full_sphere=self.full_sphere, name=self.name)
        cells = unit_sphere_from_geographic(self.cells[..., 0], self.cells[..., 1])
        return Grid("cells", SPHERICAL, cells=cells, nverts=self.nverts, name=self.name)


# ----------------------------------------------------------------- lon-lat

def lonlat_grid(lon_edges: Sequence[float], lat_edges: Sequence[float], full_sphere: Optional[bool] = None,
                name: str = "") -> Grid:
    """Lon-lat grid with great-circle cell edges between the corner points
    (the Oceananigans lon-lat convention: a vertex matrix turned into a
    CellBasedGrid, ext/ConservativeRegriddingOceananigansExt.jl:246-263)."""
    lon = np.asarray(lon_edges, np.float64)
    lat = np.asarray(lat_edges, np.float64)
    LON, LAT = np.meshgrid(lon, lat)  # (ny+1, nx+1)
    pts = unit_sphere_from_geographic(LON, LAT)
    if full_sphere is None:
        full_sphere = bool(abs((lon[-1] - lon[0]) - 360.0) < 1e-9 and lat[0] <= -90.0 and lat[-1] >= 90.0)
    return Grid("curvilinear", SPHERICAL, blocks=[pts], full_sphere=full_sphere, name=name)


def lonlat_regular(dlon: float, dlat: float, lon0: float = 0.0, lat0: float = -90.0, name: str = "") -> Grid:
    """Global lon-lat grid with spacing (dlon, dlat) starting at (lon0, lat0);
    latitude edges are clamped to [-90, 90]."""
    nx = int(round(360.0 / dlon))
    ny = int(round(180.0 / dlat))
    lon = lon0 + dlon * np.arange(nx + 1)
    lat = np.clip(lat0 + dlat * np.arange(ny + 1), -90.0, 90.0)
    return lonlat_grid(lon, lat, full_sphere=True, name=name or f"lonlat_{nx}x{ny}")


def rotated_lonlat(dlon: float, dlat: float, north_pole: Sequence[float] = (0.0, 90.0), name: str = "") -> Grid:
    """Global lon-lat grid with spacing (dlon, dlat) in a frame whose north pole
    lies at the geographic point ``north_pole`` = (lon, lat) in degrees, like
    an Oceananigans ``RotatedLatitudeLongitudeGrid`` that covers the sphere.
    The reference treats it as any Oceananigans grid: its vertex matrix becomes
    a CellBasedGrid under KnownFullSphereExtentWrapper
    (ext/ConservativeRegriddingOceananigansExt.jl:242-264).

    The regular grid's unit vectors are turned by R = Rz(lon) Ry(90 - lat),
    which carries the z axis to the pole.  A rotation maps great circles to
    great circles, so every cell is a regular cell moved rigidly; the pole rows
    still meet in one point each and the 360-degree column equals column 0."""
    g = lonlat_regular(dlon, dlat)
    sp, cp = sincosd(north_pole[1])
    sl, cl = sincosd(north_pole[0])
    ry = np.array([[sp, 0.0, cp], [0.0, 1.0, 0.0], [-cp, 0.0, sp]])  # z -> (cos lat, 0, sin lat)
    rz = np.array([[cl, -sl, 0.0], [sl, cl, 0.0], [0.0, 0.0, 1.0]])
    pts = g.blocks[0] @ (rz @ ry).T
    nx, ny = g.block_shapes[0]
    return Grid("curvilinear", SPHERICAL, blocks=[pts], full_sphere=True,
                name=name or f"rotated_lonlat_{nx}x{ny}_pole_{north_pole[0]:g}_{north_pole[1]:g}")


def lonlat_jittered(nx: int, ny: int, jitter: float, seed: int, name: str = "") -> Grid:
    """Global nx x ny lon-lat grid whose interior vertices move by
    U(-jitter, jitter) cell widths in lon and lat.  Pole rows stay on the
    poles and the 360-degree column repeats the jitter of column 0."""
    rng = np.random.default_rng(seed)
    dlon, dlat = 360.0 / nx, 180.0 / ny
    lon = dlon * np.arange(nx + 1)[None, :].repeat(ny + 1, 0)
    lat = (-90.0 + dlat * np.arange(ny + 1))[:, None].repeat(nx + 1, 1)
    jl = rng.uniform(-jitter, jitter, size=(ny + 1, nx)) * dlon
    jt = rng.uniform(-jitter, jitter, size=(ny + 1, nx)) * dlat
    jl = np.concatenate([jl, jl[:, :1]], axis=1)
    jt = np.concatenate([jt, jt[:, :1]], axis=1)
    jl[0, :] = 0.0
    jl[-1, :] = 0.0
    jt[0, :] = 0.0
    jt[-1, :] = 0.0
    pts = unit_sphere_from_geographic(lon + jl, lat + jt)
    return Grid("curvilinear", SPHERICAL, blocks=[pts], full_sphere=True, name=name or f"lonlat_jit_{nx}x{ny}")


def convex_cells(g: Grid) -> np.ndarray:
    """True for every cell whose corners all turn the same way (convex, in
    either orientation; repeated vertices such as a lon-lat cell's two pole
    corners do not count as turns).  The spherical clip needs convex
    destination cells."""
    t, nv = g.cell_table()
    n, m = t.shape[0], t.shape[1]
    nv = np.asarray(nv, np.int64)
    rows = np.arange(n)
    pos = np.zeros(n, bool)
    neg = np.zeros(n, bool)
    for k in range(m):
        valid = k < nv
        kk = np.minimum(k, nv - 1)
        a = t[rows, (kk - 1) % nv]
        b = t[rows, kk]
        c = t[rows, (kk + 1) % nv]
        if g.manifold == SPHERICAL:
            turn = np.einsum("ij,ij->i", b, np.cross(b - a, c - b))
        else:
            turn = (b[:, 0] - a[:, 0]) * (c[:, 1] - b[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - b[:, 0])
        pos |= valid & (turn > 0)
        neg |= valid & (turn < 0)
    return ~(pos & neg)


# ----------------------------------------------------------------- reordered and ring grids

def reorder_cells(g: Grid, order, name: str = "") -> Grid:
    """Cell k of the result is cell ``order[k]`` of ``g`` (same vertex ring):
    any numbering of a grid's cells, as the reference's reordered quadtree
    cursors give (src/trees/specialized_quadtree_cursors.jl:152-270), as
    per-cell polygons."""
    t, nv = g.cell_table()
    order = np.asarray(order, np.int64)
    if order.ndim != 1 or len(order) != len(t) or not np.array_equal(np.sort(order), np.arange(len(t))):
        raise ValueError("order must be a permutation of the cell indices")
    return Grid("cells", g.manifold, cells=t[order].copy(), nverts=np.asarray(nv)[order].copy(),
                full_sphere=g.full_sphere, name=name or g.name + "_reordered")


def full_ring_grid(latd, lond, name: str = "") -> Grid:
    """A RingGrids full grid (rings of equal longitude spacing) from its ring
    latitudes ``latd`` (north to south) and longitudes ``lond``, as the
    reference's RingGrids extension builds it (ext/ConservativeRegriddingRingGridsExt.jl:21-48):
    latitude edges halfway between rings and pinned to the poles, longitude
    edges half a cell either side of ``lond``, cells numbered ring by ring from
    the north (east within a ring)."""
    latd = np.asarray(latd, np.float64)
    lond = np.asarray(lond, np.float64)
    nlat, nlon = len(latd), len(lond)
    lat_edges = np.empty(nlat + 1)
    lat_edges[0], lat_edges[-1] = 90.0, -90.0
    lat_edges[1:-1] = 0.5 * (latd[:-1] + latd[1:])
    dlon = 360.0 / nlon
    lon_edges = lond[0] - dlon / 2 + dlon * np.arange(nlon + 1)
    g = lonlat_grid(lon_edges, lat_edges[::-1], full_sphere=True)   # south to north: counter-clockwise cells
    ring = np.arange(nlat)[:, None]                                  # 0 = northernmost
    order = ((nlat - 1 - ring) * nlon + np.arange(nlon)[None, :]).ravel()
    return reorder_cells(g, order, name=name or f"ring_{nlon}x{nlat}")


def full_clenshaw_grid(nlat_half: int) -> Grid:
    """Full Clenshaw-Curtis grid: 2*nlat_half - 1 rings at equally spaced
    colatitudes j*180/(2*nlat_half) (j = 1..2*nlat_half-1, the equator
    included, no pole rings), 4*nlat_half points per ring from longitude 0."""
    nlat, nlon = 2 * nlat_half - 1, 4 * nlat_half
    latd = 90.0 - np.arange(1, nlat + 1) * 180.0 / (nlat + 1)
    return full_ring_grid(latd, np.arange(nlon) * 360.0 / nlon, name=f"full_clenshaw_{nlat_half}")


def full_gaussian_grid(nlat_half: int) -> Grid:
    """Full Gaussian grid: 2*nlat_half rings at the Gauss-Legendre latitudes,
    4*nlat_half points per ring from longitude 0."""
    nlat, nlon = 2 * nlat_half, 4 * nlat_half
    x, _ = np.polynomial.legendre.leggauss(nlat)
    latd = np.degrees(np.arcsin(x))[::-1]                             # north to south
    return full_ring_grid(latd, np.arange(nlon) * 360.0 / nlon, name=f"full_gaussian_{nlat_half}")


# ----------------------------------------------------------------- folded (tripolar) grids

def folded_lonlat(nx: int, ny: int, fold_lat: float, name: str = "") -> Grid:
    """A RightCenterFolded global grid with the geometry of a tripolar ocean
    grid's fold: ny-1 lon-lat rows from the south pole up to latitude
    ``fold_lat``, then a fold row whose top vertex row is its bottom row
    reversed, so that fold cells i and nx+1-i (1-based) are the same
    quadrilateral (a strip of the cap above ``fold_lat`` between two chords).
    Every physical cell of the fold row has two slots, as in the reference's
    folded Oceananigans grids (ext/ConservativeRegriddingOceananigansExt.jl:117-175)."""
    if nx % 4:
        raise ValueError("nx must be a multiple of 4")
    lon = np.linspace(0.0, 360.0, nx + 1)
    lat = np.linspace(-90.0, fold_lat, ny)
    LON, LAT = np.meshgrid(lon, lat)
    pts = unit_sphere_from_geographic(LON, LAT)           # (ny, nx+1, 3)
    top = pts[-1][::-1][None]                             # the fold: top row = bottom row reversed
    return Grid("curvilinear", SPHERICAL, blocks=[np.concatenate([pts, top], axis=0)], full_sphere=True,
                name=name or f"folded_{nx}x{ny}")


def fold_primaries(nx: int) -> np.ndarray:
    """1-based fold-row slots that keep the cells: 1..nx/4 and nx/2+1..nx/2+nx/4;
    slot r's partner is nx+1-r."""
    nq, nh = nx // 4, nx // 2
    return np.concatenate([np.arange(1, nq + 1), np.arange(nh + 1, nh + nq + 1)])


def fold_ghosts(g: Grid) -> Grid:
    """The per-cell polygons of a one-block RightCenterFolded grid with the
    fold-row partner slots made ghosts (0 vertices: no area, never a
    candidate), numbered like the grid (i + j*nx)."""
    if g.kind != "curvilinear" or len(g.blocks) != 1:
        raise ValueError("fold_ghosts takes a one-block curvilinear grid")
    t, _ = g.cell_table()
    ny1, nx1 = g.blocks[0].shape[:2]
    nx, ny = nx1 - 1, ny1 - 1
    if nx % 4:
        raise ValueError("nx must be a multiple of 4")
    nv = np.full(t.shape[0], t.shape[1], np.int32)
    keep = np.zeros(nx, bool)
    keep[fold_primaries(nx) - 1] = True
    nv[(ny - 1) * nx + np.flatnonzero(~keep)] = 0
    return Grid("cells", g.manifold, cells=t.copy(), nverts=nv, full_sphere=g.full_sphere, name=g.name + "_ghosts")


# ----------------------------------------------------------------- cubed sphere

def _cube_face(f: int, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    one = np.ones_like(a)
    if f == 0:
        v = (one, a, b)
    elif f == 1:
        v = (-a, one, b)
    elif f == 2:
        v = (-one, -a, b)
    elif f == 3:
        v = (a, -one, b)
    elif f == 4:
        v = (-b, a, one)
    else:
        v = (b, a, -one)
    p = np.stack(v, axis=-1)
    return p / np.linalg.norm(p, axis=-1, keepdims=True)


def cubed_sphere(ne: int, jitter: float = 0.0, seed: int = 0, name: str = "") -> Grid:
    """Equiangular gnomonic cubed sphere (Ronchi, Iacono & Paolucci 1996)
    with ne x ne cells per face; face f has cell offset f*ne^2 like the
    reference's ClimaCore adapter (ext/ConservativeRegriddingClimaCoreExt.jl:56-61).
    Cells are counter-clockwise seen from outside.  With ``jitter`` > 0 the
    face-interior vertices move by U(-jitter, jitter) cell widths in both
    face angles (shared face-edge vertices stay put)."""
    rng = np.random.default_rng(seed)
    t = np.linspace(-1.0, 1.0, ne + 1) * (np.pi / 4)
    blocks = []
    for f in range(6):
        A, B = np.meshgrid(t, t)  # (ne+1, ne+1): [j, i] -> alpha_i, beta_j
        if jitter > 0:
            h = (np.pi / 2) / ne
            ja = rng.uniform(-jitter, jitter, size=A.shape) * h
            jb = rng.uniform(-jitter, jitter, size=A.shape) * h
            ja[[0, -1], :] = 0.0
            ja[:, [0, -1]] = 0.0
            jb[[0, -1], :] = 0.0
            jb[:, [0, -1]] = 0.0
            A = A + ja
            B = B + jb
        blocks.append(_cube_face(f, np.tan(A), np.tan(B)))
    return Grid("curvilinear", SPHERICAL, blocks=blocks, full_sphere=True, name=name or f"cs_C{ne}")


# ----------------------------------------------------------------- HEALPix

_JRLL = np.array([2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4], np.int64)
_JPLL = np.array([1, 3, 5, 7, 0, 2, 4, 6, 1, 3, 5, 7], np.int64)


def _compact_bits(v: np.ndarray) -> np.ndarray:
    r = np.zeros_like(v)
    for b in range(31):
        r |= ((v >> (2 * b)) & 1) << b
    return r


def healpix_nest2xyf(nside: int, pix: np.ndarray):
    npface = nside * nside
    face = pix // npface
    ipf = pix % npface
    return _compact_bits(ipf), _compact_bits(ipf >> 1), face


def _hp_loc2vec(x: np.ndarray, y: np.ndarray, face: np.ndarray) -> np.ndarray:
    """Face coordinates (x, y) in [0, 1]^2 -> unit vectors (Gorski et al. 2005)."""
    jr = _JRLL[face] - x - y
    north = jr < 1.0
    south = jr > 3.0
    nr = np.where(north, jr, np.where(south, 4.0 - jr, 1.0))
    tmp = nr * nr / 3.0
    z = np.where(north, 1.0 - tmp, np.where(south, tmp - 1.0, (2.0 - jr) * 2.0 / 3.0))
    sth = np.where(north | south, np.sqrt(np.maximum(tmp * (2.0 - tmp), 0.0)),
                   np.sqrt(np.maximum((1.0 - z) * (1.0 + z), 0.0)))
    t = _JPLL[face] * nr + x - y
    t = np.where(t < 0, t + 8, t)
    t = np.where(t >= 8, t - 8, t)
    phi = np.where(nr < 1e-15, 0.0, (np.pi / 4) * t / np.where(nr < 1e-15, 1.0, nr))
    return np.stack([sth * np.cos(phi), sth * np.sin(phi), z], axis=-1)


def healpix_corners_nested(nside: int, pix: np.ndarray) -> np.ndarray:
    """Corners (N, W, S, E) of nested pixels ``pix``: shape (len(pix), 4, 3)."""
    pix = np.asarray(pix, np.int64)
    ix, iy, face = healpix_nest2xyf(nside, pix)
    ns = float(nside)
    c = [
        _hp_loc2vec((ix + 1) / ns, (iy + 1) / ns, face),
        _hp_loc2vec(ix / ns, (iy + 1) / ns, face),
        _hp_loc2vec(ix / ns, iy / ns, face),
        _hp_loc2vec((ix + 1) / ns, iy / ns, face),
    ]
    return np.stack(c, axis=1)


def healpix_nest2ring(nside: int, pix: np.ndarray) -> np.ndarray:
    pix = np.asarray(pix, np.int64)
    ix, iy, face = healpix_nest2xyf(nside, pix)
    nl4 = 4 * nside
    npix = 12 * nside * nside
    ncap = 2 * nside * (nside - 1)
    jr = _JRLL[face] * nside - ix - iy - 1
    north = jr < nside
    south = jr > 3 * nside
    nr = np.where(north, jr, np.where(south, nl4 - jr, nside))
    nbefore = np.where(north, 2 * nr * (nr - 1), np.where(south, npix - 2 * (nr + 1) * nr, ncap + (jr - nside) * nl4))
    kshift = np.where(north | south, 0, (jr - nside) & 1)
    jp = (_JPLL[face] * nr + ix - iy + 1 + kshift) // 2
    jp = np.where(jp > nl4, jp - nl4, jp)
    jp = np.where(jp < 1, jp + nl4, jp)
    return nbefore + jp - 1


def healpix_grid(nside: int, order: str = "nested", name: str = "") -> Grid:
    """HEALPix pixels as great-circle quadrilaterals through their 4 corners
    (N, W, S, E), indexed in nested or ring order like HealpixRootNode{O}
    (ext/ConservativeRegriddingHealpixExt.jl:154-169)."""
    if nside < 1 or (nside & (nside - 1)) != 0:
        raise ValueError("nside must be a power of two")
    npix = 12 * nside * nside
    nested = np.arange(npix, dtype=np.int64)
    corners = healpix_corners_nested(nside, nested)
    if order == "ring":
        ring = healpix_nest2ring(nside, nested)
        out = np.empty_like(corners)
        out[ring] = corners
        corners = out
    elif order != "nested":
        raise ValueError("order must be 'nested' or 'ring'")
    return Grid("cells", SPHERICAL, cells=corners, full_sphere=True, healpix=(nside, order == "nested"),
                name=name or f"healpix_{nside}_{order}")


# ----------------------------------------------------------------- polygons

def polygon_grid(polys, manifold: str = PLANAR, name: str = "") -> Grid:
    """Explicit convex polygons (FlatNoTree of the reference).  Each polygon
    is a sequence of vertices; a closing repeat of the first vertex is dropped."""
    dim = 3 if manifold == SPHERICAL else 2
    rings = []
    for p in polys:
        a = np.asarray(p, np.float64).reshape(-1, dim)
        if len(a) > 1 and np.array_equal(a[0], a[-1]):
            a = a[:-1]
        rings.append(a)
    maxv = max(len(r) for r in rings)
    if maxv > 8:
        raise ValueError("polygons with more than 8 vertices are not supported")
    cells = np.zeros((len(rings), maxv, dim))
    nv = np.zeros(len(rings), np.int32)
    for k, r in enumerate(rings):
        cells[k, : len(r)] = r
        cells[k, len(r):] = r[-1]
        nv[k] = len(r)
    return Grid("cells", manifold, cells=cells, nverts=nv, name=name)


def regular_grid(x: Sequence[float], y: Sequence[float], name: str = "") -> Grid:
    """Planar RegularGrid (src/trees/grids.jl:96-115) as a vertex matrix."""
    X, Y = np.meshgrid(np.asarray(x, np.float64), np.asarray(y, np.float64))
    return Grid("curvilinear", PLANAR, blocks=[np.stack([X, Y], axis=-1)], name=name)
