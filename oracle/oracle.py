"""ctypes wrapper of the CPU oracle (crg_oracle.c).

TEST INFRASTRUCTURE ONLY: the oracle that tests/, the smoke check and the
CPU-baseline / reference legs of bench.py compare against.  The product library never uses it.

The oracle restates ConservativeRegridding.jl's build (treeify + threaded
dual DFS + per-pair clip/area + sparse()) and apply (stdlib CSC mul! then
./ areas); see the header of crg_oracle.c for the file:line citations.
Grids are described by the same arrays the product receives (objects with
the attributes of crg.grids.Grid: kind, manifold, blocks, cells, nverts,
full_sphere, healpix).
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "crg_oracle.c"
BUILD_DIR = HERE / "_build"
LIB = BUILD_DIR / "liboracle.so"
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> Path:
    stamp = BUILD_DIR / "stamp"
    fresh = (LIB.exists() and stamp.exists() and stamp.read_text() == platform.machine()
             and LIB.stat().st_mtime >= SRC.stat().st_mtime)
    if fresh and not force:
        return LIB
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    tmp = BUILD_DIR / "liboracle.so.tmp"
    cmd = ["gcc", *CFLAGS, str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(platform.machine())
    return LIB


class og_grid(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("manifold", C.c_int32), ("nblocks", C.c_int32), ("nested", C.c_int32),
        ("maxv", C.c_int32), ("full_sphere_root", C.c_int32), ("dim", C.c_int32), ("pad", C.c_int32),
        ("ncells", C.c_int64), ("nside", C.c_int64),
        ("block_nx", C.c_void_p), ("block_ny", C.c_void_p), ("block_point_off", C.c_void_p),
        ("block_cell_off", C.c_void_p), ("points", C.c_void_p), ("nverts", C.c_void_p), ("poly_verts", C.c_void_p),
    ]


_lock = threading.Lock()
_lib = None


def load() -> C.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = C.CDLL(str(LIB))
            vp, i64, i32, dbl = C.c_void_p, C.c_int64, C.c_int32, C.c_double
            sig = {
                "og_build": (vp, [C.POINTER(og_grid), C.POINTER(og_grid), C.c_int, C.c_int, C.c_int]),
                "og_nnz": (i64, [vp]), "og_ncand": (i64, [vp]), "og_overflows": (i64, [vp]),
                "og_get_csc": (None, [vp, vp, vp, vp]),
                "og_get_areas": (None, [vp, vp, vp]),
                "og_free": (None, [vp]),
                "og_apply": (None, [vp, C.c_int, vp, i64, i64, vp, i64, i64, i64, C.c_int, C.c_int]),
                "og_apply_f32": (None, [vp, C.c_int, vp, i64, i64, vp, i64, i64, i64, C.c_int, C.c_int]),
                "og_candidates": (i64, [C.POINTER(og_grid), C.POINTER(og_grid), C.c_int, C.c_int, C.POINTER(vp)]),
                "og_free_buffer": (None, [vp]),
                "og_pair_area_hook": (dbl, [C.c_int, vp, C.c_int, vp, C.c_int, C.POINTER(C.c_int)]),
                "og_cell_area_hook": (dbl, [C.c_int, vp, C.c_int]),
                "og_atan2": (dbl, [dbl, dbl]),
                "og_healpix_corners": (None, [i64, i64, vp]),
                "og_healpix_nest2ring": (i64, [i64, i64]),
                "og_num_threads": (C.c_int, []),
                "og_build_se": (vp, [C.POINTER(og_grid), C.POINTER(og_grid), C.c_int, C.c_int, dbl, vp, C.c_int,
                                     C.c_int, C.c_int, C.POINTER(C.c_int)]),
                "og_se_gll": (None, [C.c_int, vp, vp]),
                "og_se_tri_rule": (C.c_int, [C.c_int, vp, vp]),
                "og_se_lagrange_hook": (None, [C.c_int, dbl, vp]),
                "og_se_inverse_hook": (None, [vp, vp, vp]),
                "og_se_nodes_hook": (None, [vp, C.c_int, dbl, vp, vp]),
                "og_se_poly_b_hook": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int, vp]),
                "og_area_grad": (i64, [vp, C.POINTER(og_grid), C.POINTER(og_grid), vp, vp, vp, vp]),
                "og_det3_sign_hook": (C.c_int, [vp, vp, vp]),
                "og_orient2_sign_hook": (C.c_int, [dbl, dbl, dbl, dbl, dbl, dbl]),
            }
            for n, (r, a) in sig.items():
                f = getattr(lib, n)
                f.restype = r
                f.argtypes = a
            _lib = lib
        return _lib


def _desc(g):
    d = og_grid()
    keep = []
    d.manifold = 1 if g.manifold == "spherical" else 0
    d.dim = 3 if d.manifold == 1 else 2
    d.ncells = g.ncells
    d.full_sphere_root = int(bool(g.full_sphere))
    if g.kind == "curvilinear":
        shapes = [(b.shape[1] - 1, b.shape[0] - 1) for b in g.blocks]
        nx = np.array([s[0] for s in shapes], np.int64)
        ny = np.array([s[1] for s in shapes], np.int64)
        npts = np.array([(a + 1) * (b + 1) for a, b in shapes], np.int64)
        poff = np.concatenate([[0], np.cumsum(npts)[:-1]]).astype(np.int64)
        coff = np.concatenate([[0], np.cumsum(nx * ny)[:-1]]).astype(np.int64)
        pts = np.ascontiguousarray(np.concatenate([b.reshape(-1, d.dim) for b in g.blocks]), np.float64)
        keep += [nx, ny, poff, coff, pts]
        d.kind = 0
        d.nblocks = len(shapes)
        d.block_nx, d.block_ny = nx.ctypes.data, ny.ctypes.data
        d.block_point_off, d.block_cell_off = poff.ctypes.data, coff.ctypes.data
        d.points = pts.ctypes.data
    else:
        cells = np.ascontiguousarray(g.cells, np.float64)
        keep.append(cells)
        d.maxv = cells.shape[1]
        d.poly_verts = cells.ctypes.data
        if g.nverts is not None:
            nv = np.ascontiguousarray(g.nverts, np.int32)
            keep.append(nv)
            d.nverts = nv.ctypes.data
        if getattr(g, "healpix", None):
            d.kind = 1
            d.nside = int(g.healpix[0])
            d.nested = int(bool(g.healpix[1]))
        else:
            d.kind = 2
    return d, keep


class OracleRegridder:
    """CPU restatement of Regridder(dst, src; normalize) with its matrix and areas."""

    def __init__(self, dst, src, normalize=False, use_tree=True, nthreads=0):
        lib = load()
        dd, k1 = _desc(dst)
        ds, k2 = _desc(src)
        self._h = lib.og_build(C.byref(dd), C.byref(ds), int(bool(normalize)), int(bool(use_tree)), int(nthreads))
        self.nd, self.ns = dst.ncells, src.ncells
        self.nnz = lib.og_nnz(self._h)
        self.ncand = lib.og_ncand(self._h)
        self.overflows = lib.og_overflows(self._h)
        self.colptr = np.empty(self.ns + 1, np.int64)
        self.rowval = np.empty(max(self.nnz, 1), np.int64)
        self.nzval = np.empty(max(self.nnz, 1), np.float64)
        lib.og_get_csc(self._h, self.colptr.ctypes.data, self.rowval.ctypes.data, self.nzval.ctypes.data)
        self.rowval = self.rowval[: self.nnz]
        self.nzval = self.nzval[: self.nnz]
        self.dst_areas = np.empty(self.nd)
        self.src_areas = np.empty(self.ns)
        lib.og_get_areas(self._h, self.dst_areas.ctypes.data, self.src_areas.ctypes.data)
        del k1, k2

    def __del__(self):
        if getattr(self, "_h", None):
            load().og_free(self._h)
            self._h = None

    @property
    def intersections(self):
        import scipy.sparse as sp

        return sp.csc_matrix((self.nzval, self.rowval, self.colptr), shape=(self.nd, self.ns))

    def apply(self, src, transpose=False, normalize=True, nthreads=0):
        """Fields as (nfields, n) C-contiguous float64 (one field per row)."""
        src = np.ascontiguousarray(src, np.float64)
        one = src.ndim == 1
        s2 = src.reshape(1, -1) if one else src
        nout = self.ns if transpose else self.nd
        out = np.empty((s2.shape[0], nout))
        load().og_apply(self._h, int(transpose), s2.ctypes.data, 1, s2.shape[1], out.ctypes.data, 1, nout,
                        s2.shape[0], int(bool(normalize)), int(nthreads))
        return out[0] if one else out

    def apply_f32(self, src, transpose=False, normalize=True, nthreads=0, out=None):
        """The same on float32 fields (nfields, n), as the reference's regrid!
        runs on Float32 arrays: products and sums in float64, every stored
        value rounded to float32."""
        src = np.ascontiguousarray(src, np.float32)
        one = src.ndim == 1
        s2 = src.reshape(1, -1) if one else src
        nout = self.ns if transpose else self.nd
        if out is None:
            out = np.empty((s2.shape[0], nout), np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.shape == (s2.shape[0], nout)
        load().og_apply_f32(self._h, int(transpose), s2.ctypes.data, 1, s2.shape[1], out.ctypes.data, 1, nout,
                            s2.shape[0], int(bool(normalize)), int(nthreads))
        return out[0] if one else out


def area_grad(R: OracleRegridder, dst, src, row_weight=None, src_field=None, area_weight=None) -> np.ndarray:
    """Forward-mode (dual-number) derivatives through the oracle's own clip
    and area: sum_ij row_weight[i] src_field[j] dA_ij/dV + sum_i area_weight[i]
    da_i/dV over the destination vertices V of the grids R was built from
    (unnormalised areas), laid out like the library's crg_area_grad: (npoints,
    dim) in block order for curvilinear grids, (ncells, max_verts, dim) for
    polygon grids."""
    lib = load()
    dd, k1 = _desc(dst)
    ds, k2 = _desc(src)
    vec = lambda x, n: None if x is None else np.ascontiguousarray(x, np.float64).reshape(n)
    u, s, c = vec(row_weight, R.nd), vec(src_field, R.ns), vec(area_weight, R.nd)
    if (u is None) != (s is None):
        raise ValueError("row_weight and src_field are given together")
    if dst.kind == "curvilinear":
        out = np.empty((sum(b.shape[0] * b.shape[1] for b in dst.blocks), dd.dim))
    else:
        out = np.empty(np.asarray(dst.cells).shape)
    ptr = lambda a: None if a is None else a.ctypes.data
    ovf = lib.og_area_grad(R._h, C.byref(dd), C.byref(ds), ptr(u), ptr(s), ptr(c), out.ctypes.data)
    del k1, k2
    if ovf:
        raise RuntimeError(f"{ovf} clips overflowed")
    return out


def candidates(dst, src, use_tree=True, nthreads=0) -> np.ndarray:
    """Candidate pairs (src cell, dst cell) from the dual tree search."""
    lib = load()
    dd, k1 = _desc(dst)
    ds, k2 = _desc(src)
    p = C.c_void_p()
    n = lib.og_candidates(C.byref(dd), C.byref(ds), int(bool(use_tree)), int(nthreads), C.byref(p))
    arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int64)), shape=(max(n, 1) * 2,)).copy()[: 2 * n]
    lib.og_free_buffer(p)
    del k1, k2
    return arr.reshape(-1, 2)


def pair_area(s, d, spherical=True) -> float:
    s = np.ascontiguousarray(s, np.float64)
    d = np.ascontiguousarray(d, np.float64)
    ovf = C.c_int(0)
    a = load().og_pair_area_hook(int(spherical), s.ctypes.data, len(s), d.ctypes.data, len(d), C.byref(ovf))
    if ovf.value:
        raise RuntimeError("clip capacity overflow")
    return a


def cell_area(v, spherical=True) -> float:
    v = np.ascontiguousarray(v, np.float64)
    return load().og_cell_area_hook(int(spherical), v.ctypes.data, len(v))


def det3_sign(a, b, c) -> int:
    """Exact sign of det[a; b; c] (the clip's side test of c against the
    great circle through a and b, decided by error-free expansions)."""
    a, b, c = (np.ascontiguousarray(v, np.float64) for v in (a, b, c))
    return load().og_det3_sign_hook(a.ctypes.data, b.ctypes.data, c.ctypes.data)


def orient2_sign(a, b, v) -> int:
    """Exact sign of (b - a) x (v - a) on the plane."""
    return load().og_orient2_sign_hook(float(a[0]), float(a[1]), float(b[0]), float(b[1]), float(v[0]), float(v[1]))


def atan2(y, x) -> float:
    return load().og_atan2(float(y), float(x))


def healpix_corners(nside, pix) -> np.ndarray:
    out = np.empty(12)
    load().og_healpix_corners(int(nside), int(pix), out.ctypes.data)
    return out.reshape(4, 3)


def healpix_nest2ring(nside, pix) -> int:
    return load().og_healpix_nest2ring(int(nside), int(pix))


# ----------------------------------------------------------------- spectral elements

class OracleSERegridder(OracleRegridder):
    """CPU restatement of the ClimaCore extension's regridders: SE -> FV
    (se_is_dst False: ``fv`` is the destination) or FV -> SE (se_is_dst True),
    on the element grid ``elements`` with nq GLL nodes per direction."""

    def __init__(self, fv, elements, nq, se_is_dst, degree=0, radius=1.0, node_weights=None, use_tree=True,
                 nthreads=0):
        lib = load()
        df, k1 = _desc(fv)
        de, k2 = _desc(elements)
        w = None if node_weights is None else np.ascontiguousarray(node_weights, np.float64)
        err = C.c_int(0)
        self._h = lib.og_build_se(C.byref(df), C.byref(de), int(nq), int(degree), float(radius),
                                  None if w is None else w.ctypes.data, int(bool(se_is_dst)), int(bool(use_tree)),
                                  int(nthreads), C.byref(err))
        if not self._h:
            raise RuntimeError({1: "bad argument", 2: "clip capacity overflow", 3: "singular mass matrix"}
                               .get(err.value, "error"))
        nn = elements.ncells * nq * nq
        self.nd, self.ns = (nn, fv.ncells) if se_is_dst else (fv.ncells, nn)
        self.nnz = lib.og_nnz(self._h)
        self.ncand = lib.og_ncand(self._h)
        self.overflows = 0
        self.colptr = np.empty(self.ns + 1, np.int64)
        self.rowval = np.empty(max(self.nnz, 1), np.int64)
        self.nzval = np.empty(max(self.nnz, 1), np.float64)
        lib.og_get_csc(self._h, self.colptr.ctypes.data, self.rowval.ctypes.data, self.nzval.ctypes.data)
        self.rowval = self.rowval[: self.nnz]
        self.nzval = self.nzval[: self.nnz]
        self.dst_areas = np.empty(self.nd)
        self.src_areas = np.empty(self.ns)
        lib.og_get_areas(self._h, self.dst_areas.ctypes.data, self.src_areas.ctypes.data)
        del k1, k2


def se_gll(n):
    """GLL nodes and weights on [-1, 1] (n points)."""
    x, w = np.empty(n), np.empty(n)
    load().og_se_gll(int(n), x.ctypes.data, w.ctypes.data)
    return x, w


def se_tri_rule(degree):
    """Barycentric points (n, 3) and weights (summing to 1) of the triangle rule."""
    tl, tw = np.empty((16, 3)), np.empty(16)
    n = load().og_se_tri_rule(int(degree), tl.ctypes.data, tw.ctypes.data)
    if n < 0:
        raise ValueError(f"no triangle rule of degree {degree}")
    return tl[:n].copy(), tw[:n].copy()


def se_lagrange(nq, t):
    phi = np.empty(nq)
    load().og_se_lagrange_hook(int(nq), float(t), phi.ctypes.data)
    return phi


def se_inverse(corners, x):
    """(xi, eta) of the unit vector x in the element with corners (4, 3)."""
    c = np.ascontiguousarray(corners, np.float64)
    xv = np.ascontiguousarray(x, np.float64)
    out = np.empty(2)
    load().og_se_inverse_hook(c.ctypes.data, xv.ctypes.data, out.ctypes.data)
    return out[0], out[1]


def se_nodes(corners, nq, radius=1.0):
    """Node positions (nq^2, 3) and weighted Jacobians (nq^2) of one element."""
    c = np.ascontiguousarray(corners, np.float64)
    pts, wj = np.empty((nq * nq, 3)), np.empty(nq * nq)
    load().og_se_nodes_hook(c.ctypes.data, int(nq), float(radius), pts.ctypes.data, wj.ctypes.data)
    return pts, wj


def se_poly_b(corners, poly, nq, degree=0):
    """b[i + j nq] = integral over the polygon of phi_i(xi) phi_j(eta) (unit sphere)."""
    c = np.ascontiguousarray(corners, np.float64)
    p = np.ascontiguousarray(poly, np.float64)
    B = np.empty(nq * nq)
    if load().og_se_poly_b_hook(c.ctypes.data, p.ctypes.data, len(p), int(nq), int(degree), B.ctypes.data) != 0:
        raise ValueError("bad polygon or rule")
    return B
