"""Spectral-element (SE) spaces and the SE <-> FV regridders: the host mirror
of the reference's ClimaCore extension (ext/ConservativeRegriddingClimaCoreExt.jl).

``SpectralElementSpace(elements, nq)`` stands for a ClimaCore
SpectralElementSpace2D: quadrilateral elements (a spherical ``Grid`` whose
cells have 4 vertices, vertex k at reference corner (-1,-1), (1,-1), (1,1),
(-1,1)) with nq x nq Gauss-Lobatto-Legendre nodes each, placed by the
normalised bilinear element map.  An SE field is a flat vector of
nelem * nq^2 nodal values, element by element, i fastest
(se_field_to_vec, :368-370).

``Regridder(fv_grid, space)`` is the principled SE -> FV regridder
(se_to_fv_principled, :416-486) and ``Regridder(space, fv_grid)`` the FV -> SE
L2 projection (fv_to_se_l2_projection, :573-689); SE -> SE is rejected as in
the reference (:499-506).  ``regrid_field_(dst, R, src)`` is regrid! into an
SE field: the apply, then the weighted direct stiffness summation that
finalize_regridding! runs (:709-715).  All compute runs in ``libcrg_gb300.so``.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import ArgumentError, check
from .grids import SPHERICAL, Grid, cubed_sphere


class SpectralElementSpace:
    """Elements + GLL nodes per direction (ClimaCore ``n_quad_points``).

    ``node_weights`` (nelem * nq^2, ClimaCore's ``Spaces.weighted_jacobian``)
    may be given; otherwise they are J w_i w_j of the element map on a sphere
    of ``radius``."""

    def __init__(self, elements: Grid, nq: int, node_weights=None, radius: float = 1.0, name: str = ""):
        if not isinstance(elements, Grid) or elements.manifold != SPHERICAL:
            raise ArgumentError("SE elements must be a spherical Grid of quadrilaterals")
        if not 2 <= int(nq) <= 8:
            raise ArgumentError(f"nq = {nq} must be in 2..8")
        self.elements = elements
        self.nq = int(nq)
        self.radius = float(radius)
        self.name = name or f"se_{elements.name}_nq{nq}"
        self._weights_given = node_weights is not None
        self._weights = None if node_weights is None else np.ascontiguousarray(node_weights, np.float64)
        if self._weights is not None and self._weights.shape != (self.nnodes,):
            raise ArgumentError(f"node_weights must have {self.nnodes} entries")
        self._points = None
        self._groups = None
        self._dev = {}

    @classmethod
    def cubed_sphere(cls, ne: int, nq: int = 4, radius: float = 1.0, jitter: float = 0.0, seed: int = 0):
        """ClimaCore's CubedSphereSpace(h_elem = ne, n_quad_points = nq) on the
        equiangular cubed sphere, elements in face-major order (face offset
        (f - 1) ne^2, :56-61)."""
        return cls(cubed_sphere(ne, jitter=jitter, seed=seed), nq, radius=radius, name=f"se_C{ne}_nq{nq}")

    @property
    def nelem(self) -> int:
        return int(self.elements.ncells)

    @property
    def nnodes(self) -> int:
        return self.nelem * self.nq * self.nq

    # -- descriptors ---------------------------------------------------
    def _desc(self):
        from .regridder import grid_desc

        d = _lib.crg_se_space()
        gd, keep = grid_desc(self.elements)
        d.elements = gd
        d.nq = self.nq
        if self._weights_given:
            d.node_weights = self._weights.ctypes.data
            keep.append(self._weights)
        return d, keep

    def _opts(self, triangle_quad_degree: Optional[int] = None, stream=None):
        from .regridder import _stream_ptr

        return _lib.crg_se_opts(int(triangle_quad_degree or 0), 0, self.radius, _stream_ptr(stream))

    # -- nodes ---------------------------------------------------------
    def _nodes(self):
        lib = _lib.load()
        d, keep = self._desc()
        o = self._opts()
        pts = np.empty((self.nnodes, 3))
        w = np.empty(self.nnodes)
        check(lib.crg_se_nodes(C.byref(d), C.byref(o), pts.ctypes.data, w.ctypes.data))
        del keep
        self._points = pts
        if self._weights is None:
            self._weights = w

    def node_positions(self) -> np.ndarray:
        """Unit vectors of all nodes, (nnodes, 3) (se_node_positions, :139-145)."""
        if self._points is None:
            self._nodes()
        return self._points

    def node_weights(self) -> np.ndarray:
        """Weighted Jacobian of every node (se_node_weights, :153-156)."""
        if self._weights is None:
            self._nodes()
        return self._weights

    # -- direct stiffness summation -----------------------------------
    def dss_groups(self):
        """(group_ptr, group_nodes): the nodes that are the same point of the
        sphere (element edges and corners), groups of two or more copies,
        members ascending.  Copies are matched within 1e-9 (unit sphere)."""
        if self._groups is None:
            from scipy.spatial import cKDTree

            p = self.node_positions()
            parent = np.arange(len(p))

            def find(a):
                while parent[a] != a:
                    parent[a] = parent[parent[a]]
                    a = parent[a]
                return a

            for a, b in cKDTree(p).query_pairs(1e-9, output_type="ndarray"):
                ra, rb = find(a), find(b)
                if ra != rb:
                    parent[max(ra, rb)] = min(ra, rb)
            roots = np.array([find(a) for a in range(len(p))])
            order = np.lexsort((np.arange(len(p)), roots))
            r = roots[order]
            starts = np.flatnonzero(np.r_[True, r[1:] != r[:-1]])
            sizes = np.diff(np.r_[starts, len(r)])
            keep = sizes >= 2
            nodes = [order[s:s + n] for s, n in zip(starts[keep], sizes[keep])]
            ptr = np.zeros(len(nodes) + 1, np.int32)
            ptr[1:] = np.cumsum([len(n) for n in nodes])
            flat = np.concatenate(nodes).astype(np.int32) if nodes else np.zeros(0, np.int32)
            self._groups = (ptr, flat)
        return self._groups

    def _device_arrays(self, device):
        import torch

        key = str(device)
        if key not in self._dev:
            ptr, nodes = self.dss_groups()
            self._dev[key] = (torch.from_numpy(ptr).to(device), torch.from_numpy(nodes).to(device),
                              torch.from_numpy(self.node_weights()).to(device))
        return self._dev[key]

    def dss_(self, field, dims: int = 1, stream=None):
        """Weighted DSS in place (ClimaCore Spaces.weighted_dss!): the copies
        of a shared node all get sum(w f) / sum(w).  ``field`` holds the
        nnodes values along axis ``dims`` (1-based) of a 1-D or 2-D array;
        torch CUDA tensors run in place, numpy arrays go through the GPU."""
        import torch

        from .regridder import _Field, _resolve_stream

        if isinstance(field, np.ndarray):
            t = torch.from_numpy(np.ascontiguousarray(field)).cuda()
            self.dss_(t, dims, stream)
            field[...] = t.cpu().numpy()
            return field
        f = _Field(field)
        if not f.cuda:
            raise ArgumentError("dss_ takes numpy arrays or CUDA tensors")
        if len(f.shape) == 1:
            sn, sf, nf, n = f.strides[0], 0, 1, f.shape[0]
        elif len(f.shape) == 2 and dims in (1, 2):
            sn, sf, nf, n = f.strides[dims - 1], f.strides[2 - dims], f.shape[2 - dims], f.shape[dims - 1]
        else:
            raise ArgumentError("dss_ takes 1-D fields or 2-D fields with dims 1 or 2")
        if n != self.nnodes:
            raise ArgumentError(f"the field has {n} nodes along dims, the space {self.nnodes}")
        gptr, gnodes, w = self._device_arrays(field.device)
        st = _resolve_stream([f], stream)
        check(_lib.load().crg_se_dss(f.dtype, C.c_void_p(f.ptr), sn, sf, nf, C.c_void_p(gptr.data_ptr()),
                                     C.c_void_p(gnodes.data_ptr()), C.c_void_p(w.data_ptr()), len(gptr) - 1,
                                     C.c_void_p(st) if st else None))
        return field

    def __repr__(self):
        return f"SpectralElementSpace({self.nelem} elements, nq={self.nq})"


def build_se_regridder(dst, src, triangle_quad_degree: Optional[int] = None, stream=None) -> int:
    """crg_regridder* of an SE -> FV (src is the space) or FV -> SE (dst is
    the space) regridder; the caller adopts the reference."""
    from .regridder import as_grid, grid_desc

    lib = _lib.load()
    se_dst, se_src = isinstance(dst, SpectralElementSpace), isinstance(src, SpectralElementSpace)
    if se_dst and se_src:
        raise ArgumentError("SE → SE regridding is not supported. Use SE → FV → SE via two regridders.")
    space = dst if se_dst else src
    fv = as_grid(src if se_dst else dst)
    if fv.manifold != SPHERICAL:
        fv = fv.to_spherical()
    d, keep = space._desc()
    g, keep_g = grid_desc(fv)
    o = space._opts(triangle_quad_degree, stream)
    h = C.c_void_p()
    if se_dst:
        check(lib.crg_build_fv_to_se(C.byref(d), C.byref(g), C.byref(o), C.byref(h)))
    else:
        check(lib.crg_build_se_to_fv(C.byref(g), C.byref(d), C.byref(o), C.byref(h)))
    del keep, keep_g
    return h.value


def regrid_field_(dst, regridder, src, dims: int = 1, stream=None):
    """regrid! into an SE field: ``regrid_`` then, when the regridder's
    destination is an SE space, its weighted DSS (finalize_regridding!, :709-715)."""
    from .regridder import regrid_

    regrid_(dst, regridder, src, dims=dims, stream=stream)
    space = getattr(regridder, "dst_space", None)
    if space is not None:
        space.dss_(dst, dims=dims, stream=stream)
    return dst
