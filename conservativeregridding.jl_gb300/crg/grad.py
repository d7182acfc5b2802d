"""Derivatives of regridding: the pullback of ``regrid!`` with respect to the
source field and to the vertices of the destination and source grids.

The reference has no derivatives (no ChainRulesCore dependency,
Project.toml:10-23); this is the host side of ``crg_apply_adjoint`` and
``crg_area_grad``, shaped as the pieces a ``ChainRulesCore.rrule`` for
``regrid!`` / ``Regridder`` needs.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import ArgumentError, DimensionMismatch, check
from .grids import Grid
from .regridder import Regridder, _stream_ptr, as_grid, grid_desc, promote, regrid_, regrid_adjoint_


def _vec(x, n, name):
    if x is None:
        return None
    a = np.ascontiguousarray(x, np.float64)
    if a.shape != (n,):
        raise DimensionMismatch(f"{name} has shape {a.shape}, expected ({n},)")
    return a


def area_grad(R: Regridder, dst, src, row_weight=None, src_field=None, area_weight=None, stream=None) -> np.ndarray:
    """sum_ij row_weight[i] src_field[j] dA_ij/dV + sum_i area_weight[i] da_i/dV for
    the unnormalised intersection areas A and destination cell areas a, with
    respect to the destination vertices V of the grids R was built from.

    Returns an array laid out like the destination vertices: (npoints, dim) in
    ``Grid.points_flat`` order for curvilinear grids (corners shared by cells
    accumulate), (ncells, max_verts, dim) for per-cell polygons; dim is 3 on
    the sphere (derivatives with respect to the unit vector's x, y, z) and 2 on
    the plane."""
    if R._transposed:
        raise ArgumentError("area_grad takes the forward regridder (dst <- src), not a transposed view")
    dst_g, src_g = promote(as_grid(dst), as_grid(src))
    nd, ns = R.info["n_dst"], R.info["n_src"]
    u = _vec(row_weight, nd, "row_weight")
    s = _vec(src_field, ns, "src_field")
    c = _vec(area_weight, nd, "area_weight")
    if (u is None) != (s is None):
        raise ArgumentError("row_weight and src_field are given together")
    dd, keep_d = grid_desc(dst_g)
    ds, keep_s = grid_desc(src_g)
    if dst_g.kind == "curvilinear":
        out = np.empty((len(dst_g.points_flat()), dst_g.dim))
    else:
        out = np.empty(np.asarray(dst_g.cells).shape)
    ptr = lambda a: None if a is None else a.ctypes.data
    check(_lib.load().crg_area_grad(C.c_void_p(R._h.ptr), C.byref(dd), C.byref(ds), ptr(u), ptr(s), ptr(c),
                                    out.ctypes.data, _stream_ptr(stream)))
    del keep_d, keep_s
    return out


def src_area_grad(dst, src, row_weight, src_field, swapped: Regridder = None, stream=None) -> np.ndarray:
    """sum_ij row_weight[i] src_field[j] dA_ij/dW with respect to the SOURCE
    vertices W, laid out like the source vertices (as :func:`area_grad` lays
    out the destination ones).

    A_ij is the area of (destination cell i) ∩ (source cell j), a symmetric
    function of the two cells, so this is :func:`area_grad` of the regridder
    built the other way round -- ``Regridder(src, dst)``, whose destination
    grid is this source grid -- with the two weight vectors exchanged.  Pass
    that regridder as ``swapped`` to reuse it; otherwise one is built (an
    unnormalised one: the derivative is of the unnormalised areas).  The
    source cell areas never enter ``regrid!``'s forward result, so there is
    no area term."""
    dst_g, src_g = promote(as_grid(dst), as_grid(src))
    Rs = Regridder(src_g, dst_g, stream=stream) if swapped is None else swapped
    if Rs._transposed or Rs.shape != (src_g.ncells, dst_g.ncells):
        raise DimensionMismatch(f"the swapped regridder has size {Rs.shape}, expected {(src_g.ncells, dst_g.ncells)}")
    return area_grad(Rs, src_g, dst_g, row_weight=src_field, src_field=row_weight, stream=stream)


def split_points(g: Grid, flat: np.ndarray) -> list:
    """Per-block (ny+1, nx+1, dim) views of a (npoints, dim) vertex array."""
    out, o = [], 0
    for b in g.blocks:
        n = b.shape[0] * b.shape[1]
        out.append(flat[o:o + n].reshape(b.shape[0], b.shape[1], -1))
        o += n
    return out


def regrid_pullback(R: Regridder, dst, src, src_field, dst_bar, wrt_src: bool = False, swapped: Regridder = None):
    """Pullback of d = regrid(R, s) = (A s) ./ a at s = src_field for the output
    cotangent dst_bar: returns (s_bar, V_bar), s_bar = A' (dst_bar ./ a) (the
    adjoint apply) and V_bar the cotangent of the destination vertices laid
    out as in :func:`area_grad`.  With ``wrt_src=True`` it returns
    (s_bar, V_bar, W_bar), W_bar the cotangent of the source vertices
    (:func:`src_area_grad`; ``swapped`` = ``Regridder(src, dst)`` if one is
    at hand).  Normalisation cancels in d, so the derivatives are those of
    the unnormalised areas whether R is normalised or not.  FP64, one field."""
    if R._transposed:
        raise ArgumentError("regrid_pullback takes the forward regridder (dst <- src), not a transposed view")
    nd, ns = R.info["n_dst"], R.info["n_src"]
    s = _vec(src_field, ns, "src_field")
    g = _vec(dst_bar, nd, "dst_bar")
    d = np.zeros(nd)
    regrid_(d, R, s)
    s_bar = np.zeros(ns)
    regrid_adjoint_(s_bar, R, g)
    a = R.dst_areas * (R.info["normalizer"] if R.info["normalized"] else 1.0)
    u = g / a
    v_bar = area_grad(R, dst, src, u, s, -g * d / a)
    if not wrt_src:
        return s_bar, v_bar
    return s_bar, v_bar, src_area_grad(dst, src, u, s, swapped=swapped)


def lonlat_tangents(points: np.ndarray):
    """d(x, y, z)/d(longitude) and d(x, y, z)/d(latitude), per degree, at unit
    vectors ``points`` (n, 3): the chain rule from vertex-coordinate
    derivatives to longitude/latitude derivatives is a dot product with these.
    At the poles the longitude tangent is zero and the latitude tangent is
    taken along longitude 0."""
    p = np.asarray(points, np.float64)
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    rho = np.hypot(x, y)
    k = np.pi / 180.0
    cl = np.where(rho > 0, x / np.where(rho > 0, rho, 1.0), 1.0)
    sl = np.where(rho > 0, y / np.where(rho > 0, rho, 1.0), 0.0)
    t_lon = k * np.stack([-y, x, np.zeros_like(z)], axis=1)
    t_lat = k * np.stack([-z * cl, -z * sl, rho], axis=1)
    return t_lon, t_lat
