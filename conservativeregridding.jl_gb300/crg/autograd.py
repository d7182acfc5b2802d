"""torch.autograd forms of regridding: the Python counterparts of the
``ChainRulesCore.rrule`` methods of the Julia binding.  Import it as
``crg.autograd`` (``import crg`` alone does not load torch).

The reference has no derivatives (no ChainRulesCore dependency,
Project.toml:10-23).  Two differentiable functions are offered:

``regrid_ad(R, src, dims=1, normalize=True)``
    d = regrid(R, src) for a fixed regridder R (any dtype, layout and device
    ``regrid_`` takes).  Backward: src_bar = A' (d_bar ./ a_d) through the
    other stored copy of A (``crg_apply_adjoint``, no atomics).

``regrid_vertices_ad(s, dst_points, src_points, dst, src)``
    d = regrid(Regridder(dst(V), src(W)), s) as a function of the source
    field s and of the vertex coordinates V and W of both grids (FP64, one
    field).  The forward builds the regridder from the tensors' values;
    backward: s_bar by the adjoint apply, V_bar by ``crg_area_grad``, W_bar
    by ``crg_area_grad`` of the regridder built the other way round
    (``src_area_grad``).  Vertex arrays are laid out as the grids store
    them: (npoints, dim) in ``Grid.points_flat`` order for curvilinear
    grids, (ncells, max_verts, dim) for per-cell polygons; on the sphere the
    derivatives are with respect to the unit vectors' x, y, z (dot them with
    ``lonlat_tangents`` for angle derivatives; a step along them leaves the
    sphere, so renormalise moved vertices).
"""
from __future__ import annotations

import numpy as np

from ._lib import ArgumentError, DimensionMismatch
from .grad import regrid_pullback
from .grids import Grid
from .regridder import Regridder, regrid, regrid_, regrid_adjoint_

try:
    import torch
except ImportError:  # pragma: no cover - torch is a dependency of the host mirror
    torch = None


def _with_points(g: Grid, pts: np.ndarray) -> Grid:
    """The grid ``g`` with its vertex coordinates replaced by ``pts`` (laid
    out as described in the module docstring); topology and cell numbering
    are kept."""
    pts = np.ascontiguousarray(pts, np.float64)
    if g.kind == "curvilinear":
        n = sum(b.shape[0] * b.shape[1] for b in g.blocks)
        if pts.shape != (n, g.dim):
            raise DimensionMismatch(f"vertex array has shape {pts.shape}, expected {(n, g.dim)}")
        blocks, o = [], 0
        for b in g.blocks:
            m = b.shape[0] * b.shape[1]
            blocks.append(pts[o:o + m].reshape(b.shape))
            o += m
        return Grid("curvilinear", g.manifold, blocks=blocks, full_sphere=g.full_sphere, name=g.name)
    if pts.shape != g.cells.shape:
        raise DimensionMismatch(f"vertex array has shape {pts.shape}, expected {g.cells.shape}")
    return Grid("cells", g.manifold, cells=pts, nverts=g.nverts, full_sphere=g.full_sphere, name=g.name)


def grid_points(g: Grid) -> np.ndarray:
    """The vertex array of ``g`` in the layout ``regrid_vertices_ad`` takes (a copy)."""
    return np.array(g.points_flat() if g.kind == "curvilinear" else g.cells, np.float64)


if torch is not None:

    class RegridFunction(torch.autograd.Function):
        """d = regrid(R, src): forward ``crg_apply``, backward ``crg_apply_adjoint``."""

        @staticmethod
        def forward(ctx, src, R, dims, normalize):
            ctx.R, ctx.dims, ctx.normalize = R, dims, normalize
            ctx.src_shape = tuple(src.shape)
            return regrid(R, src.detach(), dims=dims, normalize=normalize)

        @staticmethod
        def backward(ctx, d_bar):
            if not ctx.needs_input_grad[0]:
                return None, None, None, None
            g = d_bar.contiguous()  # an expanded cotangent has zero strides
            s_bar = torch.empty(ctx.src_shape, dtype=g.dtype, device=g.device)
            regrid_adjoint_(s_bar, ctx.R, g, dims=ctx.dims, normalize=ctx.normalize)
            return s_bar, None, None, None

    class VertexRegridFunction(torch.autograd.Function):
        """d = regrid(Regridder(dst(V), src(W)), s) with cotangents of s, V and W."""

        @staticmethod
        def forward(ctx, s, V, W, dst, src, normalize):
            dst_g = _with_points(dst, V.detach().cpu().numpy())
            src_g = _with_points(src, W.detach().cpu().numpy())
            R = Regridder(dst_g, src_g, normalize=normalize)
            s_np = s.detach().cpu().numpy().astype(np.float64)
            d = np.zeros(R.shape[0])
            regrid_(d, R, s_np)
            ctx.state = (R, dst_g, src_g, s_np)
            ctx.like = [(t.device, t.dtype) for t in (s, V, W)]
            return torch.from_numpy(d).to(device=s.device, dtype=s.dtype)

        @staticmethod
        def backward(ctx, d_bar):
            R, dst_g, src_g, s_np = ctx.state
            need_s, need_v, need_w = ctx.needs_input_grad[:3]
            out = [None] * 6
            if not (need_s or need_v or need_w):
                return tuple(out)
            g = d_bar.detach().cpu().numpy().astype(np.float64)
            parts = regrid_pullback(R, dst_g, src_g, s_np, g, wrt_src=need_w)
            for k, need in enumerate((need_s, need_v, need_w)):
                if need:
                    device, dtype = ctx.like[k]
                    out[k] = torch.from_numpy(np.ascontiguousarray(parts[k])).to(device=device, dtype=dtype)
            return tuple(out)


def regrid_ad(R: Regridder, src, dims: int = 1, normalize: bool = True):
    """Differentiable ``regrid(R, src)`` for a torch tensor ``src`` (see the module docstring)."""
    if torch is None:
        raise RuntimeError("regrid_ad needs torch")
    return RegridFunction.apply(src, R, dims, normalize)


def regrid_vertices_ad(s, dst_points, src_points, dst: Grid, src: Grid, normalize: bool = True):
    """Differentiable d = regrid(Regridder(dst(V), src(W)), s) for FP64 torch
    tensors s (n_src,), V = dst_points and W = src_points (see the module
    docstring for their layout; ``grid_points`` gives a grid's own).  ``dst``
    and ``src`` give the topology and cell numbering; their own coordinates
    are not used.  Normalisation cancels in d, so ``normalize`` changes
    nothing but the regridder built on the way."""
    if torch is None:
        raise RuntimeError("regrid_vertices_ad needs torch")
    if dst.manifold != src.manifold:
        raise ArgumentError("regrid_vertices_ad takes two grids on the same manifold (promote them first)")
    return VertexRegridFunction.apply(s, dst_points, src_points, dst, src, normalize)
