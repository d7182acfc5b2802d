"""Values of folded (tripolar, RightCenterFolded) destinations: after
regridding onto a grid whose fold-row partner slots are ghosts
(``grids.fold_ghosts``), ``mirror_fold_`` copies each primary's value into
its partner, as the reference's ``finalize_regridding!`` does for Oceananigans
fields (ext/ConservativeRegriddingOceananigansExt.jl:194-240)."""
from __future__ import annotations

import ctypes as C

from . import _lib
from ._lib import ArgumentError, check
from .regridder import _Field, _resolve_stream


def mirror_fold_(field, nx: int, ny: int, dims: int = 1, stream=None):
    """In place: field holds nx*ny cells (numbered i + j*nx) along the axis
    ``dims`` (1-based) and any number of fields along the other axis of a
    1-D or 2-D array; numpy or torch, host or CUDA."""
    f = _Field(field)
    if len(f.shape) == 1:
        sc, sf, nf = f.strides[0], 0, 1
        ncell = f.shape[0]
    elif len(f.shape) == 2 and dims in (1, 2):
        sc, sf, nf = f.strides[dims - 1], f.strides[2 - dims], f.shape[2 - dims]
        ncell = f.shape[dims - 1]
    else:
        raise ArgumentError("mirror_fold_ takes 1-D fields or 2-D fields with dims 1 or 2")
    if ncell != nx * ny:
        raise ArgumentError(f"the field has {ncell} cells along dims, the grid {nx} x {ny}")
    st = _resolve_stream([f], stream)
    check(_lib.load().crg_mirror_fold(f.dtype, C.c_void_p(f.ptr), sc, sf, nf, nx, ny, C.c_void_p(st) if st else None))
    return field
