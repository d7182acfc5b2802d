"""Many regridders at once: ``build_batch`` (concurrent builds, crg_build_batch),
``regrid_batch_`` (concurrent applies, crg_apply_batch) and ``ApplyPlan`` (the
applies of a whole batch captured in one CUDA graph, crg_apply_plan_*).  The reference builds and applies one Regridder at a time
(src/regridder/regridder.jl:105-163, src/regridder/regrid.jl:63-118)."""
from __future__ import annotations

import ctypes as C
import weakref

from . import _lib
from ._lib import ArgumentError, DimensionMismatch, check
from .regridder import Regridder, _Field, _stream_ptr, as_grid, grid_desc, promote


def build_batch(pairs, normalize: bool = False, nthreads: int = 0) -> list:
    """Regridders for (dst, src) pairs, built concurrently by ``nthreads`` host
    threads (0: up to 8), each on its own stream."""
    pairs = [promote(as_grid(d), as_grid(s)) for d, s in pairs]
    n = len(pairs)
    if n == 0:
        return []
    dd = (_lib.crg_grid_desc * n)()
    ds = (_lib.crg_grid_desc * n)()
    keep = []
    for k, (d, s) in enumerate(pairs):
        dd[k], kd = grid_desc(d)
        ds[k], ks = grid_desc(s)
        keep += [kd, ks]
    out = (C.c_void_p * n)()
    opts = _lib.crg_build_opts(int(bool(normalize)), 0, None)
    check(_lib.load().crg_build_batch(n, dd, ds, C.byref(opts), int(nthreads), out))
    del keep
    return [Regridder._adopt(out[k]) for k in range(n)]


def _items(items, normalize, what):
    arr = (_lib.crg_apply_item * len(items))()
    keep = []
    for k, it in enumerate(items):
        dst, R, src = it[0], it[1], it[2]
        dims = it[3] if len(it) > 3 else 1
        if not isinstance(R, Regridder):
            raise ArgumentError(f"item {k}: expected a Regridder")
        fs, fd = _Field(src), _Field(dst)
        if what == "plan" and not (fs.torch and fs.cuda and fd.torch and fd.cuda):
            raise ArgumentError(f"item {k}: plan fields must be CUDA tensors")
        if fs.dtype != fd.dtype:
            raise ArgumentError(f"item {k}: source and destination dtypes differ")
        n_out, n_in = R.shape
        ssc, ssf, nf_s = _layout(fs, dims, n_in, k, "source")
        dsc, dsf, nf_d = _layout(fd, dims, n_out, k, "destination")
        if nf_s != nf_d:
            raise DimensionMismatch(f"item {k}: {nf_s} source fields but {nf_d} destination fields")
        arr[k] = _lib.crg_apply_item(R._h.ptr, int(R._transposed), fs.dtype, fs.ptr, ssc, ssf, fd.ptr, dsc, dsf,
                                     nf_s, int(bool(normalize)), 0)
        keep += [src, dst, R]
    return arr, keep


def regrid_batch_(items, normalize: bool = True, nthreads: int = 0, stream=None):
    """``regrid!`` for every item at once (crg_apply_batch): the applies run
    concurrently from ``nthreads`` host threads (0: 4), each on its own
    stream.  Items are ``(dst, R, src)`` or ``(dst, R, src, dims)`` with numpy
    arrays or torch tensors (host or CUDA; 1-D, or 2-D with the spatial axis
    ``dims``); outputs must not overlap.  With host fields the copies of the
    items share both directions of the host link; they are complete on return."""
    from .regridder import _resolve_stream

    if not items:
        return
    arr, keep = _items(items, normalize, "batch")
    fields = [_Field(x) for it in items for x in (it[0], it[2])]
    st = _resolve_stream(fields, stream)
    check(_lib.load().crg_apply_batch(len(items), arr, int(nthreads), C.c_void_p(st) if st else None))
    del keep


def _destroy(ptr):
    try:
        _lib.load(build_if_missing=False).crg_apply_plan_destroy(C.c_void_p(ptr))
    except Exception:
        pass


class ApplyPlan:
    """The applies ``regrid!(dst, R, src; dims)`` of a list of items captured
    once into a CUDA graph; ``launch()`` replays all of them with one launch.

    Items are ``(dst, R, src)`` or ``(dst, R, src, dims)`` with CUDA torch
    tensors: 1-D fields, or 2-D with the spatial axis ``dims`` (1: (cells,
    fields), the cell-major layout; 2: (fields, cells)).  ``R`` may be a
    transposed view.  Items run as parallel branches of the graph, so their
    outputs must not overlap.  The plan keeps the tensors alive and
    reads/writes them in place on every launch."""

    def __init__(self, items, normalize: bool = True):
        arr, self._keep = _items(items, normalize, "plan")
        p = C.c_void_p()
        check(_lib.load().crg_apply_plan_create(len(items), arr, C.byref(p)))
        self._p = p.value
        self._fin = weakref.finalize(self, _destroy, p.value)

    @property
    def info(self) -> dict:
        """``kernels``: kernel launches of one replay; ``batched_items``: the
        items run by the one persistent launch (the rest are their own applies)."""
        k, b = C.c_int64(), C.c_int64()
        check(_lib.load().crg_apply_plan_info(C.c_void_p(self._p), C.byref(k), C.byref(b)))
        return {"kernels": k.value, "batched_items": b.value}

    def launch(self, stream=None):
        import torch

        st = _stream_ptr(stream) if stream is not None else torch.cuda.current_stream().cuda_stream
        check(_lib.load().crg_apply_plan_launch(C.c_void_p(self._p), C.c_void_p(st) if st else None))


def _layout(f: _Field, dims, n, k, what):
    if len(f.shape) == 1:
        if f.shape[0] != n:
            raise DimensionMismatch(f"item {k}: {what} has {f.shape[0]} cells, expected {n}")
        return f.strides[0], 0, 1
    if len(f.shape) != 2 or dims not in (1, 2):
        raise ArgumentError(f"item {k}: plan fields are 1-D or 2-D with dims 1 or 2")
    cell_ax = dims - 1
    if f.shape[cell_ax] != n:
        raise DimensionMismatch(f"item {k}: {what} has {f.shape[cell_ax]} cells along dims={dims}, expected {n}")
    return f.strides[cell_ax], f.strides[1 - cell_ax], f.shape[1 - cell_ax]
