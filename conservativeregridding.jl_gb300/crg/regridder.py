"""Host-side mirror of ConservativeRegridding.jl's regridding API.

``Regridder(dst, src, normalize=False)`` builds the sparse intersection-area
matrix on the GPU (Regridder(dst, src; normalize), src/regridder/regridder.jl:105-163),
``regrid_(dst, R, src, dims=1, normalize=True)`` is ``regrid!``
(src/regridder/regrid.jl:63-118, N-D slicing :225-318) and
``R.transpose()`` is ``transpose(R)`` (src/regridder/regridder.jl:49-50):
a view that shares the device matrices, swaps the area vectors and swaps the
temporary vectors.  All compute runs in ``libcrg_gb300.so``; numpy arrays and
torch tensors (host or CUDA) are accepted as fields.
"""
from __future__ import annotations

import ctypes as C
import weakref
from typing import Optional

import numpy as np

from . import _lib
from ._lib import ArgumentError, DimensionMismatch, check
from .grids import PLANAR, SPHERICAL, Grid, polygon_grid

# crg_info fields holding [forward, transpose] pairs
_PAIR_FIELDS = ("merge_tasks", "cut_rows", "carry_slots", "empty_rows")


# ----------------------------------------------------------------- grid -> descriptor

def as_grid(x) -> Grid:
    """Accept a Grid, a point matrix of shape (ny+1, nx+1, 2|3) or a list of polygons."""
    if isinstance(x, Grid):
        return x
    if isinstance(x, np.ndarray) and x.ndim == 3 and x.shape[-1] in (2, 3):
        return Grid("curvilinear", SPHERICAL if x.shape[-1] == 3 else PLANAR, blocks=[x])
    if isinstance(x, (list, tuple)):
        return polygon_grid(x, PLANAR)
    raise ArgumentError(f"cannot turn {type(x).__name__} into a grid")


def grid_desc(g: Grid):
    """crg_grid_desc for a Grid plus the arrays that must stay alive."""
    d = _lib.crg_grid_desc()
    keep = []
    d.manifold = _lib.CRG_SPHERICAL if g.manifold == SPHERICAL else _lib.CRG_PLANAR
    d.ncells = g.ncells
    if g.kind == "curvilinear":
        nx = np.array([s[0] for s in g.block_shapes], np.int64)
        ny = np.array([s[1] for s in g.block_shapes], np.int64)
        pts = np.ascontiguousarray(g.points_flat())
        keep += [nx, ny, pts]
        d.kind = _lib.CRG_GRID_CURVILINEAR
        d.nblocks = len(g.blocks)
        d.block_nx = nx.ctypes.data_as(C.POINTER(C.c_int64))
        d.block_ny = ny.ctypes.data_as(C.POINTER(C.c_int64))
        d.points = pts.ctypes.data
    else:
        cells = np.ascontiguousarray(g.cells)
        keep.append(cells)
        d.kind = _lib.CRG_GRID_CELLS
        d.max_verts = cells.shape[1]
        d.cell_verts = cells.ctypes.data
        if g.nverts is not None:
            nv = np.ascontiguousarray(g.nverts, np.int32)
            keep.append(nv)
            d.cell_nverts = nv.ctypes.data
    return d, keep


def promote(dst: Grid, src: Grid):
    """Mixed planar/spherical inputs are promoted to the sphere
    (src/regridder/regridder.jl:109-117): planar coordinates are (lon, lat) degrees."""
    if dst.manifold != src.manifold:
        return dst.to_spherical(), src.to_spherical()
    return dst, src


class _Handle:
    """Reference-counted owner of one crg_regridder*."""

    def __init__(self, ptr: int):
        self.ptr = ptr
        self._fin = weakref.finalize(self, _release, ptr)


def _release(ptr):
    try:
        _lib.load(build_if_missing=False).crg_regridder_release(C.c_void_p(ptr))
    except Exception:
        pass


# ----------------------------------------------------------------- Regridder

class Regridder:
    """Sparse conservative regridder from ``src`` cells to ``dst`` cells.

    Attributes mirror the reference struct (src/regridder/regridder.jl:25-36):
    ``intersections`` (the nd x ns area matrix, a scipy.sparse CSC copy made
    on first access), ``dst_areas``, ``src_areas``, ``dst_temp``, ``src_temp``.
    """

    def __init__(self, dst, src, normalize: bool = False, stream=None, *, triangle_quad_degree=None, _view=None):
        if _view is not None:
            self.__dict__.update(_view)
            return
        from .se import SpectralElementSpace, build_se_regridder

        if isinstance(dst, SpectralElementSpace) or isinstance(src, SpectralElementSpace):
            # the ClimaCore methods take no normalize (ext/ConservativeRegriddingClimaCoreExt.jl:416-506)
            self._adopt_handle(build_se_regridder(dst, src, triangle_quad_degree, stream))
            self.dst_space = dst if isinstance(dst, SpectralElementSpace) else None
            self.src_space = src if isinstance(src, SpectralElementSpace) else None
            return
        lib = _lib.load()
        dst_g, src_g = promote(as_grid(dst), as_grid(src))
        dd, keep_d = grid_desc(dst_g)
        ds, keep_s = grid_desc(src_g)
        opts = _lib.crg_build_opts(int(bool(normalize)), 0, _stream_ptr(stream))
        h = C.c_void_p()
        check(lib.crg_build(C.byref(dd), C.byref(ds), C.byref(opts), C.byref(h)))
        del keep_d, keep_s
        self._adopt_handle(h.value)

    @classmethod
    def _adopt(cls, ptr: int) -> "Regridder":
        """Wrap a crg_regridder* whose one reference passes to the wrapper."""
        self = cls.__new__(cls)
        self._adopt_handle(ptr)
        return self

    def _adopt_handle(self, ptr: int):
        lib = _lib.load()
        self._h = _Handle(ptr)
        self.dst_space = self.src_space = None
        self._transposed = False
        info = _lib.crg_info()
        check(lib.crg_regridder_info(C.c_void_p(ptr), C.byref(info)))
        self.info = {k: (list(getattr(info, k)) if k in _PAIR_FIELDS else getattr(info, k))
                     for k, _ in _lib.crg_info._fields_ if k != "pad"}
        self._csc = [None]  # shared caches with transposed views
        self._areas = [None]
        self._temps = [None]

    # -- R.dst_areas / R.src_areas (copied from the device on first use) --
    def _area_pair(self):
        if self._areas[0] is None:
            lib = _lib.load()
            d = np.empty(self.info["n_dst"])
            s = np.empty(self.info["n_src"])
            check(lib.crg_get_areas(C.c_void_p(self._h.ptr), d.ctypes.data, s.ctypes.data))
            self._areas[0] = (d, s)
        return self._areas[0]

    # -- R.dst_temp / R.src_temp: the reference struct's work vectors, made on
    # first use (two host vectors of the grids' sizes; zeroing them on every
    # build cost more than a millisecond for a million cells) --
    def _temp_pair(self):
        if self._temps[0] is None:
            self._temps[0] = (np.zeros(self.info["n_dst"]), np.zeros(self.info["n_src"]))
        return self._temps[0]

    @property
    def dst_temp(self) -> np.ndarray:
        return self._temp_pair()[1 if self._transposed else 0]

    @property
    def src_temp(self) -> np.ndarray:
        return self._temp_pair()[0 if self._transposed else 1]

    @property
    def dst_areas(self) -> np.ndarray:
        return self._area_pair()[1 if self._transposed else 0]

    @property
    def src_areas(self) -> np.ndarray:
        return self._area_pair()[0 if self._transposed else 1]

    # -- shape ---------------------------------------------------------
    @property
    def shape(self):
        nd, ns = self.info["n_dst"], self.info["n_src"]
        return (ns, nd) if self._transposed else (nd, ns)

    def size(self, dim: Optional[int] = None):
        return self.shape if dim is None else self.shape[dim - 1]

    @property
    def nnz(self) -> int:
        return int(self.info["nnz"])

    # -- transpose(R) --------------------------------------------------
    def transpose(self) -> "Regridder":
        """Regridder for the backwards direction, sharing all arrays
        (src/regridder/regridder.jl:46-50)."""
        lib = _lib.load()
        check(lib.crg_regridder_retain(C.c_void_p(self._h.ptr)))
        view = dict(self.__dict__)
        view["_h"] = _Handle(self._h.ptr)
        view["_transposed"] = not self._transposed
        view["dst_space"], view["src_space"] = self.src_space, self.dst_space
        return Regridder(None, None, _view=view)

    @property
    def T(self) -> "Regridder":
        return self.transpose()

    # -- R.intersections ----------------------------------------------
    @property
    def intersections(self):
        """A (nd x ns) as scipy.sparse.csc_matrix; its transpose for a transposed view."""
        import scipy.sparse as sp

        if self._csc[0] is None:
            lib = _lib.load()
            nd, ns, nnz = self.info["n_dst"], self.info["n_src"], self.info["nnz"]
            colptr = np.empty(ns + 1, np.int64)
            rowval = np.empty(max(nnz, 1), np.int64)
            nzval = np.empty(max(nnz, 1), np.float64)
            check(lib.crg_get_csc(C.c_void_p(self._h.ptr), 0, colptr.ctypes.data, rowval.ctypes.data, nzval.ctypes.data))
            self._csc[0] = sp.csc_matrix((nzval[:nnz], rowval[:nnz], colptr), shape=(nd, ns))
        A = self._csc[0]
        return A.T if self._transposed else A

    def csc_arrays(self, index_base: int = 0):
        """(colptr, rowval, nzval) of A, exactly as crg_get_csc writes them."""
        lib = _lib.load()
        ns, nnz = self.info["n_src"], self.info["nnz"]
        colptr = np.empty(ns + 1, np.int64)
        rowval = np.empty(max(nnz, 1), np.int64)
        nzval = np.empty(max(nnz, 1), np.float64)
        check(lib.crg_get_csc(C.c_void_p(self._h.ptr), index_base, colptr.ctypes.data, rowval.ctypes.data,
                              nzval.ctypes.data))
        return colptr, rowval[:nnz], nzval[:nnz]

    def row_col_sums(self):
        """Kahan row and column sums of A (forward orientation)."""
        lib = _lib.load()
        rs = np.empty(self.info["n_dst"])
        cs = np.empty(self.info["n_src"])
        check(lib.crg_get_row_col_sums(C.c_void_p(self._h.ptr), rs.ctypes.data, cs.ctypes.data))
        return rs, cs

    def __repr__(self):
        n2, n1 = self.shape
        return f"{n2}x{n1} Regridder(nnz={self.nnz}, gpu)"


def normalize_(R: Regridder) -> Regridder:
    raise ArgumentError("normalize is a build option: use Regridder(dst, src, normalize=True)")


# ----------------------------------------------------------------- fields

def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _stream_ptr(stream) -> Optional[int]:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", 0)) or None


class _Field:
    """Pointer, dtype code, shape and element strides of a numpy array or torch tensor."""

    def __init__(self, x):
        self.obj = x
        if _is_torch(x):
            import torch

            self.torch = True
            self.shape = tuple(x.shape)
            self.strides = tuple(x.stride())
            self.ptr = x.data_ptr()
            self.cuda = x.is_cuda
            self.device = x.device.index if x.is_cuda else None
            dt = {torch.float64: _lib.CRG_F64, torch.float32: _lib.CRG_F32, torch.bfloat16: _lib.CRG_BF16}
            if x.dtype not in dt:
                raise ArgumentError(f"unsupported field dtype {x.dtype}")
            self.dtype = dt[x.dtype]
        else:
            if not isinstance(x, np.ndarray):
                raise ArgumentError(f"fields must be numpy arrays or torch tensors, got {type(x).__name__}")
            self.torch = False
            self.shape = x.shape
            isz = x.itemsize
            if any(s % isz for s in x.strides):
                raise ArgumentError("field strides must be multiples of the element size")
            self.strides = tuple(s // isz for s in x.strides)
            self.ptr = x.ctypes.data
            self.cuda = False
            self.device = None
            dt = {np.dtype(np.float64): _lib.CRG_F64, np.dtype(np.float32): _lib.CRG_F32}
            if x.dtype not in dt:
                raise ArgumentError(f"unsupported field dtype {x.dtype}")
            self.dtype = dt[x.dtype]


def _flat_field_stride(shape, strides, dim):
    """Single element stride over the non-spatial axes flattened in
    row-major order, or None when they do not flatten to one stride."""
    axes = [(s, t) for k, (s, t) in enumerate(zip(shape, strides)) if k != dim and s != 1]
    if not axes:
        return 0
    for (sa, ta), (sb, tb) in zip(axes[:-1], axes[1:]):
        if ta != tb * sb:
            return None
    return axes[-1][1]


def _moveaxis(x, src, dst):
    if _is_torch(x):
        import torch

        return torch.movedim(x, src, dst)
    return np.moveaxis(x, src, dst)


def _contiguous_like(x):
    if _is_torch(x):
        return x.contiguous()
    return np.ascontiguousarray(x)


def _call(R: Regridder, adjoint: bool, src: _Field, ssc, ssf, dst: _Field, dsc, dsf, nf, normalize, stream):
    lib = _lib.load()
    fn = lib.crg_apply_adjoint if adjoint else lib.crg_apply
    check(fn(C.c_void_p(R._h.ptr), int(R._transposed), src.dtype, C.c_void_p(src.ptr), ssc, ssf, C.c_void_p(dst.ptr),
             dsc, dsf, nf, int(bool(normalize)), C.c_void_p(stream) if stream else None))


def _resolve_stream(fields, stream):
    if stream is not None:
        return _stream_ptr(stream)
    for f in fields:
        if f.torch and f.cuda:
            import torch

            return torch.cuda.current_stream(f.obj.device).cuda_stream
    return None


def _regrid(dst_field, R: Regridder, src_field, dims: int, normalize: bool, adjoint: bool, stream):
    if adjoint:
        n_in, n_out = R.shape[0], R.shape[1]
    else:
        n_out, n_in = R.shape
    src, dst = _Field(src_field), _Field(dst_field)
    if src.dtype != dst.dtype:
        raise ArgumentError("source and destination fields must have the same element type")
    if len(src.shape) != len(dst.shape):
        raise DimensionMismatch(
            f"source and destination ranks must match; got source rank {len(src.shape)} and destination rank {len(dst.shape)}")
    N = len(src.shape)
    if N == 0:
        raise ArgumentError("fields must have at least one dimension")
    if not (isinstance(dims, (int, np.integer)) and 1 <= dims <= N):
        raise ArgumentError(f"dims={dims} is out of range for a {N}-dimensional array")
    d = dims - 1
    if src.shape[d] != n_in or dst.shape[d] != n_out:
        raise DimensionMismatch(
            f"regridder has size {(n_out, n_in)} but the source spatial axis has {src.shape[d]} cells "
            f"and the destination spatial axis has {dst.shape[d]}")
    src_other = tuple(s for k, s in enumerate(src.shape) if k != d)
    dst_other = tuple(s for k, s in enumerate(dst.shape) if k != d)
    if src_other != dst_other:
        raise DimensionMismatch(
            f"source and destination non-spatial axes must match; got source axes {src_other} and destination axes {dst_other}")
    nf = int(np.prod(src_other)) if src_other else 1
    stream = _resolve_stream([src, dst], stream)

    # 1-D vectors that are not contiguous go through R.src_temp / R.dst_temp
    # (extract_*_arraylike, src/regridder/regrid.jl:75-79, :269-274).
    if N == 1 and not src.torch and not dst.torch and src.dtype == _lib.CRG_F64:
        s_in = src_field if src.strides[0] == 1 else None
        if s_in is None:
            R.src_temp[...] = src_field
            s_in = R.src_temp
        d_out = dst_field if dst.strides[0] == 1 else R.dst_temp
        sf, df = _Field(s_in), _Field(d_out)
        _call(R, adjoint, sf, 1, 0, df, 1, 0, 1, normalize, stream)
        if d_out is not dst_field:
            dst_field[...] = d_out
        return dst_field

    ssf = _flat_field_stride(src.shape, src.strides, d)
    dsf = _flat_field_stride(dst.shape, dst.strides, d)
    ssc, dsc = src.strides[d], dst.strides[d]
    staged_dst = None
    if ssf is None:
        # the other axes do not collapse to one stride: stage a copy with the
        # spatial axis last (fields one after another)
        s_obj = _contiguous_like(_moveaxis(src_field, d, -1))
        src = _Field(s_obj)
        ssc, ssf = 1, n_in
    if dsf is None:
        staged_dst = _contiguous_like(_moveaxis(dst_field, d, -1))
        dst = _Field(staged_dst)
        dsc, dsf = 1, n_out
    if nf == 1:
        ssf = ssf or 1
        dsf = dsf or 1
    _call(R, adjoint, src, ssc, ssf, dst, dsc, dsf, nf, normalize, stream)
    if staged_dst is not None:
        _moveaxis(dst_field, d, -1)[...] = staged_dst
    return dst_field


def regrid_(dst_field, regridder: Regridder, src_field, dims: int = 1, normalize: bool = True, stream=None):
    """``regrid!(dst_field, regridder, src_field; dims=1, normalize=true)``:
    dst = (A src) ./ dst_areas along the spatial axis ``dims`` (1-based, as in
    the reference), for every combination of the other axes in one launch."""
    return _regrid(dst_field, regridder, src_field, dims, normalize, False, stream)


def regrid_adjoint_(src_grad, regridder: Regridder, dst_grad, dims: int = 1, normalize: bool = True, stream=None):
    """Backward of ``regrid_``: src_grad = A^T (dst_grad ./ dst_areas)."""
    return _regrid(src_grad, regridder, dst_grad, dims, normalize, True, stream)


def regrid(regridder: Regridder, src_field, dims: int = 1, normalize: bool = True, stream=None):
    """Allocating variant: a new destination with the source's type and device."""
    n_out = regridder.shape[0]
    if _is_torch(src_field):
        import torch

        shape = list(src_field.shape)
        shape[dims - 1] = n_out
        dst = torch.empty(shape, dtype=src_field.dtype, device=src_field.device)
    else:
        shape = list(np.shape(src_field))
        shape[dims - 1] = n_out
        dst = np.zeros(shape, dtype=np.asarray(src_field).dtype)
    return regrid_(dst, regridder, src_field, dims=dims, normalize=normalize, stream=stream)
