"""ctypes binding of ``libcrg_gb300.so`` (declared in include/crg.h).

The library is the only compute path: if it cannot be loaded the import of
the functions below raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import re
import threading

from . import _build

CRG_OK = 0
CRG_ERR_INVALID_ARGUMENT = 1
CRG_ERR_DIMENSION_MISMATCH = 2
CRG_ERR_CUDA = 3
CRG_ERR_OUT_OF_MEMORY = 4
CRG_ERR_NOT_SUPPORTED = 5
CRG_ERR_GEOMETRY = 6
CRG_ERR_INTERNAL = 7

CRG_PLANAR = 0
CRG_SPHERICAL = 1
CRG_GRID_CURVILINEAR = 0
CRG_GRID_CELLS = 1
CRG_F64 = 0
CRG_F32 = 1
CRG_BF16 = 2


class crg_grid_desc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("manifold", C.c_int32),
        ("nblocks", C.c_int32),
        ("max_verts", C.c_int32),
        ("ncells", C.c_int64),
        ("block_nx", C.POINTER(C.c_int64)),
        ("block_ny", C.POINTER(C.c_int64)),
        ("points", C.c_void_p),
        ("cell_verts", C.c_void_p),
        ("cell_nverts", C.c_void_p),
    ]


class crg_build_opts(C.Structure):
    _fields_ = [("normalize", C.c_int32), ("flags", C.c_int32), ("stream", C.c_void_p)]


class crg_se_space(C.Structure):
    _fields_ = [("elements", crg_grid_desc), ("nq", C.c_int32), ("pad", C.c_int32), ("node_weights", C.c_void_p)]


class crg_se_opts(C.Structure):
    _fields_ = [("triangle_quad_degree", C.c_int32), ("flags", C.c_int32), ("radius", C.c_double),
                ("stream", C.c_void_p)]


class crg_apply_item(C.Structure):
    _fields_ = [
        ("regridder", C.c_void_p),
        ("transpose", C.c_int32),
        ("dtype", C.c_int32),
        ("src", C.c_void_p),
        ("src_stride_cell", C.c_int64),
        ("src_stride_field", C.c_int64),
        ("dst", C.c_void_p),
        ("dst_stride_cell", C.c_int64),
        ("dst_stride_field", C.c_int64),
        ("nfields", C.c_int64),
        ("normalize", C.c_int32),
        ("adjoint", C.c_int32),
    ]


class crg_info(C.Structure):
    _fields_ = [
        ("n_dst", C.c_int64),
        ("n_src", C.c_int64),
        ("nnz", C.c_int64),
        ("n_candidates", C.c_int64),
        ("manifold", C.c_int32),
        ("normalized", C.c_int32),
        ("normalizer", C.c_double),
        ("t_build_ms", C.c_double),
        ("t_search_ms", C.c_double),
        ("t_clip_ms", C.c_double),
        ("t_assemble_ms", C.c_double),
        ("clip_overflows", C.c_int64),
        ("device", C.c_int32),
        ("pad", C.c_int32),
        ("merge_tasks", C.c_int64 * 2),
        ("cut_rows", C.c_int64 * 2),
        ("carry_slots", C.c_int64 * 2),
        ("empty_rows", C.c_int64 * 2),
        ("n_clipped", C.c_int64),
    ]


# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "crg_build": (C.c_int, [C.POINTER(crg_grid_desc), C.POINTER(crg_grid_desc), C.POINTER(crg_build_opts), C.POINTER(C.c_void_p)]),
    "crg_regridder_retain": (C.c_int, [C.c_void_p]),
    "crg_regridder_release": (C.c_int, [C.c_void_p]),
    "crg_regridder_info": (C.c_int, [C.c_void_p, C.POINTER(crg_info)]),
    "crg_apply": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p,
                            C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_void_p]),
    "crg_apply_adjoint": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p,
                                    C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_void_p]),
    "crg_apply_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p,
                                    C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_void_p]),
    "crg_area_grad": (C.c_int, [C.c_void_p, C.POINTER(crg_grid_desc), C.POINTER(crg_grid_desc), C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "crg_build_batch": (C.c_int, [C.c_int64, C.POINTER(crg_grid_desc), C.POINTER(crg_grid_desc),
                                  C.POINTER(crg_build_opts), C.c_int32, C.POINTER(C.c_void_p)]),
    "crg_apply_batch": (C.c_int, [C.c_int64, C.POINTER(crg_apply_item), C.c_int32, C.c_void_p]),
    "crg_apply_plan_create": (C.c_int, [C.c_int64, C.POINTER(crg_apply_item), C.POINTER(C.c_void_p)]),
    "crg_apply_plan_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "crg_apply_plan_destroy": (C.c_int, [C.c_void_p]),
    "crg_apply_plan_info": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "crg_get_csc": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "crg_mirror_fold": (C.c_int, [C.c_int32, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                  C.c_void_p]),
    "crg_get_esmf_weights": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p]),
    "crg_get_csr": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "crg_get_areas": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "crg_get_row_col_sums": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "crg_build_se_to_fv": (C.c_int, [C.POINTER(crg_grid_desc), C.POINTER(crg_se_space), C.POINTER(crg_se_opts),
                                     C.POINTER(C.c_void_p)]),
    "crg_build_fv_to_se": (C.c_int, [C.POINTER(crg_se_space), C.POINTER(crg_grid_desc), C.POINTER(crg_se_opts),
                                     C.POINTER(C.c_void_p)]),
    "crg_se_nodes": (C.c_int, [C.POINTER(crg_se_space), C.POINTER(crg_se_opts), C.c_void_p, C.c_void_p]),
    "crg_se_dss": (C.c_int, [C.c_int32, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                             C.c_void_p, C.c_int64, C.c_void_p]),
    "crg_last_error": (C.c_char_p, []),
    "crg_status_string": (C.c_char_p, [C.c_int]),
    "crg_abi_version": (C.c_int32, []),
}

_lock = threading.Lock()
_lib = None


def abi_version() -> int:
    """CRG_ABI_VERSION as include/crg.h defines it."""
    m = re.search(r"^#define CRG_ABI_VERSION (\d+)", (_build.INCLUDE / "crg.h").read_text(), re.M)
    if not m:
        raise RuntimeError("include/crg.h does not define CRG_ABI_VERSION")
    return int(m.group(1))


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load (building first if stale) the CUDA library."""
    global _lib
    with _lock:
        if _lib is None:
            if build_if_missing:
                _build.build()
            if not _build.LIB_PATH.exists():
                raise RuntimeError(f"{_build.LIB_PATH} is missing: the CUDA extension has not been built")
            lib = C.CDLL(str(_build.LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            want, got = abi_version(), int(lib.crg_abi_version())
            if got != want:
                raise RuntimeError(f"{_build.LIB_PATH} implements C ABI version {got}, include/crg.h declares {want}: "
                                   "rebuild the library")
            _lib = lib
        return _lib


class CrgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


class ArgumentError(ValueError):
    """Counterpart of Julia's ArgumentError (src/regridder/regrid.jl:242-245)."""


class DimensionMismatch(ValueError):
    """Counterpart of Julia's DimensionMismatch (src/regridder/regrid.jl:289-296)."""


def check(status: int) -> None:
    if status == CRG_OK:
        return
    lib = load()
    msg = lib.crg_last_error().decode(errors="replace")
    what = lib.crg_status_string(status).decode()
    if status == CRG_ERR_INVALID_ARGUMENT:
        raise ArgumentError(msg)
    if status == CRG_ERR_DIMENSION_MISMATCH:
        raise DimensionMismatch(msg)
    raise CrgError(status, f"{what}: {msg}")
