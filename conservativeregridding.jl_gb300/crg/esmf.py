"""ESMF offline-weights files: ``save_esmf_weights`` writes a regridder's
weights in the ESMF weight-file layout, as the reference's NCDatasets
extension does (ext/ConservativeRegriddingNCDatasetsExt.jl:18-60), and
``load_esmf_weights`` reads such a file back.  NetCDF is written with
scipy's NetCDF-3 writer (64-bit offsets); ESMF tools read it, with row and
col as 32-bit integers as ESMF itself writes them."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import ArgumentError, check
from .regridder import Regridder


def esmf_weights(R: Regridder, index_base: int = 1) -> dict:
    """S, row, col (CSC order), frac_a, frac_b, area_a, area_b as numpy arrays."""
    if R._transposed:
        raise ArgumentError("ESMF weights are written for the forward regridder (dst <- src)")
    nnz, na, nb = R.nnz, R.info["n_src"], R.info["n_dst"]
    out = {"row": np.empty(max(nnz, 1), np.int64), "col": np.empty(max(nnz, 1), np.int64),
           "S": np.empty(max(nnz, 1)), "frac_a": np.empty(na), "frac_b": np.empty(nb),
           "area_a": np.empty(na), "area_b": np.empty(nb)}
    check(_lib.load().crg_get_esmf_weights(C.c_void_p(R._h.ptr), int(index_base), *(
        out[k].ctypes.data for k in ("row", "col", "S", "frac_a", "frac_b", "area_a", "area_b"))))
    for k in ("row", "col", "S"):
        out[k] = out[k][:nnz]
    return out


def save_esmf_weights(path, R: Regridder, src_grid_name: str = "source", dst_grid_name: str = "destination",
                      src_shape=None, dst_shape=None, created_at=None) -> str:
    """Write R's weights to an ESMF offline-weights NetCDF file (dimensions
    n_s, n_a, n_b; variables S, row, col (1-based), frac_a, frac_b, area_a,
    area_b; "destarea" normalisation) with the reference's global attributes.
    Returns ``path``."""
    return write_esmf_file(path, esmf_weights(R, index_base=1), src_grid_name, dst_grid_name, src_shape, dst_shape,
                           created_at)


def write_esmf_file(path, w: dict, src_grid_name: str = "source", dst_grid_name: str = "destination",
                    src_shape=None, dst_shape=None, created_at=None) -> str:
    """The file of :func:`save_esmf_weights` from the arrays of
    :func:`esmf_weights` (1-based row and col)."""
    from scipy.io import netcdf_file

    if len(w["S"]) and max(w["row"].max(), w["col"].max()) >= 2**31:
        raise ArgumentError("cell indices do not fit the 32-bit row/col of an ESMF file")
    with netcdf_file(str(path), "w", version=2) as ds:
        ds.createDimension("n_s", len(w["S"]))
        ds.createDimension("n_a", len(w["area_a"]))
        ds.createDimension("n_b", len(w["area_b"]))
        names = {"S": "weight value", "row": "destination cell index (1-based)",
                 "col": "source cell index (1-based)", "frac_a": "source cell fraction covered",
                 "frac_b": "destination cell fraction covered", "area_a": "source cell areas",
                 "area_b": "destination cell areas"}
        dims = {"S": "n_s", "row": "n_s", "col": "n_s", "frac_a": "n_a", "frac_b": "n_b", "area_a": "n_a",
                "area_b": "n_b"}
        for k, long_name in names.items():
            is_index = k in ("row", "col")
            v = ds.createVariable(k, "i4" if is_index else "f8", (dims[k],))
            v[:] = w[k].astype(np.int32) if is_index else w[k]
            v.long_name = long_name
        ds.title = "ConservativeRegridding.jl weights (ESMF format)"
        ds.created_by = "ConservativeRegridding.save_esmf_weights"
        ds.source_grid = str(src_grid_name)
        ds.destination_grid = str(dst_grid_name)
        ds.normalization = "destarea"
        ds.map_method = "Conservative remapping"
        if created_at is not None:
            ds.created_at = str(created_at)
        if src_shape is not None:
            ds.source_grid_shape = np.asarray(src_shape, np.int32)
        if dst_shape is not None:
            ds.destination_grid_shape = np.asarray(dst_shape, np.int32)
    return str(path)


def load_esmf_weights(path) -> dict:
    """The arrays of an ESMF weight file (row/col as stored, 1-based) and, as
    ``matrix``, the n_b x n_a weight matrix S as scipy.sparse CSR."""
    import scipy.sparse as sp
    from scipy.io import netcdf_file

    with netcdf_file(str(path), "r", mmap=False) as ds:
        # NetCDF-3 data are big-endian on disk: native-order copies
        out = {k: np.array(ds.variables[k][:], dtype=np.int64 if k in ("row", "col") else np.float64)
               for k in ("S", "row", "col", "frac_a", "frac_b", "area_a", "area_b")}
    out["matrix"] = sp.csr_matrix((out["S"], (out["row"] - 1, out["col"] - 1)),
                                  shape=(len(out["area_b"]), len(out["area_a"])))
    return out
