"""GB300-native conservative regridding (the build and apply hot paths of
ConservativeRegridding.jl) over the C ABI of ``libcrg_gb300.so``."""
from ._lib import ArgumentError, CrgError, DimensionMismatch
from .grids import (
    Grid,
    cubed_sphere,
    full_clenshaw_grid,
    full_gaussian_grid,
    full_ring_grid,
    healpix_grid,
    lonlat_grid,
    lonlat_jittered,
    lonlat_regular,
    polygon_grid,
    regular_grid,
    reorder_cells,
    unit_sphere_from_geographic,
)
from .regridder import Regridder, regrid, regrid_, regrid_adjoint_
from .grad import area_grad, lonlat_tangents, regrid_pullback, split_points, src_area_grad
from .batch import ApplyPlan, build_batch, regrid_batch_
from .esmf import esmf_weights, load_esmf_weights, save_esmf_weights
from .fold import mirror_fold_
from .se import SpectralElementSpace, regrid_field_

__all__ = [
    "ApplyPlan",
    "ArgumentError",
    "CrgError",
    "DimensionMismatch",
    "Grid",
    "Regridder",
    "SpectralElementSpace",
    "area_grad",
    "build_batch",
    "cubed_sphere",
    "full_clenshaw_grid",
    "full_gaussian_grid",
    "full_ring_grid",
    "esmf_weights",
    "healpix_grid",
    "lonlat_grid",
    "lonlat_jittered",
    "lonlat_regular",
    "load_esmf_weights",
    "lonlat_tangents",
    "mirror_fold_",
    "polygon_grid",
    "regrid",
    "regrid_",
    "regrid_adjoint_",
    "regrid_batch_",
    "regrid_field_",
    "regrid_pullback",
    "regular_grid",
    "reorder_cells",
    "save_esmf_weights",
    "split_points",
    "src_area_grad",
    "unit_sphere_from_geographic",
]
