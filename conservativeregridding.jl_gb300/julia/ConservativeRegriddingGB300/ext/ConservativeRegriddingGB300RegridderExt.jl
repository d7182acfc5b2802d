"""
The GB300 build and apply behind ConservativeRegridding.jl's own types.

`Regridder(GB300(), dst, src; normalize)` returns the reference's
`Regridder{W,A,V}` (src/regridder/regridder.jl:25-36) with
`W = GB300Sparse`, so everything downstream is the reference's code:

- `regrid!(dst, R, src)` on vectors runs the reference's pipeline
  (src/regridder/regrid.jl:63-118); its `perform_regridding!` calls
  `mul!(dst, R.intersections, src)`, which is `crg_apply` without the
  division, and its `finalize_regridding!` (or an extension's, for
  Oceananigans, HEALPix or ClimaCore fields) divides by `R.dst_areas`.
- N-D strided arrays (`NDSliceLoop`, src/regridder/regrid.jl:225-318) go to
  the library in one call for all slices, divided on the device, instead of
  one `mul!` per slice.
- `transpose(R)` (src/regridder/regridder.jl:49-50) swaps the areas and
  wraps the matrix in a `GB300SparseT`, which applies through the stored
  copy of the transpose.
"""
module ConservativeRegriddingGB300RegridderExt

import ConservativeRegridding as CR
import ConservativeRegriddingGB300 as GB
import LinearAlgebra

const GB300Regridder = CR.Regridder{<:Union{GB.GB300Sparse,GB.GB300SparseT}}

"""
    Regridder(GB300(), dst, src; normalize = false, adapt = identity)

The reference's `Regridder(dst, src; normalize)` built on the GPU.  `dst` and
`src` are anything `ConservativeRegriddingGB300.grid` accepts: `(nx+1) x
(ny+1)` point matrices (`CellBasedGrid` vertex matrices of
`UnitSphericalPoint`s, or planar points), `dim x (nx+1) x (ny+1)` arrays, or
descriptors from `curvilinear` / `cells` (cubed-sphere faces, HEALPix
pixels, polygon lists).  Mixed planar/spherical grids are refused: promote
them first, as `Regridder(dst, src)` does (src/regridder/regridder.jl:109-117).
`adapt` is applied to the area and temporary vectors, e.g. `adapt = CuArray`
so that `regrid!` on `CuArray` fields finalises on the device.
"""
function CR.Regridder(::GB.GB300, dst, src; normalize::Bool = false, adapt = identity)
    A, dst_areas, src_areas = GB.build(dst, src; normalize)
    nd, ns = size(A)
    return CR.Regridder(A, adapt(dst_areas), adapt(src_areas), adapt(zeros(nd)), adapt(zeros(ns)))
end

# normalize! divides the matrix in place (src/regridder/regridder.jl:54-62);
# the GPU matrix is normalised by the build instead.
LinearAlgebra.normalize!(::GB300Regridder) =
    throw(ArgumentError("normalize is a build option for the GB300 regridder: Regridder(GB300(), dst, src; normalize = true)"))

function CR.perform_regridding!(dst::CR.NDSliceLoop{Dim,N,<:StridedArray{T}}, R::GB300Regridder,
                                src::CR.NDSliceLoop{Dim,N,<:StridedArray{T}};
                                normalize::Bool = true, kwargs...) where {Dim,N,T<:Union{Float32,Float64}}
    CR._validate_slice_compatibility!(dst, src)
    GB.apply!(parent(dst), R.intersections, parent(src); normalize, dims = Dim)
    return dst
end

end # module
