"""
    ConservativeRegriddingGB300

Julia binding of `libcrg_gb300.so` (declared in `include/crg.h`): the GPU build
and apply of ConservativeRegridding.jl's `Regridder`, `regrid!` and
`transpose(R)`.  The matrix, the areas and the weights live on the GPU; field
arrays may be `CuArray`s (device pointers) or host `Array`s (staged by the
library).

This file is the `ccall` layer a maintainer adds next to ConservativeRegridding.jl;
it depends only on `Libdl`, `LinearAlgebra` and `SparseArrays`.  Two package
extensions load with their trigger packages:

- `ConservativeRegriddingGB300RegridderExt` (ConservativeRegridding):
  `Regridder(GB300(), dst, src; normalize)` returns the reference's own
  `Regridder` type with a `GB300Sparse` matrix, so `regrid!`, `transpose(R)`
  and the extensions' field types run through the reference's pipeline (its
  `mul!` is `crg_apply`); N-D arrays go to the library in one call.
- `ConservativeRegriddingGB300ChainRulesCoreExt` (ChainRulesCore): `rrule`s
  for `regrid(A, s)` (the adjoint apply) and `regrid_on(V, W, s)` (also the
  destination and source vertex cotangents).
"""
module ConservativeRegriddingGB300

using Libdl
using SparseArrays
using LinearAlgebra

export GB300, GB300Sparse, GB300SparseT

const libcrg = Ref{String}("")

function __init__()
    path = get(ENV, "CRG_GB300_LIB", joinpath(@__DIR__, "..", "..", "..", "_build", "libcrg_gb300.so"))
    libcrg[] = path
end

# --- C structs (must match include/crg.h) -------------------------------------

struct CrgGridDesc
    kind::Int32          # 0 curvilinear, 1 cells
    manifold::Int32      # 0 planar, 1 spherical
    nblocks::Int32
    max_verts::Int32
    ncells::Int64
    block_nx::Ptr{Int64}
    block_ny::Ptr{Int64}
    points::Ptr{Float64}
    cell_verts::Ptr{Float64}
    cell_nverts::Ptr{Int32}
end

struct CrgBuildOpts
    normalize::Int32
    flags::Int32
    stream::Ptr{Cvoid}
end

struct CrgInfo
    n_dst::Int64; n_src::Int64; nnz::Int64; n_candidates::Int64
    manifold::Int32; normalized::Int32
    normalizer::Float64
    t_build_ms::Float64; t_search_ms::Float64; t_clip_ms::Float64; t_assemble_ms::Float64
    clip_overflows::Int64
    device::Int32; pad::Int32
    merge_tasks::NTuple{2,Int64}; cut_rows::NTuple{2,Int64}; carry_slots::NTuple{2,Int64}; empty_rows::NTuple{2,Int64}
    n_clipped::Int64
end

const CRG_F64, CRG_F32, CRG_BF16 = Int32(0), Int32(1), Int32(2)

function check(status::Cint)
    status == 0 && return nothing
    msg = unsafe_string(ccall((:crg_last_error, libcrg[]), Cstring, ()))
    status == 1 && throw(ArgumentError(msg))       # CRG_ERR_INVALID_ARGUMENT
    status == 2 && throw(DimensionMismatch(msg))   # CRG_ERR_DIMENSION_MISMATCH
    error("libcrg_gb300: " * unsafe_string(ccall((:crg_status_string, libcrg[]), Cstring, (Cint,), status)) * ": " * msg)
end

# --- the handle ---------------------------------------------------------------

mutable struct GB300Sparse
    ptr::Ptr{Cvoid}
    info::CrgInfo
    function GB300Sparse(ptr::Ptr{Cvoid})
        info = Ref{CrgInfo}()
        check(ccall((:crg_regridder_info, libcrg[]), Cint, (Ptr{Cvoid}, Ref{CrgInfo}), ptr, info))
        h = new(ptr, info[])
        finalizer(h) do x
            ccall((:crg_regridder_release, libcrg[]), Cint, (Ptr{Cvoid},), x.ptr)
        end
        return h
    end
end

"A transposed view: shares the handle (retained), swaps the direction."
struct GB300SparseT
    parent::GB300Sparse
end

Base.size(A::GB300Sparse) = (Int(A.info.n_dst), Int(A.info.n_src))
Base.size(A::GB300SparseT) = reverse(size(A.parent))
Base.size(A::Union{GB300Sparse,GB300SparseT}, d::Integer) = d <= 2 ? size(A)[d] : 1
SparseArrays.nnz(A::Union{GB300Sparse,GB300SparseT}) = Int(_direction(A)[1].info.nnz)
LinearAlgebra.transpose(A::GB300Sparse) = GB300SparseT(A)
LinearAlgebra.transpose(A::GB300SparseT) = A.parent

Base.show(io::IO, A::GB300Sparse) = print(io, "$(size(A, 1))×$(size(A, 2)) GB300Sparse with $(nnz(A)) stored entries")
Base.show(io::IO, A::GB300SparseT) = print(io, "transpose(", A.parent, ")")
# `show(::Regridder)` prints its matrix with Base.print_array (src/regridder/regridder.jl:38-44)
Base.print_array(io::IO, A::Union{GB300Sparse,GB300SparseT}) = show(io, A)

"""
    GB300()

Backend tag of `ConservativeRegridding.Regridder(GB300(), dst, src; normalize)`
(defined by the package extension for ConservativeRegridding): the build runs
in `libcrg_gb300.so` and the result is an ordinary `Regridder` whose
`intersections` is a `GB300Sparse`.
"""
struct GB300 end

"""
    curvilinear(points::Array{Float64,3})

Describe a grid of `(nx+1) x (ny+1)` vertices given as a `3 x (nx+1) x (ny+1)`
array of unit vectors (the reference's `CellBasedGrid` vertex matrix), or a
`2 x (nx+1) x (ny+1)` array of planar points.
"""
function curvilinear(points::Array{Float64,3})
    dim, nxp, nyp = size(points)
    dim in (2, 3) || throw(ArgumentError("points must be 2 or 3 coordinates per vertex, got $dim"))
    nx = Ref(Int64(nxp - 1)); ny = Ref(Int64(nyp - 1))
    desc = CrgGridDesc(0, dim == 3 ? 1 : 0, 1, 0, nx[] * ny[],
                       Base.unsafe_convert(Ptr{Int64}, nx), Base.unsafe_convert(Ptr{Int64}, ny),
                       pointer(points), C_NULL, C_NULL)
    return desc, (points, nx, ny)
end

"""
    cells(verts::Array{Float64,3}, nverts = nothing)

Describe a grid of per-cell convex polygons (HEALPix pixels, `FlatNoTree`
polygon lists): `verts` is `dim x max_verts x ncells` (ring order, not
closed; `dim` 3 on the sphere, 2 on the plane; `max_verts` 3 to 8) and
`nverts` the vertex count of each cell (`nothing`: all `max_verts`).
"""
function cells(verts::Array{Float64,3}, nverts::Union{Nothing,Vector{Int32}} = nothing)
    dim, maxv, n = size(verts)
    dim in (2, 3) || throw(ArgumentError("vertices must have 2 or 3 coordinates, got $dim"))
    nverts === nothing || length(nverts) == n ||
        throw(DimensionMismatch("nverts has $(length(nverts)) entries for $n cells"))
    desc = CrgGridDesc(1, dim == 3 ? 1 : 0, 0, maxv, n, C_NULL, C_NULL, C_NULL, pointer(verts),
                       nverts === nothing ? Ptr{Int32}(C_NULL) : pointer(nverts))
    return desc, (verts, nverts)
end

"""
    grid(x)

A grid descriptor (as returned by `curvilinear` / `cells`) for `x`: a
descriptor itself, a `dim x (nx+1) x (ny+1)` vertex array, or an
`(nx+1) x (ny+1)` matrix of points with 3 (unit sphere) or 2 (plane)
coordinates each, such as the reference's `CellBasedGrid` point matrices of
`UnitSphericalPoint`s.
"""
grid(x::Tuple{CrgGridDesc,Any}) = x
grid(points::Array{Float64,3}) = curvilinear(points)
function grid(points::AbstractMatrix)
    dim = length(first(points))
    p = Array{Float64,3}(undef, dim, size(points)...)
    for I in CartesianIndices(points)
        q = points[I]
        length(q) == dim || throw(ArgumentError("every point needs $dim coordinates"))
        for c in 1:dim
            p[c, I] = q[c]
        end
    end
    return curvilinear(p)
end

"""
    build(dst, src; normalize = false) -> (A::GB300Sparse, dst_areas, src_areas)

GPU build of `Regridder(dst, src; normalize)` (`crg_build`) for grid
descriptors (see `grid`); the areas are host copies.
"""
function build(dst, src; normalize::Bool = false)
    d, keep_d = grid(dst)
    s, keep_s = grid(src)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    opts = Ref(CrgBuildOpts(normalize, 0, C_NULL))
    GC.@preserve keep_d keep_s begin
        check(ccall((:crg_build, libcrg[]), Cint, (Ref{CrgGridDesc}, Ref{CrgGridDesc}, Ref{CrgBuildOpts}, Ref{Ptr{Cvoid}}),
                    Ref(d), Ref(s), opts, out))
    end
    A = GB300Sparse(out[])
    nd, ns = size(A)
    dst_areas = Vector{Float64}(undef, nd)
    src_areas = Vector{Float64}(undef, ns)
    check(ccall((:crg_get_areas, libcrg[]), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), A.ptr, dst_areas, src_areas))
    return A, dst_areas, src_areas
end

"Raw address of an array's first element plus `off` bytes: `Ptr` for host arrays, `CuPtr` for `CuArray`s."
_raw(p, off::Integer = 0) = reinterpret(Ptr{Cvoid}, reinterpret(UInt, p) + UInt(off))

"The handle behind `A` and the C `transpose` flag of the direction `A` applies in."
_direction(A::GB300Sparse) = (A, Int32(0))
_direction(A::GB300SparseT) = (A.parent, Int32(1))

"""
    _slice_groups(f, x, y, dims)

Cover every 1-D slice of `x` and `y` along `dims` with calls
`f(xptr, x_stride_cell, x_stride_field, yptr, y_stride_cell, y_stride_field, nfields)`.
The leading non-spatial axes whose strides chain (a dense array's axes before
and after `dims` do, separately) go into one call as `nfields` fields; the
remaining axes are looped over.  Dense arrays with `dims = 1` or
`dims = ndims` therefore take one call.
"""
function _slice_groups(f, x::StridedArray{T}, y::StridedArray{T}, dims::Int) where {T}
    other = Tuple(k for k in 1:ndims(x) if k != dims && size(x, k) != 1)   # size-1 axes add no slices
    nf, fx, fy, run = 1, 1, 1, 0
    for (r, k) in enumerate(other)
        if r == 1
            nf, fx, fy, run = size(x, k), stride(x, k), stride(y, k), 1
        elseif stride(x, k) == fx * nf && stride(y, k) == fy * nf
            nf *= size(x, k)
            run = r
        else
            break
        end
    end
    rest = other[run+1:end]
    GC.@preserve x y for I in CartesianIndices(map(k -> size(x, k), rest))
        ox = sum(ntuple(i -> (I[i] - 1) * stride(x, rest[i]), length(rest)); init = 0)
        oy = sum(ntuple(i -> (I[i] - 1) * stride(y, rest[i]), length(rest)); init = 0)
        f(_raw(pointer(x), ox * sizeof(T)), stride(x, dims), fx, _raw(pointer(y), oy * sizeof(T)), stride(y, dims), fy, nf)
    end
    return nothing
end

function _check_fields(y, x, dims, n_out, n_in)
    ndims(x) == ndims(y) ||
        throw(DimensionMismatch("source and destination ranks must match; got source rank $(ndims(x)) and destination rank $(ndims(y))"))
    1 <= dims <= ndims(x) || throw(ArgumentError("dims=$dims is out of range for a $(ndims(x))-dimensional array"))
    (size(x, dims) == n_in && size(y, dims) == n_out) ||
        throw(DimensionMismatch("regridder has size ($n_out, $n_in) but the source spatial axis has $(size(x, dims)) cells and the destination spatial axis has $(size(y, dims))"))
    ox = Tuple(size(x, k) for k in 1:ndims(x) if k != dims)
    oy = Tuple(size(y, k) for k in 1:ndims(y) if k != dims)
    ox == oy ||
        throw(DimensionMismatch("source and destination non-spatial axes must match; got source axes $ox and destination axes $oy"))
    return nothing
end

_dtype(::Type{Float64}) = CRG_F64
_dtype(::Type{Float32}) = CRG_F32

"""
    apply!(y, A, x; normalize = true, dims = 1)

`perform_regridding!` + `finalize_regridding!` for strided arrays (host
`Array`s or `CuArray`s): `y = (A x) ./ a_d` along the spatial axis `dims`
for every slice along the other axes, in one library call for a dense array
whose spatial axis is the first or the last (the reference loops `mul!` per
slice, src/regridder/regrid.jl:303-318).  `A` may be a transposed view.
"""
function apply!(y::StridedArray{T}, A::Union{GB300Sparse,GB300SparseT}, x::StridedArray{T};
                normalize::Bool = true, dims::Int = 1) where {T<:Union{Float64,Float32}}
    _check_fields(y, x, dims, size(A)...)
    h, t = _direction(A)
    _slice_groups(x, y, dims) do xp, xsc, xsf, yp, ysc, ysf, nf
        check(ccall((:crg_apply, libcrg[]), Cint,
                    (Ptr{Cvoid}, Int32, Int32, Ptr{Cvoid}, Int64, Int64, Ptr{Cvoid}, Int64, Int64, Int64, Int32, Ptr{Cvoid}),
                    h.ptr, t, _dtype(T), xp, xsc, xsf, yp, ysc, ysf, nf, normalize, C_NULL))
    end
    return y
end

"""
    adjoint!(gs, A, gd; normalize = true, dims = 1)

Pullback of `apply!` with respect to the source field: `gs = A' (gd ./ a_d)`
(or `A (gd ./ a_s)` for a transposed view), through the other stored copy of
A (`crg_apply_adjoint`, no atomics).
"""
function adjoint!(gs::StridedArray{T}, A::Union{GB300Sparse,GB300SparseT}, gd::StridedArray{T};
                  normalize::Bool = true, dims::Int = 1) where {T<:Union{Float64,Float32}}
    n_out, n_in = size(A)
    _check_fields(gs, gd, dims, n_in, n_out)
    h, t = _direction(A)
    _slice_groups(gd, gs, dims) do xp, xsc, xsf, yp, ysc, ysf, nf
        check(ccall((:crg_apply_adjoint, libcrg[]), Cint,
                    (Ptr{Cvoid}, Int32, Int32, Ptr{Cvoid}, Int64, Int64, Ptr{Cvoid}, Int64, Int64, Int64, Int32, Ptr{Cvoid}),
                    h.ptr, t, _dtype(T), xp, xsc, xsf, yp, ysc, ysf, nf, normalize, C_NULL))
    end
    return gs
end

# `mul!(y, R.intersections, x)` is the reference's perform_regridding!
# (src/regridder/regrid.jl:95-98): A x without the division, which
# finalize_regridding! then applies.  Vectors and matrices (columns = fields).
LinearAlgebra.mul!(y::StridedVecOrMat{T}, A::Union{GB300Sparse,GB300SparseT}, x::StridedVecOrMat{T}) where {T<:Union{Float64,Float32}} =
    apply!(y, A, x; normalize = false, dims = 1)

function Base.:*(A::Union{GB300Sparse,GB300SparseT}, x::StridedVecOrMat{T}) where {T<:Union{Float64,Float32}}
    y = similar(x, size(A, 1), size(x)[2:end]...)
    return mul!(y, A, x)
end

"""
    regrid(A, s; normalize = true, dims = 1) -> d

Allocating `regrid!`: `d = (A s) ./ a_d` into a new array like `s`.  Its
`ChainRulesCore.rrule` (package extension) pulls back through `adjoint!`.
"""
function regrid(A::Union{GB300Sparse,GB300SparseT}, s::StridedArray{T}; normalize::Bool = true, dims::Int = 1) where {T<:Union{Float64,Float32}}
    d = similar(s, ntuple(k -> k == dims ? size(A, 1) : size(s, k), ndims(s)))
    return apply!(d, A, s; normalize, dims)
end

"""
    area_grad(A, dst, src; row_weight, src_field, area_weight) -> Array{Float64}

Cotangent of the destination vertices for `sum_ij u_i s_j dA_ij/dV + sum_i c_i da_i/dV`
(`crg_area_grad`), laid out like `dst`'s vertex array.  For the rrule of
`d = regrid(R, s)` with output cotangent `g`: `u = g ./ a`, `c = -g .* d ./ a`
(unnormalised areas `a`).
"""
function area_grad(A::GB300Sparse, dst, src; row_weight = nothing, src_field = nothing, area_weight = nothing)
    d, keep_d = grid(dst)
    s, keep_s = grid(src)
    g = zeros(Float64, size(keep_d[1]))   # the vertex array's own layout
    ptr(v) = v === nothing ? Ptr{Float64}(C_NULL) : pointer(v)
    GC.@preserve keep_d keep_s row_weight src_field area_weight begin
        check(ccall((:crg_area_grad, libcrg[]), Cint,
                    (Ptr{Cvoid}, Ref{CrgGridDesc}, Ref{CrgGridDesc}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                     Ptr{Float64}, Ptr{Cvoid}),
                    A.ptr, Ref(d), Ref(s), ptr(row_weight), ptr(src_field), ptr(area_weight), g, C_NULL))
    end
    return g
end

"""
    src_area_grad(dst, src, row_weight, src_field; swapped = nothing) -> Array{Float64}

Cotangent of the SOURCE vertices for `sum_ij u_i s_j dA_ij/dW`, laid out like
`src`'s vertex array.  `A_ij` is the area of (destination cell i) ∩ (source
cell j), symmetric in the two cells, so this is `area_grad` of the regridder
built the other way round, `build(src, dst)` (pass its `GB300Sparse` as
`swapped` to reuse one), with the two weight vectors exchanged.
"""
function src_area_grad(dst, src, row_weight::Vector{Float64}, src_field::Vector{Float64}; swapped = nothing)
    At = swapped === nothing ? build(src, dst)[1] : swapped
    return area_grad(At, src, dst; row_weight = src_field, src_field = row_weight)
end

"""
    regrid_on(V, W, s; normalize = false) -> d

`d = regrid(R, s) = (A s) ./ a_d` with `R` built from the vertex arrays `V`
(destination) and `W` (source), each `dim x (nx+1) x (ny+1)` (see
`curvilinear`); FP64, one field.  It is a function of the coordinates as well
as of `s`: its `ChainRulesCore.rrule` (package extension) returns the
cotangents of `V` (`area_grad`), of `W` (`src_area_grad`) and of `s`
(`adjoint!`).  Normalisation cancels in `d`.
"""
function regrid_on(V::Array{Float64,3}, W::Array{Float64,3}, s::Vector{Float64}; normalize::Bool = false)
    A, _, _ = build(V, W; normalize)
    return regrid(A, s)
end

"""
    build_batch(pairs; normalize = false, nthreads = 0) -> Vector{GB300Sparse}

`crg_build_batch`: many `(dst, src)` pairs built concurrently (each grid
anything `grid` accepts).
"""
function build_batch(pairs; normalize::Bool = false, nthreads::Integer = 0)
    n = length(pairs)
    gp = [(grid(p[1]), grid(p[2])) for p in pairs]
    dd = [g[1][1] for g in gp]; ds = [g[2][1] for g in gp]
    keep = [(g[1][2], g[2][2]) for g in gp]
    out = Vector{Ptr{Cvoid}}(undef, n)
    opts = Ref(CrgBuildOpts(normalize, 0, C_NULL))
    GC.@preserve keep begin
        check(ccall((:crg_build_batch, libcrg[]), Cint,
                    (Int64, Ptr{CrgGridDesc}, Ptr{CrgGridDesc}, Ref{CrgBuildOpts}, Int32, Ptr{Ptr{Cvoid}}),
                    n, dd, ds, opts, Int32(nthreads), out))
    end
    return [GB300Sparse(p) for p in out]
end

struct CrgApplyItem
    regridder::Ptr{Cvoid}
    transpose::Int32; dtype::Int32
    src::Ptr{Cvoid}; src_stride_cell::Int64; src_stride_field::Int64
    dst::Ptr{Cvoid}; dst_stride_cell::Int64; dst_stride_field::Int64
    nfields::Int64
    normalize::Int32; adjoint::Int32
end

"""
    ApplyPlan(items) / launch(plan) / destroy(plan)

`crg_apply_plan_*`: the applies of many regridders (items built from device
arrays, e.g. `CuArray` pointers) captured as one CUDA graph.
"""
mutable struct ApplyPlan
    ptr::Ptr{Cvoid}
    function ApplyPlan(items::Vector{CrgApplyItem})
        out = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:crg_apply_plan_create, libcrg[]), Cint, (Int64, Ptr{CrgApplyItem}, Ref{Ptr{Cvoid}}),
                    length(items), items, out))
        p = new(out[])
        finalizer(p) do x
            ccall((:crg_apply_plan_destroy, libcrg[]), Cint, (Ptr{Cvoid},), x.ptr)
        end
        return p
    end
end
"""
    apply_batch!(items::Vector{CrgApplyItem}; nthreads = 0)

`crg_apply_batch`: independent applies at once (host arrays: one chunk
pipeline over all items, so their copies share both link directions).
"""
apply_batch!(items::Vector{CrgApplyItem}; nthreads::Integer = 0, stream::Ptr{Cvoid} = C_NULL) =
    check(ccall((:crg_apply_batch, libcrg[]), Cint, (Int64, Ptr{CrgApplyItem}, Int32, Ptr{Cvoid}),
                length(items), items, Int32(nthreads), stream))

launch(p::ApplyPlan; stream::Ptr{Cvoid} = C_NULL) =
    check(ccall((:crg_apply_plan_launch, libcrg[]), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), p.ptr, stream))

"""
    esmf_weights(A) -> NamedTuple

`crg_get_esmf_weights`: the arrays `save_esmf_weights` writes (S, row, col,
frac_a, frac_b, area_a, area_b; 1-based, CSC order), for the reference's
NCDatasets extension to write.
"""
function esmf_weights(A::GB300Sparse)
    nd, ns = size(A); nnz = Int(A.info.nnz)
    row = Vector{Int64}(undef, nnz); col = Vector{Int64}(undef, nnz); S = Vector{Float64}(undef, nnz)
    frac_a = Vector{Float64}(undef, ns); frac_b = Vector{Float64}(undef, nd)
    area_a = Vector{Float64}(undef, ns); area_b = Vector{Float64}(undef, nd)
    check(ccall((:crg_get_esmf_weights, libcrg[]), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                 Ptr{Float64}), A.ptr, 1, row, col, S, frac_a, frac_b, area_a, area_b))
    return (; S, row, col, frac_a, frac_b, area_a, area_b)
end

# ---------------------------------------------------------------- spectral elements

struct CrgSeSpace
    elements::CrgGridDesc
    nq::Int32
    pad::Int32
    node_weights::Ptr{Float64}
end

struct CrgSeOpts
    triangle_quad_degree::Int32
    flags::Int32
    radius::Float64
    stream::Ptr{Cvoid}
end

"""
    build_se(fv, elements, nq; se_is_dst, node_weights = nothing, triangle_quad_degree = 0, radius = 1.0)

GPU build of the ClimaCore extension's regridders: SE -> FV principled weights
(`se_is_dst = false`, `crg_build_se_to_fv`, the method `Regridder(manifold, dst, src::SESpaceOrField)`)
or the FV -> SE L2 projection (`se_is_dst = true`, `crg_build_fv_to_se`).  `elements` is the
element grid (e.g. `curvilinear` of each cube face's corner matrix), `node_weights` ClimaCore's
`Spaces.weighted_jacobian` flattened like `se_node_weights`.
"""
function build_se(fv, elements, nq::Integer; se_is_dst::Bool, node_weights = nothing,
                  triangle_quad_degree::Integer = 0, radius::Real = 1.0)
    f, keep_f = fv
    e, keep_e = elements
    w = node_weights === nothing ? Ptr{Float64}(C_NULL) : pointer(node_weights)
    space = Ref(CrgSeSpace(e, Int32(nq), 0, w))
    opts = Ref(CrgSeOpts(Int32(triangle_quad_degree), 0, Float64(radius), C_NULL))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve keep_f keep_e node_weights begin
        if se_is_dst
            check(ccall((:crg_build_fv_to_se, libcrg[]), Cint,
                        (Ref{CrgSeSpace}, Ref{CrgGridDesc}, Ref{CrgSeOpts}, Ref{Ptr{Cvoid}}), space, Ref(f), opts, out))
        else
            check(ccall((:crg_build_se_to_fv, libcrg[]), Cint,
                        (Ref{CrgGridDesc}, Ref{CrgSeSpace}, Ref{CrgSeOpts}, Ref{Ptr{Cvoid}}), Ref(f), space, opts, out))
        end
    end
    A = GB300Sparse(out[])
    nd, ns = size(A)
    dst_areas = Vector{Float64}(undef, nd)
    src_areas = Vector{Float64}(undef, ns)
    check(ccall((:crg_get_areas, libcrg[]), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), A.ptr, dst_areas, src_areas))
    return A, dst_areas, src_areas
end

"""
    se_dss!(field::CuArray, group_ptr, group_nodes, weights; nfields = 1)

`crg_se_dss`: the weighted DSS of `Spaces.weighted_dss!` on a flat nodal field
(device arrays; groups of coincident nodes as CSR).
"""
function se_dss!(field, group_ptr, group_nodes, weights; stream::Ptr{Cvoid} = C_NULL)
    T = eltype(field)
    dt = T == Float64 ? CRG_F64 : T == Float32 ? CRG_F32 : throw(ArgumentError("unsupported eltype $T"))
    n = size(field, 1)
    nf = length(field) ÷ n
    check(ccall((:crg_se_dss, libcrg[]), Cint,
                (Int32, Ptr{Cvoid}, Int64, Int64, Int64, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Int64, Ptr{Cvoid}),
                dt, pointer(field), 1, n, nf, pointer(group_ptr), pointer(group_nodes), pointer(weights),
                length(group_ptr) - 1, stream))
    return field
end

"CSC copy of A with Julia's 1-based indices: the reference's `R.intersections`."
function SparseArrays.SparseMatrixCSC(A::GB300Sparse)
    nd, ns = size(A)
    nnz = Int(A.info.nnz)
    colptr = Vector{Int64}(undef, ns + 1); rowval = Vector{Int64}(undef, nnz); nzval = Vector{Float64}(undef, nnz)
    check(ccall((:crg_get_csc, libcrg[]), Cint, (Ptr{Cvoid}, Int32, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}),
                A.ptr, 1, colptr, rowval, nzval))
    return SparseMatrixCSC(nd, ns, colptr, rowval, nzval)
end

end # module
