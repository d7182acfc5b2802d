"""
    ConservativeRegriddingGB300

Julia binding of `libcrg_gb300.so` (declared in `include/crg.h`): the GPU build
and apply of ConservativeRegridding.jl's `Regridder`, `regrid!` and
`transpose(R)`.  The matrix, the areas and the weights live on the GPU; field
arrays may be `CuArray`s (device pointers) or host `Array`s (staged by the
library).

This file is the `ccall` layer a maintainer adds next to ConservativeRegridding.jl;
it depends only on `Libdl` and `SparseArrays`.
"""
module ConservativeRegriddingGB300

using Libdl
using SparseArrays
using LinearAlgebra

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
LinearAlgebra.transpose(A::GB300Sparse) = GB300SparseT(A)
LinearAlgebra.transpose(A::GB300SparseT) = A.parent

"""
    curvilinear(points::Array{Float64,3})

Describe a grid of `(nx+1) x (ny+1)` vertices given as a `3 x (nx+1) x (ny+1)`
array of unit vectors (the reference's `CellBasedGrid` vertex matrix).
"""
function curvilinear(points::Array{Float64,3})
    dim, nxp, nyp = size(points)
    nx = Ref(Int64(nxp - 1)); ny = Ref(Int64(nyp - 1))
    desc = CrgGridDesc(0, dim == 3 ? 1 : 0, 1, 0, nx[] * ny[],
                       Base.unsafe_convert(Ptr{Int64}, nx), Base.unsafe_convert(Ptr{Int64}, ny),
                       pointer(points), C_NULL, C_NULL)
    return desc, (points, nx, ny)
end

"""
    Regridder(dst_points, src_points; normalize = false) -> ConservativeRegridding.Regridder

GPU build of `Regridder(dst, src; normalize)` for vertex-matrix grids.  The
returned struct has `intersections::GB300Sparse` and host copies of the areas.
"""
function build(dst, src; normalize::Bool = false)
    d, keep_d = dst
    s, keep_s = src
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

"""
    apply!(y, A, x; transpose = false, normalize = true, dims = 1)

`perform_regridding!` + `finalize_regridding!` for dense arrays: one call for
all slices along the non-spatial axes (the reference loops `mul!` per slice).
"""
function apply!(y::AbstractArray{T}, A::Union{GB300Sparse,GB300SparseT}, x::AbstractArray{T};
                normalize::Bool = true, dims::Int = 1) where {T<:Union{Float64,Float32}}
    ndims(x) == ndims(y) || throw(DimensionMismatch("source and destination ranks must match"))
    1 <= dims <= ndims(x) || throw(ArgumentError("dims=$dims is out of range for a $(ndims(x))-dimensional array"))
    h, t = A isa GB300SparseT ? (A.parent, Int32(1)) : (A, Int32(0))
    sx, sy = strides(x), strides(y)
    nf = length(x) ÷ size(x, dims)
    fx = nf == 1 ? 1 : sx[dims == 1 ? 2 : 1]   # slices must be uniformly strided (dense arrays)
    fy = nf == 1 ? 1 : sy[dims == 1 ? 2 : 1]
    dtype = T === Float64 ? CRG_F64 : CRG_F32
    check(ccall((:crg_apply, libcrg[]), Cint,
                (Ptr{Cvoid}, Int32, Int32, Ptr{Cvoid}, Int64, Int64, Ptr{Cvoid}, Int64, Int64, Int64, Int32, Ptr{Cvoid}),
                h.ptr, t, dtype, pointer(x), sx[dims], fx, pointer(y), sy[dims], fy, nf, normalize, C_NULL))
    return y
end

"""
    adjoint!(gs, A, gd; normalize = true, dims = 1)

Pullback of `apply!` with respect to the source field: `gs = A' (gd ./ a_d)`
(or `A gd ./ ...` for a transposed view), through the other stored copy of A.
"""
function adjoint!(gs::AbstractArray{T}, A::Union{GB300Sparse,GB300SparseT}, gd::AbstractArray{T};
                  normalize::Bool = true, dims::Int = 1) where {T<:Union{Float64,Float32}}
    h, t = A isa GB300SparseT ? (A.parent, Int32(1)) : (A, Int32(0))
    sx, sy = strides(gd), strides(gs)
    nf = length(gd) ÷ size(gd, dims)
    fx = nf == 1 ? 1 : sx[dims == 1 ? 2 : 1]
    fy = nf == 1 ? 1 : sy[dims == 1 ? 2 : 1]
    dtype = T === Float64 ? CRG_F64 : CRG_F32
    check(ccall((:crg_apply_adjoint, libcrg[]), Cint,
                (Ptr{Cvoid}, Int32, Int32, Ptr{Cvoid}, Int64, Int64, Ptr{Cvoid}, Int64, Int64, Int64, Int32, Ptr{Cvoid}),
                h.ptr, t, dtype, pointer(gd), sx[dims], fx, pointer(gs), sy[dims], fy, nf, normalize, C_NULL))
    return gs
end

"""
    area_grad(A, dst, src; row_weight, src_field, area_weight) -> Array{Float64}

Cotangent of the destination vertices for `sum_ij u_i s_j dA_ij/dV + sum_i c_i da_i/dV`
(`crg_area_grad`), laid out like `dst`'s vertex array.  For the rrule of
`d = regrid(R, s)` with output cotangent `g`: `u = g ./ a`, `c = -g .* d ./ a`
(unnormalised areas `a`).
"""
function area_grad(A::GB300Sparse, dst, src; row_weight = nothing, src_field = nothing, area_weight = nothing)
    d, keep_d = dst
    s, keep_s = src
    g = zeros(Float64, d.kind == 0 ? size(keep_d[1]) : (Int(d.ncells) * Int(d.max_verts) * 3,))
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
    build_batch(pairs; normalize = false, nthreads = 0) -> Vector{GB300Sparse}

`crg_build_batch`: many `(dst, src)` descriptor pairs built concurrently.
"""
function build_batch(pairs; normalize::Bool = false, nthreads::Integer = 0)
    n = length(pairs)
    dd = [p[1][1] for p in pairs]; ds = [p[2][1] for p in pairs]
    keep = [(p[1][2], p[2][2]) for p in pairs]
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
