"""
`ChainRulesCore.rrule`s of the GB300 regridding (the reference has no
derivative rules; its Project.toml has no ChainRulesCore).

- `regrid(A, s; normalize, dims)`: `s̄ = A' (d̄ ./ a_d)` through the other
  stored copy of A (`crg_apply_adjoint`, no atomics); `A` may be a
  transposed view.
- `regrid_on(V, W, s; normalize)`: the same `s̄`, and the cotangents of the
  destination vertices `V` (`crg_area_grad`: the derivatives of the
  intersection and destination cell areas through every clipped vertex) and
  of the source vertices `W` (`crg_area_grad` of the regridder built the
  other way round).  Each is a thunk, so a caller that needs only `s̄`
  builds nothing more.
"""
module ConservativeRegriddingGB300ChainRulesCoreExt

using ChainRulesCore
import ConservativeRegriddingGB300 as GB

const AnyGB = Union{GB.GB300Sparse,GB.GB300SparseT}

# A dense cotangent shaped and typed like `d` from whatever the caller's AD
# hands back (a lazy fill, a view, another array type).
function _dense_like(d, ḡ)
    g = similar(d)
    g .= ḡ
    return g
end

function ChainRulesCore.rrule(::typeof(GB.regrid), A::AnyGB, s::StridedArray{T};
                              normalize::Bool = true, dims::Int = 1) where {T<:Union{Float32,Float64}}
    d = GB.regrid(A, s; normalize, dims)
    function regrid_pullback(d̄)
        ḡ = unthunk(d̄)
        ḡ isa AbstractZero && return (NoTangent(), NoTangent(), ZeroTangent())
        s̄ = GB.adjoint!(similar(s), A, _dense_like(d, ḡ); normalize, dims)
        return NoTangent(), NoTangent(), s̄
    end
    return d, regrid_pullback
end

function ChainRulesCore.rrule(::typeof(GB.regrid_on), V::Array{Float64,3}, W::Array{Float64,3}, s::Vector{Float64};
                              normalize::Bool = false)
    A, a_d, _ = GB.build(V, W; normalize)
    d = GB.regrid(A, s)
    function regrid_on_pullback(d̄)
        ḡ = unthunk(d̄)
        ḡ isa AbstractZero && return (NoTangent(), ZeroTangent(), ZeroTangent(), ZeroTangent())
        g = _dense_like(d, ḡ)
        # d = (A s) ./ a is the same for normalised and unnormalised A and a:
        # differentiate the unnormalised areas
        a = A.info.normalized != 0 ? a_d .* A.info.normalizer : a_d
        u = g ./ a
        s̄ = @thunk GB.adjoint!(similar(s), A, g)
        V̄ = @thunk GB.area_grad(A, V, W; row_weight = u, src_field = s, area_weight = -g .* d ./ a)
        W̄ = @thunk GB.src_area_grad(V, W, u, s)
        return NoTangent(), V̄, W̄, s̄
    end
    return d, regrid_on_pullback
end

end # module
