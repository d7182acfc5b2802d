# Tests of the GB300 binding against ConservativeRegridding.jl itself, for a
# machine with Julia, the reference package and a GB300 with libcrg_gb300.so
# built (`python -c "import __graft_entry__ as g; g.build()"` at the
# repository root, or CRG_GB300_LIB pointing at the library):
#
#     julia --project=test -e 'using Pkg; Pkg.instantiate(); include("test/runtests.jl")'
#
# The grids are the small FP64 case of the benchmark: a 2-degree lon-lat source
# and a 3-degree destination shifted by +0.7 / +0.4 degrees (latitude edges
# clamped to the poles), great-circle edges on the unit sphere.

using Test
using LinearAlgebra, SparseArrays
import GeometryOps as GO
import ConservativeRegridding as CR
using ConservativeRegriddingGB300
import ConservativeRegriddingGB300 as GB
import ChainRulesCore

lonlat_points(lons, lats) = [GO.UnitSphereFromGeographic()((lon, lat)) for lon in lons, lat in lats]
as_array(points) = [p[c] for c in 1:3, p in points]          # 3 x (nx+1) x (ny+1)

const SRC = lonlat_points(0:2:360, -90:2:90)
const DST = lonlat_points(0.7 .+ (0:3:360), clamp.(-89.6 .+ (0:3:180), -90, 90))

# entries above `tol` of the largest: rounding-level slivers are the one place
# where GeometryOps and the GPU clip may disagree about "area > 0"
significant(A, tol) = droptol!(copy(A), tol * maximum(abs, nonzeros(A)))

@testset "Regridder(GB300(), dst, src) matches Regridder(dst, src)" begin
    R = CR.Regridder(DST, SRC; normalize = true)
    Rg = CR.Regridder(GB300(), DST, SRC; normalize = true)
    @test Rg isa CR.Regridder
    @test size(Rg) == size(R)
    A, Ag = significant(R.intersections, 1e-12), significant(SparseMatrixCSC(Rg.intersections), 1e-12)
    @test Ag.colptr == A.colptr
    @test Ag.rowval == A.rowval
    @test isapprox(nonzeros(Ag), nonzeros(A); rtol = 1e-12)
    @test isapprox(Rg.dst_areas, R.dst_areas; rtol = 1e-12)
    @test isapprox(Rg.src_areas, R.src_areas; rtol = 1e-12)
    @test_throws ArgumentError normalize!(Rg)
end

@testset "regrid! runs the reference pipeline" begin
    R = CR.Regridder(DST, SRC; normalize = true)
    Rg = CR.Regridder(GB300(), DST, SRC; normalize = true)
    nd, ns = size(R)
    s = rand(ns)
    d, dg = zeros(nd), zeros(nd)
    CR.regrid!(d, R, s)
    CR.regrid!(dg, Rg, s)
    @test isapprox(dg, d; rtol = 1e-12)
    # transpose(R) shares the handle and swaps the areas
    b, bg = zeros(ns), zeros(ns)
    CR.regrid!(b, transpose(R), d)
    CR.regrid!(bg, transpose(Rg), d)
    @test isapprox(bg, b; rtol = 1e-12)
    # a strided (non-contiguous) vector goes through dst_temp / src_temp
    big = zeros(2nd)
    CR.regrid!(view(big, 1:2:2nd), Rg, s)
    @test isapprox(big[1:2:end], d; rtol = 1e-12)
    # N-D arrays: one library call per group of slices, any spatial axis
    S = rand(ns, 3, 4)
    D = zeros(nd, 3, 4)
    CR.regrid!(D, Rg, S; dims = 1)
    @test isapprox(D, cat((R.intersections * S[:, :, k] ./ R.dst_areas for k in 1:4)...; dims = 3); rtol = 1e-12)
    S2 = permutedims(S, (2, 1, 3))                     # 3 x ns x 4: the spatial axis in the middle
    D2 = zeros(3, nd, 4)
    CR.regrid!(D2, Rg, S2; dims = 2)
    @test isapprox(permutedims(D2, (2, 1, 3)), D; rtol = 1e-12)
    # FP32 fields with FP32 weights and accumulation
    S32 = Float32.(S[:, :, 1])
    D32 = zeros(Float32, nd, 3)
    GB.apply!(D32, Rg.intersections, S32)
    @test isapprox(D32, D[:, :, 1]; rtol = 1e-5)
end

@testset "rrules" begin
    Rg = CR.Regridder(GB300(), DST, SRC; normalize = true)
    A = Rg.intersections
    nd, ns = size(A)
    s, ḡ = rand(ns), randn(nd)
    d, back = ChainRulesCore.rrule(GB.regrid, A, s)
    @test d ≈ GB.regrid(A, s)
    _, _, s̄ = back(ḡ)
    M = SparseMatrixCSC(A)
    @test isapprox(s̄, M' * (ḡ ./ Rg.dst_areas); rtol = 1e-12)
    # transposed view: the adjoint reads the forward copy
    _, backT = ChainRulesCore.rrule(GB.regrid, transpose(A), d)
    _, _, d̄ = backT(s̄)
    @test isapprox(d̄, M * (s̄ ./ Rg.src_areas); rtol = 1e-12)

    # vertex cotangents of L = w . regrid_on(V, W, s) against central
    # differences along the longitude / latitude tangents (h = 1e-7 degrees)
    V, W = as_array(DST), as_array(SRC)
    w = randn(nd)
    d, back = ChainRulesCore.rrule(GB.regrid_on, V, W, s)
    _, V̄, W̄, _ = back(w)
    V̄, W̄ = ChainRulesCore.unthunk(V̄), ChainRulesCore.unthunk(W̄)
    h = 1e-7
    loss(V, W) = dot(w, GB.regrid_on(V, W, s))
    for (X, X̄, pts, which) in ((V, V̄, DST, :dst), (W, W̄, SRC, :src)), (i, j) in ((5, 7), (40, 20), (70, 33))
        lon, lat = GO.UnitSpherical.GeographicFromUnitSphere()(pts[i, j])
        for (dl, dp) in ((h, 0.0), (0.0, h))
            Xp, Xm = copy(X), copy(X)
            Xp[:, i, j] .= GO.UnitSphereFromGeographic()((lon + dl, lat + dp))
            Xm[:, i, j] .= GO.UnitSphereFromGeographic()((lon - dl, lat - dp))
            fd = which == :dst ? (loss(Xp, W) - loss(Xm, W)) / 2h : (loss(V, Xp) - loss(V, Xm)) / 2h
            t = (X[:, i, j] .- Xm[:, i, j]) ./ h           # the tangent per degree, to O(h)
            @test isapprox(dot(X̄[:, i, j], t), fd; rtol = 1e-4, atol = 1e-6)
        end
    end
end
