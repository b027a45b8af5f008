# Tests of the ccall drop-in, in the style of the reference's test/runtests.jl
# (testsystem.jl, testmeasurements.jl) plus the engine's additions.  They need
# Julia, a CUDA GPU and PIMC_GB300_LIB pointing at the built library.
using Test
using Pimc

@testset "System (test/testsystem.jl)" begin
    s = System(Harmonic(1.0); N = 2)
    @test s.N == 2
    s = System(Harmonic(1.0); N = 5, M = 30, L = 3.0)
    @test s.N == 5 && s.M == 30
    # periodic bounds: no bead outside [-L, L] after a run
    updates = [(2, SingleCenterOfMass(s, 1.0)), (1, ReshapeLinear(s, 8)), (1, ReshapeSwapLinear(s, 8))]
    run!(s, 10_000, updates)
    for p in s.world
        @test all(abs.(p.r) .<= s.L)
    end
end

@testset "Density (test/testmeasurements.jl)" begin
    s = System(Harmonic(1.0); λ = 0.5, M = 20, N = 4, L = 5.0, T = 1.0, length_measurement_cycle = 1)
    d = Density(s; nbins = 64)
    updates = [(1, ReshapeLinear(s, 8)), (2, ReshapeSwapLinear(s, 8)), (2, SingleCenterOfMass(s, 1.0))]
    run!(s, 10_000, updates; Zmeasurements = [d])
    @test d.ndata > 0
    # the one-bin-shifted histogram drops the first row and column
    @test sum(d.dens) / d.ndata <= s.N
    @test sum(d.dens) / d.ndata > 0.8 * s.N
end

@testset "Energy of one trapped particle" begin
    # N = 1, d = 2, beta = 1: <E> = coth(1/2) in the continuum
    s = System(Harmonic(1.0); λ = 0.5, M = 64, N = 1, L = 6.0, T = 1.0, length_measurement_cycle = 1,
               semantics = 1)
    E = Energy(s, 200_000)
    updates = [(1, ReshapeLinear(s, 16)), (1, SingleCenterOfMass(s, 1.0))]
    run!(s, 20_000, updates)
    run!(s, 400_000, updates; Zmeasurements = [E])
    e = E.energy[1]
    @test abs(sum(e) / length(e) - coth(0.5)) < 0.05
end

@testset "optical lattice, contact propagator, files" begin
    V = generate_V(0.5, 2.0, :l25) + Harmonic(0.3)
    s = System(V; M = 16, N = 4, L = 6.0, T = 1.0, λ = 0.5)
    @test length(lattice_angles(:l65)) == 16
    prop = build_prop_int(5.0, 1.16, 1 / 16; n = 64)
    @test prop.table ≈ transpose(prop.table)
    @test isfinite(prop([0.3, 0.1], [0.2, 0.2], 1 / 16))
    sc = System(Harmonic(1.0); M = 16, N = 4, L = 3.0, T = 1.0, λ = 0.5, interactions = true,
                propint = prop, rₐ = 1.0)
    run!(sc, 1000, [(1, ReshapeLinear(sc, 8)), (1, ReshapeSwapLinear(sc, 8))])
    path = tempname()
    save_paths(s; path = path)
    lines = readlines(path)
    @test lines[1] == "tau,p1 x,p1 y,p2 x,p2 y,p3 x,p3 y,p4 x,p4 y"
    @test length(lines) == s.M + 2
    ck = tempname()
    save_checkpoint(s, ck)
    x0 = [p.r for p in s.world]
    run!(s, 1000, [(1, ReshapeLinear(s, 8))])
    load_checkpoint(s, ck)
    @test [p.r for p in s.world] == x0
end
