"""
    Pimc

Drop-in for oameye/PIMC.jl's user API backed by the GB300 engine
(`libpimc_gb300.so`, C ABI in `include/pimc.h`) through `ccall`.

Kept from the reference (names, keyword arguments, fields read by its
examples and tests): `System`, `ReshapeLinear`, `ReshapeSwapLinear`,
`SingleCenterOfMass`, `PolymerCenterOfMass`, `run!`, `apply!`,
`acceptance`, `Density`, `Energy`, `Counter`, `Step`, `NumbOfSlices`.
Julia closures cannot cross the ABI: the potential must be built from
`Harmonic`, `SquareLattice` (and their sum), the interaction propagator from
`GaussianPair` or `build_prop_int` (the tabulated contact propagator, its table
built on the device); any other closure raises (there is no CPU fallback).
Slices and particles are 1-based on this side as in the reference.

This file is written against the header and the Python mirror
(`pimc.jl_gb300/pimc/api.py`) that the test-suite exercises; no Julia
toolchain exists on the build machines, so it is not executed there.
"""
module Pimc

using ChainRulesCore
using LinearAlgebra

export System, run!, apply!, acceptance, ReshapeLinear, ReshapeSwapLinear,
       SingleCenterOfMass, PolymerCenterOfMass, Density, Energy, Counter, Step,
       NumbOfSlices, Harmonic, SquareLattice, GaussianPair, action_gradients,
       build_prop_int, ContactPropagator, determine_nnrange,
       RadialDistribution, Superfluid, radial_g, winding_fraction, area_fraction,
       save_paths, save_density, save_checkpoint, load_checkpoint,
       OpticalLattice, generate_V, lattice_angles

const libpimc = get(ENV, "PIMC_GB300_LIB",
                    joinpath(@__DIR__, "..", "..", "..", "lib", "libpimc_gb300.so"))

# ---------------------------------------------------------------- C structs
struct PimcParams
    dim::Cint; N::Cint; M::Cint
    L::Cdouble; T::Cdouble; lambda::Cdouble; mu::Cdouble
    harmonic_omega::Cdouble; lattice_V0::Cdouble; lattice_a::Cdouble
    interactions::Cint; pair_g::Cdouble; pair_sigma::Cdouble
    r_a::Cdouble; hardcore_a::Cdouble; semantics::Cint
    seed::UInt64; density_nbins::Cint; energy_capacity::Cint; retry_cap::Cint
end

mutable struct PimcMoveMix
    staging_phases::Cint
    stage_slices::Cint; stage_min::Cint; stage_max::Cint
    stage_minacc::Cdouble; stage_maxacc::Cdouble
    swaps_per_sweep::Cint
    swap_slices::Cint; swap_min::Cint; swap_max::Cint
    swap_minacc::Cdouble; swap_maxacc::Cdouble
    com_phases::Cint
    com_step::Cdouble; com_minstep::Cdouble; com_maxstep::Cdouble
    com_minacc::Cdouble; com_maxacc::Cdouble
    polymer_com_phases::Cint
    pcom_step::Cdouble; pcom_minstep::Cdouble; pcom_maxstep::Cdouble
    pcom_minacc::Cdouble; pcom_maxacc::Cdouble
    adapt::Cint; measure_every::Cint
end

struct PimcStats
    attempts::NTuple{4,Culonglong}; accepts::NTuple{4,Culonglong}
    skips::Culonglong; bead_updates::Cdouble; sweeps::Culonglong
    measurements::Culonglong; stage_slices::Cint; swap_slices::Cint
    com_step::Cdouble; pcom_step::Cdouble
    bead_updates_kind::NTuple{4,Cdouble}
end

function check(rc)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:pimc_last_error, libpimc), Cstring, ()))
    error("pimc error $rc: $msg")
end

# ---------------------------------------------------------------- potentials
struct Harmonic; omega::Float64; end
(h::Harmonic)(r) = 0.5 * h.omega^2 * sum(abs2, r)
struct SquareLattice; V0::Float64; a::Float64; end
(s::SquareLattice)(r) = s.V0 * sum(x -> sin(pi * x / s.a)^2, r)
"""
    OpticalLattice(angles, scale, depth; helical = false)

`depth * normalized_intensity(r, angles, scale)` of the reference's
examples/tools/potentialtools.jl:1-16 (at most 16 beams, 2D), run on the device.
"""
struct OpticalLattice
    angles::Vector{Float64}; scale::Float64; depth::Float64; helical::Bool
end
OpticalLattice(angles, scale, depth; helical::Bool = false) =
    OpticalLattice(collect(Float64, angles), scale, depth, helical)
function (o::OpticalLattice)(r)
    s, c = 0.0, 0.0
    for a in o.angles
        rk = r[1] * sin(a) + r[2] * cos(a)
        s += o.helical ? sin(2π * rk * o.scale + a) : sin(2π * rk * o.scale)
        c += o.helical ? cos(2π * rk * o.scale + a) : cos(2π * rk * o.scale)
    end
    s /= length(o.angles); c /= length(o.angles)
    return o.depth * (s * s + c * c)
end

"""
    lattice_angles(sym)

The beam sets of generate_V (potentialtools.jl:18-39): `:l25` / `:l65` point at
the integer points of x^2 + y^2 = 25 / 65 (angle a with (sin a, cos a) = (x, y)/R),
`:cubic` is 2πk/4.
"""
function lattice_angles(sym::Symbol)
    sym === :cubic && return [2π * k / 4 for k in 0:3]
    r2 = sym === :l25 ? 25 : sym === :l65 ? 65 : error("unknown lattice $sym")
    return sort([atan(x, y) for x in -9:9 for y in -9:9 if x^2 + y^2 == r2])
end

"""
    generate_V(scale, depth, sym; attractive = true)
    generate_V(angles, scale, depth; helical = false)

The reference's optical-lattice constructors (potentialtools.jl:18-39) as
engine-known potentials; `:harmonic` gives `Harmonic(1.0)`.
"""
function generate_V(scale::Float64, depth::Float64, sym::Symbol; attractive::Bool = true)
    sym === :harmonic && return Harmonic(1.0)
    return OpticalLattice(lattice_angles(sym), scale, attractive ? -depth : depth, false)
end
generate_V(angles::Vector{Float64}, scale::Float64, depth::Float64; helical::Bool = false) =
    OpticalLattice(angles, scale, depth, helical)

struct PotentialSum; terms::Vector{Any}; end
(p::PotentialSum)(r) = sum(t(r) for t in p.terms)
const PotentialTerm = Union{Harmonic,SquareLattice,OpticalLattice}
Base.:+(a::PotentialTerm, b::PotentialTerm) = PotentialSum([a, b])
Base.:+(a::PotentialSum, b::PotentialTerm) = PotentialSum([a.terms; b])
struct GaussianPair; g::Float64; sigma::Float64; end
(gp::GaussianPair)(r1, r2, tau) =
    exp(-tau / 2 * (gp.g * exp(-sum(abs2, r1) / (2gp.sigma^2)) +
                    gp.g * exp(-sum(abs2, r2) / (2gp.sigma^2))))

"""
    build_prop_int(L, g0, τ; n = 600)

The contact-interaction propagator of the reference (src/propagator.jl:35-89):
the n x n table of its Bessel integrals over the radii range(1e-20, L, n),
computed on the device (`pimc_contact_table`), and a callable
`prop_int(r1_rel, r2_rel, τ) = 1 + T(|r1|, |r2|) / prop_rel0(r1, r2, τ)` by
linear interpolation of it.  As a System's `propint` it runs on the device.
"""
struct ContactPropagator
    range::Float64; g0::Float64; tau::Float64; n::Int; table::Matrix{Float64}
end
function build_prop_int(L::Float64, g0::Float64, τ::Float64; n::Int = 600)
    t = Matrix{Float64}(undef, n, n)
    check(ccall((:pimc_contact_table, libpimc), Cint,
                (Cdouble, Cdouble, Cdouble, Cint, Ptr{Cdouble}), g0, τ, L, n, t))
    return ContactPropagator(L, g0, τ, n, t)   # symmetric: row- and column-major agree
end
function contact_terms(cp::ContactPropagator, r1::Float64, r2::Float64)
    h = (cp.range - 1e-20) / (cp.n - 1)
    function cell(r)
        p = (clamp(r, 1e-20, cp.range) - 1e-20) / h
        f = min(floor(p), cp.n - 2)
        return Int(f) + 1, p - f
    end
    (i, wx), (j, wy) = cell(r1), cell(r2)
    t = cp.table
    c0 = (1 - wy) * t[i, j] + wy * t[i, j+1]
    c1 = (1 - wy) * t[i+1, j] + wy * t[i+1, j+1]
    return (1 - wx) * c0 + wx * c1
end
(cp::ContactPropagator)(r1_rel, r2_rel, τ) =
    1 + contact_terms(cp, norm(r1_rel), norm(r2_rel)) /
        (exp(-dot(r1_rel - r2_rel, r1_rel - r2_rel) / (4τ)) / (4π * τ))

"""
    determine_nnrange(propint, τ, a, b)

The radius r where `propint([r], [r], τ) = 0.999` above the curve's minimum
(src/system.jl:10-15): the minimiser on a 4097-point grid of [a, b], then
bisection to the last bit.
"""
function determine_nnrange(propint, τ::Float64, a::Float64, b::Float64)
    f(r) = propint([r], [r], τ) - 0.999
    rs = range(a, b, length = 4097)
    lo, hi = rs[argmin(f.(rs))], b
    flo = f(lo)
    flo * f(hi) > 0 && error("determine_nnrange: no sign change on (r_min, b)")
    while true
        mid = (lo + hi) / 2
        (mid <= lo || mid >= hi) && break
        fm = f(mid)
        fm == 0 && return mid
        if (fm < 0) == (flo < 0)
            lo, flo = mid, fm
        else
            hi = mid
        end
    end
    return abs(flo) <= abs(f(hi)) ? lo : hi
end

function potential_terms(V)
    omega, V0, a, beams = 0.0, 0.0, 1.0, nothing
    for t in (V isa PotentialSum ? V.terms : [V])
        if t isa Harmonic
            omega = t.omega
        elseif t isa SquareLattice
            V0, a = t.V0, t.a
        elseif t isa OpticalLattice
            beams === nothing || error("one optical lattice per potential")
            beams = t
        elseif t === zero || t isa Function && t(zeros(2)) == 0 && t(ones(2)) == 0
            nothing
        else
            error("potential must be Harmonic, SquareLattice, OpticalLattice or their sum")
        end
    end
    return omega, V0, a, beams
end

function attach_beams(h::Ptr{Cvoid}, b)
    b === nothing && return nothing
    check(ccall((:pimc_set_beams, libpimc), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint, Cdouble, Cdouble, Cint),
                h, -1, b.angles, length(b.angles), b.scale, b.depth, b.helical))
end

# ---------------------------------------------------------------- System
mutable struct System
    handle::Ptr{Cvoid}
    dim::Int64; M::Int64; N::Int64; Ninit::Int64
    μ::Float64; λ::Float64; L::Float64; vol::Float64; β::Float64; τ::Float64
    V::Any; dV::Any; propint::Any; a::Float64; ctr::Int64
    measure_scheme::Symbol
    N_MC::Dict{Int64,Int64}; Nctr::Dict{Int64,Int64}; Ncycle::Int64
    params::PimcParams
    eser_seen::Int
end

function System(potential; dV = zero, dim::Int64 = 2, M::Int64 = 100, N::Int64 = 2,
                μ::Float64 = 0.0, L::Float64 = 4.0, T::Float64 = 1.0, λ::Float64 = 1.0,
                interactions::Bool = false, propint = _ -> 0.0, g::Float64 = 0.0,
                rₐ::Float64 = 0.0, length_measurement_cycle::Int64 = 10,
                measure_scheme::Symbol = :c, semantics::Int = 0, seed::UInt64 = UInt64(20261203))
    omega, V0, a_lat, beams = potential_terms(potential)
    pg, ps = 0.0, 1.0
    if interactions
        if propint isa GaussianPair
            rₐ > 0 || error("pass rₐ with a GaussianPair")
            pg, ps = propint.g, propint.sigma
        elseif propint isa ContactPropagator
            # init_int (src/system.jl:17-34)
            rₐ == 0.0 && (rₐ = determine_nnrange(propint, 1 / (T * M), 1e-20, L))
        else
            error("interactions=true needs propint = GaussianPair(g, σ) or build_prop_int(L, g0, τ)")
        end
    end
    a = interactions && g > 0 ? exp(-2π / g) : 0.0
    p = PimcParams(dim, N, M, L, T, λ, μ, omega, V0, a_lat, interactions, pg, ps, rₐ, a,
                   semantics, seed, 0, 0, 0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:pimc_create, libpimc), Cint, (Ref{PimcParams}, Ref{Ptr{Cvoid}}), p, h))
    s = System(h[], dim, M, N, N, μ, λ, L, (2L)^dim, 1 / T, 1 / (T * M), potential, dV,
               propint, a, 10_000, measure_scheme, Dict(N => 0), Dict(N => 0),
               length_measurement_cycle, p, 0)
    finalizer(s -> ccall((:pimc_destroy, libpimc), Cint, (Ptr{Cvoid},), s.handle), s)
    attach_beams(s.handle, beams)
    if interactions && propint isa ContactPropagator
        tab = Matrix(transpose(propint.table))   # the C side reads it row-major
        check(ccall((:pimc_set_contact_table, libpimc), Cint,
                    (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint, Cdouble),
                    s.handle, -1, tab, propint.n, propint.range))
    end
    return s
end

"""Positions as the reference's `s.world[n].r` (M x dim per particle)."""
function Base.getproperty(s::System, f::Symbol)
    if f === :world
        x = Vector{Float64}(undef, s.dim * s.N * s.M)
        check(ccall((:pimc_get_beads, libpimc), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), s.handle, x))
        nx = Vector{Cint}(undef, s.N)
        check(ccall((:pimc_get_next, libpimc), Cint, (Ptr{Cvoid}, Ptr{Cint}), s.handle, nx))
        X = reshape(x, s.M, s.N, s.dim)   # x[d][n][j] row-major == X[j, n, d]
        return [(r = X[:, n, :], next = nx[n] + 1) for n in 1:s.N]
    end
    return getfield(s, f)
end

# ---------------------------------------------------------------- updates
Base.@kwdef mutable struct Counter
    queue::Vector{Bool} = Bool[]; tries::Int64 = 0; range::Int64 = 100_000; adj::Int64 = 10
end
mutable struct Step; size::Float64; minstep::Float64; maxstep::Float64; minacc::Float64; maxacc::Float64; end
mutable struct NumbOfSlices; m::Int64; minslices::Int64; maxslices::Int64; minacc::Float64; maxacc::Float64; end
acceptance(q) = sum(q) / length(q)

abstract type Update end
for (T, V) in ((:ReshapeLinear, :NumbOfSlices), (:ReshapeSwapLinear, :NumbOfSlices))
    @eval struct $T <: Update
        counter::Counter; var::$V; counter_var::Counter
        $T(s::System, slices::Int64; minslices = 2, maxslices = s.M - 2, minacc = 0.6,
           maxacc = 0.8, adj = 10, range = 10_000) =
            new(Counter(), NumbOfSlices(min(slices, maxslices), minslices, maxslices, minacc, maxacc),
                Counter(adj = adj, range = range))
    end
end
for T in (:SingleCenterOfMass, :PolymerCenterOfMass)
    @eval struct $T <: Update
        counter::Counter; var::Step; counter_var::Counter
        $T(s::System, step::Float64; minstep = 1e-1, maxstep = s.L / 2, minacc = 0.4,
           maxacc = 0.6, adj = 10, range = 10_000) =
            new(Counter(), Step(step, minstep, maxstep, minacc, maxacc), Counter(adj = adj, range = range))
    end
end

# single attempts with host-drawn random numbers (src/updates/*.jl call sites)
function (u::ReshapeLinear)(s::System)
    n, j0 = rand(0:s.N-1), rand(0:s.M-1)
    m = min(u.var.maxslices, rand(2:u.var.m))
    nr, un = randn((m - 1) * s.dim * (s.a > 0 ? 64 : 1)), rand(1)
    res = Ref{Cint}(0)
    check(ccall((:pimc_attempt_staging, libpimc), Cint,
                (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ref{Cint}, Ptr{Cdouble}),
                s.handle, n, j0, m, nr, length(nr), un, 1, res, C_NULL))
    acc = res[] == 1
    push!(u.counter_var.queue, acc); u.counter_var.tries += 1
    return acc
end

function (u::ReshapeSwapLinear)(s::System)
    s.N <= 1 && return false
    j0, m, n1 = rand(0:s.M-1), min(u.var.maxslices, rand(2:u.var.m)), rand(0:s.N-1)
    nr, un = randn(2 * (m - 1) * s.dim * (s.a > 0 ? 64 : 1)), rand(1)
    res, n2 = Ref{Cint}(0), Ref{Cint}(0)
    check(ccall((:pimc_attempt_swap, libpimc), Cint,
                (Ptr{Cvoid}, Cint, Cint, Cint, Cdouble, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint,
                 Ref{Cint}, Ref{Cint}, Ptr{Cdouble}),
                s.handle, j0, m, n1, rand(), nr, length(nr), un, 1, res, n2, C_NULL))
    res[] == 2 && return false
    acc = res[] == 1
    push!(u.counter_var.queue, acc); u.counter_var.tries += 1
    return acc
end

for (T, fn) in ((:SingleCenterOfMass, :pimc_attempt_com), (:PolymerCenterOfMass, :pimc_attempt_polymer_com))
    @eval function (u::$T)(s::System)
        nx = Vector{Cint}(undef, s.N)
        check(ccall((:pimc_get_next, libpimc), Cint, (Ptr{Cvoid}, Ptr{Cint}), s.handle, nx))
        cand = $(T === :SingleCenterOfMass) ? [i - 1 for i in 1:s.N if nx[i] == i - 1] : collect(0:s.N-1)
        isempty(cand) && return false
        un = rand(s.dim + 1)
        res = Ref{Cint}(0)
        check(ccall(($(QuoteNode(fn)), libpimc), Cint,
                    (Ptr{Cvoid}, Cint, Cdouble, Ptr{Cdouble}, Cint, Ref{Cint}),
                    s.handle, rand(cand), u.var.size, un, length(un), res))
        acc = res[] == 1
        push!(u.counter_var.queue, acc); u.counter_var.tries += 1
        return acc
    end
end

# ---------------------------------------------------------------- measurements
mutable struct Density
    nbins::Int64; bin::Float64; dens::Array{Float64}; ndata::Int64
    Density(s::System; nbins = 500) = new(nbins, 2s.L / nbins, zeros(ntuple(_ -> nbins, s.dim)), 0)
end
mutable struct Energy
    energy::Dict{Int64,Vector{Float64}}; energy_virial::Dict{Int64,Vector{Float64}}; n::Int
    Energy(s::System, n = 20_000) = new(Dict(0 => Float64[]), Dict(0 => Float64[]), n)
end

"""
    RadialDistribution(s; nbins = 100, rmax = s.L)

Pair radial distribution (the TODO of src/measurement.jl:125): every
measurement bins, at every slice, each unordered pair's minimum-image distance.
`radial_g(rd, s)` gives g(r) at the bin centres.
"""
mutable struct RadialDistribution
    nbins::Int64; rmax::Float64; bin::Float64; hist::Vector{Float64}; ndata::Int64
    RadialDistribution(s::System; nbins = 100, rmax = s.L) =
        new(nbins, rmax, rmax / nbins, zeros(nbins), 0)
end
function radial_g(rd::RadialDistribution, s::System)
    e = (0:rd.nbins) .* rd.bin
    shell = s.dim == 2 ? π .* diff(e .^ 2) : 2 .* diff(e)
    pairs = rd.ndata * s.M * s.N * (s.N - 1) / 2
    return rd.hist ./ (pairs .* shell ./ (2s.L)^s.dim)
end

"""
    Superfluid(s, n = 20_000)

Superfluid-fraction estimators (the TODO of src/measurement.jl:126), series
keyed by N: the squared winding `W2`, the signed area `area` about the origin
and `I` = sum r^2 / M.  `winding_fraction(sf, s, N)` = <W^2>/(2 dim λ β N) in a
periodic box; `area_fraction(sf, s, N)` = 2<A_z^2>/(λ β <I>) in a trap.
"""
mutable struct Superfluid
    W2::Dict{Int64,Vector{Float64}}; area::Dict{Int64,Vector{Float64}}
    I::Dict{Int64,Vector{Float64}}; n::Int
    Superfluid(s::System, n = 20_000) =
        new(Dict(0 => Float64[]), Dict(0 => Float64[]), Dict(0 => Float64[]), n)
end
mean_(v) = sum(v) / length(v)
winding_fraction(sf::Superfluid, s::System, N::Int) = mean_(sf.W2[N]) / (2 * s.dim * s.λ * s.β * N)
area_fraction(sf::Superfluid, s::System, N::Int) =
    2 * mean_(sf.area[N] .^ 2) / (s.λ * s.β * mean_(sf.I[N]))

# a handle with room for the requested histogram and series: the state moves
# over verbatim (positions, cached links, permutation)
function ensure_engine!(s::System, nb::Int, cap::Int)
    p = s.params
    (p.density_nbins == nb && p.energy_capacity >= cap) && return nothing
    x = Vector{Float64}(undef, s.dim * s.N * s.M)
    V = Vector{Float64}(undef, s.N * s.M)
    nx = Vector{Cint}(undef, s.N)
    check(ccall((:pimc_get_beads, libpimc), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), s.handle, x))
    check(ccall((:pimc_get_links, libpimc), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), s.handle, V))
    check(ccall((:pimc_get_next, libpimc), Cint, (Ptr{Cvoid}, Ptr{Cint}), s.handle, nx))
    q = PimcParams(p.dim, p.N, p.M, p.L, p.T, p.lambda, p.mu, p.harmonic_omega, p.lattice_V0,
                   p.lattice_a, p.interactions, p.pair_g, p.pair_sigma, p.r_a, p.hardcore_a,
                   p.semantics, p.seed, nb, max(p.energy_capacity, cap), p.retry_cap)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:pimc_create, libpimc), Cint, (Ref{PimcParams}, Ref{Ptr{Cvoid}}), q, h))
    check(ccall((:pimc_set_raw, libpimc), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cint}),
                h[], x, V, nx))
    if s.propint isa ContactPropagator && p.interactions != 0
        tab = Matrix(transpose(s.propint.table))
        check(ccall((:pimc_set_contact_table, libpimc), Cint,
                    (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint, Cdouble),
                    h[], -1, tab, s.propint.n, s.propint.range))
    end
    attach_beams(h[], potential_terms(s.V)[4])
    ccall((:pimc_destroy, libpimc), Cint, (Ptr{Cvoid},), s.handle)
    s.handle = h[]
    s.params = q
    s.eser_seen = 0
    return nothing
end

# ---------------------------------------------------------------- files
"""`save_paths(s)` (examples/tools/savetools.jl:30-34): paths.csv from the device state."""
save_paths(s::System; path::AbstractString = "paths.csv") =
    check(ccall((:pimc_write_paths_csv, libpimc), Cint, (Ptr{Cvoid}, Cint, Cstring), s.handle, 0, path))

"""`save_density(s, d, g, name, V)` (savetools.jl:52-65): the normalised density
table under the reference's file name."""
function save_density(s::System, d::Density, g, name, V)
    path = "density$(name)M$(s.M)beta$(s.β)N$(s.N)g$(g)V$(V).csv"
    counts = Vector{Float64}(vec(d.dens))
    check(ccall((:pimc_write_density_csv, libpimc), Cint,
                (Cstring, Cint, Cint, Cdouble, Ptr{Cdouble}, Culonglong),
                path, s.dim, d.nbins, s.L, counts, d.ndata))
    println("saved density")
    return path
end

"""Every chain's state in a checksummed file; `load_checkpoint` resumes it bit for bit."""
save_checkpoint(s::System, path::AbstractString) =
    check(ccall((:pimc_save_checkpoint, libpimc), Cint, (Ptr{Cvoid}, Cstring), s.handle, path))
load_checkpoint(s::System, path::AbstractString) =
    check(ccall((:pimc_load_checkpoint, libpimc), Cint, (Ptr{Cvoid}, Cstring), s.handle, path))

# ---------------------------------------------------------------- run!
"""
    run!(s, n, updates; Zmeasurements)

`n` attempts of the update list (src/simulation.jl:29-42) become sweeps of the
engine: one staging phase per sweep (N ceil(M/l) windows), swaps and
centre-of-mass moves in the 1/every proportions, measurements every
ceil(Ncycle / attempts-per-sweep) sweeps.
"""
function run!(s::System, n::Int64, updates; Zmeasurements = Any[])
    w = Dict{Symbol,Float64}(); obj = Dict{Symbol,Any}()
    for (every, u) in updates
        k = nameof(typeof(u)); w[k] = get(w, k, 0.0) + 1 / every; obj[k] = u
    end
    ws = sum(values(w))
    st = get(obj, :ReshapeLinear, nothing)
    ell = st === nothing ? 2 : st.var.m
    k = cld(s.M, ell)
    per = st === nothing ? s.N * ws / maximum(values(w)) : s.N * k * ws / w[:ReshapeLinear]
    sweeps = max(1, round(Int, n / per)); unit = per / ws
    frac(key) = get(w, key, 0.0) * unit
    sw = get(obj, :ReshapeSwapLinear, nothing); cm = get(obj, :SingleCenterOfMass, nothing)
    pc = get(obj, :PolymerCenterOfMass, nothing)
    mix = PimcMoveMix(st === nothing ? 0 : 1, ell, st === nothing ? 2 : st.var.minslices,
                      st === nothing ? 2 : min(st.var.maxslices, 64),
                      st === nothing ? 0.6 : st.var.minacc, st === nothing ? 0.8 : st.var.maxacc,
                      sw === nothing ? 0 : round(Int, frac(:ReshapeSwapLinear)),
                      sw === nothing ? 2 : sw.var.m, 2, sw === nothing ? 2 : min(sw.var.maxslices, 64),
                      sw === nothing ? 0.6 : sw.var.minacc, sw === nothing ? 0.8 : sw.var.maxacc,
                      cm === nothing ? 0 : max(1, round(Int, frac(:SingleCenterOfMass) / s.N)),
                      cm === nothing ? 1.0 : cm.var.size, 0.1, s.L / 2, 0.4, 0.6,
                      pc === nothing ? 0 : max(1, round(Int, frac(:PolymerCenterOfMass) / s.N)),
                      pc === nothing ? 1.0 : pc.var.size, 0.1, s.L / 2, 0.4, 0.6, 1,
                      isempty(Zmeasurements) ? 0 : max(1, round(Int, s.Ncycle / per)))
    dens = [z for z in Zmeasurements if z isa Density]
    series = [z for z in Zmeasurements if z isa Energy || z isa Superfluid]
    rdfs = [z for z in Zmeasurements if z isa RadialDistribution]
    if !isempty(Zmeasurements)
        nmeas = cld(sweeps, mix.measure_every) + 1
        ensure_engine!(s, isempty(dens) ? 0 : dens[1].nbins, isempty(series) ? 0 : nmeas)
        check(ccall((:pimc_reset_measurements, libpimc), Cint, (Ptr{Cvoid},), s.handle))
        s.eser_seen = 0
        check(ccall((:pimc_set_radial, libpimc), Cint, (Ptr{Cvoid}, Cint, Cint, Cdouble), s.handle, -1,
                    isempty(rdfs) ? 0 : rdfs[1].nbins, isempty(rdfs) ? 0.0 : rdfs[1].rmax))
    end
    check(ccall((:pimc_set_move_mix, libpimc), Cint, (Ptr{Cvoid}, Cint, Ref{PimcMoveMix}), s.handle, -1, mix))
    check(ccall((:pimc_run, libpimc), Cint, (Ptr{Cvoid}, Clonglong), s.handle, sweeps))
    isempty(Zmeasurements) && return nothing
    cnt = Ref{Cint}(0)
    check(ccall((:pimc_get_observables, libpimc), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint, Ref{Cint}),
                s.handle, 0, C_NULL, 0, cnt))
    rows = Vector{Float64}(undef, 8 * max(cnt[], 1))
    check(ccall((:pimc_get_observables, libpimc), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint, Ref{Cint}),
                s.handle, 0, rows, cnt[], cnt))
    R = reshape(rows, 8, :)[:, s.eser_seen+1:cnt[]]
    phys = s.params.semantics == 1
    for z in series
        if z isa Energy
            append!(get!(z.energy, s.N, Float64[]), R[1, :] .+ (phys ? R[3, :] : 0.0))
            append!(get!(z.energy_virial, s.N, Float64[]), R[2, :] .+ (phys ? R[4, :] : 0.0))
        else
            append!(get!(z.W2, s.N, Float64[]), R[5, :])
            append!(get!(z.area, s.N, Float64[]), R[6, :])
            append!(get!(z.I, s.N, Float64[]), R[7, :])
        end
    end
    s.N_MC[s.N] = get(s.N_MC, s.N, 0) + cnt[] - s.eser_seen
    s.eser_seen = cnt[]
    for d in dens
        nd = Ref{Culonglong}(0)
        h = Vector{Float64}(undef, d.nbins^s.dim)
        check(ccall((:pimc_get_density, libpimc), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ref{Culonglong}),
                    s.handle, 0, h, nd))
        d.dens .+= reshape(h, size(d.dens))
        d.ndata += nd[]
    end
    for r in rdfs
        nm = Ref{Culonglong}(0)
        h = Vector{Float64}(undef, r.nbins)
        check(ccall((:pimc_get_radial, libpimc), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ref{Culonglong}),
                    s.handle, 0, h, nm))
        r.hist .+= h
        r.ndata += nm[]
    end
    return nothing
end

function apply!(s::System, f::Update)
    acc = f(s)
    push!(f.counter.queue, acc); f.counter.tries += 1
    if f.counter_var.tries % f.counter_var.adj == 0 && !isempty(f.counter_var.queue)
        a = acceptance(f.counter_var.queue)
        if f.var isa Step
            f.var.size = clamp(a < f.var.minacc ? f.var.size * 0.9 : a > f.var.maxacc ? f.var.size * 1.1 : f.var.size,
                               f.var.minstep, f.var.maxstep)
        else
            f.var.m = clamp(a < f.var.minacc ? f.var.m - 1 : a > f.var.maxacc ? f.var.m + 1 : f.var.m,
                            f.var.minslices, f.var.maxslices)
        end
    end
    return nothing
end

# ---------------------------------------------------------------- adjoint
"""
    action_gradients(s) -> (S_pot, dS/dr [dim, N, M] as x[d][n][j], dS/d(V0, ω, g))

The potential part of the action and its adjoint from the device kernel.
"""
function action_gradients(s::System)
    g = Vector{Float64}(undef, s.dim * s.N * s.M)
    th = zeros(3); ex = zeros(4)
    check(ccall((:pimc_adjoint, libpimc), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                s.handle, 0, g, th, ex))
    return ex[1] + ex[2], g, th
end

struct PotentialParams; V0::Float64; ω::Float64; g::Float64; end

"""
    potential_action(s, θ::PotentialParams) -> S_pot

The potential action of the current paths at parameters θ; differentiable in
θ through a ChainRulesCore rrule backed by the adjoint kernel.
"""
function potential_action(s::System, θ::PotentialParams)
    check(ccall((:pimc_set_potential, libpimc), Cint, (Ptr{Cvoid}, Cint, Cdouble, Cdouble, Cdouble),
                s.handle, 0, θ.V0, θ.ω, θ.g))
    S, _, _ = action_gradients(s)
    return S
end

function ChainRulesCore.rrule(::typeof(potential_action), s::System, θ::PotentialParams)
    check(ccall((:pimc_set_potential, libpimc), Cint, (Ptr{Cvoid}, Cint, Cdouble, Cdouble, Cdouble),
                s.handle, 0, θ.V0, θ.ω, θ.g))
    S, _, dθ = action_gradients(s)
    pullback(ΔS) = (NoTangent(), NoTangent(),
                    Tangent{PotentialParams}(V0 = ΔS * dθ[1], ω = ΔS * dθ[2], g = ΔS * dθ[3]))
    return S, pullback
end

end # module
