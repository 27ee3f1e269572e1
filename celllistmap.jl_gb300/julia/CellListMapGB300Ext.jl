# CellListMap.jl package extension binding libcelllist_cuda.so (the C ABI of include/celllistmap_gb300.h).
#
# A maintainer of CellListMap.jl adds this file as `ext/CellListMapGB300Ext.jl`; its methods route the
# built-in pair operators to the GPU library and leave every other closure on the package's CPU path.
# Julia is not part of this repository's build and test environment: the file is written against the C
# ABI and checked only for covering every entry point of the header (tests/test_abi.py); the same ABI is
# driven by the Python mirror (celllistmap.jl_gb300/api.py) and the test-suite.

module CellListMapGB300Ext

using CellListMap, StaticArrays
import CellListMap: pairwise!, neighborlist

const lib = "libcelllist_cuda"   # resolved from the artifact / LD_LIBRARY_PATH

const CLM_OK = Int32(0)
const ARGERR = (1, 2, 3, 10, 11)

function check(h, st)
    st == CLM_OK && return nothing
    buf = Vector{UInt8}(undef, 512)
    ccall((:clm_last_error, lib), Int32, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, buf, 512)
    msg = unsafe_string(pointer(buf))
    st in ARGERR && throw(ArgumentError(msg))
    st == 4 && throw(DimensionMismatch(msg))
    error(msg)
end

mutable struct GPUSystem{T,N}
    h::Ptr{Cvoid}
    nsets::Int
end

function GPUSystem(::Type{T}, ::Val{N}, nsets) where {T,N}
    h = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:clm_create, lib), Int32, (Int32, Int32, Int32, Ptr{Ptr{Cvoid}}),
               T === Float64 ? 1 : 0, N, nsets, h)
    st == CLM_OK || error("clm_create failed ($st)")
    s = GPUSystem{T,N}(h[], nsets)
    finalizer(x -> ccall((:clm_destroy, lib), Int32, (Ptr{Cvoid},), x.h), s)
    return s
end

# Box: kind 0 = OrthorhombicCell, 1 = TriclinicCell, 2 = NonPeriodicCell; M column-major N x N
set_box!(s::GPUSystem{T,N}, M::AbstractMatrix, kind, cutoff, lcell) where {T,N} =
    check(s.h, ccall((:clm_set_box, lib), Int32, (Ptr{Cvoid}, Ptr{Float64}, Int32, Float64, Int32),
                     s.h, Matrix{Float64}(M), kind, cutoff, lcell))

# positions: a Vector{SVector{N,T}} is N x n column-major memory, exactly what the ABI takes
set_positions!(s::GPUSystem{T,N}, set, x::Vector{SVector{N,T}}) where {T,N} =
    GC.@preserve x check(s.h, ccall((:clm_set_positions, lib), Int32,
                                    (Ptr{Cvoid}, Int32, Ptr{Cvoid}, Int64, Int32),
                                    s.h, set, pointer(x), length(x), 0))

struct OpParams          # clm_op_params
    p::NTuple{8,Float64}
    ntypes::Int32; nbins::Int32
    types_x::Ptr{Int32}; types_y::Ptr{Int32}
    eps_table::Ptr{Float64}; sig_table::Ptr{Float64}
    vel_x::Ptr{Cvoid}; vel_y::Ptr{Cvoid}; bins::Ptr{Float64}
    params_on_device::Int32; reserved::Int32
    weights_x::Ptr{Float64}; weights_y::Ptr{Float64}
end

mutable struct Outputs   # clm_outputs
    scalar::Float64; count::Int64; min_i::Int64; min_j::Int64; min_d::Float64
    forces_x::Ptr{Cvoid}; forces_y::Ptr{Cvoid}
    hist_count::Ptr{Int64}; hist_sum::Ptr{Float64}
    out_on_device::Int32; index_base::Int32
    adjoint::Ptr{Float64}
end

run!(s, op::Integer, p::OpParams, o::Outputs) =
    check(s.h, ccall((:clm_run, lib), Int32, (Ptr{Cvoid}, Int32, Ref{OpParams}, Ref{Outputs}), s.h, op, p, o))

# neighborlist(...) on the GPU: pairs with 1-based indices, as the reference returns them
function gpu_neighborlist(s::GPUSystem{T}) where {T}
    run!(s, 1, OpParams(ntuple(_ -> 0.0, 8), 0, 0, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, 0, 0, C_NULL, C_NULL),
         Outputs(0, 0, 0, 0, 0, C_NULL, C_NULL, C_NULL, C_NULL, 0, 1, C_NULL))
    n = Ref{Int64}(0)
    check(s.h, ccall((:clm_nl_count, lib), Int32, (Ptr{Cvoid}, Ptr{Int64}), s.h, n))
    i = Vector{Int64}(undef, n[]); j = similar(i); d = Vector{T}(undef, n[])
    check(s.h, ccall((:clm_nl_fetch, lib), Int32,
                     (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Ptr{Cvoid}, Int64, Int32, Int32),
                     s.h, i, j, d, n[], 1, 0))
    return [(i[k], j[k], d[k]) for k in eachindex(i)]
end


struct BatchOutputs      # clm_batch_outputs
    scalar::Ptr{Float64}; count::Ptr{Int64}; forces::Ptr{Cvoid}
    out_on_device::Int32; reserved::Int32
end

# systems: Vector of (positions::Vector{SVector{3,Float64}}, sides::SVector{3,Float64})
function gpu_batch_energies(systems, cutoff; graph=true)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    ccall((:clm_batched_create, lib), Int32, (Int32, Int32, Ptr{Ptr{Cvoid}}), 1, 3, h) == 0 || error("create")
    offsets = Int64[0; cumsum(length(first(s)) for s in systems)]
    sides = reduce(vcat, [collect(last(s)) for s in systems])
    check(h[], ccall((:clm_batched_set_systems, lib), Int32,
                     (Ptr{Cvoid}, Int64, Ptr{Int64}, Ptr{Float64}, Int32, Float64, Int32),
                     h[], length(systems), offsets, sides, 0, cutoff, 1))
    x = reduce(vcat, first.(systems))                    # concatenated Vector{SVector{3,Float64}}
    GC.@preserve x check(h[], ccall((:clm_set_positions, lib), Int32,
                                    (Ptr{Cvoid}, Int32, Ptr{Cvoid}, Int64, Int32), h[], 0, pointer(x), length(x), 0))
    check(h[], ccall((:clm_batched_set_graph, lib), Int32, (Ptr{Cvoid}, Int32), h[], graph))
    u = Vector{Float64}(undef, length(systems)); n = Vector{Int64}(undef, length(systems))
    out = Ref(BatchOutputs(pointer(u), pointer(n), C_NULL, 0, 0))
    ops = Int32[6]                                       # CLM_OP_SOFT_ENERGY
    params = Ref(OpParams(ntuple(_ -> 0.0, 8), 0, 0, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, 0, 0, C_NULL, C_NULL))
    GC.@preserve u n check(h[], ccall((:clm_batched_run, lib), Int32,
                                      (Ptr{Cvoid}, Int32, Ptr{Int32}, Ref{OpParams}, Ref{BatchOutputs}),
                                      h[], 1, ops, params, out))
    st = Vector{Int32}(undef, length(systems))
    ccall((:clm_batched_status, lib), Int32, (Ptr{Cvoid}, Ptr{Int32}, Int64), h[], st, length(st))
    ccall((:clm_destroy, lib), Int32, (Ptr{Cvoid},), h[])
    return u, st
end

# ---- the adjoint as a ChainRulesCore rrule of the energy
using ChainRulesCore

function ChainRulesCore.rrule(::typeof(lj_energy), x::Vector{SVector{3,Float32}}, M::Matrix{Float64},
                              ε::Matrix{Float64}, σ::Matrix{Float64}, types::Vector{Int32}; cutoff)
    s = GPUSystem(Float32, Val(3), 1)
    set_box!(s, M, isdiag(M) ? 0 : 1, cutoff, 1); set_positions!(s, 0, x)
    f = similar(x); adj = zeros(32)
    εr = permutedims(ε); σr = permutedims(σ)             # row-major tables, rooted across the call
    p = OpParams((1.0, 1.0, 4.0, 4.0, 0.0, 0.0, 0.0, 0.0), Int32(size(ε, 1)), 0, pointer(types), C_NULL,
                 pointer(εr), pointer(σr), C_NULL, C_NULL, C_NULL, 0, 0, C_NULL, C_NULL)
    o = Outputs(0, 0, 0, 0, 0, pointer(f), C_NULL, C_NULL, C_NULL, 0, 0, pointer(adj))
    GC.@preserve x f adj types εr σr check(s.h, ccall((:clm_lj_adjoint, lib), Int32,
                                                     (Ptr{Cvoid}, Ref{OpParams}, Ref{Outputs}), s.h, p, o))
    U = o.scalar
    W = permutedims(reshape(adj[1:9], 3, 3))             # row-major virial
    nt = size(ε, 1); ncls = nt * (nt + 1) ÷ 2
    function pullback(ΔU)
        dx = -ΔU .* f                                    # dU/dx = -F
        dM = ΔU .* (W * inv(M)')                         # scaled coordinates fixed
        dε = symmetric_from_upper(ΔU .* adj[10:9+ncls], nt)
        dσ = symmetric_from_upper(ΔU .* adj[10+ncls:9+2ncls], nt)
        return NoTangent(), dx, dM, dε, dσ, NoTangent()
    end
    return U, pullback
end

function gpu_gravity!(forces::Vector{SVector{3,Float64}}, s::GPUSystem{Float64}, mass::Vector{Float64})
    p = OpParams((9.8, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0), 0, 0, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL,
                 C_NULL, C_NULL, 0, 0, pointer(mass), C_NULL)
    o = Outputs(0, 0, 0, 0, 0, pointer(forces), C_NULL, C_NULL, C_NULL, 0, 0, C_NULL)
    GC.@preserve forces mass run!(s, 14, p, o)   # o.scalar = sum of -9.8 m_i m_j / d
    return forces
end

build!(s) = check(s.h, ccall((:clm_build, lib), Int32, (Ptr{Cvoid},), s.h))          # UpdateCellList!
set_precision!(s, split::Bool) =
    check(s.h, ccall((:clm_set_precision, lib), Int32, (Ptr{Cvoid}, Int32), s.h, split))
set_stream!(s, stream::Ptr{Cvoid}) =                                                 # e.g. CUDA.jl's stream().handle
    check(s.h, ccall((:clm_set_stream, lib), Int32, (Ptr{Cvoid}, Ptr{Cvoid}), s.h, stream))

function box_fields(s::GPUSystem{T,N}) where {T,N}                                   # the fields of Box
    nc = zeros(Int64, N); h = zeros(N); lo = zeros(N); hi = zeros(N)
    Mal = zeros(N, N); R = zeros(N, N); Rinv = zeros(N, N); cut = Ref(0.0)
    check(s.h, ccall((:clm_get_box, lib), Int32,
                     (Ptr{Cvoid}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                      Ptr{Float64}, Ptr{Float64}, Ptr{Float64}), s.h, nc, h, lo, hi, Mal, R, Rinv, cut))
    return (nc=nc, cell_size=h, computing_box=(lo, hi), unit_cell=Mal, rotation=R, inv_rotation=Rinv,
            cutoff=cut[])
end

function celllist(s::GPUSystem{T,N}, set=0) where {T,N}                               # the fields of CellList
    nr = Ref{Int64}(0); np = Ref{Int64}(0); ncp = Ref{Int64}(0); ncr = Ref{Int64}(0)
    check(s.h, ccall((:clm_get_celllist_info, lib), Int32,
                     (Ptr{Cvoid}, Int32, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}), s.h, set, nr, np, ncp, ncr))
    cell = Vector{Int64}(undef, np[]); index = similar(cell); real = Vector{Int8}(undef, np[])
    x = Vector{SVector{N,T}}(undef, np[])
    GC.@preserve x check(s.h, ccall((:clm_fetch_celllist, lib), Int32,
                                    (Ptr{Cvoid}, Int32, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{Int8}, Ptr{Cvoid}, Int32),
                                    s.h, set, np[], cell, index, real, pointer(x), 1))
    return (n_real=nr[], n_cells_with_particles=ncp[], n_cells_with_real=ncr[],
            cell=cell .+ 1, index=index, real=Bool.(real), x=x)
end

# scalar reductions with no device allocation (after build!), for callers under their own device pool
run_noalloc!(s, op::Integer, p::OpParams, o::Outputs) =
    check(s.h, ccall((:clm_run_noalloc, lib), Int32, (Ptr{Cvoid}, Int32, Ref{OpParams}, Ref{Outputs}), s.h, op, p, o))

function last_timings(s)                                                             # device ms of build and map
    b = Ref{Float32}(0); m = Ref{Float32}(0)
    check(s.h, ccall((:clm_last_timings, lib), Int32, (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}), s.h, b, m))
    return (build_ms=b[], map_ms=m[])
end
function kernel_launches(s)
    n = Ref{Int64}(0)
    check(s.h, ccall((:clm_stats, lib), Int32, (Ptr{Cvoid}, Ptr{Int64}), s.h, n))
    return n[]
end
function device_allocations()                                                       # for allocation tests
    c = Ref{Int64}(0); b = Ref{Int64}(0)
    ccall((:clm_device_allocations, lib), Int32, (Ptr{Int64}, Ptr{Int64}), c, b)
    return (count=c[], bytes=b[])
end
version() = unsafe_string(ccall((:clm_version, lib), Cstring, ()))

# batches: cell tiles and block shape, the autotuner, the last step's device time
batched_config!(h, lcell, parts, grid_div) =
    check(h, ccall((:clm_batched_set_config, lib), Int32, (Ptr{Cvoid}, Int32, Int32, Int32), h, lcell, parts, grid_div))
function batched_autotune!(h, ops::Vector{Int32}, params::Vector{OpParams}; reps=5)
    cfg = zeros(Int32, 3); best = Ref{Float32}(0)
    check(h, ccall((:clm_batched_autotune, lib), Int32,
                   (Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{OpParams}, Int32, Ptr{Int32}, Ptr{Float32}),
                   h, length(ops), ops, params, reps, cfg, best))
    return (lcell=cfg[1], parts=cfg[2], grid_div=cfg[3], step_ms=best[])
end
function batched_last_step(h)
    t = Ref{Float32}(0); n = Ref{Int64}(0)
    check(h, ccall((:clm_batched_last_step, lib), Int32, (Ptr{Cvoid}, Ptr{Float32}, Ptr{Int64}), h, t, n))
    return (step_ms=t[], launches=n[])
end

# ---- the user-facing dispatch: pairwise! methods for built-in operator objects
module GPU
abstract type Op end
struct NeighborList <: Op end
struct Count <: Op end
struct SoftEnergy <: Op; c::Float64; end                       # c = 0: the cutoff
SoftEnergy() = SoftEnergy(0.0)
struct SoftForces <: Op; c::Float64; end
struct LennardJones <: Op; eps::Float64; sigma::Float64; c12::Float64; c6::Float64; forces::Bool; end
LennardJones(eps, sigma; c12=4.0, c6=4.0, forces=true) = LennardJones(eps, sigma, c12, c6, forces)
struct MinimumDistance <: Op end
struct RadialHistogram{V} <: Op; bins::Vector{Float64}; vx::V; vy::Union{Nothing,V}; end
struct WeightedInverseDistance <: Op; wx::Vector{Float64}; wy::Union{Nothing,Vector{Float64}}; c::Float64; end
end

const HANDLES = WeakKeyDict{Any,GPUSystem}()
op_id(::GPU.NeighborList) = 1;  op_id(::GPU.Count) = 2;  op_id(::GPU.SoftEnergy) = 6;  op_id(::GPU.SoftForces) = 7
op_id(o::GPU.LennardJones) = o.forces ? 9 : 8;  op_id(::GPU.MinimumDistance) = 10;  op_id(::GPU.RadialHistogram) = 11
op_id(::GPU.WeightedInverseDistance) = 14

function handle!(sys::CellListMap.AbstractParticleSystem)
    T = eltype(eltype(sys.xpositions.x)); N = CellListMap.dim(sys)
    two = sys isa CellListMap.ParticleSystem2
    s = get!(() -> GPUSystem(T, Val(N), two ? 2 : 1), HANDLES, sys)
    kind = Dict(CellListMap.OrthorhombicCell => 0, CellListMap.TriclinicCell => 1,
                CellListMap.NonPeriodicCell => 2)[CellListMap.unitcelltype(sys)]
    set_box!(s, CellListMap.unitcell(sys), kind, CellListMap.cutoff(sys), CellListMap.box(sys).lcell)
    if sys.xpositions.updated[]
        set_positions!(s, 0, sys.xpositions.x); sys.xpositions.updated[] = false
    end
    if two && sys.ypositions.updated[]
        set_positions!(s, 1, sys.ypositions.x); sys.ypositions.updated[] = false
    end
    return s
end

noparams() = OpParams(ntuple(_ -> 0.0, 8), 0, 0, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, 0, 0,
                      C_NULL, C_NULL)
nooutputs(; forces_x=C_NULL, forces_y=C_NULL, hc=C_NULL, hs=C_NULL, base=1) =
    Outputs(0, 0, 0, 0, 0, forces_x, forces_y, hc, hs, 0, base, C_NULL)

# scalar sums: the output is the sum (output::Number), as pairwise!(f, sys) returns it
function CellListMap.pairwise!(op::Union{GPU.Count,GPU.SoftEnergy}, sys; kw...)
    s = handle!(sys); o = nooutputs()
    p = op isa GPU.SoftEnergy ? setparams(noparams(), (op.c,)) : noparams()
    run!(s, op_id(op), p, o)
    return op isa GPU.Count ? o.count : o.scalar
end

# forces: sys.output is the Vector{SVector{N,T}} of forces (f[i] -= df; f[j] += df), the energy is returned
function CellListMap.pairwise!(op::Union{GPU.SoftForces,GPU.LennardJones,GPU.WeightedInverseDistance}, sys; kw...)
    s = handle!(sys); f = sys.output
    fy = sys isa CellListMap.ParticleSystem2 ? similar(f, length(sys.ypositions.x)) : nothing
    p = op isa GPU.SoftForces ? setparams(noparams(), (op.c,)) :
        op isa GPU.LennardJones ? setparams(noparams(), (op.eps, op.sigma, op.c12, op.c6)) :
        weighted_params(op)
    o = nooutputs(forces_x=pointer(f), forces_y=isnothing(fy) ? C_NULL : pointer(fy))
    GC.@preserve f fy op run!(s, op_id(op), p, o)
    return o.scalar
end

# minimum distance: the reference's MinimumDistance(i, j, d) output (test/examples/nearest_neighbor.jl)
function CellListMap.pairwise!(::GPU.MinimumDistance, sys; kw...)
    s = handle!(sys); o = nooutputs(base=1)
    run!(s, 10, noparams(), o)
    return (o.min_i, o.min_j, o.min_d)
end

# radial histogram with the per-bin velocity sums (test/examples/pairwise_velocities.jl)
function CellListMap.pairwise!(op::GPU.RadialHistogram, sys; kw...)
    s = handle!(sys); nb = length(op.bins) - 1
    hc = zeros(Int64, nb); hs = zeros(Float64, nb)
    p = hist_params(op)
    o = nooutputs(hc=pointer(hc), hs=pointer(hs))
    GC.@preserve hc hs op run!(s, 11, p, o)
    return hc, hs
end

# neighborlist(Val(:cuda); xpositions, cutoff, unitcell): the reference's (i, j, d) tuples, 1-based.  A new
# positional method, so the reference's own neighborlist(; ...) keeps its CPU path.
function CellListMap.neighborlist(::Val{:cuda}; xpositions, ypositions=nothing, cutoff, unitcell=nothing, kw...)
    sys = isnothing(ypositions) ? ParticleSystem(; xpositions, cutoff, unitcell, output=0.0) :
                                  ParticleSystem(; xpositions, ypositions, cutoff, unitcell, output=0.0)
    gpu_neighborlist(handle!(sys))
end

end # module CellListMapGB300Ext
