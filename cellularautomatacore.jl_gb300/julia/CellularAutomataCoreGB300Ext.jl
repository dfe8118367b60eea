# CellularAutomataCoreGB300Ext — the GB300 backend of CellularAutomataCore.jl, as the package
# extension a maintainer adds beside ext/CellularAutomataCoreKernelAbstractionsExt.jl: a new
# `GB300Backend <: AbstractBackend` that implements the backend contract (src/backends.jl:4-14)
# by `ccall`ing libgbca.so, whose C ABI is include/gbca.h. No KernelAbstractions, no Julia kernel
# and no CPU fallback sit on this path: every sweep is a hand-written sm_103a kernel of the library.
#
#   solve(CAProblem(Life(:highlife), u0, 200), Synchronous(); backend=GB300Backend(), saveat=20)
#   solve(EnsembleProblem(prob), Synchronous(), EnsembleGB300(); trajectories=4096)
#   abc_rejection(prob, proposals, distance, observed; ensemblealg=EnsembleGB300())
#
# Closures cannot cross a ccall, so the backend runs typed rules: Life and Generations (their
# masks), Lenia (its numbers), and the two LocalRules the reference writes as closures, the
# README's forest fire and the conformance battery's kernel-field SI epidemic, restated below as
# rule types whose `local_rule` is the closure's own body, so ReferenceBackend and ArrayBackend
# remain their oracle. `check_problem` rejects anything else.
#
# Set the library with ENV["GBCA_LIB"] (default "libgbca.so" on the loader path).
module CellularAutomataCoreGB300Ext

using CellularAutomataCore
using CellularAutomataCore: AbstractBackend, AbstractRule, AbstractScheme, Synchronous, Stochastic, Checkerboard,
                            Lattice, Periodic, Reflecting, Constant, Moore, VonNeumann, Life, Generations, Lenia,
                            IncompatibleSpaceError, UnsupportedCombinationError, InvalidStateError, bernoulli,
                            field, covariate
using SciMLBase

const CAC = CellularAutomataCore

export GB300Backend, EnsembleGB300, ForestFire, KernelSI, GB300Server

const libgbca = get(ENV, "GBCA_LIB", "libgbca.so")

# ------------------------------------------------------------------ the C ABI's constants

const GBCA_OK = Int32(0)
const GBCA_ERR_ARGUMENT = Int32(1)
const GBCA_ERR_INCOMPATIBLE_SPACE = Int32(2)
const GBCA_ERR_UNSUPPORTED = Int32(3)
const GBCA_ERR_STATE = Int32(4)
const GBCA_ERR_CUDA = Int32(5)
const GBCA_ERR_OUT_OF_MEMORY = Int32(6)
const GBCA_ERR_TIMEOUT = Int32(7)
const GBCA_ERR_BUSY = Int32(8)

const GBCA_RULE_LIFE = Int32(1)
const GBCA_RULE_GENERATIONS = Int32(2)
const GBCA_RULE_FOREST_FIRE = Int32(3)
const GBCA_RULE_LENIA = Int32(4)
const GBCA_RULE_SI_FIELD = Int32(5)
const GBCA_SOURCE_INDICATOR = Int32(0)
const GBCA_SOURCE_IDENTITY = Int32(1)
const GBCA_MOORE = Int32(1)
const GBCA_VON_NEUMANN = Int32(2)
const GBCA_PERIODIC = Int32(0)
const GBCA_REFLECTING = Int32(1)
const GBCA_CONSTANT = Int32(2)
const GBCA_SYNCHRONOUS = Int32(0)
const GBCA_STOCHASTIC = Int32(1)
const GBCA_CHECKERBOARD = Int32(2)
const GBCA_DIRECT = Int32(0)
const GBCA_FFT = Int32(1)
const GBCA_MAX_PEAKS = 8

# gbca_desc, field by field and in order (isbits, so Julia lays it out as C does)
struct GbcaDesc
    rule::Int32
    nbhd::Int32
    radius::Int32
    states::Int32
    birth::UInt64
    survive::UInt64
    n1::Int64
    n2::Int64
    boundary::NTuple{2,Int32}
    constant::NTuple{2,Float64}
    seed::UInt64
    scheme::Int32
    scheme_p_f32::Int32
    scheme_p::Float64
    params_f32::Int32
    lenia_method::Int32
    lenia_R::Int32
    lenia_npeaks::Int32
    lenia_f64::Int32
    reserved::Int32
    lenia_peaks::NTuple{8,Float64}
    lenia_mu::Float64
    lenia_sigma::Float64
    lenia_dt::Float64
end

# gbca_server_config
struct GbcaServerConfig
    hbm_budget::UInt64
    chunk_steps::Int32
    big_cells::Int32
    max_big::Int32
    big_chunk_us::Int32
end

# gbca_result
struct GbcaResult
    id::UInt64
    status::Int32
    reserved::Int32
    counts::NTuple{8,Int64}
    other::Int64
    morans::Float64
    t_submit::Float64
    t_admit::Float64
    t_done::Float64
end

# ------------------------------------------------------------------ typed rules

"""
    ForestFire(; neighbourhood=VonNeumann(1), precision=Float64)

The forest fire of the package README (README.md:56-60) on Int8 codes 0 = empty, 1 = tree,
2 = fire, as a rule type: a fire burns out; an empty cell grows a tree with probability `p.p`
(draw 1); a tree catches fire from a burning neighbour, or by lightning with probability `p.f`
(draw 2). `precision = Float32` draws with Float32 `p` and `f`.
"""
struct ForestFire{T<:AbstractFloat,N} <: AbstractRule
    neighbourhood::N
end
function ForestFire(; neighbourhood=VonNeumann(1), precision::Type{<:AbstractFloat}=Float64)
    return ForestFire{precision,typeof(neighbourhood)}(neighbourhood)
end
CAC.neighbourhood(r::ForestFire) = r.neighbourhood
@inline function CAC.local_rule(::ForestFire{T}, cell, nbrs, ctx) where {T}
    cell == 2 && return oftype(cell, 0)
    cell == 0 && return bernoulli(ctx, T(ctx.p.p), 1) ? oftype(cell, 1) : oftype(cell, 0)
    any(==(2), nbrs) && return oftype(cell, 2)
    return bernoulli(ctx, T(ctx.p.f), 2) ? oftype(cell, 2) : oftype(cell, 1)
end

"""
    KernelSI(; field=:pressure, covariate=nothing, precision=Float64)

The kernel-field SI epidemic of test/backend_conformance.jl:52-57 (and :72-75 in Float32) as a
rule type: an infected cell (1) stays infected; any other becomes infected with probability
`1 - exp(-p.β * covariate * field)` (draw 1), the covariate factor left out when `covariate`
is `nothing`. `field` names a KernelField of the problem.
"""
struct KernelSI{T<:AbstractFloat} <: AbstractRule
    field::Symbol
    covariate::Union{Symbol,Nothing}
end
function KernelSI(; field::Symbol=:pressure, covariate::Union{Symbol,Nothing}=nothing,
                  precision::Type{<:AbstractFloat}=Float64)
    return KernelSI{precision}(field, covariate)
end
CAC.neighbourhood(::KernelSI) = nothing
@inline function CAC.local_rule(r::KernelSI{T}, cell, nbrs, ctx) where {T}
    cell == 1 && return cell
    λ = r.covariate === nothing ? T(ctx.p.β) * field(ctx, r.field) :
        T(ctx.p.β) * covariate(ctx, r.covariate) * field(ctx, r.field)
    return bernoulli(ctx, 1 - exp(-λ), 1) ? one(cell) : cell
end

# ------------------------------------------------------------------ errors

# status codes to the reference's exception types (src/errors.jl); no exception crosses the ABI
function check(rc::Integer; what::AbstractString="GB300Backend", space::AbstractString="its space")
    rc == GBCA_OK && return nothing
    msg = unsafe_string(ccall((:gbca_last_error, libgbca), Cstring, ()))
    rc == GBCA_ERR_ARGUMENT && throw(ArgumentError(msg))
    rc == GBCA_ERR_INCOMPATIBLE_SPACE && throw(IncompatibleSpaceError(what, space, msg))
    rc == GBCA_ERR_UNSUPPORTED && throw(UnsupportedCombinationError(what, msg))
    rc == GBCA_ERR_STATE && throw(InvalidStateError(what, nothing, nothing, msg))
    rc == GBCA_ERR_OUT_OF_MEMORY && throw(OutOfMemoryError())
    return throw(ErrorException("libgbca: " * msg))
end

# ------------------------------------------------------------------ problem -> gbca_desc

_boundary_kind(::Periodic) = GBCA_PERIODIC
_boundary_kind(::Reflecting) = GBCA_REFLECTING
_boundary_kind(::Constant) = GBCA_CONSTANT
_boundary_value(b::Constant) = Float64(b.value)
_boundary_value(_) = 0.0

function _neighbourhood(prob)
    nb = CAC.neighbourhood(prob.rule)
    nb === nothing && (nb = CAC.default_neighbourhood(prob.space))
    nb isa Moore && return GBCA_MOORE, Int32(nb.radius)
    nb isa VonNeumann && return GBCA_VON_NEUMANN, Int32(nb.radius)
    return throw(ArgumentError("GB300Backend runs Moore(r) and VonNeumann(r) neighbourhoods, got $nb"))
end

_scheme_fields(::Synchronous) = (GBCA_SYNCHRONOUS, Int32(0), 1.0)
_scheme_fields(s::Stochastic) = (GBCA_STOCHASTIC, Int32(s.p isa Float32), Float64(s.p))
_scheme_fields(::Checkerboard) = (GBCA_CHECKERBOARD, Int32(0), 1.0)
function _scheme_fields(s)
    return throw(UnsupportedCombinationError("GB300Backend", string(typeof(s))))
end

_f32(::Type{Float32}) = Int32(1)
_f32(::Type) = Int32(0)

"""
    gbca_desc(prob, scheme) -> GbcaDesc

The C description of a problem (what check_problem and allocate_state receive): the rule's
kind and masks (Life, Generations: rules.jl:267-275, 354-358, 424-429), the neighbourhood's
kind and radius, the lattice's dims, boundary kinds and Constant values (spaces.jl:16-51,
94-110), the seed, the scheme (schemes.jl:22-51) and Lenia's numbers (lenia.jl:17-31,
kernels.jl:87-98). Raises the reference's errors for what the backend cannot run.
"""
function gbca_desc(prob, scheme)
    space = prob.space
    (space isa Lattice && length(space.dims) == 2 && space.geometry isa CAC.Square) ||
        throw(IncompatibleSpaceError("GB300Backend", CAC._describe(space), "needs a two-dimensional square lattice"))
    n1, n2 = Int64(space.dims[1]), Int64(space.dims[2])
    bnd = (_boundary_kind(space.boundaries[1]), _boundary_kind(space.boundaries[2]))
    cst = (_boundary_value(space.boundaries[1]), _boundary_value(space.boundaries[2]))
    sch, sp32, sp = _scheme_fields(scheme)
    rule = prob.rule
    kind, nbhd, radius, states = Int32(0), GBCA_MOORE, Int32(1), Int32(2)
    birth, survive = UInt64(0), UInt64(0)
    params_f32 = Int32(0)
    method, R, npeaks, f64 = GBCA_DIRECT, Int32(0), Int32(0), Int32(0)
    peaks = ntuple(_ -> 0.0, GBCA_MAX_PEAKS)
    mu, sigma, dt = 0.0, 0.0, 0.0
    if rule isa Lenia
        kind = GBCA_RULE_LENIA
        method = rule.fft ? GBCA_FFT : GBCA_DIRECT
        R = Int32(rule.kernel.radius)
        pk = rule.kernel.peaks
        length(pk) <= GBCA_MAX_PEAKS ||
            throw(ArgumentError("GB300Backend runs Lenia with at most $GBCA_MAX_PEAKS peaks"))
        npeaks = Int32(length(pk))
        peaks = ntuple(k -> k <= length(pk) ? Float64(pk[k]) : 0.0, GBCA_MAX_PEAKS)
        f64 = Int32(rule.μ isa Float64)
        mu, sigma, dt = Float64(rule.μ), Float64(rule.σ), Float64(rule.dt)
        eltype(prob.u0) == typeof(rule.μ) ||
            throw(ArgumentError("Lenia(precision=$(typeof(rule.μ))) needs a $(typeof(rule.μ)) state"))
    else
        eltype(prob.u0) == Int8 ||
            throw(ArgumentError("GB300Backend runs Life, Generations and the typed rules on Int8 states"))
        nbhd, radius = _neighbourhood(prob)
        if rule isa Life
            kind, birth, survive = GBCA_RULE_LIFE, rule.birth, rule.survive
        elseif rule isa Generations
            kind, birth, survive, states = GBCA_RULE_GENERATIONS, rule.birth, rule.survive, Int32(rule.states)
        elseif rule isa ForestFire
            kind = GBCA_RULE_FOREST_FIRE
            params_f32 = _f32(typeof(rule).parameters[1])
        elseif rule isa KernelSI
            kind = GBCA_RULE_SI_FIELD
            params_f32 = _f32(typeof(rule).parameters[1])
            haskey(prob.fields, rule.field) ||
                throw(ArgumentError("the rule reads field :$(rule.field), which the problem does not define"))
            rule.covariate === nothing || haskey(prob.covariates, rule.covariate) ||
                throw(ArgumentError("the rule reads covariate :$(rule.covariate), which the problem does not define"))
        else
            throw(ArgumentError("GB300Backend cannot run $(typeof(rule)): arbitrary LocalRules cannot cross the " *
                                "C ABI; use Life, Generations, ForestFire, KernelSI or Lenia"))
        end
    end
    return GbcaDesc(kind, nbhd, radius, states, birth, survive, n1, n2, bnd, cst, prob.seed % UInt64, sch, sp32,
                    sp, params_f32, method, R, npeaks, f64, Int32(0), peaks, mu, sigma, dt)
end

# the integrator's p as the ABI's parameter vector: forest fire (p, f), SI (β), else none
function params_of(prob, p)
    prob.rule isa ForestFire && return (Float64(p.p), Float64(p.f)), Int32(2)
    prob.rule isa KernelSI && return (Float64(p.β), 0.0), Int32(1)
    return (0.0, 0.0), Int32(0)
end

# ------------------------------------------------------------------ the backend

"""
    GB300Backend(; background=nothing, tilesize=64, tune=false)

The GB300 backend: every sweep runs in libgbca.so's sm_103a kernels. With `background`, only
tiles holding another state (or next to one) are swept, as SparseBackend(background; tilesize)
does (src/sparse.jl). With `tune = true`, allocate_state times the candidate sweep geometries on
the initial state and caches the fastest for the problem's shape.
"""
struct GB300Backend <: AbstractBackend
    background::Union{Nothing,Int}
    tilesize::Int
    tune::Bool
end
GB300Backend(; background=nothing, tilesize::Integer=64, tune::Bool=false) = GB300Backend(background, tilesize, tune)

mutable struct GB300State{T}
    handle::Ptr{Cvoid}
    dims::NTuple{2,Int}
    pending::Int64                 # queued steps; consecutive advance! calls run as one call
    t0::Int64
    params::NTuple{2,Float64}
    nparams::Int32
end

CAC.supports(::GB300Backend, ::Union{Synchronous,Stochastic,Checkerboard}) = true

function CAC.check_problem(::GB300Backend, prob, scheme)
    d = gbca_desc(prob, scheme)
    return check(ccall((:gbca_check, libgbca), Cint, (Ref{GbcaDesc},), d); space=CAC._describe(prob.space))
end

# the SI rule's kernel field source as the ABI's kind: an Int8 state has 256 values, so the
# source function is compared with x == 1 and identity on all of them
function _source_kind(src)
    src === identity && return GBCA_SOURCE_IDENTITY
    vals = typemin(Int8):typemax(Int8)
    all(v -> src(v) == (v == 1), vals) && return GBCA_SOURCE_INDICATOR
    all(v -> src(v) == v, vals) && return GBCA_SOURCE_IDENTITY
    return throw(ArgumentError("GB300Backend reads kernel fields of x == 1 or x itself"))
end

function _attach_environment(h::Ptr{Cvoid}, b::GB300Backend, prob)
    if prob.mask !== nothing
        m = UInt8.(collect(prob.mask))
        check(ccall((:gbca_set_mask, libgbca), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, m, sizeof(m)))
    end
    if prob.rule isa KernelSI
        rf = prob.fields[prob.rule.field]            # a _ResolvedField: offsets already negated
        taps = Int32[x for o in rf.offsets for x in Tuple(o)]
        w = Float64.(rf.weights)
        check(ccall((:gbca_set_field, libgbca), Cint,
                    (Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{Float64}, Int32, Int32, Int32),
                    h, length(w), taps, w, _f32(eltype(rf.weights)), _source_kind(rf.source),
                    rf.fft ? GBCA_FFT : GBCA_DIRECT))
        if prob.rule.covariate !== nothing
            c = prob.covariates[prob.rule.covariate]
            cf = eltype(c) == Float32 ? Array{Float32}(c) : Array{Float64}(c)
            check(ccall((:gbca_set_covariate, libgbca), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int32),
                        h, cf, ndims(cf) == 3 ? size(cf, 3) : 1, _f32(eltype(cf))))
        end
    end
    if b.background !== nothing
        check(ccall((:gbca_set_sparse, libgbca), Cint, (Ptr{Cvoid}, Int32, Int32, Int32),
                    h, 1, b.background, b.tilesize))
    end
    return nothing
end

function CAC.allocate_state(b::GB300Backend, prob, scheme)
    d = gbca_desc(prob, scheme)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gbca_create, libgbca), Cint, (Ref{GbcaDesc}, Ref{Ptr{Cvoid}}), d, h);
          space=CAC._describe(prob.space))
    ps, np = params_of(prob, prob.p)
    st = GB300State{eltype(prob.u0)}(h[], (Int(d.n1), Int(d.n2)), 0, 0, ps, np)
    finalizer(s -> ccall((:gbca_destroy, libgbca), Cint, (Ptr{Cvoid},), s.handle), st)
    _attach_environment(h[], b, prob)
    CAC.set_state!(b, st, prob.u0)
    if b.tune
        k, rows, staging = Ref{Int32}(0), Ref{Int32}(0), Ref{Int32}(0)
        pv = Ref(ps)
        check(ccall((:gbca_tune, libgbca), Cint,
                    (Ptr{Cvoid}, Ptr{Float64}, Int32, Ref{Int32}, Ref{Int32}, Ref{Int32}),
                    st.handle, pv, np, k, rows, staging))
    end
    return st
end

# run the queued steps as one temporally blocked gbca_advance
function flush!(st::GB300State)
    st.pending == 0 && return nothing
    pv = Ref(st.params)
    check(ccall((:gbca_advance, libgbca), Cint, (Ptr{Cvoid}, Int64, Int64, Ptr{Float64}, Int32),
                st.handle, st.t0, st.pending, pv, st.nparams))
    st.pending = 0
    return nothing
end

function CAC.advance!(::GB300Backend, st::GB300State, prob, scheme, p, t)
    ps, np = params_of(prob, p)
    if st.pending > 0 && st.t0 + st.pending == t && ps == st.params
        st.pending += 1
    else
        flush!(st)
        st.t0, st.pending, st.params, st.nparams = Int64(t), 1, ps, np
    end
    return nothing
end

function CAC.current_state(::GB300Backend, st::GB300State{T}) where {T}
    flush!(st)
    u = Array{T}(undef, st.dims)
    check(ccall((:gbca_get_state, libgbca), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t), st.handle, u, sizeof(u)))
    return u
end

function CAC.set_state!(::GB300Backend, st::GB300State{T}, u) where {T}
    flush!(st)
    size(u) == st.dims || throw(CAC.StateShapeError("the state", st.dims, size(u)))
    a = convert(Array{T}, u)
    check(ccall((:gbca_set_state, libgbca), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t), st.handle, a, sizeof(a)))
    return nothing
end

# Queued copies (gbca_set_state_async / gbca_get_state_async): `buf` should be page-locked
# (Base.Libc.malloc'd memory registered with CUDA.Mem.register, say) and must be left alone
# until sync!(st); they let one lattice's or one step's copies overlap another's sweeps.
function set_state_async!(st::GB300State{T}, buf::Array{T}) where {T}
    flush!(st)
    size(buf) == st.dims || throw(CAC.StateShapeError("the state", st.dims, size(buf)))
    check(ccall((:gbca_set_state_async, libgbca), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t), st.handle, buf,
                sizeof(buf)))
    return nothing
end

function get_state_async!(buf::Array{T}, st::GB300State{T}) where {T}
    flush!(st)
    size(buf) == st.dims || throw(CAC.StateShapeError("the buffer", st.dims, size(buf)))
    check(ccall((:gbca_get_state_async, libgbca), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t), st.handle, buf,
                sizeof(buf)))
    return buf
end

function sync!(st::GB300State)
    flush!(st)
    check(ccall((:gbca_sync, libgbca), Cint, (Ptr{Cvoid},), st.handle))
    return nothing
end

function CAC.read_cell(::GB300Backend, st::GB300State{T}, I) where {T}
    flush!(st)
    v = Ref{T}()
    check(ccall((:gbca_read_cell, libgbca), Cint, (Ptr{Cvoid}, Int64, Int64, Ptr{Cvoid}), st.handle, I[1], I[2], v))
    return v[]
end

function CAC.write_cell!(::GB300Backend, st::GB300State{T}, I, v) where {T}
    flush!(st)
    x = Ref{T}(convert(T, v))
    check(ccall((:gbca_write_cell, libgbca), Cint, (Ptr{Cvoid}, Int64, Int64, Ptr{Cvoid}), st.handle, I[1], I[2], x))
    return nothing
end

"""
    device_summaries(st; nvals=3) -> (counts, other, morans)

state_counts (src/measures.jl:14-20) and Moran's I with VonNeumann(1) (src/measures.jl:91-107)
of the current Int8 state, computed on the device.
"""
function device_summaries(st::GB300State{Int8}; nvals::Integer=3)
    flush!(st)
    counts = zeros(Int64, nvals)
    other, morans = Ref{Int64}(0), Ref{Float64}(0.0)
    check(ccall((:gbca_summaries, libgbca), Cint, (Ptr{Cvoid}, Ptr{Int64}, Int32, Ref{Int64}, Ref{Float64}),
                st.handle, counts, nvals, other, morans))
    return counts, other[], morans[]
end

# the geometry a sweep uses, and pinning one (results never depend on it)
function geometry(st::GB300State)
    k, rows, staging = Ref{Int32}(0), Ref{Int32}(0), Ref{Int32}(0)
    pv = Ref(st.params)
    check(ccall((:gbca_geometry, libgbca), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ref{Int32}, Ref{Int32}, Ref{Int32}),
                st.handle, pv, k, rows, staging))
    return (steps_per_pass=k[], tile_rows=rows[], staging=staging[])
end
function set_geometry!(st::GB300State; steps_per_pass::Integer=0, tile_rows::Integer=0, staging::Integer=0)
    return check(ccall((:gbca_set_geometry, libgbca), Cint, (Ptr{Cvoid}, Int32, Int32, Int32),
                       st.handle, steps_per_pass, tile_rows, staging))
end

# ------------------------------------------------------------------ saved states on the device

# queue a copy of the state after the queued steps; fetch it later (src/problem.jl:336-370)
function snapshot!(st::GB300State)
    flush!(st)
    ticket = Ref{Int64}(0)
    check(ccall((:gbca_snapshot, libgbca), Cint, (Ptr{Cvoid}, Ref{Int64}), st.handle, ticket))
    return ticket[]
end
function fetch_snapshot(st::GB300State{T}, ticket::Integer) where {T}
    u = Array{T}(undef, st.dims)
    check(ccall((:gbca_snapshot_fetch, libgbca), Cint, (Ptr{Cvoid}, Int64, Ptr{Cvoid}, Csize_t),
                st.handle, ticket, u, sizeof(u)))
    return u
end

# ------------------------------------------------------------------ slabs of one lattice

"""
    set_slab!(st, col0, n2_global)

Places the state's n1 x n2 lattice as columns col0 .. col0 + n2 - 1 (mod n2_global) of a lattice
of n2_global columns: cell ids, hence draws, and Checkerboard parities become the larger
lattice's (src/backends.jl:457-479 splits that lattice among threads; here among ranks). The
caller pads each rank's slab with h = r K gates columns on each side and refreshes them from its
neighbours every K steps (columns are contiguous in `device_state`'s buffer).
"""
set_slab!(st::GB300State, col0::Integer, n2_global::Integer) =
    check(ccall((:gbca_set_slab, libgbca), Cint, (Ptr{Cvoid}, Int64, Int64), st.handle, col0, n2_global))

"""
    slab_sums(st, j_lo, j_hi) -> Vector{Int64}

The exact integer sums behind state_counts and morans_i (src/measures.jl:14-20,91-107) over
columns j_lo:j_hi-1 (0-based) of the current state: 256 value counts, then S, S2, P, Q, W. Summed
over the ranks' owned columns (an MPI Allreduce), they are the whole lattice's.
"""
function slab_sums(st::GB300State{Int8}, j_lo::Integer, j_hi::Integer)
    flush!(st)
    sums = zeros(Int64, 261)
    check(ccall((:gbca_slab_sums, libgbca), Cint, (Ptr{Cvoid}, Int64, Int64, Ptr{Int64}), st.handle, j_lo, j_hi, sums))
    return sums
end

# ------------------------------------------------------------------ batched ensembles

"""
    EnsembleGB300(; tune=true)

An ensemble algorithm that runs every trajectory of an EnsembleProblem built on an Int8
CAProblem (Synchronous, radius <= 8) in one persistent, graph-captured launch of libgbca.so, in
place of solving them one at a time (src/problem.jl:571-589; abc_rejection,
src/calibration.jl:66-91). Each trajectory's problem comes from the ensemble's `prob_func`
(seed_trajectory by default: seed prob.seed + i); `output_func` receives a solution holding the
initial and the final state (save_everystep = false semantics). The context handed to
`prob_func` and `output_func` carries `sim_id` and `sim_seed` (nothing: a `seed` keyword is not
supported).
"""
struct EnsembleGB300 <: SciMLBase.EnsembleAlgorithm
    tune::Bool
end
EnsembleGB300(; tune::Bool=true) = EnsembleGB300(tune)

function SciMLBase.__solve(ens::SciMLBase.AbstractEnsembleProblem, alg::AbstractScheme, ealg::EnsembleGB300;
                           trajectories::Integer, seed=nothing, kwargs...)
    seed === nothing || throw(ArgumentError("EnsembleGB300 takes no `seed` keyword; use prob_func"))
    alg isa Synchronous || throw(UnsupportedCombinationError("EnsembleGB300", string(typeof(alg))))
    start = time()
    ctx(i) = (sim_id=i, sim_seed=nothing)
    probs = [ens.prob_func(ens.prob, ctx(i)) for i in 1:trajectories]
    descs = [gbca_desc(pr, alg) for pr in probs]
    n = length(descs)
    e = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gbca_ensemble_create, libgbca), Cint, (Ptr{GbcaDesc}, Int32, Ref{Ptr{Cvoid}}), descs, n, e))
    try
        for (i, pr) in enumerate(probs)
            u = convert(Array{Int8}, pr.u0)
            check(ccall((:gbca_ensemble_set_state, libgbca), Cint, (Ptr{Cvoid}, Int32, Ptr{Cvoid}, Csize_t),
                        e[], i - 1, u, sizeof(u)))
        end
        t0 = Int64[pr.tspan[1] for pr in probs]
        nsteps = Int64[pr.tspan[2] - pr.tspan[1] for pr in probs]
        ps = Float64[x for pr in probs for x in params_of(pr, pr.p)[1]]
        if ealg.tune
            tile, depth = Ref{Int32}(0), Ref{Int32}(0)
            check(ccall((:gbca_ensemble_tune, libgbca), Cint,
                        (Ptr{Cvoid}, Int64, Ptr{Float64}, Int32, Ref{Int32}, Ref{Int32}), e[], 16, ps, 2, tile, depth))
        end
        check(ccall((:gbca_ensemble_run, libgbca), Cint, (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Int32),
                    e[], t0, nsteps, ps, 2))
        check(ccall((:gbca_ensemble_sync, libgbca), Cint, (Ptr{Cvoid},), e[]))
        us = map(enumerate(probs)) do (i, pr)
            u = Array{Int8}(undef, size(pr.u0))
            check(ccall((:gbca_ensemble_get_state, libgbca), Cint, (Ptr{Cvoid}, Int32, Ptr{Cvoid}, Csize_t),
                        e[], i - 1, u, sizeof(u)))
            sol = CAC.CASolution([copy(pr.u0), u], [pr.tspan[1], pr.tspan[2]], pr, alg, GB300Backend(),
                                 SciMLBase.ReturnCode.Success)
            out, _ = ens.output_func(sol, ctx(i))
            out
        end
        return SciMLBase.EnsembleSolution(us, time() - start, true)
    finally
        ccall((:gbca_ensemble_destroy, libgbca), Cint, (Ptr{Cvoid},), e[])
    end
end

# ------------------------------------------------------------------ serving

"""
    GB300Server(; hbm_budget=8 << 30, chunk_steps=64, big_cells=1 << 20, max_big=8, big_chunk_us=0)

The continuous-batching request loop of libgbca.so: `submit(srv, prob)` queues a simulation
(Int8 rules, Synchronous) and returns its id at once; `poll(srv)` returns finished requests'
state counts and Moran's I. No counterpart in the reference, whose unit of work is one solve.
"""
mutable struct GB300Server
    ptr::Ptr{Cvoid}
end
function GB300Server(; hbm_budget::Integer=8 << 30, chunk_steps::Integer=64, big_cells::Integer=1 << 20,
                     max_big::Integer=8, big_chunk_us::Integer=0)
    cfg = GbcaServerConfig(hbm_budget, chunk_steps, big_cells, max_big, big_chunk_us)
    p = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gbca_server_start, libgbca), Cint, (Ref{GbcaServerConfig}, Ref{Ptr{Cvoid}}), cfg, p))
    srv = GB300Server(p[])
    finalizer(stop!, srv)
    return srv
end

function submit(srv::GB300Server, prob; density::Union{Nothing,Real}=nothing, init_seed::Integer=0)
    d = gbca_desc(prob, Synchronous())
    ps, np = params_of(prob, prob.p)
    pv = Ref(ps)
    id = Ref{UInt64}(0)
    t0, nsteps = Int64(prob.tspan[1]), Int64(prob.tspan[2] - prob.tspan[1])
    if density === nothing
        u = convert(Array{Int8}, prob.u0)
        check(ccall((:gbca_server_submit, libgbca), Cint,
                    (Ptr{Cvoid}, Ref{GbcaDesc}, Ptr{Cvoid}, Csize_t, Float64, UInt64, Int64, Int64, Ptr{Float64},
                     Int32, Ref{UInt64}), srv.ptr, d, u, sizeof(u), 0.0, 0, t0, nsteps, pv, np, id))
    else
        check(ccall((:gbca_server_submit, libgbca), Cint,
                    (Ptr{Cvoid}, Ref{GbcaDesc}, Ptr{Cvoid}, Csize_t, Float64, UInt64, Int64, Int64, Ptr{Float64},
                     Int32, Ref{UInt64}), srv.ptr, d, C_NULL, 0, density, init_seed, t0, nsteps, pv, np, id))
    end
    return id[]
end

function poll(srv::GB300Server; max::Integer=4096)
    out = Vector{GbcaResult}(undef, max)
    n = Ref{Int32}(0)
    check(ccall((:gbca_server_poll, libgbca), Cint, (Ptr{Cvoid}, Ptr{GbcaResult}, Int32, Ref{Int32}),
                srv.ptr, out, max, n))
    return out[1:n[]]
end

function status(srv::GB300Server)
    q, a, c = Ref{Int64}(0), Ref{Int64}(0), Ref{Float64}(0.0)
    check(ccall((:gbca_server_status, libgbca), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}, Ref{Float64}),
                srv.ptr, q, a, c))
    return (queued=q[], active=a[], clock=c[])
end

# seconds each large-request lane and the small stream had work in flight, clock, chunks run
function stats(srv::GB300Server)
    busy = zeros(Float64, 64)
    n, small, wall, chunks = Ref{Int32}(0), Ref{Float64}(0.0), Ref{Float64}(0.0), Ref{Int64}(0)
    check(ccall((:gbca_server_stats, libgbca), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Int32, Ref{Int32}, Ref{Float64}, Ref{Float64}, Ref{Int64}),
                srv.ptr, busy, 64, n, small, wall, chunks))
    return (lane_busy_s=busy[1:min(n[], 64)], small_busy_s=small[], wall_s=wall[], chunks=chunks[])
end

function stop!(srv::GB300Server)
    srv.ptr == C_NULL && return nothing
    ccall((:gbca_server_stop, libgbca), Cint, (Ptr{Cvoid},), srv.ptr)
    srv.ptr = C_NULL
    return nothing
end

# ------------------------------------------------------------------ without allocation

"""
    advance_noalloc!(prob, scheme, state::Ptr{Int8}, pitch, t, nsteps; stream=C_NULL, p=prob.p)

Advance an Int8 state the caller keeps in device memory (a CuArray's pointer, say: n2 columns
of n1 bytes, `pitch` bytes apart, 16-byte aligned) by `nsteps` steps in place, for callers that
cannot allocate device memory when they need a sweep (a pool that owns the device, a real-time
loop). At most 16 MiB of state (pitch * n2); calls must not overlap on one device.
"""
function advance_noalloc!(prob, scheme, state::Ptr{Int8}, pitch::Integer, t::Integer, nsteps::Integer;
                          stream::Ptr{Cvoid}=C_NULL, p=prob.p)
    d = gbca_desc(prob, scheme)
    ps, np = params_of(prob, p)
    pv = Ref(ps)
    return check(ccall((:gbca_advance_noalloc, libgbca), Cint,
                       (Ref{GbcaDesc}, Ptr{Cvoid}, Int64, Int64, Int64, Ptr{Float64}, Int32, Ptr{Cvoid}),
                       d, state, pitch, t, nsteps, pv, np, stream))
end

# ------------------------------------------------------------------ diagnostics

kernel_launches() = ccall((:gbca_kernel_launches, libgbca), Int64, ())
library_version() = ccall((:gbca_version, libgbca), Int32, ())
device_count() = ccall((:gbca_device_count, libgbca), Int32, ())
threshold(p::Real, f32::Bool=false) = ccall((:gbca_threshold, libgbca), UInt64, (Float64, Int32), p, f32)

end # module
