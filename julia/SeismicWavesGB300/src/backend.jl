# The wavesim side of the GB300 backend.
#
# build_wavesim constructs the reference's own wavesim structs; their array
# type parameter A is `backend.Data.Array{T, N}` (acou_models.jl:112,
# ela_models.jl).  Returning `GB300Backend` from select_backend for
# `parall = :GB300` therefore gives those wavesims a type of their own,
# `AcousticCDCPMLWaveSimulation{T, N, GB300Array{T, N}, GB300Array{T, 1}}`, and
# the run_swforward! / run_swgradient! methods of this package, which dispatch
# on it, are more specific than the core's loops (src/apis/forward.jl:71,
# src/apis/gradient.jl:93): no change to SeismicWaves itself.  The arrays stay
# host memory; the GPU state lives in the library, one handle per wavesim.

"""
    GB300Array{T, N}

Host array used for the bookkeeping fields of a wavesim built with
`parall = :GB300` (model parameters, C-PML coefficients, checkpointer
copies).  Its only role beyond `Array` is to mark the wavesim type.
"""
struct GB300Array{T, N} <: DenseArray{T, N}
    data::Array{T, N}
end
GB300Array{T, N}(a::AbstractArray) where {T, N} = GB300Array{T, N}(convert(Array{T, N}, a))
GB300Array{T, N}(::UndefInitializer, dims::Dims{N}) where {T, N} = GB300Array{T, N}(Array{T, N}(undef, dims))
GB300Array(a::AbstractArray{T, N}) where {T, N} = GB300Array{T, N}(Array{T, N}(a))

Base.size(x::GB300Array) = size(x.data)
Base.IndexStyle(::Type{<:GB300Array}) = IndexLinear()
Base.@propagate_inbounds Base.getindex(x::GB300Array, i::Int) = x.data[i]
Base.@propagate_inbounds Base.setindex!(x::GB300Array, v, i::Int) = (x.data[i] = v; x)
Base.similar(x::GB300Array, ::Type{S}, dims::Dims) where {S} = GB300Array(similar(x.data, S, dims))
Base.copy(x::GB300Array) = GB300Array(copy(x.data))
Base.unsafe_convert(::Type{Ptr{T}}, x::GB300Array{T}) where {T} = Base.unsafe_convert(Ptr{T}, x.data)
Base.strides(x::GB300Array) = strides(x.data)
Base.elsize(::Type{GB300Array{T, N}}) where {T, N} = sizeof(T)
Base.convert(::Type{Array{T, N}}, x::GB300Array{T, N}) where {T, N} = x.data
Base.Array(x::GB300Array) = copy(x.data)

"""
The backend module select_backend returns for `parall = :GB300`: the array
constructors a wavesim needs (`Data.Array`, `zeros`, `ones`).  The per-step
functions of the reference's backends (`forward_onestep_CPML!`, ...) are not
provided: every time step of every shot runs inside one library call.
"""
module GB300Backend
using ..SeismicWavesGB300: GB300Array
module Data
using ...SeismicWavesGB300: GB300Array
const Array = GB300Array
end
zeros(::Type{T}, dims::Integer...) where {T} = GB300Array(Base.zeros(T, dims...))
ones(::Type{T}, dims::Integer...) where {T} = GB300Array(Base.ones(T, dims...))
end

const FT = Union{Float32, Float64}
SeismicWaves.select_backend(::CPMLBoundaryCondition, ::LocalGrid,
                            ::Type{<:AcousticCDCPMLWaveSimulation{<:FT, 2}}, ::Type{Val{:GB300}}) = GB300Backend
SeismicWaves.select_backend(::CPMLBoundaryCondition, ::LocalGrid,
                            ::Type{<:AcousticCDCPMLWaveSimulation{<:FT, 3}}, ::Type{Val{:GB300}}) = GB300Backend
SeismicWaves.select_backend(::CPMLBoundaryCondition, ::LocalGrid,
                            ::Type{<:AcousticVDStaggeredCPMLWaveSimulation{<:FT, 2}}, ::Type{Val{:GB300}}) = GB300Backend
SeismicWaves.select_backend(::CPMLBoundaryCondition, ::LocalGrid,
                            ::Type{<:ElasticIsoCPMLWaveSimulation{<:FT, 2}}, ::Type{Val{:GB300}}) = GB300Backend

const GB300CD{T, N} = AcousticCDCPMLWaveSimulation{T, N, GB300Array{T, N}, GB300Array{T, 1}}
const GB300VD{T} = AcousticVDStaggeredCPMLWaveSimulation{T, 2, GB300Array{T, 2}, GB300Array{T, 1}}
const GB300Elastic{T} = ElasticIsoCPMLWaveSimulation{T, 2, GB300Array{T, 2}, GB300Array{T, 1}}
const GB300Sim = Union{GB300CD, GB300VD, GB300Elastic}

# ---------------------------------------------------------------------------
# One library context and one library simulation per wavesim, created at the
# first call and reused by every later one (the device fields and graphs stay
# allocated, like the reference's preallocated wavesim).  The handle is keyed
# by the wavesim's field dictionary (mutable and unique to the wavesim) in a
# WeakKeyDict: when the wavesim is collected, the handle becomes unreachable
# and its finalizer releases the device memory.
# ---------------------------------------------------------------------------
mutable struct GB300Handle
    ctx::Ptr{Cvoid}
    sim::Ptr{Cvoid}
    destroy::Symbol          # sw_wavesim_destroy, sw_acoustic_vd_destroy or sw_elastic_destroy
    function GB300Handle(ctx, sim, destroy)
        h = new(ctx, sim, destroy)
        finalizer(release!, h)
        return h
    end
end

function release!(h::GB300Handle)
    if h.sim != C_NULL
        if h.destroy === :sw_elastic_destroy
            ccall((:sw_elastic_destroy, libsw[]), Cint, (Ptr{Cvoid},), h.sim)
        elseif h.destroy === :sw_acoustic_vd_destroy
            ccall((:sw_acoustic_vd_destroy, libsw[]), Cint, (Ptr{Cvoid},), h.sim)
        else
            ccall((:sw_wavesim_destroy, libsw[]), Cint, (Ptr{Cvoid},), h.sim)
        end
        h.sim = C_NULL
    end
    if h.ctx != C_NULL
        ccall((:sw_ctx_destroy, libsw[]), Cint, (Ptr{Cvoid},), h.ctx)
        h.ctx = C_NULL
    end
    return nothing
end

const HANDLES = WeakKeyDict{Any, GB300Handle}()
const HANDLES_LOCK = ReentrantLock()
const DEVICE = Ref{Int32}(0)

"""
    set_device!(ordinal)

CUDA device of the simulations created from now on (default 0).
"""
set_device!(d::Integer) = (DEVICE[] = Int32(d); nothing)

"""
    release!(wavesim)

Frees the wavesim's device memory now instead of at garbage collection.
"""
function release!(wavesim::GB300Sim)
    lock(HANDLES_LOCK) do
        h = pop!(HANDLES, wavesim.grid.fields, nothing)
        h === nothing || release!(h)
    end
    return nothing
end

function new_context()
    ctx = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:sw_ctx_create, libsw[]), Cint, (Cint, Ptr{Cvoid}, Ref{Ptr{Cvoid}}), DEVICE[], C_NULL, ctx),
          C_NULL, "sw_ctx_create")
    return ctx[]
end

isgradsim(model) = model.checkpointer !== nothing

function grad_params(model)
    gp = model.gradparams
    if gp === nothing
        return SwGradParams(1, 0, 0, 0, 0)
    end
    return SwGradParams(gp.check_freq, gp.mute_radius_src, gp.mute_radius_rec, gp.compute_misfit, 0)
end

function handle(create::Function, model)
    lock(HANDLES_LOCK) do
        get!(HANDLES, model.grid.fields) do
            ctx = new_context()
            try
                return create(ctx)
            catch
                ccall((:sw_ctx_destroy, libsw[]), Cint, (Ptr{Cvoid},), ctx)
                rethrow()
            end
        end
    end
end

# cpml coefficients of the current shot (after init_shot! -> init_bdc!), packed
# [a, a_h, b, b_h] per axis as the library expects
cpml_block(model) = Float32.(vcat([vcat(c.a.data, c.a_h.data, c.b.data, c.b_h.data) for c in model.cpmlcoeffs]...))
