# The C structs of include/swgb300.h, field for field (names, order and types),
# and the library handle.  Julia lays these immutable structs out like C, so a
# Vector of them is the array the batched entry points take.

const libsw = Ref{String}(get(ENV, "SWGB300_LIB", "libswgb300.so"))

"""
    set_library!(path)

Path of `libswgb300.so` (default: the `SWGB300_LIB` environment variable, else
the dynamic loader's search path).
"""
set_library!(path::AbstractString) = (libsw[] = String(path); nothing)

const SW_OK = Int32(0)
const SW_STATUS = Dict(1 => "SW_ERR_ARG", 2 => "SW_ERR_OOM", 3 => "SW_ERR_CUDA", 4 => "SW_ERR_TIMEOUT",
                       5 => "SW_ERR_STATE", 6 => "SW_ERR_UNSUPPORTED", 7 => "SW_ERR_CAPACITY")

# InputParametersAcoustic + CPMLBoundaryConditionParameters (sw_acoustic_params)
struct SwAcousticParams
    ndim::Int32
    n::NTuple{3, Int32}
    h::NTuple{3, Float64}
    dt::Float64
    halo::Int32
    rcoef::Float64
    freetop::Int32
end

# one ScalarShot as possrcrec_scaletf hands it to a backend (sw_acoustic_shot)
struct SwAcousticShot
    nt::Int32
    nsrc::Int32
    src_idx::Ptr{Int32}      # (nsrc, ndim) 1-based grid indices
    srctf::Ptr{Float32}      # (nt, nsrc) scaled source time functions
    nrec::Int32
    rec_idx::Ptr{Int32}      # (nrec, ndim)
    traces::Ptr{Float32}     # (nt, nrec) output
    cpml::Ptr{Float32}       # ndim blocks [a, a_h, b, b_h]
    observed::Ptr{Float32}   # gradient: (nt, nrec)
    invcov_diag::Ptr{Float32}
    nwin::Int32
    windows::Ptr{Int32}      # (2, nwin)
    src_pos::Ptr{Float64}    # muting
    rec_pos::Ptr{Float64}
    invcov::Ptr{Float32}     # dense (nt, nt) C^-1 or C_NULL (takes precedence over invcov_diag)
    misfit_kind::Int32       # 0 L2Misfit, 1 CCTSMisfit
    misfit_dt::Float64       # CCTSMisfit.dt
    cpml64::Ptr{Float64}     # C_NULL or the cpml coefficients in Float64 (compensated forward)
end

# GradParameters (sw_grad_params)
struct SwGradParams
    check_freq::Int32
    mute_radius_src::Int32
    mute_radius_rec::Int32
    compute_misfit::Int32
    snapshot_bf16::Int32
end

# InputParametersElastic (sw_elastic_params)
struct SwElasticParams
    n::NTuple{2, Int32}
    h::NTuple{2, Float64}
    dt::Float64
    halo::Int32
    rcoef::Float64
    freetop::Int32
    interp_rho::Int32        # 0 arithmetic, 1 harmonic
    interp_mu::Int32
end

# grid points of one source/receiver table in CSR form (sw_point_table)
struct SwPointTable
    offsets::Ptr{Int32}
    ij::Ptr{Int32}
    coef::Ptr{Float32}
end

# one MomentTensorShot / ExternalForceShot (sw_elastic_shot)
struct SwElasticShot
    nt::Int32
    kind::Int32              # 0 moment tensor, 1 external force
    nsrc::Int32
    srctf::Ptr{Float32}
    momtens::Ptr{Float32}    # (3, nsrc): Mxx, Mzz, Mxz
    src::NTuple{2, SwPointTable}
    nrec::Int32
    rec::NTuple{2, SwPointTable}
    traces::Ptr{Float32}     # (nt, 2, nrec)
    cpml::Ptr{Float32}
    observed::Ptr{Float32}
    invcov_diag::Ptr{Float32}
    nwin::Int32
    windows::Ptr{Int32}
    src_pos::Ptr{Float64}
    rec_pos::Ptr{Float64}
    invcov::Ptr{Float32}
    misfit_kind::Int32       # 0 L2Misfit, 1 CCTSMisfit (per component trace)
    misfit_dt::Float64       # CCTSMisfit.dt
end

last_error(ctx::Ptr{Cvoid}) =
    ctx == C_NULL ? "" : unsafe_string(ccall((:sw_ctx_last_error, libsw[]), Cstring, (Ptr{Cvoid},), ctx))

function check(rc::Integer, ctx::Ptr{Cvoid}, what::AbstractString)
    rc == SW_OK && return nothing
    error("swgb300 ", what, ": ", get(SW_STATUS, Int(rc), string(rc)), ": ", last_error(ctx))
end

optptr(x) = x === nothing ? C_NULL : pointer(x)
