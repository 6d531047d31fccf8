# run_swforward! / run_swgradient! for the acoustic wavesims built with
# parall = :GB300 (constant density 2D/3D, variable density 2D).  Host logic
# stays the reference's: check_sim_consistency, set_wavesim_matprop!,
# init_shot! (checks + init_bdc!), possrcrec_scaletf; then one library call
# runs every time step of every shot.

function cd_params(model::GB300CD{T, N}) where {T, N}
    n = ntuple(d -> Int32(d <= N ? model.grid.size[d] : 1), 3)
    h = ntuple(d -> Float64(d <= N ? model.grid.spacing[d] : 1), 3)
    cp = model.cpmlparams
    return SwAcousticParams(Int32(N), n, h, Float64(model.dt), Int32(cp.halo), Float64(cp.rcoef), Int32(cp.freeboundtop))
end

function cd_handle(model::GB300CD)
    handle(model) do ctx
        p = cd_params(model)
        g = grad_params(model)
        ws = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:sw_wavesim_create, libsw[]), Cint,
                    (Ptr{Cvoid}, Ref{SwAcousticParams}, Int32, Ref{SwGradParams}, Ref{Ptr{Cvoid}}),
                    ctx, p, Int32(isgradsim(model)), g, ws), ctx, "sw_wavesim_create")
        GB300Handle(ctx, ws[], :sw_wavesim_destroy)
    end
end

function vd_handle(model::GB300VD)
    handle(model) do ctx
        nx, nz = model.grid.size
        hx, hz = model.grid.spacing
        cp = model.cpmlparams
        p = SwAcousticParams(Int32(2), (Int32(nx), Int32(nz), Int32(1)), (Float64(hx), Float64(hz), 1.0),
                             Float64(model.dt), Int32(cp.halo), Float64(cp.rcoef), Int32(cp.freeboundtop))
        g = grad_params(model)
        interp = model.matprop.interp_method isa SeismicWaves.HarmonicAverageInterpolation ? Int32(1) : Int32(0)
        vd = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:sw_acoustic_vd_create, libsw[]), Cint,
                    (Ptr{Cvoid}, Ref{SwAcousticParams}, Int32, Int32, Ref{SwGradParams}, Ref{Ptr{Cvoid}}),
                    ctx, p, interp, Int32(isgradsim(model)), g, vd), ctx, "sw_acoustic_vd_create")
        GB300Handle(ctx, vd[], :sw_acoustic_vd_destroy)
    end
end

function set_material!(h::GB300Handle, model::GB300CD)
    vp = Float32.(model.matprop.vp)
    check(ccall((:sw_wavesim_set_vp, libsw[]), Cint, (Ptr{Cvoid}, Ptr{Float32}, Int32), h.sim, vp, 0),
          h.ctx, "sw_wavesim_set_vp")
end

function set_material!(h::GB300Handle, model::GB300VD)
    vp = Float32.(model.matprop.vp)
    rho = Float32.(model.matprop.rho)
    check(ccall((:sw_acoustic_vd_set_material, libsw[]), Cint, (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}),
                h.sim, vp, rho), h.ctx, "sw_acoustic_vd_set_material")
end

# The misfit fields of one shot: (invcov_diag, dense invcov, windows (2, nwin), kind, dt).
function misfit_fields(m::SeismicWaves.L2Misfit)
    ic = m.invcov
    d, dense = isdiag(ic) ? (Float32.(diag(ic)), nothing) : (nothing, Float32.(Matrix(ic)))
    win = isempty(m.windows) ? Int32[] : Int32.(vcat([[w.first, w.second] for w in m.windows]...))
    return d, dense, win, Int32(0), 0.0
end
misfit_fields(m::SeismicWaves.CCTSMisfit) = (nothing, nothing, Int32[], Int32(1), Float64(m.dt))

# Everything a shot struct points to, kept alive across the call (GC.@preserve).
struct ScalarShotBuffers
    si::Matrix{Int32}
    ri::Matrix{Int32}
    tf::Matrix{Float32}
    tr::Matrix{Float32}
    cp::Vector{Float32}
    obs::Union{Nothing, Matrix{Float32}}
    icd::Union{Nothing, Vector{Float32}}
    icf::Union{Nothing, Matrix{Float32}}
    win::Vector{Int32}
    sp::Matrix{Float64}
    rp::Matrix{Float64}
    kind::Int32
    mdt::Float64
end

function scalar_shot_buffers(model, shot, misfit)
    init_shot!(model, shot)                      # checks + init_bdc! for this shot's f0
    possrcs, posrecs, scal = possrcrec_scaletf(model, shot)
    tr = zeros(Float32, size(shot.recs.seismograms))
    obs, icd, icf, win, kind, mdt = nothing, nothing, nothing, Int32[], Int32(0), 0.0
    if misfit !== nothing
        icd, icf, win, kind, mdt = misfit_fields(misfit)
        obs = misfit isa SeismicWaves.L2Misfit ? Float32.(misfit.observed) : Float32.(misfit.observed)
    end
    return ScalarShotBuffers(Int32.(possrcs), Int32.(posrecs), Float32.(scal), tr, cpml_block(model), obs, icd, icf,
                             win, Float64.(shot.srcs.positions), Float64.(shot.recs.positions), kind, mdt)
end

sw_struct(b::ScalarShotBuffers) =
    SwAcousticShot(Int32(size(b.tr, 1)), Int32(size(b.si, 1)), pointer(b.si), pointer(b.tf), Int32(size(b.ri, 1)),
                   pointer(b.ri), pointer(b.tr), pointer(b.cp), optptr(b.obs), optptr(b.icd),
                   Int32(length(b.win) ÷ 2), isempty(b.win) ? Ptr{Int32}(C_NULL) : pointer(b.win),
                   pointer(b.sp), pointer(b.rp), optptr(b.icf), b.kind, b.mdt, Ptr{Float64}(C_NULL))

const GB300Acoustic = Union{GB300CD, GB300VD}

forward_symbol(::GB300CD) = :sw_acoustic_forward
forward_symbol(::GB300VD) = :sw_acoustic_vd_forward
acoustic_handle(model::GB300CD) = cd_handle(model)
acoustic_handle(model::GB300VD) = vd_handle(model)

# the fields savesnapshot! receives per snapshot step: CD "pcur"; VD "pcur" and "vcur"
function save_snapshots!(model::GB300CD{T, N}, buf::Vector{Float32}, nt::Int) where {T, N}
    n = prod(model.grid.size)
    k = 0
    for it in 1:nt
        it % model.snapshotter.snapevery == 0 || continue
        f = reshape(T.(buf[(k * n + 1):((k + 1) * n)]), model.grid.size)
        SeismicWaves.savesnapshot!(model.snapshotter, "pcur" => SeismicWaves.ScalarVariableField(f), it)
        k += 1
    end
end

function save_snapshots!(model::GB300VD{T}, buf::Vector{Float32}, nt::Int) where {T}
    nx, nz = model.grid.size
    sizes = ((nx, nz), (nx - 1, nz), (nx, nz - 1))
    B = sum(prod, sizes)
    k = 0
    for it in 1:nt
        it % model.snapshotter.snapevery == 0 || continue
        o = k * B
        parts = Array{T, 2}[]
        for s in sizes
            push!(parts, reshape(T.(buf[(o + 1):(o + prod(s))]), s))
            o += prod(s)
        end
        SeismicWaves.savesnapshot!(model.snapshotter, "pcur" => SeismicWaves.ScalarVariableField(parts[1]), it)
        SeismicWaves.savesnapshot!(model.snapshotter, "vcur" => SeismicWaves.MultiVariableField(parts[2:3]), it)
        k += 1
    end
end
snapshot_block(model::GB300CD) = prod(model.grid.size)
snapshot_block(model::GB300VD) = (n = model.grid.size; n[1] * n[2] + (n[1] - 1) * n[2] + n[1] * (n[2] - 1))

function SeismicWaves.run_swforward!(model::GB300Acoustic, matprop::SeismicWaves.MaterialProperties{T, N},
                                     shots::Vector{<:SeismicWaves.Shot{T}}) where {T, N}
    check_sim_consistency(model, matprop, shots)
    set_wavesim_matprop!(model, matprop)        # the reference's checks; also keeps model.matprop current
    h = acoustic_handle(model)
    set_material!(h, model)
    bufs = [scalar_shot_buffers(model, shot, nothing) for shot in shots]
    structs = [sw_struct(b) for b in bufs]
    if snapenabled(model)
        every = model.snapshotter.snapevery
        snaps = [zeros(Float32, snapshot_block(model) * (size(b.tr, 1) ÷ every)) for b in bufs]
        ptrs = [pointer(s) for s in snaps]
        sym = model isa GB300CD ? :sw_acoustic_forward_snapshots : :sw_acoustic_vd_forward_snapshots
        GC.@preserve bufs snaps ptrs structs begin
            rc = if sym === :sw_acoustic_forward_snapshots
                ccall((:sw_acoustic_forward_snapshots, libsw[]), Cint,
                      (Ptr{Cvoid}, Int32, Ptr{SwAcousticShot}, Int32, Int32, Ptr{Ptr{Float32}}),
                      h.sim, length(structs), structs, 0, every, ptrs)
            else
                ccall((:sw_acoustic_vd_forward_snapshots, libsw[]), Cint,
                      (Ptr{Cvoid}, Int32, Ptr{SwAcousticShot}, Int32, Int32, Ptr{Ptr{Float32}}),
                      h.sim, length(structs), structs, 0, every, ptrs)
            end
            check(rc, h.ctx, String(sym))
        end
        out = []
        for (shot, b, s) in zip(shots, bufs, snaps)
            shot.recs.seismograms .= b.tr
            save_snapshots!(model, s, size(b.tr, 1))
            push!(out, deepcopy(model.snapshotter.snapshots))
        end
        return out
    end
    GC.@preserve bufs structs begin
        rc = if model isa GB300CD
            ccall((:sw_acoustic_forward, libsw[]), Cint, (Ptr{Cvoid}, Int32, Ptr{SwAcousticShot}, Int32),
                  h.sim, length(structs), structs, 0)
        else
            ccall((:sw_acoustic_vd_forward, libsw[]), Cint, (Ptr{Cvoid}, Int32, Ptr{SwAcousticShot}, Int32),
                  h.sim, length(structs), structs, 0)
        end
        check(rc, h.ctx, String(forward_symbol(model)))
    end
    for (shot, b) in zip(shots, bufs)
        shot.recs.seismograms .= b.tr
    end
    return nothing
end

function SeismicWaves.run_swgradient!(model::GB300Acoustic, matprop::SeismicWaves.MaterialProperties{T, N},
                                      shots::Vector{<:SeismicWaves.Shot{T}},
                                      misfit::Vector{<:SeismicWaves.AbstractMisfit{T}}) where {T, N}
    @assert model.checkpointer !== nothing "The wavesim object was not built for gradient computations. (Was `gradient=true` specified?)"
    check_sim_consistency(model, matprop, shots)
    set_wavesim_matprop!(model, matprop)
    h = acoustic_handle(model)
    set_material!(h, model)
    bufs = [scalar_shot_buffers(model, shot, m) for (shot, m) in zip(shots, misfit)]
    structs = [sw_struct(b) for b in bufs]
    msf = Ref(0.0)
    if model isa GB300CD
        grad = zeros(Float64, model.grid.size)
        GC.@preserve bufs structs check(ccall((:sw_acoustic_gradient, libsw[]), Cint,
                                              (Ptr{Cvoid}, Int32, Ptr{SwAcousticShot}, Int32, Ptr{Float64},
                                               Ref{Float64}),
                                              h.sim, length(structs), structs, 0, grad, msf), h.ctx,
                                        "sw_acoustic_gradient")
        g = Dict("vp" => T.(grad))
    else
        gvp = zeros(Float64, model.grid.size)
        grho = zeros(Float64, model.grid.size)
        GC.@preserve bufs structs check(ccall((:sw_acoustic_vd_gradient, libsw[]), Cint,
                                              (Ptr{Cvoid}, Int32, Ptr{SwAcousticShot}, Int32, Ptr{Float64},
                                               Ptr{Float64}, Ref{Float64}),
                                              h.sim, length(structs), structs, 0, gvp, grho, msf), h.ctx,
                                        "sw_acoustic_vd_gradient")
        g = Dict("vp" => T.(gvp), "rho" => T.(grho))
    end
    for (shot, b) in zip(shots, bufs)
        shot.recs.seismograms .= b.tr
    end
    return model.gradparams.compute_misfit ? (g, T(msf[])) : g
end
